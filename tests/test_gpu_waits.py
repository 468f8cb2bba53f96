"""The engine's two bounded device-side waits, run to their limits on purpose.

Neither wait is expected to run out in normal operation: a CTA of the
preparation kernel waits for a work unit another CTA is still publishing,
and a step-kernel CTA waits for its bulk copy of positions into shared
memory.  Each has a limit (sop_engine_config.queue_wait_ns / stage_wait_ns).
Here the host makes them run out without any fault: it asks the producers to
stall before publishing (longer than the queue limit), or the step kernel to
expect its copies without issuing them.  The call must return
SOP_ERR_TIMEOUT in bounded time, name the wait (sop_engine_wait_errors), and
leave the engine usable: once the stall is lifted, a re-added replica runs
bit-identically to one on a fresh engine, under the same short limits.
"""
import time

import numpy as np
import pytest

from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

QUEUE_NS, STAGE_NS = 2_000_000, 1_000_000  # 2 ms, 1 ms


def script():
    # the reference cadence at nnlup 1: a list build (units to publish) every step
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", "neighborlist"),
            ("set", "nnlup", "1"), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


def engine():
    return Engine(0, max_beads=1 << 14, max_replicas=8, max_list_entries=1 << 21,
                  queue_wait_ns=QUEUE_NS, stage_wait_ns=STAGE_NS)


@pytest.fixture(scope="module")
def system():
    return S.synth_chain(9700, 900)  # staged in shared memory (<= 1664 beads)


@pytest.fixture(scope="module")
def reference(system):
    with Engine(0, max_beads=1 << 14, max_replicas=8, max_list_entries=1 << 21) as e:
        r = e.add(system, make_params(script(), seed=97))
        e.run(60)
        return e.state(r)[1]


def recovered(e, system, bad):
    """Lift the stall, replace the replica the failed call touched, run."""
    e.inject_stall(0, False)
    e.remove(bad)
    r = e.add(system, make_params(script(), seed=97))
    e.run(60)
    assert e.status(r)[0] == 0
    return e.state(r)[1]


def test_queue_wait_runs_out_and_the_engine_recovers(system, reference):
    with engine() as e:
        r = e.add(system, make_params(script(), seed=97))
        e.run(5)  # the short limits do not trip in normal operation
        e.inject_stall(publish_delay_ns=50_000_000)  # 50 ms > the 2 ms limit
        t0 = time.time()
        with pytest.raises(L.SopError) as err:
            e.run(3)
        assert time.time() - t0 < 30
        assert err.value.code == L.ERR_TIMEOUT
        assert e.wait_errors() & 2
        np.testing.assert_array_equal(recovered(e, system, r), reference)


def test_stage_wait_runs_out_and_the_engine_recovers(system, reference):
    with engine() as e:
        r = e.add(system, make_params(script(), seed=97))
        e.run(5)
        e.inject_stall(skip_stage_copy=True)  # the copy's barrier phase never completes
        t0 = time.time()
        with pytest.raises(L.SopError) as err:
            e.run(2)
        assert time.time() - t0 < 30
        assert err.value.code == L.ERR_TIMEOUT
        assert e.wait_errors() & 1
        np.testing.assert_array_equal(recovered(e, system, r), reference)


def test_inject_stall_rejects_unbounded_delays():
    with engine() as e:
        with pytest.raises(L.SopError):
            e.inject_stall(publish_delay_ns=2_000_000_000)
        with pytest.raises(L.SopError):
            e.inject_stall(publish_delay_ns=-1)
