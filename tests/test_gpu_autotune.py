"""Autotuner (sop_autotune_ex).  Its trials are real steps of one run window:
tuning must leave every trajectory bit-identical to a plain sop_run of the
same step count, and skin / cell-edge tuning must keep the pair list feeding
each step equal to the reference's (3.2x / nnlup) pair sets.  Forces are
exact fixed-point sums of their contributions, so the tolerance is bit
identity throughout."""
import re

import numpy as np
import pytest

from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
SIZES = [40, 90, 150, 300, 600, 1100, 1700, 2600, 5000]


def script():
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", "neighborlist"),
            ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


def engine():
    return Engine(0, max_beads=1 << 16, max_replicas=32, max_list_entries=1 << 24)


def steps_of(report):
    m = re.search(r"(\d+) trials, (\d+) steps", report)
    assert m, report
    return int(m.group(2))


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def test_shape_tuning_equals_plain_run():
    systems = [S.synth_chain(8200 + k, n) for k, n in enumerate(SIZES)]
    params = [make_params(script(), seed=4100 + k, list_mode="skin", skin=2.0)
              for k in range(len(systems))]
    with engine() as a:
        ids = [a.add(s, p) for s, p in zip(systems, params)]
        report = a.autotune(steps_per_trial=6, shape=True, lists=False)
        total = steps_of(report)
        want = [(a.state(r), a.energy(r), a.status(r)) for r in ids]
    assert "chosen threads=" in report and "shape threads=" in report
    with engine() as b:
        ids = [b.add(s, p) for s, p in zip(systems, params)]
        b.run(total)
        for k, r in enumerate(ids):
            (_, xa, va), ea, sa = want[k]
            _, xb, vb = b.state(r)
            np.testing.assert_array_equal(xb, xa)
            np.testing.assert_array_equal(vb, va)
            np.testing.assert_array_equal(b.energy(r), ea)
            assert b.status(r) == sa and sa[0] == 0


def test_list_tuning_keeps_reference_pair_sets():
    system = S.synth_chain(8300, 700)
    with engine() as e:
        a = e.add(system, make_params(script(), force_terms=DET))  # reference cadence, untouched
        b = e.add(system, make_params(script(), force_terms=DET, list_mode="skin", skin=2.0))
        report = e.autotune(steps_per_trial=10, shape=False, lists=True)
        assert "chosen bucket n=[256,1024)" in report
        for _ in range(2):
            for k in (2, 3):
                np.testing.assert_array_equal(pairset(*e.pairs(a, k)), pairset(*e.pairs(b, k)))
            np.testing.assert_array_equal(e.state(a)[1], e.state(b)[1])
            assert e.status(a)[0] == 0 and e.status(b)[0] == 0
            e.run(150)  # and the tuned list keeps tracking after the tuner


@pytest.mark.parametrize("cfg", [dict(step_strategy=1), dict(step_strategy=1, step_min_blocks=2),
                                 dict(step_min_blocks=3, stage_limit=2048), dict(step_min_blocks=2),
                                 dict(stage_limit=-1), dict(build_slice_beads=128, chunk_beads=64),
                                 dict(item_cost_beads=-1), dict(item_cost_beads=16, chunk_beads=64),
                                 dict(queue_blocks=-1), dict(queue_blocks=8, chunk_beads=32),
                                 dict(queue_blocks=1, lanes_per_bead=1, block_threads=512),
                                 dict(queue_blocks=2, stage_limit=-1),
                                 dict(lanes_per_bead=4), dict(lanes_per_bead=1), dict(block_threads=64),
                                 dict(block_threads=128, lanes_per_bead=4, chunk_beads=512),
                                 dict(group_rebuild_pct=-1), dict(group_rebuild_pct=90),
                                 dict(block_threads=512), dict(block_threads=512, step_min_blocks=3,
                                                               chunk_beads=256),
                                 dict(block_threads=512, lanes_per_bead=4, stage_limit=-1)])
def test_launch_shapes_bit_identical(cfg):
    """Every launch shape, both step strategies (CTA items staged in shared
    memory, warp tasks through L1/L2), fixed or queued CTA blocks, every lane
    count and rebuild grouping give the same trajectories: each force is an exact integer sum of its
    pair contributions, whatever the list order or the build times."""
    systems = [S.synth_chain(8400 + k, n) for k, n in enumerate([60, 700, 2600, 5000, 130])]
    params = [make_params(script(), seed=4400 + k, list_mode="skin" if k % 2 else "neighborlist",
                          skin=2.0) for k in range(len(systems))]
    out = []
    for c in ({}, cfg):
        with Engine(0, max_beads=1 << 15, max_replicas=16, max_list_entries=1 << 23, **c) as e:
            ids = [e.add(s, p) for s, p in zip(systems, params)]
            e.run(250)
            out.append([e.state(r)[1] for r in ids])
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("edge", [6.0, 8.0, 10.0, 12.0, 16.0])
def test_cell_edges_keep_pair_sets_and_trajectories(edge):
    """Absolute cell edges of the list build's grid (list cutoff 2.5 sigma +
    2 A = 11.5 A: 6-10 A cells with the 5x5x5 stencil, 12 and 16 A with the
    3x3x3 one): the same pair sets and trajectory as the reference cadence."""
    systems = [S.synth_chain(8500 + k, n) for k, n in enumerate([90, 700, 2600])]
    with engine() as e:
        ref = [e.add(s, make_params(script(), force_terms=DET)) for s in systems]
        skin = [e.add(s, make_params(script(), force_terms=DET, list_mode="skin", skin=2.0,
                                     cell_edge=edge)) for s in systems]
        for _ in range(2):
            e.run(200)
            for a, b in zip(ref, skin):
                for k in (2, 3):
                    np.testing.assert_array_equal(pairset(*e.pairs(a, k)), pairset(*e.pairs(b, k)))
                np.testing.assert_array_equal(e.state(a)[1], e.state(b)[1])
                assert e.status(b)[0] == 0


def test_block_size_outside_the_supported_shapes_is_refused():
    with pytest.raises(Exception):
        Engine(0, max_beads=1 << 12, max_replicas=4, max_list_entries=1 << 20, block_threads=512,
               step_strategy=1)
    with pytest.raises(Exception):
        Engine(0, max_beads=1 << 12, max_replicas=4, max_list_entries=1 << 20, block_threads=576)
