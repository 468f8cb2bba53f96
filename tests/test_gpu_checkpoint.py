"""Per-replica checkpoint / restore: a snapshot taken between runs and
restored into the same system on another engine (other launch shape, other
replicas beside it) continues bit for bit: positions, velocities, energies,
observables and pair lists equal the uninterrupted run's."""
import numpy as np
import pytest

from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu


def script(mode):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.7"),
            ("set", "nstep", "1000"), ("set", "nup", "50"), ("set", "cutofftype", mode),
            ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


@pytest.mark.parametrize("mode,kw", [("neighborlist", {}), ("celllist", {}),
                                     ("neighborlist", dict(list_mode="skin", skin=1.5))])
def test_checkpoint_restore_continues_exactly(mode, kw):
    system = S.synth_chain(8800, 900)
    params = make_params(script(mode), seed=8801, **kw)
    with Engine(0, max_beads=1 << 14, max_replicas=8, max_list_entries=1 << 22) as a:
        r = a.add(system, params)
        a.run(230)  # an output step (nup 50) inside, and cadence mid-way
        snap = a.checkpoint(r)
        a.run(170)
        want = (a.state(r), a.energy(r), a.observables(r), [a.pairs(r, k) for k in range(4)])
    with Engine(0, max_beads=1 << 15, max_replicas=8, max_list_entries=1 << 23,
                lanes_per_bead=4, chunk_beads=64) as b:
        other = b.add(S.synth_chain(8900, 300), make_params(script(mode), seed=1))
        r = b.add(system, params)
        b.restore(r, snap)
        b.run(170)
        (_, xa, va), ea, oa, pa = want
        _, xb, vb = b.state(r)
        np.testing.assert_array_equal(xb, xa)
        np.testing.assert_array_equal(vb, va)
        np.testing.assert_array_equal(b.energy(r), ea)
        np.testing.assert_array_equal(b.observables(r), oa)
        for k in range(4):
            np.testing.assert_array_equal(pairset(*b.pairs(r, k)), pairset(*pa[k]))
        assert b.status(other)[0] == 0


def test_restore_rejects_another_system():
    with Engine(0, max_beads=1 << 14, max_replicas=4, max_list_entries=1 << 21) as e:
        a = e.add(S.synth_chain(8810, 200), make_params(script("neighborlist")))
        b = e.add(S.synth_chain(8811, 300), make_params(script("neighborlist")))
        snap = e.checkpoint(a)
        with pytest.raises(Exception):
            e.restore(b, snap)
        with pytest.raises(Exception):
            e.restore(a, snap[:-4])
