"""Large single systems: multi-chain globules of 10,000 and 50,000 beads, whose
lists are built from global-memory cell bins (one binning CTA, list slices on
every SM).  Oracle: the restatement over the pruned candidate set (pairs
within the list cutoff plus margin at the start positions, plus all natives),
which the CPU suite pins bit for bit to the full implicit set.

Tolerances as the other parity tests: pair lists bit-exact as integer sets;
forces and energies within 1e-5 relative; noise-off trajectories within
1e-4 A RMSD; skin lists give the reference's pair sets."""
import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
F_TOL, E_TOL, RMSD_TOL = 1e-5, 1e-5, 1e-4
PRUNE = 3.2 * 3.8 + 8.0  # neighbor-list cutoff + 8 A of motion


def script():
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", "neighborlist"),
            ("set", "nnlup", "10"), ("set", "boxl", "2000"), ("set", "ncell", "250"),
            ("set", "run", "1")]


_sys = {}


def globule(nchain, chain_len):
    key = (nchain, chain_len)
    if key not in _sys:
        _sys[key] = S.synth_globule(3000 + nchain, nchain, chain_len)
    return _sys[key]


def port_for(system):
    p = O.Port()
    p.set_system(system, prune=PRUNE)
    for _, k, v in script():
        p.command(k, v)
    p.set_force_terms(0, 1, 1, 1)
    return p


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def rmsd(a, b):
    return float(np.sqrt(((np.asarray(a) - np.asarray(b)) ** 2).sum(1).mean()))


@pytest.fixture(scope="module")
def eng():
    e = Engine(0, max_beads=1 << 17, max_replicas=8, max_list_entries=1 << 25)
    yield e
    e.close()


@pytest.mark.parametrize("nchain", [20, 100])
def test_large_lists_forces_energies(eng, nchain):
    system = globule(nchain, 500)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system)
        port.setup(True)
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)),
                                          err_msg="list %d" % k)
        assert rel(eng.force(r), port.coords(3)) < F_TOL
        e = eng.energy(r)
        for k, name in enumerate(O.ENERGY_NAMES):
            want = port.energy(name)
            assert abs(e[k] - want) <= E_TOL * max(abs(want), 1e-3), (name, e[k], want)
        assert eng.status(r)[0] == 0
    finally:
        eng.remove(r)


def test_large_noise_off_trajectory(eng):
    system = globule(20, 500)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system)
        port.setup(True)
        eng.run_plain(r, 300)
        port.run(300)
        _, x, v = eng.state(r)
        assert rmsd(x, port.coords(1)) < RMSD_TOL
        assert rel(v, port.coords(2)) < 1e-4
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
    finally:
        eng.remove(r)


def test_large_skin_list_gives_reference_pair_sets(eng):
    """50,000 beads: the displacement-triggered skin list feeds each step the
    pair sets of the reference's 3.2x / nnlup schedule, batched."""
    system = globule(100, 500)
    a = eng.add(system, make_params(script(), force_terms=DET))
    b = eng.add(system, make_params(script(), force_terms=DET, list_mode="skin", skin=2.0))
    try:
        eng.run(200)
        for k in (2, 3):
            np.testing.assert_array_equal(pairset(*eng.pairs(a, k)), pairset(*eng.pairs(b, k)))
        np.testing.assert_array_equal(eng.state(a)[1], eng.state(b)[1])
        assert eng.status(a)[0] == 0 and eng.status(b)[0] == 0
        assert eng.info(b)["builds"] >= 1
    finally:
        eng.remove(a)
        eng.remove(b)
