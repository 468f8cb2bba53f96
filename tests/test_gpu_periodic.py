"""Minimum images on the GPU: replicas whose extent reaches half the box.

The reference applies dx -= boxl rnd(dx / boxl) to every pair, bond and angle
(global.cpp:223-227) and wraps its cell list by ncell (cell_list.cpp:37-39).
When a replica's extent plus two list cutoffs reaches boxl / 2, the engine
switches it to image mode: its list build scans every bead pair with the
images in both the FP32 screen and the FP64 decision, and its step, energies,
observables and pair filter apply the images too.  Checked against the oracle
(pinned to the reference with images in tests/test_oracle.py) at boxes
smaller than twice the chains: lists bit-exact as sets, forces and energies
within 1e-5, 1,000-step noise-off trajectories within 1e-4 A RMSD (FP64
precision: 1e-10 and 1e-8 A), Q exact, Rg^2 within 1e-9; an image-mode
replica inside a batch equals itself alone; a box shrunk between runs takes
effect at once.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
F_TOL, E_TOL, RMSD_TOL = 1e-5, 1e-5, 1e-4


def script(mode="neighborlist", boxl="40", ncell="5", temp="0.6"):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", mode),
            ("set", "nnlup", "10"), ("set", "boxl", boxl), ("set", "ncell", ncell),
            ("set", "run", "1")]


@pytest.fixture(scope="module")
def eng():
    e = Engine(0, max_beads=1 << 17, max_replicas=64, max_list_entries=1 << 24)
    yield e
    e.close()


def port_for(system, scr, terms=(0, 1, 1, 1)):
    p = O.Port()
    p.set_system(system)
    for _, k, v in scr:
        p.command(k, v)
    p.set_force_terms(*terms)
    return p


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def rmsd(a, b):
    return float(np.sqrt(((np.asarray(a) - np.asarray(b)) ** 2).sum(1).mean()))


_chains = {}


def chain(n):
    if n not in _chains:
        _chains[n] = S.synth_chain(9500 + n, n)
    return _chains[n]


def box_for(system, frac=1.1):
    """A box edge of frac times the chain's extent: pairs farther apart than
    half of it along an axis are imaged; at 1.1 extents some imaged pairs
    fall within the list cutoffs (6-90 for these chains) and none closer than
    a bond length."""
    ext = float((system.xyz.max(0) - system.xyz.min(0)).max())
    return "%.3f" % (frac * ext)


CASES = [(150, "neighborlist"), (150, "celllist"), (300, "neighborlist"), (120, "none"),
         (1500, "neighborlist"), (600, "celllist")]


def scr_for(n, mode):
    system = chain(n)
    boxl = box_for(system)
    return system, script(mode, boxl=boxl, ncell="%.6f" % (float(boxl) / 8.0))


@pytest.mark.parametrize("n,mode", CASES)
def test_image_lists_forces_energies(eng, n, mode):
    system, scr = scr_for(n, mode)
    r = eng.add(system, make_params(scr, force_terms=DET))
    try:
        port = port_for(system, scr)
        port.setup(True)
        for k in range(4):
            if mode == "none" and k < 2:
                continue
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)),
                                          err_msg="list %d" % k)
        assert rel(eng.force(r), port.coords(3)) < F_TOL
        e = eng.energy(r)
        for k, name in enumerate(O.ENERGY_NAMES):
            want = port.energy(name)
            assert abs(e[k] - want) <= E_TOL * max(abs(want), 1e-3), (name, e[k], want)
        for bit, terms in ((L.TERM_FENE, (0, 1, 0, 0)), (L.TERM_ANGLE, (0, 0, 1, 0)),
                           (L.TERM_VDW, (0, 0, 0, 1))):
            eng.set_params(r, make_params(scr, force_terms=bit))
            port.set_force_terms(*terms)
            port.force_eval()
            assert rel(eng.force(r), port.coords(3)) < F_TOL, bit
        assert eng.status(r)[0] == 0
    finally:
        eng.remove(r)


@pytest.mark.parametrize("n,mode", [(150, "neighborlist"), (150, "celllist"), (120, "none"),
                                    (1500, "neighborlist")])
def test_image_noise_off_trajectory(eng, n, mode):
    system, scr = scr_for(n, mode)
    steps = 300 if n > 1000 else 1000
    r = eng.add(system, make_params(scr, force_terms=DET))
    try:
        port = port_for(system, scr)
        port.setup(True)
        eng.run_plain(r, steps)
        port.run(steps)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD_TOL
        for k in range(4):
            if mode == "none" and k < 2:
                continue
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
        port.energy_eval()
        e = eng.energy(r)
        assert abs(e[5] - port.energy("rna_etot")) <= E_TOL * abs(port.energy("rna_etot"))
        port.observables()
        o = eng.observables(r)
        assert o[0] == port.energy("Q")
        assert abs(o[2] - port.energy("rgsq")) <= 1e-9 * port.energy("rgsq")
        assert abs(o[3] - port.energy("kinT")) <= 1e-4 * port.energy("kinT")
        assert eng.status(r)[0] == 0
    finally:
        eng.remove(r)


def test_image_fp64_precision(eng):
    system, scr = scr_for(300, "neighborlist")
    r = eng.add(system, make_params(scr, force_terms=DET, precision=L.PREC_FP64))
    try:
        port = port_for(system, scr)
        port.setup(True)
        assert rel(eng.force(r), port.coords(3)) < 1e-10
        eng.run_plain(r, 1000)
        port.run(1000)
        assert rmsd(eng.state(r)[1], port.coords(1)) < 1e-8
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
    finally:
        eng.remove(r)


def test_image_replica_in_a_batch_and_in_skin_mode(eng):
    """Image-mode replicas (skin lists and the reference cadence) next to
    open-boundary ones, noise on: each equals itself alone, bit for bit; the
    skin-list one also equals its cadence twin."""
    sys_img, scr_img = scr_for(300, "neighborlist")
    others = [chain(76), chain(600)]
    params = [make_params(scr_img, seed=51),
              make_params(scr_img, seed=51, list_mode="skin", skin=1.5),
              make_params(script(boxl="500", ncell="62.5"), seed=52),
              make_params(script(boxl="500", ncell="62.5"), seed=53)]
    systems = [sys_img, sys_img] + others
    alone = []
    for s, p in zip(systems, params):
        r = eng.add(s, p)
        eng.run(200)
        alone.append(eng.state(r)[1])
        eng.remove(r)
    ids = [eng.add(s, p) for s, p in zip(systems, params)]
    eng.run(200)
    for k, r in enumerate(ids):
        np.testing.assert_array_equal(eng.state(r)[1], alone[k])
        assert eng.status(r)[0] == 0
    np.testing.assert_array_equal(alone[0], alone[1])
    for r in ids:
        eng.remove(r)


def test_box_shrunk_between_runs(eng):
    """Open boundaries first, then a box smaller than the chain set between
    runs: the next steps already use images, as the oracle does."""
    system = chain(150)
    open_scr = script(boxl="500", ncell="62.5")
    small = box_for(system)
    small_scr = script(boxl=small, ncell="%.6f" % (float(small) / 8.0))
    r = eng.add(system, make_params(open_scr, force_terms=DET))
    try:
        port = port_for(system, open_scr)
        port.setup(True)
        eng.run_plain(r, 200)
        port.run(200)
        eng.set_params(r, make_params(small_scr, force_terms=DET))
        for _, k, v in small_scr:
            if k in ("boxl", "ncell"):
                port.command(k, v)
        port.neighbor_list()
        port.pair_list()
        port.force_eval()
        assert rel(eng.force(r), port.coords(3)) < F_TOL
        eng.run_plain(r, 300)
        port.run(300)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD_TOL
    finally:
        eng.remove(r)
