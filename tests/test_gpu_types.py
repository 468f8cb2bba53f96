"""GPU parity on the rest of the reference's input space, through the C ABI:

* bead types 1 and 2 -- sigma 3.8 / 5.4 / 7.0 A, rcut_nat 8 / 11 / 14 A and
  the type-dependent native coefficients (global.cpp:60-92);
* vdw files that leave out part of the non-native candidates: a pair missing
  from the file never interacts (params.cpp:186-232), given to the engine as
  exclusions (sop_system_desc.nexcl);
* the constant pulling force on two beads (no reference term) against the
  oracle's CPU restatement of it.

Against the oracle (pinned to the reference on these inputs by
tests/test_oracle.py) and the reference's own golden vectors
(tests/golden/sop_golden_types_N150.npz).  Tolerances as everywhere: pair
lists bit-exact as integer sets; forces (normwise, per term too) and
energies within 1e-5 relative; 1,000-step noise-off trajectories within
1e-4 A RMSD.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

GOLDEN_TYPED = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden",
                                             "sop_golden_types_N*.npz")))
DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW  # random term off
F_TOL, E_TOL, RMSD_TOL = 1e-5, 1e-5, 1e-4
PN = 1.0 / 69.48  # kcal/mol/A per pN


def script(mode="neighborlist", temp="0.6"):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", mode),
            ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


@pytest.fixture(scope="module")
def eng():
    e = Engine(0, max_beads=1 << 18, max_replicas=256, max_list_entries=1 << 25)
    yield e
    e.close()


_cache = {}


def typed(n, frac):
    """A chain with a seeded mix of bead types (about 40% type 2) whose vdw
    file leaves out a seeded fraction of the non-native candidates."""
    key = (n, frac)
    if key not in _cache:
        seed = 7700 + n
        xyz = L.synth_chain(seed, n)
        types = np.where(np.random.default_rng(seed + 1).random(n) < 0.4, 2, 1).astype(np.int32)
        system = S.system_from_xyz(xyz, bead_type=types)
        _cache[key] = S.with_exclusions(system, frac, seed + 2) if frac > 0 else system
    return _cache[key]


def port_for(system, scr, terms=(0, 1, 1, 1), **pull):
    p = O.Port()
    p.set_system(system)
    for _, k, v in scr:
        p.command(k, v)
    for k, v in pull.items():
        p.set_param(k, v)
    p.set_force_terms(*terms)
    return p


def pairset(ii, jj):
    a = np.stack([np.minimum(ii, jj), np.maximum(ii, jj)], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def rmsd(a, b):
    return float(np.sqrt(((np.asarray(a) - np.asarray(b)) ** 2).sum(1).mean()))


CASES = [(76, 0.0), (76, 0.3), (300, 0.25), (1500, 0.25)]


@pytest.mark.parametrize("n,frac", CASES)
@pytest.mark.parametrize("mode", ["neighborlist", "celllist", "none"])
def test_typed_lists_bit_exact(eng, n, frac, mode):
    if mode == "none" and n > 300:
        pytest.skip("full candidate list is O(N^2)")
    system = typed(n, frac)
    r = eng.add(system, make_params(script(mode), force_terms=DET))
    try:
        port = port_for(system, script(mode))
        port.setup(False)
        for k in range(4):
            if mode == "none" and k < 2:
                continue
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)),
                                          err_msg="list %d" % k)
    finally:
        eng.remove(r)


@pytest.mark.parametrize("n,frac", CASES)
def test_typed_forces_and_energies(eng, n, frac):
    system = typed(n, frac)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system, script())
        port.setup(True)
        assert rel(eng.force(r), port.coords(3)) < F_TOL
        e = eng.energy(r)
        for k, name in enumerate(O.ENERGY_NAMES):
            want = port.energy(name)
            assert abs(e[k] - want) <= E_TOL * max(abs(want), 1e-3), (name, e[k], want)
        for bit, terms in ((L.TERM_FENE, (0, 1, 0, 0)), (L.TERM_ANGLE, (0, 0, 1, 0)),
                           (L.TERM_VDW, (0, 0, 0, 1))):
            eng.set_params(r, make_params(script(), force_terms=bit))
            port.set_force_terms(*terms)
            port.force_eval()
            assert rel(eng.force(r), port.coords(3)) < F_TOL, bit
    finally:
        eng.remove(r)


@pytest.mark.parametrize("n,frac", [(76, 0.3), (300, 0.25), (1500, 0.25)])
def test_typed_noise_off_trajectory(eng, n, frac):
    """1,000 noise-off steps: positions within 1e-4 A RMSD, lists bit-exact,
    energies and observables."""
    system = typed(n, frac)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system, script())
        port.setup(True)
        eng.run_plain(r, 1000)
        port.run(1000)
        _, x, _ = eng.state(r)
        assert rmsd(x, port.coords(1)) < RMSD_TOL
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
        port.energy_eval()
        e = eng.energy(r)
        assert abs(e[5] - port.energy("rna_etot")) <= E_TOL * abs(port.energy("rna_etot"))
        port.observables()
        o = eng.observables(r)
        assert o[0] == port.energy("Q")
        assert abs(o[2] - port.energy("rgsq")) <= 1e-9 * port.energy("rgsq")
        assert eng.status(r)[0] == 0
    finally:
        eng.remove(r)


def test_typed_skin_and_batched_paths(eng):
    """Typed, partially listed replicas in skin mode inside a batch: the same
    trajectory as the reference cadence run alone (exact sums, exact pair
    filter), and the oracle within tolerance."""
    systems = [typed(300, 0.25), typed(76, 0.3), typed(1500, 0.25)]
    cadence = []
    for s in systems:
        r = eng.add(s, make_params(script(), force_terms=DET))
        eng.run_plain(r, 400)
        cadence.append(eng.state(r)[1])
        eng.remove(r)
    ids = [eng.add(s, make_params(script(), force_terms=DET, list_mode="skin", skin=2.0))
           for s in systems]
    eng.run(400)
    for k, (r, s) in enumerate(zip(ids, systems)):
        np.testing.assert_array_equal(eng.state(r)[1], cadence[k])
        port = port_for(s, script())
        port.setup(True)
        port.run(400)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD_TOL
        eng.remove(r)


def system_from_golden(g):
    return S.System(xyz=g["xyz"], bonds=(g["ib"], g["jb"], g["r0"]),
                    angles=(g["ia"], g["ja"], g["ka"], g["a0"]),
                    natives=(g["in_"], g["jn"], g["rn"]), bead_type=g["bead_type"],
                    exclusions=(g["ie"], g["je"]))


@pytest.mark.parametrize("path", GOLDEN_TYPED, ids=[os.path.basename(p) for p in GOLDEN_TYPED])
def test_typed_golden_vectors(eng, path):
    """The reference's own lists, forces, energies and 100-step trajectory
    for a typed chain with a partial vdw file, and sop.x's steepest descent."""
    g = np.load(path)
    system = system_from_golden(g)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)),
                                          pairset(g[name][:, 0], g[name][:, 1]))
        assert rel(eng.force(r), g["f_all"]) < F_TOL
        np.testing.assert_allclose(eng.energy(r), g["e0"], rtol=E_TOL, atol=1e-8)
        for bit, name in ((L.TERM_FENE, "f_fene"), (L.TERM_ANGLE, "f_ang"), (L.TERM_VDW, "f_vdw")):
            eng.set_params(r, make_params(script(), force_terms=bit))
            assert rel(eng.force(r), g[name]) < F_TOL, name
        eng.set_params(r, make_params(script(), force_terms=DET))
        eng.force(r)
        eng.run_plain(r, 100)
        _, x, _ = eng.state(r)
        assert rmsd(x, g["traj_unc"]) < RMSD_TOL
        np.testing.assert_allclose(eng.energy(r), g["traj_e"], rtol=E_TOL, atol=1e-8)
        for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)),
                                          pairset(g["traj_" + name][:, 0], g["traj_" + name][:, 1]))
    finally:
        eng.remove(r)
    r = eng.add(system, make_params(script("celllist"), force_terms=DET))
    try:
        for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)),
                                          pairset(g["cell_" + name][:, 0], g["cell_" + name][:, 1]))
    finally:
        eng.remove(r)
    r = eng.add(system, make_params(script(temp="0.0")))
    try:
        eng.run_plain(r, 100)
        _, x, _ = eng.state(r)
        np.testing.assert_allclose(x, g["sd_unc"], rtol=0, atol=1e-5)
        e = eng.energy(r)
        row = g["sd_update"][-1]
        np.testing.assert_allclose([e[0], e[1], e[2], e[5]], [row[3], row[4], row[5], row[6]],
                                   rtol=1e-5, atol=2e-6)
    finally:
        eng.remove(r)


@pytest.mark.parametrize("pull", [(15.0, 0, -1), (7.5, 5, 250)])
def test_pull_force_matches_oracle(eng, pull):
    """Constant pulling force (pN, pulled beads; -1 = the last bead): the
    force with it against the oracle's restatement, then 1,000 noise-off steps
    (plain path) and 500 batched steps in skin mode against the oracle."""
    f_pn, pi, pj = pull
    system = S.synth_chain(7900, 300)
    kw = dict(pull_force=f_pn * PN, pull_i=pi, pull_j=pj)
    r = eng.add(system, make_params(script(), force_terms=DET, **kw))
    try:
        port = port_for(system, script(), **kw)
        port.setup(True)
        f = eng.force(r)
        assert rel(f, port.coords(3)) < F_TOL
        # the pulled beads' own forces carry the term to FP32 accuracy
        for b in (pi, pj if pj >= 0 else system.nbead - 1):
            assert np.linalg.norm(f[b] - port.coords(3)[b]) < 1e-5 * max(1.0, np.linalg.norm(port.coords(3)[b]))
        eng.run_plain(r, 1000)
        port.run(1000)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD_TOL
        # the chain is stretched relative to the unpulled run
        assert eng.status(r)[0] == 0
    finally:
        eng.remove(r)
    r = eng.add(system, make_params(script(), force_terms=DET, list_mode="skin", skin=2.0, **kw))
    try:
        port = port_for(system, script(), **kw)
        port.setup(True)
        eng.run(500)
        port.run(500)
        assert rmsd(eng.state(r)[1], port.coords(1)) < RMSD_TOL
    finally:
        eng.remove(r)


def test_pull_stretches_chain(eng):
    """Over a noisy run the pulled chain's end-to-end distance grows beyond
    the unpulled chain's (sanity of the sign: the termini are pulled apart)."""
    system = S.synth_chain(7950, 120)
    a = eng.add(system, make_params(script(), seed=11))
    b = eng.add(system, make_params(script(), seed=11, pull_force=15.0 * PN * 20))
    eng.run(3000)
    ea = eng.observables(a)[4]
    eb = eng.observables(b)[4]
    assert eb > ea, (ea, eb)
    eng.remove(a)
    eng.remove(b)
