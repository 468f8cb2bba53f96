"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and
the reference's golden vectors.

Tolerances: pair lists bit-exact as integer sets;
per-step forces and energies within 1e-5 relative (forces normwise over all
beads: |F_gpu - F_ref|_2 / |F_ref|_2); 1,000-step noise-off trajectories
within 1e-4 A RMSD.
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

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sop_golden_N*.npz")))
DET = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW  # random term off
F_TOL, E_TOL, RMSD_TOL = 1e-5, 1e-5, 1e-4


def script(mode="neighborlist", temp="0.6", nnlup="10"):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", "1000"), ("set", "nup", "1000"), ("set", "cutofftype", mode),
            ("set", "nnlup", nnlup), ("set", "boxl", "500"), ("set", "ncell", "62.5"),
            ("set", "run", "1")]


@pytest.fixture(scope="module")
def eng():
    e = Engine(0, max_beads=1 << 18, max_replicas=256, max_list_entries=1 << 25)
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


_systems = {}


def chain(n):
    if n not in _systems:
        _systems[n] = S.synth_chain(3000 + n, n)
    return _systems[n]


@pytest.mark.parametrize("n", [30, 76, 300, 1500])
@pytest.mark.parametrize("mode", ["neighborlist", "celllist", "none"])
def test_lists_bit_exact(eng, n, mode):
    if mode == "none" and n > 300:
        pytest.skip("full candidate list is O(N^2)")
    system = chain(n)
    r = eng.add(system, make_params(script(mode), force_terms=DET))
    try:
        port = port_for(system, script(mode))
        port.setup(False)
        for k in range(4):
            if mode == "none" and k < 2:
                continue  # no neighbor list without a cutoff type
            got = pairset(*eng.pairs(r, k))
            want = pairset(*port.pairs(k))
            np.testing.assert_array_equal(got, want, err_msg="list %d" % k)
    finally:
        eng.remove(r)


@pytest.mark.parametrize("n", [30, 76, 300, 1500, 3000])
def test_forces_and_energies(eng, n):
    system = chain(n)
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


@pytest.mark.parametrize("n,steps", [(76, 1000), (300, 1000), (1500, 300), (3000, 1000)])
def test_noise_off_trajectory(eng, n, steps):
    """Noise-off trajectories against the oracle, up to the 3000-bead chain's
    1,000 steps: positions within 1e-4 A RMSD, lists bit-exact as sets."""
    system = chain(n)
    r = eng.add(system, make_params(script(), force_terms=DET))
    try:
        port = port_for(system, script())
        port.setup(True)
        eng.run_plain(r, steps)
        port.run(steps)
        _, x, v = eng.state(r)
        assert rmsd(x, port.coords(1)) < RMSD_TOL
        assert rel(v, port.coords(2)) < 1e-4
        for k in range(4):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(*port.pairs(k)))
        port.energy_eval()
        e = eng.energy(r)
        assert abs(e[5] - port.energy("rna_etot")) <= E_TOL * abs(port.energy("rna_etot"))
        port.observables()
        o = eng.observables(r)
        assert o[0] == port.energy("Q")
        assert abs(o[2] - port.energy("rgsq")) <= 1e-9 * port.energy("rgsq")
        assert abs(o[3] - port.energy("kinT")) <= 1e-4 * port.energy("kinT")
    finally:
        eng.remove(r)


@pytest.mark.parametrize("n,mode", [(76, "neighborlist"), (300, "celllist"), (1500, "neighborlist")])
def test_overdamped_noise_off_trajectory(eng, n, mode):
    """set dynamics overdamped: overdamped_iteration (sop.cpp:331-363) with
    a5 = h/zeta, kinT from the increments (sop.cpp:270-278)."""
    system = chain(n)
    scr = [("set", "dynamics", "overdamped")] + script(mode)
    r = eng.add(system, make_params(scr, force_terms=DET))
    try:
        port = port_for(system, scr)
        assert port.param("sim_type") == 2
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
        assert abs(o[3] - port.energy("kinT")) <= 1e-3 * port.energy("kinT")
    finally:
        eng.remove(r)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_vectors(eng, path):
    g = np.load(path)
    system = S.System(xyz=g["xyz"], bonds=(g["ib"], g["jb"], g["r0"]),
                      angles=(g["ia"], g["ja"], g["ka"], g["a0"]),
                      natives=(g["in_"], g["jn"], g["rn"]), bead_type=np.ones(len(g["xyz"]), np.int32))
    sc = script()
    r = eng.add(system, make_params(sc, force_terms=DET))
    try:
        for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)), pairset(g[name][:, 0], g[name][:, 1]))
        assert rel(eng.force(r), g["f_all"]) < F_TOL
        e = eng.energy(r)
        np.testing.assert_allclose(e, g["e0"], rtol=E_TOL, atol=1e-8)
        eng.run_plain(r, 100)
        _, x, v = eng.state(r)
        assert rmsd(x, g["traj_unc"]) < RMSD_TOL
        e = eng.energy(r)
        np.testing.assert_allclose(e, g["traj_e"], rtol=E_TOL, atol=1e-8)
        for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
            np.testing.assert_array_equal(pairset(*eng.pairs(r, k)),
                                          pairset(g["traj_" + name][:, 0], g["traj_" + name][:, 1]))
    finally:
        eng.remove(r)
    # steepest descent (T = 0): sop.x's own update.out and final coordinates
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


def test_plain_and_batched_paths_agree(eng):
    """The same replica stepped one-system-per-launch and inside the packed,
    graph-captured batch gives bit-identical state."""
    system = chain(300)
    p = make_params(script(), force_terms=DET)
    r = eng.add(system, p)
    eng.run_plain(r, 120)
    _, xa, va = eng.state(r)
    eng.remove(r)
    r = eng.add(system, p)
    eng.run(120)
    _, xb, vb = eng.state(r)
    eng.remove(r)
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(va, vb)


def test_thermostat_matches_oracle(eng):
    """Noise on: the mean kinetic temperature of a Langevin run equals the
    oracle's over its own noisy run (same integrator and protocol, independent
    counter-based streams), so the noise has the reference's amplitude and
    distribution.  Statistical tolerance: 5% on the means of 120 samples of a
    300-bead chain (one sample fluctuates by ~4.7%; the two means by ~1.2%)."""
    system = chain(300)
    scr = script()
    r = eng.add(system, make_params(scr, seed=7301))
    try:
        port = port_for(system, scr, terms=(1, 1, 1, 1))
        port.setup(True)
        eng.run_plain(r, 2000)
        port.run(2000)
        g, c = [], []
        for _ in range(120):
            eng.run_plain(r, 100)
            g.append(eng.observables(r)[3])
            port.run(100)
            port.observables()
            c.append(port.energy("kinT"))
        assert eng.status(r)[0] == 0
        assert abs(np.mean(g) - np.mean(c)) < 0.05 * np.mean(c), (np.mean(g), np.mean(c))
        assert abs(np.std(g) - np.std(c)) < 0.35 * np.std(c), (np.std(g), np.std(c))
    finally:
        eng.remove(r)


def test_many_replicas_per_prep_cta():
    """700 small replicas: every prep CTA owns two or three of them, hundreds
    of producers publish build units while others consume, skin and cadence
    rebuilds interleave.  A sample of the replicas equals the same replica run
    alone, bit for bit (noise on)."""
    from sop_gb300 import _lib as Lb
    count = 700
    sizes = [30 + (k * 37) % 90 for k in range(count)]
    xyzs = Lb.synth_many([(52000 + k, n) for k, n in enumerate(sizes)])
    systems = [S.system_from_xyz(x) for x in xyzs]
    params = [make_params(script(temp=str(0.4 + 0.001 * (k % 400))), seed=5200 + k,
                          list_mode="skin" if k % 2 else "neighborlist", skin=1.0)
              for k in range(count)]
    sample = [0, 1, 151, 302, 455, 699]
    with Engine(0, max_beads=1 << 17, max_replicas=count + 8, max_list_entries=1 << 24) as e:
        ids = [e.add(s, p) for s, p in zip(systems, params)]
        e.run(200)
        got = {k: e.state(ids[k])[1] for k in sample}
        assert all(e.status(r)[0] == 0 for r in ids)
    with Engine(0, max_beads=1 << 12, max_replicas=4, max_list_entries=1 << 20) as e:
        for k in sample:
            r = e.add(systems[k], params[k])
            e.run(200)
            np.testing.assert_array_equal(e.state(r)[1], got[k])
            e.remove(r)


def test_batch_invariance_with_noise(eng):
    """Each replica alone and inside a mix of uneven sizes: bit-identical,
    noise on (counter-based streams keyed by replica seed)."""
    sizes = [40, 333, 1200, 77, 600]
    systems = [S.synth_chain(7100 + k, n) for k, n in enumerate(sizes)]
    params = [make_params(script(temp=str(0.4 + 0.1 * k)), seed=900 + k) for k in range(len(sizes))]
    alone = []
    for s, p in zip(systems, params):
        r = eng.add(s, p)
        eng.run(100)
        alone.append(eng.state(r)[1])
        eng.remove(r)
    ids = [eng.add(s, p) for s, p in zip(systems, params)]
    eng.run(100)
    for k, r in enumerate(ids):
        np.testing.assert_array_equal(eng.state(r)[1], alone[k])
    for r in ids:
        eng.remove(r)


def test_skin_list_gives_reference_pair_sets(eng):
    """Displacement-triggered Verlet list (2.5 sigma + skin): the pair list it
    feeds each step equals the reference's 3.2x/nnlup schedule."""
    system = chain(300)
    a = eng.add(system, make_params(script(), force_terms=DET))
    b = eng.add(system, make_params(script(), force_terms=DET, list_mode="skin", skin=1.5))
    eng.run(400)
    for k in (2, 3):
        np.testing.assert_array_equal(pairset(*eng.pairs(a, k)), pairset(*eng.pairs(b, k)))
    # same pair sets every step and exact integer force sums: same trajectory
    np.testing.assert_array_equal(eng.state(a)[1], eng.state(b)[1])
    eng.remove(a)
    eng.remove(b)


def test_status_flags_fene_overstretch(eng):
    """A bond stretched past R0 is reported on that replica only."""
    system = chain(76)
    bad = system.xyz.copy()
    bad[40:] += np.array([2.5, 0.0, 0.0])  # bond 39-40 stretched by ~2.5 A
    s_bad = S.System(xyz=bad, bonds=system.bonds, angles=system.angles, natives=system.natives,
                     bead_type=system.bead_type)
    good = eng.add(system, make_params(script(), force_terms=DET))
    badr = eng.add(s_bad, make_params(script(), force_terms=DET))
    eng.run(10)
    assert eng.status(badr)[0] & L.ST_FENE
    assert eng.status(good)[0] == 0
    eng.remove(good)
    eng.remove(badr)
