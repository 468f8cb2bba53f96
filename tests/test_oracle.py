"""The CPU oracle pinned against the reference (CPU only).

* oracle/sop_oracle.c (the restatement) against oracle/_ref (the unmodified
  reference sources) on fresh seeded inputs: lists, forces, energies,
  trajectories and observables bit for bit;
* the restatement against the committed golden vectors (made by the
  reference, tests/golden/make_golden.py), which also exist on hosts without
  the reference tree;
* the Philox-4x32-10 stream against published known-answer vectors.
"""
import glob
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import systems as S

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sop_golden_N*.npz")))
GOLDEN_TYPED = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden",
                                             "sop_golden_types_N*.npz")))
needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference tree not built here")


def golden_script(mode="neighborlist", temp="0.6", nstep=100, nup=50, dynamics=None, boxl="500",
                  ncell="62.5"):
    pre = [("set", "dynamics", dynamics)] if dynamics else []
    return pre + [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", str(nstep)), ("set", "nup", str(nup)),
            ("set", "cutofftype", mode), ("set", "nnlup", "10"), ("set", "boxl", boxl),
            ("set", "ncell", ncell), ("set", "run", "1")]


def system_from_golden(g):
    typed = "bead_type" in g.files
    return S.System(xyz=g["xyz"], bonds=(g["ib"], g["jb"], g["r0"]),
                    angles=(g["ia"], g["ja"], g["ka"], g["a0"]),
                    natives=(g["in_"], g["jn"], g["rn"]),
                    bead_type=g["bead_type"] if typed else np.ones(len(g["xyz"]), np.int32),
                    exclusions=(g["ie"], g["je"]) if typed else None)


def typed_chain(seed, n, frac=0.25):
    """A chain with a seeded mix of bead types 1/2 whose vdw file leaves out
    a seeded fraction of the non-native candidates."""
    xyz = S._lib.synth_chain(seed, n)
    types = np.where(np.random.default_rng(seed + 1).random(n) < 0.4, 2, 1).astype(np.int32)
    system = S.system_from_xyz(xyz, bead_type=types)
    return S.with_exclusions(system, frac, seed + 2) if frac > 0 else system


def port_for(system, script):
    p = O.Port()
    p.set_system(system)
    for _, k, v in script:
        p.command(k, v)
    return p


def pairs(o, k):
    ii, jj = o.pairs(k)
    return np.stack([ii, jj], 1)


@needs_ref
@pytest.mark.parametrize("n,mode,dyn", [(30, "neighborlist", None), (76, "neighborlist", None),
                                        (76, "celllist", None), (120, "none", None),
                                        (250, "neighborlist", None),
                                        (76, "neighborlist", "overdamped"),
                                        (150, "celllist", "overdamped")])
def test_port_equals_reference(n, mode, dyn):
    system = S.synth_chain(5000 + n, n)
    ref, port = O.Ref(), O.Port()
    with tempfile.TemporaryDirectory() as d:
        path = S.write_reference_files(system, d, golden_script(mode, dynamics=dyn), run=False)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            ref.load_script(path)
            port.load_script(path)  # file names resolve against the cwd, as in io.cpp
        finally:
            os.chdir(cwd)
    for o in (ref, port):
        o.set_force_terms(0, 1, 1, 1)
        o.setup(True)
    for k in range(4):
        np.testing.assert_array_equal(pairs(ref, k), pairs(port, k))
    np.testing.assert_array_equal(ref.energies(), port.energies())
    np.testing.assert_array_equal(ref.coords(3), port.coords(3))
    for terms in ((0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1)):
        for o in (ref, port):
            o.set_force_terms(*terms)
            o.force_eval()
        np.testing.assert_array_equal(ref.coords(3), port.coords(3))
    for o in (ref, port):
        o.set_force_terms(0, 1, 1, 1)
        o.force_eval()
        o.run(60)
        o.energy_eval()
        o.observables()
    for which in (1, 2):
        np.testing.assert_array_equal(ref.coords(which), port.coords(which))
    np.testing.assert_array_equal(ref.energies(), port.energies())
    for k in ("Q", "rgsq", "kinT"):
        assert ref.energy(k) == port.energy(k)
    for k in range(4):
        np.testing.assert_array_equal(pairs(ref, k), pairs(port, k))


@needs_ref
@pytest.mark.parametrize("n,mode,frac", [(76, "neighborlist", 0.0), (120, "neighborlist", 0.25),
                                         (150, "celllist", 0.4), (90, "none", 0.3)])
def test_port_equals_reference_types_and_exclusions(n, mode, frac):
    """Bead types 1 and 2 (sigma, rcut_nat and the type-dependent native
    coefficients, global.cpp:60-92) and a vdw file that leaves out part of the
    non-native candidates (params.cpp:186-232): the reference reading the
    files, the restatement reading the same files, and the restatement given
    the system directly (sopo_set_topology / sopo_set_topology_implicit) agree
    bit for bit."""
    system = typed_chain(6100 + n, n, frac)
    # the reference keeps its globals between loads: reset the integrator
    scr = golden_script(mode, dynamics="underdamped")
    ref, port_files = O.Ref(), O.Port()
    port_direct = port_for(system, scr)
    with tempfile.TemporaryDirectory() as d:
        path = S.write_reference_files(system, d, scr, run=False)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            ref.load_script(path)
            port_files.load_script(path)
        finally:
            os.chdir(cwd)
    assert ref.count("ncon_att") == len(system.natives[0])
    assert ref.count("ncon_rep") == len(S.candidate_pairs(system)[0])
    ports = (port_files, port_direct)
    for o in (ref,) + ports:
        o.set_force_terms(0, 1, 1, 1)
        o.setup(True)
    for p in ports:
        for k in range(4):
            np.testing.assert_array_equal(pairs(ref, k), pairs(p, k))
        np.testing.assert_array_equal(ref.energies(), p.energies())
        np.testing.assert_array_equal(ref.coords(3), p.coords(3))
    for terms in ((0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1)):
        for o in (ref,) + ports:
            o.set_force_terms(*terms)
            o.force_eval()
        for p in ports:
            np.testing.assert_array_equal(ref.coords(3), p.coords(3))
    for o in (ref,) + ports:
        o.set_force_terms(0, 1, 1, 1)
        o.force_eval()
        o.run(60)
        o.energy_eval()
        o.observables()
    for p in ports:
        for which in (1, 2):
            np.testing.assert_array_equal(ref.coords(which), p.coords(which))
        np.testing.assert_array_equal(ref.energies(), p.energies())
        for k in ("Q", "rgsq", "kinT"):
            assert ref.energy(k) == p.energy(k)
        for k in range(4):
            np.testing.assert_array_equal(pairs(ref, k), pairs(p, k))


@needs_ref
@pytest.mark.parametrize("n,mode,boxl,ncell", [(150, "neighborlist", "40", "5"),
                                               (150, "celllist", "40", "5"),
                                               (120, "none", "35", "4.375"),
                                               (300, "neighborlist", "47.5", "5.9375")])
def test_port_equals_reference_with_periodic_images(n, mode, boxl, ncell):
    """A box smaller than twice the chain's extent: the minimum image
    (global.cpp:223-227) applies to list decisions, forces, energies and
    observables, and the cell list wraps by ncell.  Restatement and reference
    agree bit for bit."""
    system = S.synth_chain(6400 + n, n)
    ext = (system.xyz.max(0) - system.xyz.min(0)).max()
    assert ext > 0.5 * float(boxl)  # images do apply
    scr = golden_script(mode, dynamics="underdamped", boxl=boxl, ncell=ncell)
    ref, port = O.Ref(), O.Port()
    with tempfile.TemporaryDirectory() as d:
        path = S.write_reference_files(system, d, scr, run=False)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            ref.load_script(path)
            port.load_script(path)
        finally:
            os.chdir(cwd)
    for o in (ref, port):
        o.set_force_terms(0, 1, 1, 1)
        o.setup(True)
    for k in range(4):
        np.testing.assert_array_equal(pairs(ref, k), pairs(port, k))
    np.testing.assert_array_equal(ref.energies(), port.energies())
    np.testing.assert_array_equal(ref.coords(3), port.coords(3))
    for o in (ref, port):
        o.run(60)
        o.energy_eval()
        o.observables()
    for which in (1, 2):
        np.testing.assert_array_equal(ref.coords(which), port.coords(which))
    np.testing.assert_array_equal(ref.energies(), port.energies())
    for k in ("Q", "rgsq", "kinT"):
        assert ref.energy(k) == port.energy(k)


def test_typed_system_files_hold_what_the_system_says():
    """write_reference_files of a typed system with exclusions: every
    non-native line carries a distance at or above its pair's rcut_nat (so
    it stays non-native), excluded pairs are absent, types are per bead."""
    system = typed_chain(6200, 60, 0.3)
    with tempfile.TemporaryDirectory() as d:
        S.write_reference_files(system, d, golden_script(), run=False)
        rows = np.loadtxt(os.path.join(d, "vdw.dat"), skiprows=1)
    i, j = rows[:, 0].astype(int) - 1, rows[:, 1].astype(int) - 1
    t = system.bead_type
    np.testing.assert_array_equal(rows[:, 3], t[i])
    np.testing.assert_array_equal(rows[:, 4], t[j])
    native = rows[:, 2] < S.RCUT_NAT[t[i], t[j]]
    assert native.sum() == len(system.natives[0])
    listed = set(zip(i.tolist(), j.tolist()))
    assert not listed & set(zip(system.exclusions[0].tolist(), system.exclusions[1].tolist()))
    assert len(listed) == system.candidate_count() - len(system.exclusions[0])


def test_pull_force_term():
    """The pulling term (no reference counterpart): f along the separation of
    the two pulled beads, pushing them apart, added after the other terms;
    equal and opposite, so the force sum is unchanged."""
    system = S.synth_chain(6300, 80)
    scr = golden_script()
    base = port_for(system, scr)
    pulled = port_for(system, scr)
    f = 10.0 / 69.48  # 10 pN
    pulled.set_param("pull_force", f)
    pulled.set_param("pull_i", 3)
    pulled.set_param("pull_j", 70)
    for p in (base, pulled):
        p.set_force_terms(0, 1, 1, 1)
        p.setup(True)
    x = system.xyz
    u = x[70] - x[3]
    d = np.sqrt((u * u).sum())
    want = base.coords(3).copy()
    want[3] -= f * u / d
    want[70] += f * u / d
    np.testing.assert_allclose(pulled.coords(3), want, rtol=0, atol=1e-12)
    assert abs(pulled.coords(3).sum(0) - base.coords(3).sum(0)).max() < 1e-10
    # default pulled pair: the first and the last bead
    ends = port_for(system, scr)
    ends.set_param("pull_force", f)
    ends.set_force_terms(0, 1, 1, 1)
    ends.setup(True)
    u = x[-1] - x[0]
    want = base.coords(3).copy()
    want[0] -= f * u / np.sqrt((u * u).sum())
    want[-1] += f * u / np.sqrt((u * u).sum())
    np.testing.assert_allclose(ends.coords(3), want, rtol=0, atol=1e-12)


def test_standalone_generator_equals_engine_library_generator():
    """The workload generator built on its own (oracle/_build/libsopsynth.so,
    loaded by the benchmark's reference arm) and the engine library's copy
    give the same coordinates for the same seeds."""
    from sop_gb300 import _lib as L
    try:
        L.lib()
    except Exception:
        pytest.skip("engine library not built")
    for seed, n in ((11, 30), (2000, 700), (2511, 1500)):
        np.testing.assert_array_equal(O.synth_chain(seed, n), L.synth_chain(seed, n))


@needs_ref
def test_reference_files_round_trip():
    """The vdw file the generator writes splits into exactly the natives it holds."""
    system = S.synth_chain(77, 60)
    ref = O.Ref()
    with tempfile.TemporaryDirectory() as d:
        path = S.write_reference_files(system, d, golden_script(), run=False)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            ref.load_script(path)
        finally:
            os.chdir(cwd)
    assert ref.count("ncon_att") == len(system.natives[0])
    assert ref.count("ncon_att") + ref.count("ncon_rep") == system.candidate_count()
    np.testing.assert_array_equal(ref.coords(1), system.xyz)


@pytest.mark.parametrize("path", GOLDEN + GOLDEN_TYPED,
                         ids=[os.path.basename(p) for p in GOLDEN + GOLDEN_TYPED])
def test_port_matches_golden(path):
    g = np.load(path)
    system = system_from_golden(g)
    port = port_for(system, golden_script())
    np.testing.assert_array_equal([port.param(k) for k in ("T", "zeta", "h", "a1", "a2", "a3", "a4")],
                                  g["params"])
    port.set_force_terms(0, 1, 1, 1)
    port.setup(True)
    for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
        np.testing.assert_array_equal(pairs(port, k), g[name])
    # FP64 results: bit-exact on the x86 host that made them; 1e-12 elsewhere
    np.testing.assert_allclose(port.energies(), g["e0"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(port.coords(3), g["f_all"], rtol=1e-11, atol=1e-11)
    for name, terms in (("f_fene", (0, 1, 0, 0)), ("f_ang", (0, 0, 1, 0)), ("f_vdw", (0, 0, 0, 1))):
        port.set_force_terms(*terms)
        port.force_eval()
        np.testing.assert_allclose(port.coords(3), g[name], rtol=1e-11, atol=1e-11)
    port.set_force_terms(0, 1, 1, 1)
    port.force_eval()
    port.run(100)
    port.energy_eval()
    port.observables()
    np.testing.assert_allclose(port.coords(1), g["traj_unc"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(port.coords(2), g["traj_vel"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(port.energies(), g["traj_e"], rtol=1e-10, atol=1e-10)
    obs = [port.energy("Q"), port.count("contct_nat"), port.energy("rgsq"), port.energy("kinT")]
    np.testing.assert_allclose(obs, g["traj_obs"], rtol=1e-10)
    for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
        np.testing.assert_array_equal(pairs(port, k), g["traj_" + name])


@pytest.mark.parametrize("path", GOLDEN + GOLDEN_TYPED,
                         ids=[os.path.basename(p) for p in GOLDEN + GOLDEN_TYPED])
def test_port_cell_list_matches_golden(path):
    g = np.load(path)
    port = port_for(system_from_golden(g), golden_script("celllist"))
    port.setup(False)
    for k, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
        np.testing.assert_array_equal(pairs(port, k), g["cell_" + name])


@pytest.mark.parametrize("path", GOLDEN + GOLDEN_TYPED,
                         ids=[os.path.basename(p) for p in GOLDEN + GOLDEN_TYPED])
def test_port_steepest_descent_matches_reference_program(path):
    """sop.x at T=0 (v stays 0, x += a2 F, sop.cpp:316) against update.out,
    and the positions at the start and at every output step against the
    frames it appended to traj.bin / traj_uncorrected.bin (io.cpp:280-303)."""
    g = np.load(path)
    n = len(g["xyz"])
    frames = g["sd_traj"].reshape(-1, n, 3)
    frames_unc = g["sd_traj_unc"].reshape(-1, n, 3)
    assert len(frames) == len(frames_unc) == 1 + len(g["sd_update"])
    port = port_for(system_from_golden(g), golden_script(temp="0.0"))
    port.setup(True)
    np.testing.assert_allclose(port.coords(0), frames[0], rtol=0, atol=1e-6)  # %f columns
    np.testing.assert_allclose(port.coords(1), frames_unc[0], rtol=0, atol=1e-6)
    for k, row in enumerate(g["sd_update"]):
        step = int(row[0])
        port.run(step - int(port.param("force_evals")) + 1)
        port.energy_eval()
        port.observables()
        got = [port.energy("kinT"), port.energy("e_bnd"), port.energy("e_ang_ss"),
               port.energy("e_vdw_rr"), port.energy("rna_etot"), port.energy("Q"),
               port.count("contct_nat"), port.energy("rgsq")]
        np.testing.assert_allclose(got, row[2:], rtol=0, atol=2e-6)  # %f columns
        np.testing.assert_allclose(port.coords(0), frames[k + 1], rtol=0, atol=1e-6)
        np.testing.assert_allclose(port.coords(1), frames_unc[k + 1], rtol=0, atol=1e-6)
    np.testing.assert_allclose(port.coords(1), g["sd_unc"], rtol=0, atol=2e-6)


def test_philox_known_answers():
    """Random123 known-answer vectors for Philox-4x32-10."""
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        assert tuple(O.philox(ctr, key)) == want


@pytest.mark.parametrize("mode", ["neighborlist", "celllist"])
def test_pruned_candidates_equal_implicit(mode):
    """The pruned candidate set (the large-system oracle) forms the same lists,
    forces, energies and trajectory as the full implicit set, bit for bit,
    while no pair from beyond the pruning cutoff enters a list."""
    system = S.synth_chain(6600, 400)
    scr = golden_script(mode)
    full, pruned = O.Port(), O.Port()
    full.set_system(system)
    # cell mode lists every candidate in adjacent 8 A cells: up to 2 sqrt(3) 8 A apart
    pruned.set_system(system, prune=3.2 * 3.8 + 8.0 if mode == "neighborlist" else 30.0)
    assert pruned.count("ncon_rep") < full.count("ncon_rep")
    for p in (full, pruned):
        for _, k, v in scr:
            p.command(k, v)
        p.set_force_terms(0, 1, 1, 1)
        p.setup(True)
    for k in range(4):  # same entries in the same order
        np.testing.assert_array_equal(pairs(pruned, k), pairs(full, k))
    np.testing.assert_array_equal(pruned.coords(3), full.coords(3))
    full.run(200)
    pruned.run(200)
    np.testing.assert_array_equal(pruned.coords(1), full.coords(1))
    full.energy_eval()
    pruned.energy_eval()
    np.testing.assert_array_equal(pruned.energies(), full.energies())
