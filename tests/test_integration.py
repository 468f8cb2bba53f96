"""The SOP-CPU-side GPU backend (sop-cpu_gb300/integration/gpu_backend.cpp).

* It compiles against the reference's own headers with -Wall -Werror and
  links with the reference's globals and libsopgpu.so.
* Linked instead with the reference's own command reader and loaders
  (io.cpp, params.cpp) and a recording stub of the C ABI, it hands the
  engine what the reference loaded from a vdw file with bead types 1 and 2
  that leaves out part of the non-native candidates: per-bead types, the
  natives, the bonds and angles 0-based, the left-out candidates as
  exclusions, the integrator constants, and force_term_on[] / nforce_term as
  the term mask; results come back into the 1-based globals.
* A failed status from any call ends the program with the library's message
  and exit(-1).

No GPU calls.  Skipped where the reference tree is absent (the tree is the
one the oracle was built from, or the REF environment variable).
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import systems as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIR = os.path.join(ROOT, "sop-cpu_gb300", "integration")
LIB = os.path.join(ROOT, "sop-cpu_gb300", "lib", "libsopgpu.so")
REF = os.environ.get("REF") or O.ref_tree()

needs_ref = pytest.mark.skipif(not (REF and os.path.exists(os.path.join(REF, "global.h"))),
                               reason="reference tree not present")
needs_tools = pytest.mark.skipif(shutil.which("make") is None or shutil.which("g++") is None,
                                 reason="no make / g++")

SCRIPT = [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.7"),
          ("set", "nstep", "100"), ("set", "nup", "50"), ("set", "cutofftype", "neighborlist"),
          ("set", "nnlup", "10"), ("set", "boxl", "500"), ("set", "ncell", "62.5"), ("set", "run", "3")]


def make(target):
    p = subprocess.run(["make", "-s", "-C", DIR, target, "REF=" + REF], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    return os.path.join(DIR, "_build", {"check": "gpu_backend_check", "shim-test": "shim_test"}[target])


@needs_ref
@needs_tools
def test_backend_compiles_and_links_against_the_reference():
    if not os.path.exists(LIB):
        pytest.skip("libsopgpu.so not built")
    exe = make("check")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "14 entry points" in out.stdout
    if shutil.which("nm"):
        syms = subprocess.run(["nm", "-C", os.path.join(DIR, "_build", "gpu_backend.o")],
                              capture_output=True, text=True).stdout
        for f in ("update_neighbor_list()", "update_cell_list()", "update_pair_list()",
                  "force_eval()", "energy_eval()", "underdamped_iteration(coord*)",
                  "overdamped_iteration(coord*)"):
            assert " T " + f in syms, f


def typed_system():
    xyz = S._lib.synth_chain(4242, 40) if os.path.exists(LIB) else O.synth_chain(4242, 40)
    types = np.where(np.random.default_rng(4243).random(40) < 0.4, 2, 1).astype(np.int32)
    return S.with_exclusions(S.system_from_xyz(xyz, bead_type=types), 0.3, 4244)


def run_shim(system, fail=None):
    exe = make("shim-test")
    with tempfile.TemporaryDirectory() as d:
        inp = S.write_reference_files(system, d, SCRIPT, run=False)
        env = dict(os.environ, SOP_STUB_LOG=os.path.join(d, "stub.log"))
        if fail:
            env["SOP_STUB_FAIL"] = fail
        p = subprocess.run([exe, inp], cwd=d, env=env, capture_output=True, text=True, timeout=60)
        log = open(os.path.join(d, "stub.log")).read().splitlines()
    return p, log


def field(log, key, nth=0):
    rows = [l.split()[1:] for l in log if l.split() and l.split()[0] == key]
    return rows[nth]


def kv(row):
    return {row[k]: row[k + 1] for k in range(0, len(row), 2)}


@needs_ref
@needs_tools
def test_backend_hands_the_reference_inputs_to_the_engine():
    system = typed_system()
    p, log = run_shim(system)
    assert p.returncode == 0, p.stderr
    n = system.nbead
    assert int(field(log, "nbead")[0]) == n
    np.testing.assert_array_equal(np.array(field(log, "type"), int), system.bead_type)
    np.testing.assert_array_equal(np.array(field(log, "xyz"), float).reshape(n, 3), system.xyz)
    b = field(log, "bonds")
    bonds = np.array(b[1:], float).reshape(int(b[0]), 3)
    np.testing.assert_array_equal(bonds[:, 0], system.bonds[0])
    np.testing.assert_array_equal(bonds[:, 1], system.bonds[1])
    np.testing.assert_array_equal(bonds[:, 2], system.bonds[2])
    a = field(log, "angles")
    ang = np.array(a[1:], int).reshape(int(a[0]), 2)
    np.testing.assert_array_equal(ang[:, 0], system.angles[0])
    np.testing.assert_array_equal(ang[:, 1], system.angles[2])
    nt = field(log, "natives")
    nat = np.array(nt[1:], float).reshape(int(nt[0]), 3)
    want = {(int(i), int(j), float(r)) for i, j, r in zip(*system.natives)}
    assert {(int(i), int(j), r) for i, j, r in nat} == want
    ex = field(log, "exclusions")
    exc = np.array(ex[1:], int).reshape(int(ex[0]), 2)
    assert len(system.exclusions[0]) > 0
    assert {tuple(e) for e in exc} == set(zip(system.exclusions[0].tolist(),
                                              system.exclusions[1].tolist()))
    prm = kv(field(log, "params"))
    sp = S.script_params(SCRIPT)
    for k in ("T", "zeta", "h", "a1", "a2", "a3", "a4", "a5", "boxl", "lcell", "ncell"):
        assert float(prm[k]) == sp[k], k
    assert int(prm["nnlup"]) == 10 and int(prm["nup"]) == 50
    assert int(prm["list_mode"]) == 1 and int(prm["dynamics"]) == 0
    assert int(prm["force_terms"]) == 0xF  # random, FENE, angles, vdw (global.cpp:200-202)
    assert int(prm["seed"]) == -100 - 3    # run 3
    assert float(prm["k_bnd"]) == 20.0 and float(prm["R0"]) == 2.0
    # the switches the program flipped, as set_forces would install them
    out = dict(l.split(" ", 1) for l in p.stdout.splitlines() if " " in l)
    terms = [l.split()[1] for l in p.stdout.splitlines() if l.startswith("terms")]
    assert terms == ["15", "14", "2"]
    sets = [int(kv(l.split()[1:])["force_terms"]) for l in log if l.startswith("set_params")]
    assert sets[:3] == [15, 14, 2]
    # results into the 1-based globals
    np.testing.assert_array_equal(np.array(out["force1"].split(), float), [0, 0.25, 0.5])
    np.testing.assert_array_equal(np.array(out["forceN"].split(), float),
                                  [n - 1, n - 1 + 0.25, n - 1 + 0.5])
    np.testing.assert_array_equal(np.array(out["energy"].split(), float),
                                  [1.5, 2.5, 3.5, 4.5, 5.5, 6.5])
    np.testing.assert_array_equal(np.array(out["pos1"].split(), float), [0, 1, 2])
    np.testing.assert_array_equal(np.array(out["uncN"].split(), float),
                                  [10 * (n - 1) + c + 0.5 for c in range(3)])
    np.testing.assert_array_equal(np.array(out["vel2"].split(), float), [-10, -11, -12])
    np.testing.assert_array_equal(np.array(out["output"].split(), float),
                                  [100, 101, 102, 105, 300, 301, 302, 303])
    calls = [l.split()[1] for l in log if l.startswith("call")]
    for name in ("sop_update_neighbor_list", "sop_update_cell_list", "sop_update_pair_list",
                 "sop_force_eval", "sop_energy_eval", "sop_underdamped_iteration",
                 "sop_replica_start", "sop_run_chunk", "sop_replica_outputs", "sop_observables",
                 "sop_replica_get_state", "sop_engine_destroy"):
        assert name in calls, name
    assert calls.count("sop_underdamped_iteration") == 2  # underdamped and overdamped forwards
    assert p.stdout.rstrip().endswith("done")


@needs_ref
@needs_tools
@pytest.mark.parametrize("name", ["sop_engine_create", "sop_replica_add", "sop_update_neighbor_list",
                                  "sop_update_pair_list", "sop_force_eval", "sop_energy_eval",
                                  "sop_underdamped_iteration", "sop_run_chunk",
                                  "sop_replica_get_state"])
def test_backend_stops_on_a_failed_status(name):
    p, log = run_shim(typed_system(), fail=name)
    assert p.returncode == 255, (p.returncode, p.stdout)
    assert ("GPU backend: %s failed: stub failure" % name) in p.stderr
    assert "done" not in p.stdout


@needs_ref
@needs_tools
def test_backend_refuses_close_non_native_candidates():
    """A vdw file listing a non-native pair with |i-j| <= 2 has no image in
    the engine's candidate set: refused with a message, not dropped."""
    system = typed_system()
    exe = make("shim-test")
    with tempfile.TemporaryDirectory() as d:
        inp = S.write_reference_files(system, d, SCRIPT, run=False)
        vdw = os.path.join(d, "vdw.dat")
        lines = open(vdw).read().splitlines()
        head = lines[0].split()
        lines[0] = "%s %s %s %d" % (head[0], head[1], head[2], int(head[3]) + 1)
        lines.append("5 7 9.500000 1 1")
        open(vdw, "w").write("\n".join(lines) + "\n")
        env = dict(os.environ, SOP_STUB_LOG=os.path.join(d, "stub.log"))
        p = subprocess.run([exe, inp], cwd=d, env=env, capture_output=True, text=True, timeout=60)
    assert p.returncode == 255
    assert "|i-j| <= 2" in p.stderr
