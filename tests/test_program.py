"""sop_gpu.x, the reference program's command-line drop-in: the same input
script and data files in, the same update.out rows and coordinate files out.
Against sop.x's own output for a T = 0 (steepest-descent) run, carried by the
golden fixtures: rows within 1e-5 relative (2e-6 absolute, the printed
precision), final coordinates and every trajectory frame within 1e-5 A.
The fixtures include a chain of bead types 1 and 2 whose vdw file leaves out
a quarter of the non-native candidates."""
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

from sop_gb300 import systems as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "sop-cpu_gb300", "lib", "sop_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sop_golden_N*.npz")) +
                glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sop_golden_types_N*.npz")))


def golden_script(temp="0.0", nstep=100, nup=50):  # as tests/golden/make_golden.py
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", temp),
            ("set", "nstep", str(nstep)), ("set", "nup", str(nup)),
            ("set", "cutofftype", "neighborlist"), ("set", "nnlup", "10"), ("set", "boxl", "500"),
            ("set", "ncell", "62.5"), ("set", "run", "1")]


def system_from_golden(g):
    """The fixture's system; sop_golden_types_* add bead types 1/2 and the
    candidates their vdw file leaves out."""
    typed = "bead_type" in g.files
    return S.System(xyz=g["xyz"], bonds=(g["ib"], g["jb"], g["r0"]),
                    angles=(g["ia"], g["ja"], g["ka"], g["a0"]),
                    natives=(g["in_"], g["jn"], g["rn"]),
                    bead_type=g["bead_type"] if typed else np.ones(len(g["xyz"]), np.int32),
                    exclusions=(g["ie"], g["je"]) if typed else None)


def test_program_usage():
    if not os.path.exists(EXE):
        pytest.skip("sop_gpu.x not built")
    p = subprocess.run([EXE], capture_output=True, text=True)
    assert p.returncode == 1 and "Usage" in p.stderr


def rewrite(path, edit):
    lines = open(path).read().splitlines(keepends=True)
    open(path, "w").write("".join(edit(lines)))


# Bad input, refused while the files are read (before any device call): the
# program names the file and the entry and exits 1.
BAD_INPUTS = {
    "missing file": ("bonds.dat", None, "cannot open"),
    "truncated init": ("init.dat", lambda L: L[:-3], "missing (the header declares more)"),
    "bead index 0 in vdw": ("vdw.dat", lambda L: L[:1] + ["0 5 4.0 1 1\n"] + L[2:], "bead index out of range"),
    "negative bead in bonds": ("bonds.dat", lambda L: L[:1] + ["-3 2 3.8\n"] + L[2:], "bead index out of range"),
    "huge bead in angles": ("angles.dat", lambda L: L[:1] + ["1 2 99999999 0\n"] + L[2:],
                            "bead index out of range"),
    "short vdw entry": ("vdw.dat", lambda L: L[:1] + ["4 9 5.0\n"] + L[2:], "fewer than 5 fields"),
}


@pytest.mark.parametrize("case", sorted(BAD_INPUTS))
def test_program_refuses_bad_input(case):
    if not os.path.exists(EXE):
        pytest.skip("sop_gpu.x not built")
    fname, edit, message = BAD_INPUTS[case]
    system = S.synth_chain(4242, 40)
    with tempfile.TemporaryDirectory() as d:
        inp = S.write_reference_files(system, d, golden_script(), run=True)
        path = os.path.join(d, fname)
        if edit is None:
            os.remove(path)
        else:
            rewrite(path, edit)
        p = subprocess.run([EXE, inp], cwd=d, capture_output=True, text=True, timeout=120)
    assert p.returncode == 1, (p.returncode, p.stderr)
    assert message in p.stderr, p.stderr


def test_program_refuses_run_without_coordinates():
    if not os.path.exists(EXE):
        pytest.skip("sop_gpu.x not built")
    with tempfile.TemporaryDirectory() as d:
        inp = os.path.join(d, "input")
        open(inp, "w").write("set temp 0.6;\nrun;\n")
        p = subprocess.run([EXE, inp], cwd=d, capture_output=True, text=True, timeout=120)
    assert p.returncode == 1 and "no initial coordinates" in p.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_program_matches_reference_program(path):
    g = np.load(path)
    system = system_from_golden(g)
    with tempfile.TemporaryDirectory() as d:
        inp = S.write_reference_files(system, d, golden_script(), run=True)
        p = subprocess.run([EXE, inp], cwd=d, capture_output=True, text=True, timeout=300)
        assert p.returncode == 0, p.stderr
        rows = np.array([list(map(float, l.split())) for l in open(os.path.join(d, "update.out"))])
        unc = np.loadtxt(os.path.join(d, "unccoord.out"))[:, 1:]
        traj = np.loadtxt(os.path.join(d, "traj.bin"))
        traj_unc = np.loadtxt(os.path.join(d, "traj_uncorrected.bin"))
    want = g["sd_update"]
    assert rows.shape == want.shape
    np.testing.assert_array_equal(rows[:, 0], want[:, 0])          # istep
    np.testing.assert_allclose(rows[:, 1:], want[:, 1:], rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(unc, g["sd_unc"], rtol=0, atol=1e-5)
    # record_traj frames: the start (printed from the same input, so equal) and one per nup
    n = len(g["xyz"])
    assert traj.shape == g["sd_traj"].shape and traj_unc.shape == g["sd_traj_unc"].shape
    np.testing.assert_array_equal(traj_unc[:n], g["sd_traj_unc"][:n])
    np.testing.assert_allclose(traj_unc, g["sd_traj_unc"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(traj, g["sd_traj"], rtol=0, atol=1e-5)


@pytest.mark.gpu
def test_program_restart_continues_the_run():
    """`set restart on` (sop.cpp:132-136): a run of 400 steps equals a run of
    200 steps continued from its unccoord.out / veloc.out by a second run with
    istep_restart 200 -- the same update.out step numbers, energies and final
    coordinates within the files' printed precision (T = 0, deterministic).
    A restart whose coordinate file is missing is refused."""
    system = S.synth_chain(4343, 60)

    def run(d, nstep, restart=False):
        scr = golden_script(nstep=nstep, nup=100)
        if restart:
            scr = scr[:-1] + [("set", "restart", "on"), ("set", "istep_restart", "200")] + scr[-1:]
        inp = S.write_reference_files(system, d, scr, run=True)
        return subprocess.run([EXE, inp], cwd=d, capture_output=True, text=True, timeout=300)

    def rows(d):
        return np.array([list(map(float, l.split())) for l in open(os.path.join(d, "update.out"))])

    with tempfile.TemporaryDirectory() as a, tempfile.TemporaryDirectory() as b, \
            tempfile.TemporaryDirectory() as c:
        assert run(a, 200).returncode == 0
        p = run(b, 400, restart=True)  # no coordinate files yet
        assert p.returncode == 1 and "restart: cannot read" in p.stderr, p.stderr
        for f in ("unccoord.out", "veloc.out"):
            open(os.path.join(b, f), "w").write(open(os.path.join(a, f)).read())
        os.remove(os.path.join(b, "update.out")) if os.path.exists(os.path.join(b, "update.out")) else None
        p = run(b, 400, restart=True)
        assert p.returncode == 0, p.stderr
        assert run(c, 400).returncode == 0
        rb, rc = rows(b), rows(c)
        xb = np.loadtxt(os.path.join(b, "unccoord.out"))[:, 1:]
        xc = np.loadtxt(os.path.join(c, "unccoord.out"))[:, 1:]
    np.testing.assert_array_equal(rb[:, 0], [300.0, 400.0])
    np.testing.assert_allclose(rb, rc[-2:], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(xb, xc, rtol=0, atol=1e-4)
