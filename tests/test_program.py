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
