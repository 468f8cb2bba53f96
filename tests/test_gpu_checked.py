"""The checked build, libsopgpu_checked.so: the kernels test every partner
index they read from a list row, cell bin, native, bond or angle record
against the bead range of its replica before the gather, and a bad one fails
the call with SOP_ERR_INDEX instead of reading outside the replica (the
GPUs here have no compute-sanitizer).  The GPU parity suites -- every list
mode, bead types and exclusions, minimum images, FP64 precision, 10,000- and
50,000-bead globules, lean and full preparation launches -- run through it in
a child process (SOP_GB300_CHECKED=1): every call must succeed and every
parity check hold as with the default build."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_types.py", "tests/test_gpu_periodic.py",
          "tests/test_gpu_fp64.py", "tests/test_gpu_large.py", "tests/test_gpu_prep.py"]


def child(args, **kw):
    env = dict(os.environ, SOP_GB300_CHECKED="1")
    return subprocess.run([sys.executable] + args, cwd=ROOT, env=env, capture_output=True, text=True,
                          **kw)


def test_child_loads_the_checked_library():
    r = child(["-c", "import sys; sys.path[:0] = ['.', 'sop-cpu_gb300']; "
                     "from sop_gb300 import _lib as L; L.lib(); print(L.LIB_PATH)"], timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().endswith("libsopgpu_checked.so")


def test_parity_suites_on_the_checked_build():
    r = child(["-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider"] + SUITES, timeout=2400)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
