"""The SOP-CPU-side GPU backend (sop-cpu_gb300/integration/gpu_backend.cpp):
it compiles against the reference's own headers with -Wall -Werror and links
with the reference's globals and libsopgpu.so, so every reference global it
reads and every C-ABI call it makes resolves; the linked program defines the
reference's entry points (update_neighbor_list, update_cell_list,
update_pair_list, force_eval, energy_eval) with the reference's C++
signatures.  No GPU calls.  Skipped where the reference tree is absent."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIR = os.path.join(ROOT, "sop-cpu_gb300", "integration")
LIB = os.path.join(ROOT, "sop-cpu_gb300", "lib", "libsopgpu.so")
REF = os.environ.get("REF", "/root/reference")


def test_backend_compiles_and_links_against_the_reference():
    if not os.path.exists(os.path.join(REF, "global.h")):
        pytest.skip("reference tree not present")
    if not os.path.exists(LIB):
        pytest.skip("libsopgpu.so not built")
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no make / g++")
    p = subprocess.run(["make", "-C", DIR, "check", "REF=" + REF], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    exe = os.path.join(DIR, "_build", "gpu_backend_check")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "10 entry points" in out.stdout
    if shutil.which("nm"):
        syms = subprocess.run(["nm", "-C", os.path.join(DIR, "_build", "gpu_backend.o")],
                              capture_output=True, text=True).stdout
        for f in ("update_neighbor_list()", "update_cell_list()", "update_pair_list()",
                  "force_eval()", "energy_eval()"):
            assert " T " + f in syms, f
