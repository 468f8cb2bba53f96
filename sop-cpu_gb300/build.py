"""Build libsopgpu.so (and the drop-in program sop_gpu.x) in-tree for sm_103a,
and libsopgpu_checked.so: the same library with the kernels' partner-index
checks compiled in (-DSOP_CHECKED; a bad index is reported as SOP_ERR_INDEX).

    python sop-cpu_gb300/build.py            # library + program
    python sop-cpu_gb300/build.py --check    # also print -Xptxas -v resource usage

Translation units compile in parallel; outputs go to sop-cpu_gb300/_build
(objects) and sop-cpu_gb300/lib (the shared library), both git-ignored.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["csrc/kernels.cu", "csrc/engine.cu", "csrc/noalloc.cu", "csrc/autotune.cu",
              "csrc/checkpoint.cu", "csrc/probe.cu"]
CXX_SOURCES = ["csrc/server.cpp", "host/synth.cpp"]
PROGRAM = "host/sop_main.cpp"


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, cwd=HERE, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(HERE, "csrc", h) for h in ("sop_common.cuh", "kernels.cuh", "engine.h")]
    headers.append(os.path.join(ROOT, "include", "sop_gpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
        objs.append(obj)
        if force or verbose_ptxas or _stale(obj, [os.path.join(HERE, src)] + headers):
            cmd = [nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-Xcompiler", "-ffp-contract=off", "-c", src, "-o", obj]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    # the checked kernels (bounds checks on every partner index)
    checked_obj = os.path.join(BUILD, "kernels_checked.o")
    if force or verbose_ptxas or _stale(checked_obj, [os.path.join(HERE, "csrc/kernels.cu")] + headers):
        jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                     "-Xcompiler", "-ffp-contract=off", "-DSOP_CHECKED", "-c",
                                     "csrc/kernels.cu", "-o", checked_obj])
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cpp", ".o"))
        objs.append(obj)
        if force or _stale(obj, [os.path.join(HERE, src)] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I/usr/local/cuda/include", "-c", src, "-o", obj])
    logs = []
    with ThreadPoolExecutor(max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    lib = os.path.join(LIBDIR, "libsopgpu.so")
    if force or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    lib_checked = os.path.join(LIBDIR, "libsopgpu_checked.so")
    objs_checked = [checked_obj if o.endswith(os.sep + "kernels.o") else o for o in objs]
    if force or _stale(lib_checked, objs_checked):
        _run([nvcc] + ARCH + ["-shared", "-o", lib_checked] + objs_checked + ["-lcudart"])
    prog_src = os.path.join(HERE, PROGRAM)
    if os.path.exists(prog_src):
        prog = os.path.join(LIBDIR, "sop_gpu.x")
        if force or _stale(prog, [prog_src, lib]):
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", prog, prog_src,
                  "-L" + LIBDIR, "-lsopgpu", "-Wl,-rpath,$ORIGIN"])
    return "\n".join(l for l in logs if l.strip())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true", help="print -Xptxas -v resource usage")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    out = build(verbose_ptxas=a.check, force=a.force)
    if out:
        print(out)
    print("built", os.path.join(LIBDIR, "libsopgpu.so"))


if __name__ == "__main__":
    sys.exit(main())
