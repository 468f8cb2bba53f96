"""Test infrastructure: the CPU restatement (oracle/sop_oracle.c) timed against
the reference program itself (oracle/_ref/sop.x, built from the reference
tree with its own Makefile flags) on the same inputs, one core each.

Sample: replicas of the batched-replica workload (512 chains, N log-uniform
30-1500, seed 2000, T uniform 0.4-0.9), stratified by size; the reference
cadence (neighbor list 3.2x every 10 steps, pair list 2.5x every step,
zeta 50, dt 0.05).  For sop.x the step loop alone is timed as
wall(nstep) - wall(0) of two runs of the program on the same files (loading
and set-up cancel); for the restatement, a timer around its step loop.

    make -C oracle port synth ref && python oracle/time_reference.py [--steps 1000]

Prints one JSON line: per replica and in total, bead-steps/s of each, and
their ratio.  Runs where the reference tree was built (oracle/_ref).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory would shadow the oracle package
sys.path = [ROOT, os.path.join(ROOT, "sop-cpu_gb300")] + [
    p for p in sys.path if os.path.abspath(p or ".") != HERE]

from oracle import oracle as O  # noqa: E402
from sop_gb300 import systems as S  # noqa: E402


def script(temp, nstep):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "%.6f" % temp),
            ("set", "nstep", str(nstep)), ("set", "nup", str(max(nstep, 1) * 10)),
            ("set", "cutofftype", "neighborlist"), ("set", "nnlup", "10"),
            ("set", "boxl", "2000"), ("set", "ncell", "250"), ("set", "run", "1")]


def time_program(system, temp, nstep, d):
    """Wall seconds of sop.x on the system's files for nstep steps."""
    path = S.write_reference_files(system, d, script(temp, nstep), run=True)
    t0 = time.perf_counter()
    subprocess.run([O.REF_EXE, path], cwd=d, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    return time.perf_counter() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--sample", type=int, default=8)
    a = ap.parse_args()
    if not os.path.exists(O.REF_EXE):
        sys.exit("oracle/_ref/sop.x not built (make -C oracle ref)")
    systems, temps = S.mixed_batch(512, 30, 1500, seed=2000, synth_many=O.synth_many)
    order = np.argsort([s.nbead for s in systems])
    pick = order[np.linspace(0, len(order) - 1, a.sample).round().astype(int)]
    rows = []
    for k in pick:
        s, T = systems[k], float(temps[k])
        with tempfile.TemporaryDirectory() as d:
            w0 = time_program(s, T, 0, d)
            w1 = time_program(s, T, a.steps, d)
        ref_s = max(w1 - w0, 1e-9)
        p = O.Port()
        p.set_system(s)
        for _, key, v in script(T, a.steps):
            p.command(key, v)
        p.setup(True)
        port_s = O.run_many([p], a.steps, 1)
        rows.append({"replica": int(k), "nbead": s.nbead, "ref_s": ref_s, "port_s": port_s,
                     "ref_bead_steps_per_s": s.nbead * a.steps / ref_s,
                     "port_bead_steps_per_s": s.nbead * a.steps / port_s})
    beads = sum(r["nbead"] for r in rows)
    tot_ref = sum(r["ref_s"] for r in rows)
    tot_port = sum(r["port_s"] for r in rows)
    print(json.dumps({
        "steps": a.steps, "replicas": len(rows), "beads": beads,
        "ref_bead_steps_per_s": beads * a.steps / tot_ref,
        "port_bead_steps_per_s": beads * a.steps / tot_port,
        "port_over_ref": tot_ref / tot_port, "cores": 1,
        "host": os.uname().machine, "rows": rows}))


if __name__ == "__main__":
    main()
