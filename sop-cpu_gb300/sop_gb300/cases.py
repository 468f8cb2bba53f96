"""Small fixed workloads for profiling the kernels (ncu launch lists and
single-kernel captures).  Run as

    PYTHONPATH=sop-cpu_gb300 python -m sop_gb300.cases mix --steps 3
    PYTHONPATH=sop-cpu_gb300 python -m sop_gb300.cases build --steps 4
    PYTHONPATH=sop-cpu_gb300 python -m sop_gb300.cases mixbuild --steps 3
    PYTHONPATH=sop-cpu_gb300 python -m sop_gb300.cases globule --steps 3

mix      512 replicas, N log-uniform 30-1500 (seed 2000), T 0.4-0.9, skin lists
         (3.0 A): the batched step workload; one CUDA-graph-free batched step
         per --steps.
mixwide  the same with 384 replicas, N log-uniform 30-5000: the serving mix,
         74 replicas above the stage limit (the CTA queue on, unless
         --queue-blocks -1).
build    one 1500-bead chain, neighbor list rebuilt before every step (nnlup 1):
         every prologue is a full list build.
mixbuild the mix with the reference's neighbor-list cadence at nnlup 1: every
         replica rebuilds its lists before every step (the load of a grouped
         skin rebuild of the whole batch).
globule  100 chains x 500 beads in one compact globule (50,000 beads), skin
         lists: the large single-system workload.

Each case prints the per-kernel CUDA-event times of sop_profile_steps_ex.
"""
from __future__ import annotations

import argparse
import sys

from . import systems as S
from .engine import Engine, make_params

WORKLOAD_SCRIPT = [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
                   ("set", "nstep", "200000"), ("set", "nup", "1000000"),
                   ("set", "cutofftype", "neighborlist"), ("set", "nnlup", "10"),
                   ("set", "boxl", "2000"), ("set", "ncell", "250"), ("set", "run", "1")]


def mix_engine(count=512, lo=30, hi=1500, skin=3.0, every_step=False, **cfg):
    systems, temps = S.mixed_batch(count, lo, hi, seed=2000)
    nb = sum(s.nbead for s in systems)
    eng = Engine(0, max_beads=max(1 << 16, int(nb * 1.3)), max_replicas=count + 16,
                 max_list_entries=int(nb * 200), **cfg)
    script = [c if c[1] != "nnlup" else ("set", "nnlup", "1") for c in WORKLOAD_SCRIPT]
    for k, (s, T) in enumerate(zip(systems, temps)):
        if every_step:
            p = make_params(script, T=float(T), seed=77_000 + k)
        else:
            p = make_params(WORKLOAD_SCRIPT, T=float(T), seed=77_000 + k, list_mode="skin", skin=skin)
        eng.add(s, p)
    return eng, systems


def build_engine(n=1500):
    s = S.synth_chain(9000 + n, n)
    eng = Engine(0, max_beads=max(1 << 14, 2 * n), max_replicas=8, max_list_entries=n * 400)
    sc = [c if c[1] != "nnlup" else ("set", "nnlup", "1") for c in WORKLOAD_SCRIPT]
    eng.add(s, make_params(sc, seed=5))
    return eng, [s]


def globule_engine(nchain=100, chain_len=500, skin=2.0):
    s = S.synth_globule(3000, nchain, chain_len)
    n = s.nbead
    eng = Engine(0, max_beads=n + 1024, max_replicas=4, max_list_entries=n * 200)
    eng.add(s, make_params(WORKLOAD_SCRIPT, seed=3000, list_mode="skin", skin=skin))
    return eng, [s]


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case", choices=("mix", "mixwide", "mixbuild", "build", "globule"))
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warm", type=int, default=10, help="batched steps before the profiled ones")
    ap.add_argument("--tune", type=int, default=0,
                    help="autotune with this many steps per trial before profiling")
    ap.add_argument("--queue-blocks", type=int, default=0,
                    help="the engine's queue_blocks (0: automatic, <0: fixed CTA blocks)")
    a = ap.parse_args(argv)
    q = a.queue_blocks
    eng, systems = {"mix": lambda: mix_engine(queue_blocks=q),
                    "mixwide": lambda: mix_engine(count=384, lo=30, hi=5000, queue_blocks=q),
                    "mixbuild": lambda: mix_engine(every_step=True, queue_blocks=q),
                    "build": build_engine, "globule": globule_engine}[a.case]()
    if a.warm:
        eng.run(a.warm)
    if a.tune:
        t = eng.profile_split(a.steps)
        print("untuned: " + " ".join("%s_ms=%.4f" % kv for kv in t.items()))
        print(eng.autotune(a.tune), end="")
    t = eng.profile_split(a.steps)
    print("case=%s replicas=%d beads=%d prologue_ms=%.4f build_ms=%.4f step_ms=%.4f"
          % (a.case, len(systems), sum(s.nbead for s in systems), t["prologue"], t["build"],
             t["step"]))
    eng.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
