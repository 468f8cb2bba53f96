"""Benchmark: bead-steps/s of the batched SOP engine on one GB300.

Workload (the batched-replica configuration): 512 seeded chains with bead
counts log-uniform in [30, 1500], temperatures uniform in [0.4, 0.9], the
SOP force field of the reference (FENE k=20 R0=2, native LJ, non-native
repulsion sigma=3.8, i,i+2 soft sphere), underdamped Langevin zeta=50,
dt=0.05, pair list filtered at 2.5x every step.  Synthetic seeded inputs
stand in for real structures (no public dataset is named).

A bench "step" is one block of --md-steps MD steps over every replica.
value      bead-steps/s, device-timed (CUDA events on the engine stream),
           inputs resident in HBM; L2 flushed (256 MB write) before each step.
e2e        the same metric through sop_run_host: every step uploads all
           positions/velocities from pinned host memory, runs, downloads them.
plain      the plain one-system-per-launch GPU path (no graph, no batching)
           over the same mix, for the batched/plain ratio.
roofline   the fused step kernel: algorithmic bytes per launch over its
           CUDA-event duration against MEASURED_PEAKS.json hbm_gbs.
cpu_baseline  the CPU oracle (the reference algorithm restated in C) on a
           stratified sample of the replicas, all host threads.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "sop-cpu_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "bead-steps/s batched+served vs plain GPU path (1 GB300); p50/p99 latency; F err<1e-5"
UNIT = "bead-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--md-steps", type=int, default=100)
    ap.add_argument("--replicas", type=int, default=512)
    ap.add_argument("--lo", type=int, default=30)
    ap.add_argument("--hi", type=int, default=1500)
    ap.add_argument("--list-mode", default="skin", choices=["neighborlist", "skin"])
    ap.add_argument("--skin", type=float, default=2.0)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_script():
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "200000"), ("set", "nup", "1000000"), ("set", "cutofftype", "neighborlist"),
            ("set", "nnlup", "10"), ("set", "boxl", "2000"), ("set", "ncell", "250"), ("set", "run", "1")]


def build_workload(args, rank):
    from sop_gb300 import systems as S
    systems, temps = S.mixed_batch(args.replicas, args.lo, args.hi, seed=2000 + 100000 * rank)
    return systems, temps


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(systems, temps, seconds, threads=None):
    """The oracle port (reference algorithm: explicit candidate lists, 3.2x
    neighbor list every 10 steps, 2.5x pair list every step) on a stratified
    sample of the replicas; all host threads; bead-steps/s of the sample."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    order = np.argsort([s.nbead for s in systems])
    pick = order[np.linspace(0, len(order) - 1, min(2 * threads, len(order))).round().astype(int)]
    ports = []
    for k in pick:
        p = O.Port()
        p.set_system(systems[k])
        for _, key, v in workload_script():
            p.command(key, v)
        p.set_param("T", float(temps[k]))
        p.setup(True)
        ports.append(p)
    beads = sum(systems[k].nbead for k in pick)
    # size the step count so the sample takes about `seconds`
    t1 = O.run_many(ports, 10, threads)
    nsteps = max(10, int(10 * seconds / max(t1, 1e-3)))
    wall = O.run_many(ports, nsteps, threads)
    return {"value": beads * nsteps / wall, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of %d replicas (stratified by size, %d beads), %d steps, %.1f s wall"
                      % (len(pick), len(systems), beads, nsteps, wall)}


def make_engine(systems, temps, args):
    from sop_gb300 import _lib as L
    from sop_gb300.engine import Engine, make_params
    nb = sum(s.nbead for s in systems)
    eng = Engine(0, max_beads=max(1 << 16, int(nb * 1.2)), max_replicas=len(systems) + 16,
                 max_list_entries=int(nb * 160))
    ids = []
    for k, (s, T) in enumerate(zip(systems, temps)):
        p = make_params(workload_script(), T=float(T), seed=77_000 + k,
                        list_mode=args.list_mode, skin=args.skin)
        ids.append(eng.add(s, p))
    return eng, ids


def algorithmic_bytes(eng, ids, systems):
    """Bytes per fused step over all replicas: 96 N (FP64 positions and
    velocity state read + write) + 12 P_att + 8 P_rep (pair-list entries) +
    8 N_bond + 8 N_ang; pair counts from the current pair lists."""
    tot = 0
    for r, s in zip(ids, systems):
        p_att = len(eng.pairs(r, 2)[0])
        p_rep = len(eng.pairs(r, 3)[0])
        tot += 96 * s.nbead + 12 * p_att + 8 * p_rep + 8 * len(s.bonds[0]) + 8 * len(s.angles[0])
    return tot


def flush_l2():
    import torch
    buf = getattr(flush_l2, "buf", None)
    if buf is None:
        buf = flush_l2.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    buf.fill_(1.0)
    torch.cuda.synchronize()


def run_gb300(args):
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    systems, temps = build_workload(args, rank)
    eng, ids = make_engine(systems, temps, args)
    beads = sum(s.nbead for s in systems)
    md = args.md_steps
    for _ in range(args.warmup):
        eng.run(md)
    # timed: K steps, L2 flushed before each, device time by CUDA events
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = eng.launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush_l2()
            eng.run(md)
            times.append(eng.timing()[0])
    launches = eng.launches() - l0  # every kernel the engine launched in the timed region
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = beads * md * args.steps * world / (total_ms / 1e3)

    # roofline of the fused step kernel
    step_ms, pro_ms = eng.profile_steps(md)
    algo = algorithmic_bytes(eng, ids, systems)
    peak, peak_kind = read_peaks()
    achieved = algo / (step_ms / 1e3) / 1e9

    # end to end through the host-buffer C call
    nb3 = 3 * beads
    xin = torch.empty(nb3, dtype=torch.float64, pin_memory=True).numpy()
    vin = torch.empty(nb3, dtype=torch.float64, pin_memory=True).numpy()
    xout = torch.empty(nb3, dtype=torch.float64, pin_memory=True).numpy()
    vout = torch.empty(nb3, dtype=torch.float64, pin_memory=True).numpy()
    o = 0
    for r, s in zip(ids, systems):
        _, x, v = eng.state(r)
        xin[o:o + 3 * s.nbead] = x.ravel()
        vin[o:o + 3 * s.nbead] = v.ravel()
        o += 3 * s.nbead
    e2e_steps = max(2, args.steps // 2)
    eng.run_host(xin, vin, md, xout, vout)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.run_host(xin, vin, md, xout, vout)
    e2e_s = time.perf_counter() - t0
    e2e = beads * md * e2e_steps * world / e2e_s

    # the plain one-system-per-launch path over the same mix
    t0 = time.perf_counter()
    plain_ms = 0.0
    for r, s in zip(ids, systems):
        eng.run_plain(r, args.plain_steps)
        plain_ms += eng.timing()[0]
    plain = beads * args.plain_steps / (plain_ms / 1e3)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair forces / f64 state",
        "data": "synthetic (seeded chains)",
        "config": {"workload": "batched replicas: %d chains, N log-uniform %d-%d (%d beads), "
                               "T 0.4-0.9, zeta 50, dt 0.05" % (len(systems), args.lo, args.hi, beads),
                   "md_steps_per_step": md, "list_mode": args.list_mode, "skin": args.skin,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "flushed (256 MB write) before each timed step; working set is L2-resident within a step"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * nb3 * 8,
                "d2h_bytes_per_step": 2 * nb3 * 8},
        "gpu_launches": int(launches),
        "plain_gpu_path": {"value": plain, "unit": UNIT, "steps": args.plain_steps,
                           "batched_over_plain": value / plain},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                     "kernel": "k_step (fused force + Langevin)", "kernel_ms": step_ms,
                     "prologue_ms": pro_ms, "algorithmic_bytes_per_launch": algo},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(systems, temps, args.cpu_seconds)
    eng.close()
    if rank == 0:
        print(json.dumps(line))


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    systems, temps = build_workload(args, 0)
    threads = os.cpu_count() or 1
    per_step = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    vals = []
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(systems, temps, per_step, threads)
        if k >= args.warmup:
            vals.append(cb["value"])
    value = float(np.mean(vals))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded chains)", "impl": "reference",
        "config": {"workload": "batched replicas: %d chains, N log-uniform %d-%d, T 0.4-0.9, "
                               "zeta 50, dt 0.05" % (len(systems), args.lo, args.hi)},
        "cpu_baseline": dict(cb, value=value),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
