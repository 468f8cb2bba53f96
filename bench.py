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
           CUDA-event duration against the measured HBM copy bandwidth;
           traffic = DRAM bytes per launch of the same kernel on the same
           workload from the recorded ncu capture (caches flushed before the
           captured pass), or null when the kernel source changed since that
           capture; the same achieved GB/s against the L2 read bandwidth
           measured in the run; issue_frac = the kernel's warp instructions
           (recorded capture) over the SMs' issue slots in its live duration.
cpu_baseline  the CPU oracle (the reference algorithm restated in C) on a
           stratified sample of the replicas, all host threads.
served     Poisson arrivals into the continuous-batching server: throughput,
           p50 / p99 latency.
large_system  a 50,000-bead globule: mixed and FP64 throughput, mixed-vs-FP64
           force error and energy drift.
single_system  one 3000-bead chain on its own (the plain single-system
           path): throughput, force error against the oracle every 1000 steps.

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
    ap.add_argument("--md-steps", type=int, default=500)
    ap.add_argument("--autotune", type=int, default=150,
                    help="steps per autotuner trial during warm-up (0 = off)")
    ap.add_argument("--replicas", type=int, default=512)
    ap.add_argument("--lo", type=int, default=30)
    ap.add_argument("--hi", type=int, default=1500)
    ap.add_argument("--list-mode", default="skin", choices=["neighborlist", "skin"])
    ap.add_argument("--skin", type=float, default=3.0)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--full-steps", type=int, default=200000,
                    help="MD steps of every replica in one run after the timed region (0 = skip)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-steps", default="100,10000", help="log-uniform step-count range")
    ap.add_argument("--serve-chunk", type=int, default=100)
    ap.add_argument("--serve-active", type=int, default=2048,
                    help="most requests the server keeps resident (stepped together)")
    ap.add_argument("--large-chains", type=int, default=100,
                    help="single large system: chains x --large-len beads (0 = skip)")
    ap.add_argument("--large-len", type=int, default=500)
    ap.add_argument("--single-len", type=int, default=3000,
                    help="single-system leg: one chain of this many beads")
    ap.add_argument("--single-steps", type=int, default=10000,
                    help="single-system leg: steps, in windows of 1000 (0 = skip)")
    ap.add_argument("--large-steps", type=int, default=2000)
    ap.add_argument("--leg", default="all", choices=["all", "serve", "large", "single"],
                    help="run one secondary leg alone and print its JSON (no headline line)")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_script():
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "0.6"),
            ("set", "nstep", "200000"), ("set", "nup", "1000000"), ("set", "cutofftype", "neighborlist"),
            ("set", "nnlup", "10"), ("set", "boxl", "2000"), ("set", "ncell", "250"), ("set", "run", "1")]


def job_totals(units, seconds, world, device="cpu"):
    """Whole-job figures of a replicas-only run: the units all ranks processed
    (sum) and the job's time (max over ranks)."""
    if world == 1:
        return float(units), float(seconds)
    import torch
    import torch.distributed as dist
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item())


def build_workload(args, rank, synth_many=None):
    """Each rank its own seeded mix (replicas only: no data is shared).
    ``synth_many`` swaps the engine library's generator for the stand-alone
    build of the same source (the reference arm loads no engine code)."""
    from sop_gb300 import systems as S
    systems, temps = S.mixed_batch(args.replicas, args.lo, args.hi, seed=2000 + 100000 * rank,
                                   synth_many=synth_many)
    return systems, temps


def workload_name(args, systems):
    return ("batched replicas: %d chains, N log-uniform %d-%d (%d beads), T 0.4-0.9, zeta 50, "
            "dt 0.05" % (len(systems), args.lo, args.hi, sum(s.nbead for s in systems)))


def default_workload(args):
    """The workload of the recorded capture: 512 chains, N 30-1500, seed 2000."""
    return (args.replicas, args.lo, args.hi) == (512, 30, 1500) and args.list_mode == "skin"


TRAFFIC_RECORD = os.path.join(ROOT, "profiles", "k_step_mix512.md")
KERNEL_SOURCE = os.path.join(ROOT, "sop-cpu_gb300", "csrc", "kernels.cu")


def blob_hash(path):
    """git's blob hash of a file (what `git hash-object` prints)."""
    import hashlib
    data = open(path, "rb").read()
    return hashlib.sha1(b"blob %d\0" % len(data) + data).hexdigest()


def read_capture():
    """From the recorded ncu capture of k_step on the default workload: DRAM
    bytes (read + write) and warp instructions per launch, and the blob hash
    of the kernel source it was captured from.  Values are None when the
    record is missing or was captured from another source than the one
    built here."""
    rec = {"traffic": None, "warp_instructions": None, "source": None}
    try:
        with open(TRAFFIC_RECORD) as f:
            for line in f:
                if line.startswith("traffic:"):
                    rec["traffic"] = int(line.split()[1])
                elif line.startswith("warp instructions:"):
                    rec["warp_instructions"] = int(line.split()[2])
                elif line.startswith("kernels.cu blob:"):
                    rec["source"] = line.split()[2]
    except (OSError, ValueError, IndexError):
        return rec
    try:
        current = blob_hash(KERNEL_SOURCE)
    except OSError:
        current = None
    rec["current"] = current
    if rec["source"] != current:
        rec["traffic"] = rec["warp_instructions"] = None
    return rec


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


PN_PER_KCAL_MOL_A = 69.48


def large_system(args):
    """100 chains x 500 beads in one compact globule (50,000 beads), skin
    lists, noise on: the mixed-precision run and the FP64-precision run (the
    drift reference) side by side in one engine, same seed and noise stream.
    Every --large-steps / 10 steps: each run's mean total energy over the
    block (20 samples), and the force error of the mixed-precision path
    against the FP64 path at the FP64 run's current positions (random term
    off on both).  Throughput of each precision alone over a short window."""
    from sop_gb300 import _lib as L
    from sop_gb300 import systems as S
    from sop_gb300.engine import Engine, make_params
    s = S.synth_globule(3000, args.large_chains, args.large_len)
    n = s.nbead
    steps = args.large_steps
    blocks = 10 if steps >= 10 * 20 else 1
    per = max(1, steps // (blocks * 20))
    sc = workload_script()
    out = {"workload": "%d chains x %d beads, one globule (%d beads), skin lists, T 0.6"
                       % (args.large_chains, args.large_len, n), "steps": per * 20 * blocks}
    det = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
    with Engine(0, max_beads=4 * n + 4096, max_replicas=8, max_list_entries=n * 800) as eng:
        # throughput of each precision alone
        for prec, key in ((L.PREC_MIXED, "mixed"), (L.PREC_FP64, "fp64")):
            r = eng.add(s, make_params(sc, seed=31337, list_mode="skin", skin=2.0, precision=prec))
            eng.run(20)
            eng.run(1000 if prec == L.PREC_MIXED else 200)
            t = eng.timing()[0]
            out[key + "_bead_steps_per_s"] = n * (1000 if prec == L.PREC_MIXED else 200) / (t / 1e3)
            eng.remove(r)
        runs = {key: eng.add(s, make_params(sc, seed=31337, list_mode="skin", skin=2.0, precision=prec))
                for prec, key in ((L.PREC_MIXED, "mixed"), (L.PREC_FP64, "fp64"))}
        # probes in an engine of their own, which never steps
        probes = Engine(0, max_beads=2 * n + 4096, max_replicas=4, max_list_entries=n * 400)
        probe_m = probes.add(s, make_params(sc, force_terms=det, list_mode="skin", skin=2.0))
        probe_d = probes.add(s, make_params(sc, force_terms=det, list_mode="skin", skin=2.0,
                                            precision=L.PREC_FP64))

        def force_error():
            _, x, _ = eng.state(runs["fp64"])
            for p in (probe_m, probe_d):
                probes.set_state(p, x)
                probes.neighbor_list(p)
                probes.pair_list(p)
            fd = probes.force(probe_d)
            return float(np.linalg.norm(probes.force(probe_m) - fd) / np.linalg.norm(fd))

        ferr = [force_error()]
        block_mean = {"mixed": [], "fp64": []}
        block_std = {"mixed": [], "fp64": []}
        t0 = time.perf_counter()
        for _ in range(blocks):
            samples = {"mixed": [], "fp64": []}
            for _ in range(20):
                eng.run(per)
                for key, r in runs.items():
                    samples[key].append(float(eng.energy(r)[5]))
            for key in samples:
                block_mean[key].append(float(np.mean(samples[key])))
                block_std[key].append(float(np.std(samples[key])))
            ferr.append(force_error())
        wall = time.perf_counter() - t0
        status = {key: eng.status(r)[0] for key, r in runs.items()}
        probes.close()
    bm, bd = np.array(block_mean["mixed"]), np.array(block_mean["fp64"])
    # the block means of the two runs: equal within their spread (the runs
    # separate chaotically, so single energies differ by thermal noise)
    se = np.sqrt((np.array(block_std["mixed"]) ** 2 + np.array(block_std["fp64"]) ** 2) / 20)
    out.update({
        "force_rel_err_mixed_vs_fp64": ferr, "force_rel_err_max": max(ferr),
        "check_every_steps": per * 20, "etot_block_mean_mixed": block_mean["mixed"],
        "etot_block_mean_fp64": block_mean["fp64"],
        "etot_block_rel_diff_max": float(np.max(np.abs(bm - bd) / np.abs(bd))),
        "etot_block_diff_over_se_max": float(np.max(np.abs(bm - bd) / np.maximum(se, 1e-30))),
        "etot_drift_rel_mixed": float((bm[-1] - bm[0]) / abs(bm[0])),
        "etot_drift_rel_fp64": float((bd[-1] - bd[0]) / abs(bd[0])),
        "status": status, "wall_s": wall})
    return out


def serve_stream(args, rank):
    """The serving stream: Poisson arrivals at --serve-rate of seeded chains
    (N log-uniform 30-5000 from a pre-generated pool, steps log-uniform in
    --serve-steps, T 0.4-0.9, constant pulling force 0-15 pN on the termini)
    into the continuous-batching server for --serve-seconds."""
    from sop_gb300 import _lib as L
    from sop_gb300 import systems as S
    from sop_gb300.engine import make_params
    from sop_gb300.server import Server
    rng = np.random.default_rng(4000 + 100000 * rank)
    pool_sizes = np.unique(S.loguniform_sizes(4100 + rank, 48, 30, 5000))
    xyzs = L.synth_many([(41000 + k, int(n)) for k, n in enumerate(pool_sizes)])
    pool = [S.system_from_xyz(x) for x in xyzs]
    lo, hi = (float(v) for v in args.serve_steps.split(","))
    nreq = max(1, int(args.serve_rate * args.serve_seconds))
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, nreq))
    target = np.exp(rng.uniform(math.log(30), math.log(5000), nreq))
    pick = np.abs(np.log(pool_sizes)[None, :] - np.log(target)[:, None]).argmin(1)
    steps = np.exp(rng.uniform(math.log(lo), math.log(hi), nreq)).round().astype(int)
    temps = rng.uniform(0.4, 0.9, nreq)
    pulls = rng.uniform(0.0, 15.0, nreq) / PN_PER_KCAL_MOL_A
    params = [make_params(workload_script(), T=float(temps[k]), seed=90_000 + k,
                          list_mode=args.list_mode, skin=args.skin, pull_force=float(pulls[k]))
              for k in range(nreq)]
    srv = Server(0, max_active=args.serve_active, chunk_steps=args.serve_chunk, max_beads=1 << 21,
                 max_replicas=2100, max_list_entries=(1 << 21) * 96)
    # warm-up requests, not timed
    for k in range(8):
        srv.submit(pool[k % len(pool)], 200, params[k])
    while srv.pump():
        pass
    srv.poll()
    t_start = srv.clock()
    done, nxt, pending = [], 0, 0
    while nxt < nreq or pending:
        now = srv.clock() - t_start
        while nxt < nreq and arrivals[nxt] <= now:
            srv.submit(pool[pick[nxt]], int(steps[nxt]), params[nxt])
            nxt += 1
        pending = srv.pump()
        done += srv.poll()
        if pending == 0 and nxt < nreq:
            time.sleep(max(0.0, min(0.005, arrivals[nxt] - (srv.clock() - t_start))))
    done += srv.poll()
    phases = srv.timing()
    srv.close()
    lat = np.array([r["finish"] - r["submit"] for r in done])
    svc = np.array([r["finish"] - r["start"] for r in done])
    que = np.array([r["start"] - r["submit"] for r in done])
    work = sum(r["nbead"] * r["steps"] for r in done)
    span = max(r["finish"] for r in done) - t_start
    offered = float(np.sum(pool_sizes[pick] * steps)) / float(arrivals[-1])
    return {"value": work / span, "unit": UNIT, "requests": len(done), "window_s": float(arrivals[-1]),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "p50_service_s": float(np.percentile(svc, 50)), "p99_service_s": float(np.percentile(svc, 99)),
            "p50_queue_s": float(np.percentile(que, 50)), "p99_queue_s": float(np.percentile(que, 99)),
            "span_s": float(span), "bead_steps": float(work),
            "offered_bead_steps_per_s": offered, "pump_phases_s": phases,
            "errors": int(sum(1 for r in done if r["status"] or r["replica_status"])),
            "stream": "Poisson %.0f req/s for %.0f s, then drained, N log-uniform 30-5000 (pool of %d "
                      "seeded chains), steps log-uniform %g-%g%s, T 0.4-0.9, pull 0-15 pN"
                      % (args.serve_rate, args.serve_seconds, len(pool), lo, hi,
                         "" if (lo, hi) == (1e4, 1e6) else
                         " (the serving configuration's 1e4-1e6 scaled)"),
            "max_active": args.serve_active}


def force_err(eng, r, s):
    """Normwise relative force error of replica r against the CPU oracle (the
    reference's FP64 formulas) at its current state, lists rebuilt there on
    both sides, random term off on both sides; r's parameters are restored."""
    from oracle import oracle as O
    from sop_gb300 import _lib as L
    keep = eng.params(r)
    p = eng.params(r)
    p.force_terms = L.TERM_FENE | L.TERM_ANGLE | L.TERM_VDW
    eng.set_params(r, p)
    eng.neighbor_list(r)
    eng.pair_list(r)
    f = eng.force(r)
    _, x, _ = eng.state(r)
    eng.set_params(r, keep)
    port = O.Port()
    port.set_system(s)
    for _, key, v in workload_script():
        port.command(key, v)
    port.set_coords(0, x)
    port.set_coords(1, x)
    port.set_force_terms(0, 1, 1, 1)
    port.neighbor_list()
    port.pair_list()
    port.force_eval()
    fr = port.coords(3)
    return float(np.linalg.norm(f - fr) / np.linalg.norm(fr))


def force_check(eng, ids, systems, count=4):
    """Force error of sampled replicas against the CPU oracle at their current
    state (random term off on both sides): max normwise relative error."""
    order = np.argsort([s.nbead for s in systems])
    pick = order[np.linspace(0, len(order) - 1, count).round().astype(int)]
    return max(force_err(eng, ids[k], systems[k]) for k in pick)


def single_system(args):
    """One compact chain of --single-len beads (3000, seed 1000) on its own: the
    plain single-system path (one replica, the reference's neighbor-list
    cadence, nnlup 10, underdamped, T 0.6, noise on), the launch shape tuned for
    it during warm-up (--autotune steps per trial; trials are real steps),
    --single-steps steps in windows of 1000; after each window the force at the
    current state against the CPU oracle (FP64 reference formulas), as the
    check every 1000 steps."""
    from sop_gb300 import systems as S
    from sop_gb300.engine import Engine, make_params
    s = S.synth_chain(1000, args.single_len)
    n = s.nbead
    windows = max(1, args.single_steps // 1000)
    with Engine(0, max_beads=max(1 << 14, 2 * n), max_replicas=4, max_list_entries=n * 400) as eng:
        r = eng.add(s, make_params(workload_script(), seed=1000))
        eng.run(50)  # warm
        tuned = None
        if args.autotune > 0:  # launch shape for one replica (its trials are real steps,
            # ~20 us each here, so at least 1000 per trial to rank the shapes)
            report = eng.autotune(max(args.autotune, 1000), shape=True, lists=False)
            tuned = [l for l in report.splitlines() if l.startswith("chosen")]
        total, errs = 0.0, []
        for _ in range(windows):
            eng.run(1000)
            total += eng.timing()[0]
            errs.append(force_err(eng, r, s))
        status = eng.status(r)[0]
    return {"workload": "one compact chain of %d beads, neighbor-list cadence (nnlup 10), T 0.6" % n,
            "steps": 1000 * windows, "bead_steps_per_s": n * 1000 * windows / (total / 1e3),
            "force_rel_err_max": max(errs), "force_checks": len(errs), "status": status,
            "autotuned": tuned}


def measure_l2_gbs(device):
    """L2 read bandwidth of this GPU from the library's probe: a 32 MB buffer
    (L2-resident) read 40 times by one kernel with L1-bypassing 16-byte loads,
    best of five launches."""
    import ctypes as C
    from sop_gb300 import _lib as L
    g = C.c_double()
    L.check(L.lib().sop_probe_l2_read(device, 32 << 20, 40, C.byref(g)), "sop_probe_l2_read")
    return g.value


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
    tuned = None
    if args.autotune > 0:  # its trials are real steps: part of the warm-up
        report = eng.autotune(args.autotune)
        tuned = [l for l in report.splitlines() if l.startswith("chosen")]
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
    units, total_s = job_totals(beads * md * args.steps, total_ms / 1e3, world, "cuda")
    total_ms = total_s * 1e3
    value = units / total_s

    # roofline of the fused step kernel
    step_ms, pro_ms = eng.profile_steps(md)
    cap = read_capture() if default_workload(args) else {"traffic": None, "warp_instructions": None}
    props = torch.cuda.get_device_properties(local)
    clk_mhz = clk.summary().get("sm_mhz") or 2070.0
    issue_frac = (cap["warp_instructions"] / (props.multi_processor_count * 4 * clk_mhz * 1e6 *
                                              step_ms / 1e3)
                  if cap.get("warp_instructions") else None)
    algo = algorithmic_bytes(eng, ids, systems)
    peak, peak_kind = read_peaks()
    achieved = algo / (step_ms / 1e3) / 1e9
    l2_gbs = measure_l2_gbs(local)

    # the batched configuration's whole horizon (--full-steps MD steps of every
    # replica, grouped rebuilds included) in one run call
    full = None
    if args.full_steps > 0:
        eng.run(args.full_steps)
        full_ms = eng.timing()[0]
        bad = sum(1 for r in ids if eng.status(r)[0])
        full = {"md_steps": args.full_steps, "bead_steps": beads * args.full_steps,
                "bead_steps_per_s": beads * args.full_steps / (full_ms / 1e3), "wall_s": full_ms / 1e3,
                "replicas_with_error_status": bad}

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
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.run_host(xin, vin, md, xout, vout)
    e2e_s = time.perf_counter() - t0
    e2e_units, e2e_s = job_totals(beads * md * e2e_steps, e2e_s, world, "cuda")
    e2e = e2e_units / e2e_s

    # the plain one-system-per-launch path over the same mix
    t0 = time.perf_counter()
    plain_ms = 0.0
    for r, s in zip(ids, systems):
        eng.run_plain(r, args.plain_steps)
        plain_ms += eng.timing()[0]
    plain = beads * args.plain_steps / (plain_ms / 1e3)
    ferr = force_check(eng, ids, systems)
    eng.close()
    served = serve_stream(args, rank) if args.serve_seconds > 0 else None
    large = large_system(args) if (args.large_chains > 0 and rank == 0) else None
    single = single_system(args) if (args.single_steps > 0 and rank == 0) else None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair forces / f64 state",
        "data": "synthetic (seeded chains)",
        "config": {"workload": workload_name(args, systems),
                   "md_steps_per_step": md, "list_mode": args.list_mode, "skin": args.skin,
                   "autotuned": tuned,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "flushed (256 MB write) before each timed step; working set is L2-resident within a step"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * nb3 * 8,
                "d2h_bytes_per_step": 2 * nb3 * 8},
        "gpu_launches": int(launches),
        "plain_gpu_path": {"value": plain, "unit": UNIT, "steps": args.plain_steps,
                           "batched_over_plain": value / plain},
        "full_horizon": full,
        "served": served,
        "large_system": large,
        "single_system": single,
        "force_rel_err": ferr,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": cap["traffic"],
                     "traffic_note": ("ncu, caches flushed before the captured pass; captured from "
                                      "kernels.cu blob %s, built from %s" % (cap.get("source"),
                                                                           cap.get("current"))),
                     "issue_frac": issue_frac,
                     "kernel": "k_step (fused force + Langevin)", "kernel_ms": step_ms,
                     "prologue_ms": pro_ms, "algorithmic_bytes_per_launch": algo,
                     "l2": {"peak": l2_gbs, "frac": achieved / l2_gbs,
                            "peak_source": "measured here: sop_probe_l2_read, 32 MB read 40x"}},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(systems, temps, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line))


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as O
    systems, temps = build_workload(args, 0, synth_many=O.synth_many)
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
        "config": {"workload": workload_name(args, systems)},
        "cpu_baseline": dict(cb, value=value),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.leg != "all":
        import torch
        torch.cuda.set_device(0)
        fn = {"serve": lambda: serve_stream(args, 0), "large": lambda: large_system(args),
              "single": lambda: single_system(args)}[args.leg]
        with ClockSampler(0) as clk:
            res = fn()
        res["leg"] = args.leg
        res["clocks"] = clk.summary()
        print(json.dumps(res))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
