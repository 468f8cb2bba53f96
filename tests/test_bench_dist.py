"""The replicas-only multi-GPU logic of bench.py on CPU: two gloo ranks
(127.0.0.1) each take their own seeded mix, and the whole-job figures are the
sum of the units over ranks and the max of their times."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "sop-cpu_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    class Args:
        replicas, lo, hi = 6, 30, 120
    systems, _ = bench.build_workload(Args, rank)
    beads = sum(s.nbead for s in systems)
    units, secs = bench.job_totals(beads * 10, 1.0 + rank, world)
    out.put((rank, beads, units, secs, systems[0].xyz[0].tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_sum_units_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (_, b0, u0, t0, x0), (_, b1, u1, t1, x1) = res
    assert u0 == u1 == float(10 * (b0 + b1))  # every rank sees the job's total
    assert t0 == t1 == 2.0                     # and the slowest rank's time
    assert x0 != x1                            # each rank its own seeded mix
