"""Continuous batching: requests that arrive while others run are admitted as
slots and memory free up, share the device, and each result equals the same
system run alone.  Tolerance: bit-identical (every per-replica computation is
independent of what else is packed beside it)."""
import numpy as np
import pytest

from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params
from sop_gb300.server import Server

pytestmark = pytest.mark.gpu

PN_PER_KCAL_MOL_A = 69.48  # 1 kcal/mol/A in pN


def script(temp):
    return [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "temp", "%.3f" % temp),
            ("set", "cutofftype", "neighborlist"), ("set", "nnlup", "10"), ("set", "boxl", "2000"),
            ("set", "nup", "100000"), ("set", "run", "1")]


def requests():
    sizes = [40, 150, 700, 1300, 90, 2500, 333]
    steps = [60, 410, 230, 170, 333, 120, 275]
    out = []
    for k, (n, st) in enumerate(zip(sizes, steps)):
        p = make_params(script(0.4 + 0.07 * k), seed=5000 + k, list_mode="skin", skin=2.0,
                        pull_force=(2.0 * k) / PN_PER_KCAL_MOL_A)
        out.append((S.synth_chain(6100 + k, n), st, p))
    return out


def alone(system, nsteps, params):
    with Engine(0, max_beads=1 << 14, max_replicas=4, max_list_entries=1 << 22) as eng:
        r = eng.add(system, params)
        eng.run(nsteps)
        return eng.energy(r), eng.observables(r)


def test_served_results_equal_alone_and_overlap():
    reqs = requests()
    want = [alone(s, st, p) for s, st, p in reqs]
    with Server(0, max_active=16, chunk_steps=50, max_beads=1 << 16, max_replicas=32,
                max_list_entries=1 << 24) as srv:
        ids = [srv.submit(s, st, p) for s, st, p in reqs[:4]]
        srv.pump()
        in_flight = srv.stats()["active"]
        ids += [srv.submit(s, st, p) for s, st, p in reqs[4:]]  # arrive while others run
        results = {}
        for _ in range(1000):
            pending = srv.pump()
            for r in srv.poll():
                results[r["id"]] = r
            if pending == 0:
                break
        for r in srv.poll():
            results[r["id"]] = r
    assert in_flight >= 1
    assert sorted(results) == sorted(ids)
    for k, rid in enumerate(ids):
        r = results[rid]
        assert r["status"] == 0 and r["replica_status"] == 0
        assert r["submit"] <= r["start"] <= r["finish"]
        np.testing.assert_array_equal(r["energy"], want[k][0])
        np.testing.assert_array_equal(r["obs"], want[k][1])
    # the late arrivals were admitted while earlier requests were still running
    late_start = min(results[i]["start"] for i in ids[4:])
    early_finish = max(results[i]["finish"] for i in ids[:4])
    assert late_start < early_finish


def test_admission_waits_for_memory():
    reqs = requests()
    eng = Engine(0, max_beads=1 << 14, max_replicas=4, max_list_entries=1 << 22)
    sizes = [eng.system_bytes(s, p) for s, _, p in reqs]
    eng.close()
    budget = sorted(sizes)[-1] + sorted(sizes)[-2]  # room for about two large systems
    seen = 0
    with Server(0, max_active=16, memory_budget=budget, chunk_steps=40, max_beads=1 << 16,
                max_replicas=32, max_list_entries=1 << 24) as srv:
        ids = [srv.submit(s, st, p) for s, st, p in reqs]
        done = []
        for _ in range(2000):
            pending = srv.pump()
            seen = max(seen, srv.stats()["active"])
            done += srv.poll()
            if pending == 0:
                break
        done += srv.poll()
    assert len(done) == len(reqs)
    assert all(r["status"] == 0 for r in done)
    assert 1 <= seen < len(reqs)
    # at every admission the systems then resident fit the budget
    nbytes = dict(zip(ids, sizes))
    for a in done:
        resident = sum(nbytes[r["id"]] for r in done if r["start"] <= a["start"] < r["finish"])
        assert resident <= budget
