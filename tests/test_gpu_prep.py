"""The lean preparation launch.  A step's k_prep skips its work-queue phase
when the previous step flagged no possible work for any replica (no skin
trigger, output step, pending observables or cadence build).  Against the same
engine with the lean path off (every k_prep runs its queue): positions,
velocities, output-step energies, observables and status bit-identical, over
every list mode, output cadences that do and do not divide the graph length,
overdamped dynamics, noise, and run windows that end at different steps; and
no lean launch ever found queued work (the fallback counter stays 0)."""
import ctypes as C

import numpy as np
import pytest

from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu


def script(mode="neighborlist", nnlup="10", nup="7", dyn=None):
    s = [("set", "zeta", "50"), ("set", "t_step", "0.05")]
    if dyn:
        s.append(("set", "dynamics", dyn))
    return s + [("set", "temp", "0.7"), ("set", "nstep", "1000"), ("set", "nup", nup),
                ("set", "cutofftype", mode), ("set", "nnlup", nnlup), ("set", "boxl", "500"),
                ("set", "ncell", "62.5"), ("set", "run", "1")]


CASES = [  # (beads, script, extra params)
    (60, script("neighborlist", "10", "7"), {}),
    (140, script("celllist", "3", "11"), {}),
    (300, script("neighborlist", "10", "1000"), {"list_mode": "skin", "skin": 1.0}),
    (90, script("neighborlist", "10", "25"), {"list_mode": "skin", "skin": 0.5}),
    (500, script("neighborlist", "1", "13"), {}),
    (75, script("neighborlist", "5", "9", dyn="overdamped"), {}),
    (120, script("neighborlist", "10", "6"), {"list_mode": "none"}),
    (800, script("neighborlist", "10", "1000"), {"list_mode": "skin", "skin": 2.0}),
]


def outputs(e, r):
    en, ob = (C.c_double * 6)(), (C.c_double * 5)()
    L.check(L.lib().sop_replica_outputs(e.h, r, en, ob), "sop_replica_outputs")
    return np.array(en[:]), np.array(ob[:])


def snapshot(e, ids):
    out = []
    for r in ids:
        _, x, v = e.state(r)
        en, ob = outputs(e, r)
        out.append((x, v, en, ob, e.status(r)))
    return out


def build(lean):
    e = Engine(0, max_beads=1 << 15, max_replicas=16, max_list_entries=1 << 22, graph_steps=8,
               lean_prep=0 if lean else -1)
    ids = [e.add(S.synth_chain(6100 + k, n), make_params(sc, seed=610 + k, **kw))
           for k, (n, sc, kw) in enumerate(CASES)]
    return e, ids


def compare(a, b):
    for (xa, va, ea, oa, sa), (xb, vb, eb, ob, sb) in zip(a, b):
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(va, vb)
        np.testing.assert_array_equal(ea, eb)
        np.testing.assert_array_equal(oa, ob)
        assert sa == sb and sa[0] == 0


def test_lean_prep_equals_full_prep_batched():
    res = {}
    for lean in (True, False):
        e, ids = build(lean)
        with e:
            snaps = []
            for n in (203, 57, 5):  # graph replays, graph tails, host work between runs
                e.run(n)
                snaps.append(snapshot(e, ids))
            res[lean] = (snaps, e.prep_fallbacks())
    for sa, sb in zip(res[True][0], res[False][0]):
        compare(sa, sb)
    assert res[True][1] == 0 and res[False][1] == 0


def test_lean_prep_equals_full_prep_run_windows():
    windows = [37, 160, 91, 64, 23, 130, 77, 101]
    res = {}
    for lean in (True, False):
        e, ids = build(lean)
        with e:
            for r, w in zip(ids, windows):
                L.check(L.lib().sop_replica_start(e.h, r, w), "sop_replica_start")
            fin = (C.c_int * 16)()
            nfin = C.c_int()
            done = []
            for _ in range(20):  # chunks of 17 steps: windows close mid-chunk
                L.check(L.lib().sop_run_chunk(e.h, 17, fin, 16, C.byref(nfin)), "sop_run_chunk")
                done += list(fin[:nfin.value])
            assert sorted(done) == sorted(ids)
            res[lean] = (snapshot(e, ids), e.prep_fallbacks())
    compare(res[True][0], res[False][0])
    assert res[True][1] == 0
