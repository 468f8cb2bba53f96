"""Python handle on the continuous-batching server (sop_server_* in the C ABI)."""
from __future__ import annotations

import ctypes as C

from . import _lib as L
from .engine import _Desc, make_params


class Server:
    def __init__(self, device=0, max_active=1024, memory_budget=0, chunk_steps=200, **engine_cfg):
        cfg = L.ServerConfig()
        cfg.engine = L.default_engine_config()
        cfg.engine.device = device
        for k, v in engine_cfg.items():
            setattr(cfg.engine, k, v)
        cfg.max_active = max_active
        cfg.memory_budget = memory_budget
        cfg.chunk_steps = chunk_steps
        h = C.c_void_p()
        L.check(L.lib().sop_server_create(C.byref(cfg), C.byref(h)), "sop_server_create")
        self.h = h

    def close(self):
        if self.h:
            L.lib().sop_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, system, nsteps, params=None, vel=None, **kw) -> int:
        d = _Desc(system, params if params is not None else make_params(**kw), vel)
        rid = C.c_int64()
        L.check(L.lib().sop_server_submit(self.h, C.byref(d.desc), int(nsteps), C.byref(rid)),
                "sop_server_submit")
        return rid.value

    def pump(self) -> int:
        pending = C.c_int()
        L.check(L.lib().sop_server_pump(self.h, C.byref(pending)), "sop_server_pump")
        return pending.value

    def poll(self, cap=4096):
        buf = (L.RequestResult * cap)()
        n = C.c_int()
        L.check(L.lib().sop_server_poll(self.h, buf, cap, C.byref(n)), "sop_server_poll")
        out = []
        for k in range(n.value):
            r = buf[k]
            out.append(dict(id=r.request_id, status=r.status, replica_status=r.replica_status,
                            nbead=r.nbead, steps=r.steps, submit=r.submit_s, start=r.start_s,
                            finish=r.finish_s, energy=list(r.energy), obs=list(r.observables)))
        return out

    def clock(self) -> float:
        t = C.c_double()
        L.check(L.lib().sop_server_clock(self.h, C.byref(t)), "sop_server_clock")
        return t.value

    def stats(self):
        bs, a, q = C.c_int64(), C.c_int(), C.c_int()
        L.check(L.lib().sop_server_stats(self.h, C.byref(bs), C.byref(a), C.byref(q)), "sop_server_stats")
        return dict(bead_steps=bs.value, active=a.value, queued=q.value)

    def timing(self):
        """Seconds the pumps spent admitting, running chunks and retiring."""
        a, r, t = C.c_double(), C.c_double(), C.c_double()
        L.check(L.lib().sop_server_timing(self.h, C.byref(a), C.byref(r), C.byref(t)), "sop_server_timing")
        return dict(admit_s=a.value, run_s=r.value, retire_s=t.value)
