"""Python handle on the engine C ABI (include/sop_gpu.h).

Every call goes to libsopgpu.so; errors raise :class:`SopError`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .systems import System, script_params

LIST_MODES = {"none": L.LIST_NONE, "neighborlist": L.LIST_NEIGHBOR, "celllist": L.LIST_CELL,
              "skin": L.LIST_SKIN}


def make_params(script=None, **kw) -> L.Params:
    """sop_params from reference "set" commands and/or keyword overrides.

    ``script`` is a list of ("set", key, value) tuples replayed with the side
    effects of set_params (params.cpp:12-101); keywords override fields by
    name (T, zeta, h, a1..a4, boxl, lcell, ncell, nnlup, nup, list_mode, skin,
    cell_edge, seed, force_terms, pull_force, pull_i, pull_j).
    """
    p = L.default_params()
    if script is not None:
        sp = script_params(script)
        for k in ("T", "zeta", "h", "a1", "a2", "a3", "a4", "a5", "boxl", "lcell", "ncell"):
            setattr(p, k, sp[k])
        p.dynamics = L.DYN_OVERDAMPED if sp["sim_type"] == 2 else L.DYN_UNDERDAMPED
        p.nnlup = int(sp["nnlup"])
        p.nup = int(sp["nup"])
        p.seed = (-100 - int(sp["run"])) & 0xFFFFFFFFFFFFFFFF
        p.list_mode = (L.LIST_NEIGHBOR if sp["neighborlist"] else
                       L.LIST_CELL if sp["celllist"] else L.LIST_NONE)
    for k, v in kw.items():
        if k == "list_mode" and isinstance(v, str):
            v = LIST_MODES[v]
        if k == "seed":
            v = int(v) & 0xFFFFFFFFFFFFFFFF
        setattr(p, k, v)
    return p


class _Desc:
    """sop_system_desc with its arrays kept alive."""

    def __init__(self, system: System, params: L.Params, vel=None):
        n = system.nbead
        self.keep = []

        def iarr(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
            self.keep.append(a)
            return a

        def darr(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
            self.keep.append(a)
            return a

        d = L.SystemDesc()
        d.nbead = n
        d.xyz = L.dptr(darr(system.xyz.reshape(-1)))
        d.vel = L.dptr(darr(np.asarray(vel).reshape(-1))) if vel is not None else None
        d.bead_type = L.iptr(iarr(system.bead_type)) if system.bead_type is not None else None
        d.chain = L.iptr(iarr(system.chain)) if system.chain is not None else None
        ib, jb, r0 = system.bonds
        d.nbnd = len(ib)
        d.ib, d.jb, d.r0 = L.iptr(iarr(ib)), L.iptr(iarr(jb)), L.dptr(darr(r0))
        ia, _, ka, _ = system.angles
        d.nang = len(ia)
        d.ia, d.ka = L.iptr(iarr(ia)), L.iptr(iarr(ka))
        in_, jn, rn = system.natives
        d.nnat = len(in_)
        d.in_, d.jn, d.rn = L.iptr(iarr(in_)), L.iptr(iarr(jn)), L.dptr(darr(rn))
        if system.exclusions is not None and len(system.exclusions[0]):
            ie, je = system.exclusions
            d.nexcl = len(ie)
            d.ie, d.je = L.iptr(iarr(ie)), L.iptr(iarr(je))
        else:
            d.nexcl = 0
        d.params = params
        self.desc = d


class Engine:
    def __init__(self, device: int = 0, **cfg):
        c = L.default_engine_config()
        c.device = device
        for k, v in cfg.items():
            setattr(c, k, v)
        h = C.c_void_p()
        L.check(L.lib().sop_engine_create(C.byref(c), C.byref(h)), "sop_engine_create")
        self.h = h
        self.nbead = {}

    def close(self):
        if self.h:
            L.lib().sop_engine_destroy(self.h)
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

    # -- replicas
    def add(self, system: System, params: L.Params | None = None, vel=None, **kw) -> int:
        p = params if params is not None else make_params(**kw)
        d = _Desc(system, p, vel)
        r = C.c_int()
        L.check(L.lib().sop_replica_add(self.h, C.byref(d.desc), C.byref(r)), "sop_replica_add")
        self.nbead[r.value] = system.nbead
        return r.value

    def system_bytes(self, system: System, params: L.Params | None = None) -> int:
        d = _Desc(system, params if params is not None else make_params())
        b = C.c_int64()
        L.check(L.lib().sop_system_bytes(self.h, C.byref(d.desc), C.byref(b)), "sop_system_bytes")
        return b.value

    def remove(self, r: int):
        L.check(L.lib().sop_replica_remove(self.h, r), "sop_replica_remove")
        self.nbead.pop(r, None)

    def set_params(self, r: int, params: L.Params):
        L.check(L.lib().sop_replica_set_params(self.h, r, C.byref(params)), "sop_replica_set_params")

    def params(self, r: int) -> L.Params:
        p = L.Params()
        L.check(L.lib().sop_replica_get_params(self.h, r, C.byref(p)), "sop_replica_get_params")
        return p

    def state(self, r: int):
        n = self.nbead[r]
        pos, unc, vel = (np.zeros((n, 3)) for _ in range(3))
        L.check(L.lib().sop_replica_get_state(self.h, r, L.dptr(pos), L.dptr(unc), L.dptr(vel)),
                "sop_replica_get_state")
        return pos, unc, vel

    def set_state(self, r: int, unc_pos, vel=None):
        u = np.ascontiguousarray(unc_pos, np.float64)
        v = None if vel is None else np.ascontiguousarray(vel, np.float64)
        L.check(L.lib().sop_replica_set_state(self.h, r, L.dptr(u), L.dptr(v)), "sop_replica_set_state")

    def checkpoint(self, r: int) -> bytes:
        """Exact snapshot of replica r (sop_replica_checkpoint)."""
        n = C.c_int64()
        L.check(L.lib().sop_replica_checkpoint(self.h, r, None, 0, C.byref(n)), "sop_replica_checkpoint")
        buf = C.create_string_buffer(n.value)
        L.check(L.lib().sop_replica_checkpoint(self.h, r, buf, n.value, C.byref(n)),
                "sop_replica_checkpoint")
        return buf.raw

    def restore(self, r: int, data: bytes):
        """Continue replica r from a snapshot of the same system."""
        buf = C.create_string_buffer(data, len(data))
        L.check(L.lib().sop_replica_restore(self.h, r, buf, len(data)), "sop_replica_restore")

    def status(self, r: int):
        st = C.c_int()
        steps = C.c_int64()
        L.check(L.lib().sop_replica_status(self.h, r, C.byref(st), C.byref(steps)), "sop_replica_status")
        return st.value, steps.value

    def info(self, r: int) -> dict:
        o = (C.c_int64 * 8)()
        L.check(L.lib().sop_replica_info(self.h, r, o), "sop_replica_info")
        keys = ("nbead", "L", "max_row", "builds", "t", "status", "natives", "offset")
        return dict(zip(keys, list(o)))

    # -- reference-named operations
    def neighbor_list(self, r: int):
        L.check(L.lib().sop_update_neighbor_list(self.h, r), "sop_update_neighbor_list")

    def cell_list(self, r: int):
        L.check(L.lib().sop_update_cell_list(self.h, r), "sop_update_cell_list")

    def pair_list(self, r: int):
        L.check(L.lib().sop_update_pair_list(self.h, r), "sop_update_pair_list")

    def pairs(self, r: int, which: int):
        cnt = C.c_int()
        L.check(L.lib().sop_get_pair_list(self.h, r, which, None, None, 0, C.byref(cnt)),
                "sop_get_pair_list")
        n = cnt.value
        ii = np.zeros(max(n, 1), np.int32)
        jj = np.zeros(max(n, 1), np.int32)
        L.check(L.lib().sop_get_pair_list(self.h, r, which, L.iptr(ii), L.iptr(jj), n, C.byref(cnt)),
                "sop_get_pair_list")
        return ii[:n], jj[:n]

    def force(self, r: int):
        f = np.zeros((self.nbead[r], 3))
        L.check(L.lib().sop_force_eval(self.h, r, L.dptr(f)), "sop_force_eval")
        return f

    def energy(self, r: int):
        e = np.zeros(6)
        L.check(L.lib().sop_energy_eval(self.h, r, L.dptr(e)), "sop_energy_eval")
        return e

    def observables(self, r: int):
        o = np.zeros(5)
        L.check(L.lib().sop_observables(self.h, r, L.dptr(o)), "sop_observables")
        return o

    def iteration(self, r: int):
        L.check(L.lib().sop_underdamped_iteration(self.h, r), "sop_underdamped_iteration")

    # -- stepping
    def run_plain(self, r: int, nsteps: int):
        L.check(L.lib().sop_run_plain(self.h, r, int(nsteps)), "sop_run_plain")

    def run(self, nsteps: int):
        L.check(L.lib().sop_run(self.h, int(nsteps)), "sop_run")

    def run_host(self, xyz_in, vel_in, nsteps, xyz_out, vel_out):
        L.check(L.lib().sop_run_host(self.h, L.dptr(xyz_in), L.dptr(vel_in), int(nsteps),
                                     L.dptr(xyz_out), L.dptr(vel_out)), "sop_run_host")

    def timing(self):
        t, s = C.c_double(), C.c_double()
        n = C.c_int64()
        L.check(L.lib().sop_last_run_timing(self.h, C.byref(t), C.byref(s), C.byref(n)),
                "sop_last_run_timing")
        return t.value, s.value, n.value

    def profile_steps(self, nsteps: int):
        """(step-kernel ms, prologue ms) per launch, CUDA events per kernel."""
        s, p = C.c_double(), C.c_double()
        L.check(L.lib().sop_profile_steps(self.h, int(nsteps), C.byref(s), C.byref(p)),
                "sop_profile_steps")
        return s.value, p.value

    def profile_split(self, nsteps: int):
        """Mean ms per step of the preparation (k_prep: bookkeeping, binning,
        list builds), the gap after it and k_step (CUDA events)."""
        out = (C.c_double * 4)()
        L.check(L.lib().sop_profile_steps_ex(self.h, int(nsteps), out), "sop_profile_steps_ex")
        return {"prologue": out[0] + out[1], "build": out[2], "step": out[3]}

    def launches(self) -> int:
        n = C.c_int64()
        L.check(L.lib().sop_engine_launches(self.h, C.byref(n)), "sop_engine_launches")
        return n.value

    def prep_fallbacks(self) -> int:
        """Lean preparation launches that found queued work (expected 0)."""
        n = C.c_int64()
        L.check(L.lib().sop_engine_prep_fallbacks(self.h, C.byref(n)), "sop_engine_prep_fallbacks")
        return n.value

    def inject_stall(self, publish_delay_ns: int = 0, skip_stage_copy: bool = False):
        """Diagnostics: stalls that make the device-side waits run out (tests
        of the timeout path); both zero = normal operation."""
        L.check(L.lib().sop_engine_inject_stall(self.h, int(publish_delay_ns), int(skip_stage_copy)),
                "sop_engine_inject_stall")

    def wait_errors(self) -> int:
        """Waits that ran out in the last call that timed out: bit 0 staging
        copy, bit 1 work queue."""
        b = C.c_int()
        L.check(L.lib().sop_engine_wait_errors(self.h, C.byref(b)), "sop_engine_wait_errors")
        return b.value

    def sync(self):
        L.check(L.lib().sop_engine_sync(self.h), "sop_engine_sync")

    def autotune(self, steps_per_trial: int = 50, shape: bool = True, lists: bool = True) -> str:
        """Tune launch shape and/or per-size-bucket skin and cell edge; the
        trials are real steps (see sop_autotune_ex).  Returns the trial table."""
        what = (L.TUNE_SHAPE if shape else 0) | (L.TUNE_LISTS if lists else 0)
        buf = C.create_string_buffer(1 << 16)
        L.check(L.lib().sop_autotune_ex(self.h, steps_per_trial, what, buf, len(buf)),
                "sop_autotune_ex")
        return buf.value.decode()
