"""ctypes binding of libsopgpu.so (the C ABI declared in include/sop_gpu.h).

The library is built in-tree by ``build.py`` (``__graft_entry__.build()``).
Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# SOP_GB300_CHECKED=1 selects the checked build (every partner index tested
# against its replica's range; a bad one fails the call with SOP_ERR_INDEX)
LIB_PATH = os.path.join(PKG_DIR, "lib", "libsopgpu_checked.so"
                        if os.environ.get("SOP_GB300_CHECKED") == "1" else "libsopgpu.so")

SOP_OK = 0
ERRORS = {
    -1: "SOP_ERR_ARG", -2: "SOP_ERR_CUDA", -3: "SOP_ERR_NOMEM", -4: "SOP_ERR_STATE",
    -5: "SOP_ERR_OVERFLOW", -6: "SOP_ERR_UNSUPPORTED", -7: "SOP_ERR_NODEV",
    -8: "SOP_ERR_REPLICA", -9: "SOP_ERR_FULL", -10: "SOP_ERR_TIMEOUT", -11: "SOP_ERR_INDEX",
}
ERR_TIMEOUT = -10
ERR_INDEX = -11
ST_NONFINITE, ST_FENE, ST_LIST_OVERFLOW, ST_PERIODIC, ST_GRID = 1, 2, 4, 8, 16
LIST_NONE, LIST_NEIGHBOR, LIST_CELL, LIST_SKIN = 0, 1, 2, 3
TERM_RANDOM, TERM_FENE, TERM_ANGLE, TERM_VDW, TERM_ALL = 1, 2, 4, 8, 15
TUNE_SHAPE, TUNE_LISTS = 1, 2
PREC_MIXED, PREC_FP64 = 0, 1
DYN_UNDERDAMPED, DYN_OVERDAMPED = 0, 1


class SopError(RuntimeError):
    def __init__(self, code, where):
        detail = ""
        try:
            detail = ": " + lib().sop_status_string(code).decode()
        except Exception:
            pass
        super().__init__("%s failed: %s (%d)%s" % (where, ERRORS.get(code, "?"), code, detail))
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("T", C.c_double), ("zeta", C.c_double), ("h", C.c_double),
        ("a1", C.c_double), ("a2", C.c_double), ("a3", C.c_double), ("a4", C.c_double),
        ("boxl", C.c_double), ("lcell", C.c_double), ("ncell", C.c_double),
        ("k_bnd", C.c_double), ("R0", C.c_double),
        ("sigma_ss", C.c_double), ("epsilon_ss", C.c_double),
        ("skin", C.c_double), ("cell_edge", C.c_double), ("pull_force", C.c_double),
        ("seed", C.c_uint64),
        ("nnlup", C.c_int), ("nup", C.c_int), ("list_mode", C.c_int),
        ("force_terms", C.c_int), ("precision", C.c_int),
        ("pull_i", C.c_int), ("pull_j", C.c_int),
        ("dynamics", C.c_int), ("a5", C.c_double),
    ]


IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)


class SystemDesc(C.Structure):
    _fields_ = [
        ("nbead", C.c_int), ("xyz", DP), ("vel", DP), ("bead_type", IP), ("chain", IP),
        ("nbnd", C.c_int), ("ib", IP), ("jb", IP), ("r0", DP),
        ("nang", C.c_int), ("ia", IP), ("ka", IP),
        ("nnat", C.c_int), ("in_", IP), ("jn", IP), ("rn", DP),
        ("nexcl", C.c_int), ("ie", IP), ("je", IP),
        ("params", Params),
    ]


class EngineConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("max_beads", C.c_int), ("max_replicas", C.c_int),
        ("max_list_entries", C.c_int64), ("block_threads", C.c_int),
        ("lanes_per_bead", C.c_int), ("graph_steps", C.c_int),
        ("stage_limit", C.c_int), ("chunk_beads", C.c_int), ("build_slice_beads", C.c_int),
        ("step_min_blocks", C.c_int), ("step_strategy", C.c_int), ("group_rebuild_pct", C.c_int),
        ("lean_prep", C.c_int), ("queue_wait_ns", C.c_int64), ("stage_wait_ns", C.c_int64),
        ("item_cost_beads", C.c_int), ("row_bands", C.c_int),
        ("queue_blocks", C.c_int),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("engine", EngineConfig), ("max_active", C.c_int),
        ("memory_budget", C.c_int64), ("chunk_steps", C.c_int),
    ]


class RequestResult(C.Structure):
    _fields_ = [
        ("request_id", C.c_int64), ("status", C.c_int), ("replica_status", C.c_int),
        ("nbead", C.c_int), ("steps", C.c_int64),
        ("submit_s", C.c_double), ("start_s", C.c_double), ("finish_s", C.c_double),
        ("energy", C.c_double * 6), ("observables", C.c_double * 5),
    ]


VP = C.c_void_p
_PROTOS = {
    "sop_version": (C.c_char_p, []),
    "sop_struct_size": (C.c_int, [C.c_char_p]),
    "sop_status_string": (C.c_char_p, [C.c_int]),
    "sop_params_default": (None, [C.POINTER(Params)]),
    "sop_engine_config_default": (None, [C.POINTER(EngineConfig)]),
    "sop_engine_create": (C.c_int, [C.POINTER(EngineConfig), C.POINTER(VP)]),
    "sop_engine_destroy": (C.c_int, [VP]),
    "sop_engine_sync": (C.c_int, [VP]),
    "sop_system_bytes": (C.c_int, [VP, C.POINTER(SystemDesc), C.POINTER(C.c_int64)]),
    "sop_engine_free_bytes": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sop_engine_launches": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sop_engine_prep_fallbacks": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sop_engine_inject_stall": (C.c_int, [VP, C.c_int64, C.c_int]),
    "sop_engine_wait_errors": (C.c_int, [VP, IP]),
    "sop_probe_l2_read": (C.c_int, [C.c_int, C.c_int64, C.c_int, C.POINTER(C.c_double)]),
    "sop_replica_add": (C.c_int, [VP, C.POINTER(SystemDesc), IP]),
    "sop_replica_remove": (C.c_int, [VP, C.c_int]),
    "sop_replica_set_params": (C.c_int, [VP, C.c_int, C.POINTER(Params)]),
    "sop_replica_get_params": (C.c_int, [VP, C.c_int, C.POINTER(Params)]),
    "sop_replica_get_state": (C.c_int, [VP, C.c_int, DP, DP, DP]),
    "sop_replica_set_state": (C.c_int, [VP, C.c_int, DP, DP]),
    "sop_replica_status": (C.c_int, [VP, C.c_int, IP, C.POINTER(C.c_int64)]),
    "sop_replica_count": (C.c_int, [VP, IP]),
    "sop_replica_info": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int64)]),
    "sop_update_neighbor_list": (C.c_int, [VP, C.c_int]),
    "sop_update_cell_list": (C.c_int, [VP, C.c_int]),
    "sop_update_pair_list": (C.c_int, [VP, C.c_int]),
    "sop_get_pair_list": (C.c_int, [VP, C.c_int, C.c_int, IP, IP, C.c_int, IP]),
    "sop_force_eval": (C.c_int, [VP, C.c_int, DP]),
    "sop_energy_eval": (C.c_int, [VP, C.c_int, DP]),
    "sop_underdamped_iteration": (C.c_int, [VP, C.c_int]),
    "sop_observables": (C.c_int, [VP, C.c_int, DP]),
    "sop_run_plain": (C.c_int, [VP, C.c_int, C.c_int64]),
    "sop_run": (C.c_int, [VP, C.c_int64]),
    "sop_replica_start": (C.c_int, [VP, C.c_int, C.c_int64]),
    "sop_run_chunk": (C.c_int, [VP, C.c_int64, IP, C.c_int, IP]),
    "sop_run_chunk_begin": (C.c_int, [VP, C.c_int64]),
    "sop_run_chunk_end": (C.c_int, [VP, IP, C.c_int, IP]),
    "sop_prepare": (C.c_int, [C.POINTER(SystemDesc), C.POINTER(VP)]),
    "sop_prepared_bytes": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sop_prepared_free": (None, [VP]),
    "sop_replicas_admit": (C.c_int, [VP, C.POINTER(VP), C.POINTER(C.c_int64), C.c_int, IP, IP]),
    "sop_replicas_retire": (C.c_int, [VP, IP, C.c_int, DP, DP, IP]),
    "sop_run_host": (C.c_int, [VP, DP, DP, C.c_int64, DP, DP]),
    "sop_last_run_timing": (C.c_int, [VP, DP, DP, C.POINTER(C.c_int64)]),
    "sop_profile_steps": (C.c_int, [VP, C.c_int64, DP, DP]),
    "sop_profile_steps_ex": (C.c_int, [VP, C.c_int64, DP]),
    "sop_replica_outputs": (C.c_int, [VP, C.c_int, DP, DP]),
    "sop_replica_set_step": (C.c_int, [VP, C.c_int, C.c_int64]),
    "sop_replica_checkpoint": (C.c_int, [VP, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "sop_replica_restore": (C.c_int, [VP, C.c_int, C.c_void_p, C.c_int64]),
    "sop_autotune": (C.c_int, [VP, C.c_int, C.c_char_p, C.c_int]),
    "sop_autotune_ex": (C.c_int, [VP, C.c_int, C.c_int, C.c_char_p, C.c_int]),
    "sop_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(VP)]),
    "sop_server_destroy": (C.c_int, [VP]),
    "sop_server_submit": (C.c_int, [VP, C.POINTER(SystemDesc), C.c_int64, C.POINTER(C.c_int64)]),
    "sop_server_pump": (C.c_int, [VP, IP]),
    "sop_server_poll": (C.c_int, [VP, C.POINTER(RequestResult), C.c_int, IP]),
    "sop_server_clock": (C.c_int, [VP, DP]),
    "sop_server_stats": (C.c_int, [VP, C.POINTER(C.c_int64), IP, IP]),
    "sop_server_timing": (C.c_int, [VP, DP, DP, DP]),
    "sop_synth_chain": (C.c_int, [C.c_uint64, C.c_int, C.c_int, DP]),
    "sop_synth_globule": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.c_int, DP]),
    "sop_neighbor_list_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "sop_selftest_split": (None, [C.c_double, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "sop_selftest_philox": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32)]),
}

_lib = None


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsopgpu.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        missing = [n for n in _PROTOS if not hasattr(L, n)]
        if missing:
            raise RuntimeError("libsopgpu.so lacks exports: %s" % ", ".join(missing))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        wrong = ["%s (library %d bytes, binding %d)" % (n, L.sop_struct_size(n.encode()), C.sizeof(s))
                 for n, s in STRUCTS.items() if L.sop_struct_size(n.encode()) != C.sizeof(s)]
        if wrong:
            raise RuntimeError("struct layouts differ from %s: %s" % (LIB_PATH, "; ".join(wrong)))
        _lib = L
    return _lib


def check(code, where):
    if code != SOP_OK:
        raise SopError(code, where)
    return code


# the header's structs and their bindings (checked against the library at load)
STRUCTS = {"sop_params": Params, "sop_system_desc": SystemDesc, "sop_engine_config": EngineConfig,
           "sop_server_config": ServerConfig, "sop_request_result": RequestResult}


def exported_symbols():
    return list(_PROTOS)


def dptr(a):
    return a.ctypes.data_as(DP) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(IP) if a is not None else None


def synth_chain(seed, nbead, compact_steps=2000):
    out = np.zeros((nbead, 3), np.float64)
    check(lib().sop_synth_chain(C.c_uint64(seed), nbead, compact_steps, dptr(out)), "sop_synth_chain")
    return out


def synth_globule(seed, nchain, chain_len, compact_steps=2000):
    out = np.zeros((nchain * chain_len, 3), np.float64)
    check(lib().sop_synth_globule(C.c_uint64(seed), nchain, chain_len, compact_steps, dptr(out)),
          "sop_synth_globule")
    return out


def synth_many(jobs, compact_steps=2000, workers=None):
    """[(seed, nbead)] -> list of (nbead,3) arrays, generated on host threads
    (ctypes drops the GIL during the call)."""
    workers = workers or min(32, os.cpu_count() or 1)
    with ThreadPoolExecutor(workers) as ex:
        return list(ex.map(lambda j: synth_chain(j[0], j[1], compact_steps), jobs))


def default_params():
    p = Params()
    lib().sop_params_default(C.byref(p))
    return p


def default_engine_config():
    c = EngineConfig()
    lib().sop_engine_config_default(C.byref(c))
    return c
