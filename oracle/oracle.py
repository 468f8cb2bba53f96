"""Test infrastructure only: ctypes handles on the CPU oracle.

``Port``  -- oracle/sop_oracle.c, the C restatement (builds on any host).
``Ref``   -- oracle/_ref/libsopref.so, the unmodified SOP-CPU sources behind
             oracle/ref_harness.cpp (built only where the reference tree is).
``synth_chain`` / ``synth_many`` -- oracle/_build/libsopsynth.so, the seeded
             workload generator built on its own (host code only), so a CPU
             baseline builds its inputs without loading the engine library.

Both expose the same methods so a test can run one script through either.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the GPU product never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libsoporacle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsopref.so")
REF_EXE = os.path.join(HERE, "_ref", "sop.x")
REF_TREE_FILE = os.path.join(HERE, "_ref", "ref_tree")
SYNTH_LIB = os.path.join(HERE, "_build", "libsopsynth.so")
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)

_port = None
_ref = None


def _port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            raise RuntimeError("oracle port not built: make -C oracle port")
        L = C.CDLL(PORT_LIB)
        L.sopo_create.restype = C.c_void_p
        L.sopo_destroy.argtypes = [C.c_void_p]
        L.sopo_load_script.argtypes = [C.c_void_p, C.c_char_p]
        L.sopo_set_topology_implicit.argtypes = [
            C.c_void_p, C.c_int, IP, IP, C.c_int, IP, IP, DP, C.c_int, IP, IP, IP,
            C.c_int, IP, IP, DP]
        L.sopo_set_topology_pruned.argtypes = [
            C.c_void_p, C.c_int, IP, IP, C.c_int, IP, IP, DP, C.c_int, IP, IP, IP,
            C.c_int, IP, IP, DP, DP, C.c_double]
        L.sopo_set_topology.argtypes = [
            C.c_void_p, C.c_int, C.c_int, IP, IP, DP, C.c_int, IP, IP, IP,
            C.c_int, IP, IP, DP, IP, IP]
        L.sopo_set_coords.argtypes = [C.c_void_p, C.c_int, DP]
        L.sopo_get_coords.argtypes = [C.c_void_p, C.c_int, DP]
        L.sopo_set_param.argtypes = [C.c_void_p, C.c_char_p, C.c_double]
        L.sopo_get_param.argtypes = [C.c_void_p, C.c_char_p]
        L.sopo_get_param.restype = C.c_double
        L.sopo_set_command.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
        L.sopo_set_force_terms.argtypes = [C.c_void_p] + [C.c_int] * 4
        for fn in ("sopo_neighbor_list", "sopo_cell_list", "sopo_pair_list", "sopo_force_eval",
                   "sopo_energy_eval", "sopo_observables", "sopo_iteration"):
            getattr(L, fn).argtypes = [C.c_void_p]
        L.sopo_setup.argtypes = [C.c_void_p, C.c_int]
        L.sopo_run.argtypes = [C.c_void_p, C.c_int]
        L.sopo_get_list.argtypes = [C.c_void_p, C.c_int, IP, IP]
        L.sopo_get_count.argtypes = [C.c_void_p, C.c_char_p]
        L.sopo_get_energy.argtypes = [C.c_void_p, C.c_char_p]
        L.sopo_get_energy.restype = C.c_double
        L.sopo_run_many.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int]
        L.sopo_run_many.restype = C.c_double
        L.sopo_philox4x32_10.argtypes = [C.POINTER(C.c_uint32)] * 3
        _port = L
    return _port


def _ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            raise RuntimeError("reference oracle not built: make -C oracle ref")
        L = C.CDLL(REF_LIB)
        L.sopref_load_script.argtypes = [C.c_char_p]
        L.sopref_setup.argtypes = [C.c_int]
        L.sopref_set_force_terms.argtypes = [C.c_int] * 4
        L.sopref_run.argtypes = [C.c_int]
        L.sopref_get_int.argtypes = [C.c_char_p]
        L.sopref_get_double.argtypes = [C.c_char_p]
        L.sopref_get_double.restype = C.c_double
        L.sopref_set_double.argtypes = [C.c_char_p, C.c_double]
        L.sopref_get_coords.argtypes = [C.c_int, DP]
        L.sopref_set_coords.argtypes = [C.c_int, DP]
        L.sopref_get_list.argtypes = [C.c_int, IP, IP]
        _ref = L
    return _ref


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_tree():
    """The reference source tree oracle/_ref was built from, or None."""
    try:
        with open(REF_TREE_FILE) as f:
            path = f.read().strip()
        return path if os.path.isdir(path) else None
    except OSError:
        return None


_synth = None


def _synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_LIB):
            raise RuntimeError("workload generator not built: make -C oracle synth")
        L = C.CDLL(SYNTH_LIB)
        L.sop_synth_chain.argtypes = [C.c_uint64, C.c_int, C.c_int, DP]
        L.sop_synth_globule.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, DP]
        _synth = L
    return _synth


def synth_chain(seed, nbead, compact_steps=2000):
    """The seeded compact chain of sop_synth_chain, from the stand-alone build."""
    out = np.zeros((nbead, 3), np.float64)
    rc = _synth_lib().sop_synth_chain(C.c_uint64(seed), nbead, compact_steps, out.ctypes.data_as(DP))
    if rc != 0:
        raise RuntimeError("sop_synth_chain = %d" % rc)
    return out


def synth_many(jobs, compact_steps=2000, workers=None):
    """[(seed, nbead)] -> list of (nbead,3) arrays on host threads."""
    from concurrent.futures import ThreadPoolExecutor
    workers = workers or min(32, os.cpu_count() or 1)
    with ThreadPoolExecutor(workers) as ex:
        return list(ex.map(lambda j: synth_chain(j[0], j[1], compact_steps), jobs))


ENERGY_NAMES = ("e_bnd", "e_ang_ss", "e_vdw_rr", "e_vdw_rr_att", "e_vdw_rr_rep", "rna_etot")


class Port:
    """One oracle system (reentrant; many may coexist)."""

    def __init__(self):
        self.L = _port_lib()
        self.h = C.c_void_p(self.L.sopo_create())

    def __del__(self):
        try:
            self.L.sopo_destroy(self.h)
        except Exception:
            pass

    @property
    def nbead(self):
        return self.L.sopo_get_count(self.h, b"nbead")

    def load_script(self, path):
        rc = self.L.sopo_load_script(self.h, path.encode())
        if rc != 0:
            raise RuntimeError("sopo_load_script(%s) = %d" % (path, rc))
        return self.nbead

    def set_system(self, system, prune=None):
        """Implicit-candidate topology from a sop_gb300.systems.System; with
        `prune` (A), only the pairs closer than that at the system's positions
        plus the natives (sopo_set_topology_pruned, for large systems).  A
        system with exclusions goes in as the explicit candidate list a vdw
        file would hold (sopo_set_topology: natives and the non-natives the
        file lists, lexicographic order, each with its bead types)."""
        if system.exclusions is not None and prune is None:
            return self._set_explicit(system)
        n = system.nbead
        ib, jb, r0 = [np.ascontiguousarray(a) for a in system.bonds]
        ia, ja, ka, _ = [np.ascontiguousarray(a) for a in system.angles]
        in_, jn, rn = [np.ascontiguousarray(a) for a in system.natives]
        ib, jb, ia, ja, ka, in_, jn = [a.astype(np.int32) for a in (ib, jb, ia, ja, ka, in_, jn)]
        r0 = r0.astype(np.float64)
        rn = rn.astype(np.float64)
        typ = (np.ones(n, np.int32) if system.bead_type is None
               else np.ascontiguousarray(system.bead_type, np.int32))
        ch = None if system.chain is None else np.ascontiguousarray(system.chain, np.int32)
        ip = lambda a: a.ctypes.data_as(IP) if a is not None else None
        dp = lambda a: a.ctypes.data_as(DP)
        xyz = np.ascontiguousarray(system.xyz, np.float64)
        self._keep = (ib, jb, r0, ia, ja, ka, in_, jn, rn, typ, ch, xyz)
        if prune is None:
            rc = self.L.sopo_set_topology_implicit(self.h, n, ip(typ), ip(ch), len(ib), ip(ib),
                                                   ip(jb), dp(r0), len(ia), ip(ia), ip(ja), ip(ka),
                                                   len(in_), ip(in_), ip(jn), dp(rn))
        else:
            rc = self.L.sopo_set_topology_pruned(self.h, n, ip(typ), ip(ch), len(ib), ip(ib),
                                                 ip(jb), dp(r0), len(ia), ip(ia), ip(ja), ip(ka),
                                                 len(in_), ip(in_), ip(jn), dp(rn), dp(xyz),
                                                 float(prune))
        if rc != 0:
            raise RuntimeError("sopo_set_topology = %d" % rc)
        self.set_coords(0, xyz)
        self.set_coords(1, xyz)

    def _set_explicit(self, system):
        from sop_gb300 import systems as S  # candidate enumeration only
        n = system.nbead
        ib, jb, r0 = [np.ascontiguousarray(a) for a in system.bonds]
        ia, ja, ka, _ = [np.ascontiguousarray(a) for a in system.angles]
        in_, jn, rn = [np.asarray(a) for a in system.natives]
        ib, jb, ia, ja, ka = [a.astype(np.int32) for a in (ib, jb, ia, ja, ka)]
        r0 = r0.astype(np.float64)
        typ = (np.ones(n, np.int32) if system.bead_type is None
               else np.asarray(system.bead_type, np.int32))
        ri, rj = S.candidate_pairs(system)
        ic = np.concatenate([np.asarray(in_, np.int64), ri.astype(np.int64)])
        jc = np.concatenate([np.asarray(jn, np.int64), rj.astype(np.int64)])
        # non-natives carry a distance at or above rcut_nat of their types
        rc = np.concatenate([np.asarray(rn, np.float64),
                             S.RCUT_NAT[typ[ri], typ[rj]] + 1.0])
        order = np.lexsort((jc, ic))
        ic = np.ascontiguousarray(ic[order], np.int32)
        jc = np.ascontiguousarray(jc[order], np.int32)
        rc = np.ascontiguousarray(rc[order])
        ti = np.ascontiguousarray(typ[ic], np.int32)
        tj = np.ascontiguousarray(typ[jc], np.int32)
        ip = lambda a: a.ctypes.data_as(IP)
        dp = lambda a: a.ctypes.data_as(DP)
        xyz = np.ascontiguousarray(system.xyz, np.float64)
        self._keep = (ib, jb, r0, ia, ja, ka, ic, jc, rc, ti, tj, xyz)
        rc_ = self.L.sopo_set_topology(self.h, n, len(ib), ip(ib), ip(jb), dp(r0), len(ia), ip(ia),
                                       ip(ja), ip(ka), len(ic), ip(ic), ip(jc), dp(rc), ip(ti), ip(tj))
        if rc_ != 0:
            raise RuntimeError("sopo_set_topology = %d" % rc_)
        self.set_coords(0, xyz)
        self.set_coords(1, xyz)

    def command(self, key, value=None):
        self.L.sopo_set_command(self.h, key.encode(), value.encode() if value is not None else None)

    def set_param(self, name, v):
        if self.L.sopo_set_param(self.h, name.encode(), float(v)) != 0:
            raise KeyError(name)

    def param(self, name):
        return self.L.sopo_get_param(self.h, name.encode())

    def set_force_terms(self, random_on, fene_on, ang_on, vdw_on):
        self.L.sopo_set_force_terms(self.h, int(random_on), int(fene_on), int(ang_on), int(vdw_on))

    def setup(self, initial_eval=True):
        self.L.sopo_setup(self.h, int(initial_eval))

    def neighbor_list(self):
        self.L.sopo_neighbor_list(self.h)

    def cell_list(self):
        self.L.sopo_cell_list(self.h)

    def pair_list(self):
        self.L.sopo_pair_list(self.h)

    def force_eval(self):
        self.L.sopo_force_eval(self.h)

    def energy_eval(self):
        self.L.sopo_energy_eval(self.h)

    def observables(self):
        self.L.sopo_observables(self.h)

    def iteration(self):
        self.L.sopo_iteration(self.h)

    def run(self, n):
        self.L.sopo_run(self.h, int(n))

    def coords(self, which):
        out = np.zeros((self.nbead, 3), np.float64)
        self.L.sopo_get_coords(self.h, which, out.ctypes.data_as(DP))
        return out

    def set_coords(self, which, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64)
        self.L.sopo_set_coords(self.h, which, xyz.ctypes.data_as(DP))

    def pairs(self, which):
        n = self.L.sopo_get_list(self.h, which, None, None)
        ii = np.zeros(max(n, 1), np.int32)
        jj = np.zeros(max(n, 1), np.int32)
        self.L.sopo_get_list(self.h, which, ii.ctypes.data_as(IP), jj.ctypes.data_as(IP))
        return ii[:n], jj[:n]

    def count(self, name):
        return self.L.sopo_get_count(self.h, name.encode())

    def energy(self, name):
        return self.L.sopo_get_energy(self.h, name.encode())

    def energies(self):
        return np.array([self.energy(k) for k in ENERGY_NAMES])


class Ref:
    """The reference itself (process-global state: one system at a time)."""

    def __init__(self):
        self.L = _ref_lib()

    @property
    def nbead(self):
        return self.L.sopref_get_int(b"nbead")

    def load_script(self, path):
        return self.L.sopref_load_script(path.encode())

    def set_force_terms(self, random_on, fene_on, ang_on, vdw_on):
        self.L.sopref_set_force_terms(int(random_on), int(fene_on), int(ang_on), int(vdw_on))

    def param(self, name):
        if name in ("nnlup", "nup", "neighborlist", "celllist"):
            return self.L.sopref_get_int(name.encode())
        return self.L.sopref_get_double(name.encode())

    def set_param(self, name, v):
        self.L.sopref_set_double(name.encode(), float(v))

    def setup(self, initial_eval=True):
        self.L.sopref_setup(int(initial_eval))

    def neighbor_list(self):
        self.L.sopref_neighbor_list()

    def cell_list(self):
        self.L.sopref_cell_list()

    def pair_list(self):
        self.L.sopref_pair_list()

    def force_eval(self):
        self.L.sopref_force_eval()

    def energy_eval(self):
        self.L.sopref_energy_eval()

    def observables(self):
        self.L.sopref_observables()

    def iteration(self):
        self.L.sopref_iteration()

    def run(self, n):
        self.L.sopref_run(int(n))

    def coords(self, which):
        out = np.zeros((self.nbead, 3), np.float64)
        self.L.sopref_get_coords(which, out.ctypes.data_as(DP))
        return out

    def set_coords(self, which, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64)
        self.L.sopref_set_coords(which, xyz.ctypes.data_as(DP))

    def pairs(self, which):
        n = self.L.sopref_get_list(which, None, None)
        ii = np.zeros(max(n, 1), np.int32)
        jj = np.zeros(max(n, 1), np.int32)
        self.L.sopref_get_list(which, ii.ctypes.data_as(IP), jj.ctypes.data_as(IP))
        return ii[:n], jj[:n]

    def count(self, name):
        return self.L.sopref_get_int(name.encode())

    def energy(self, name):
        return self.L.sopref_get_double(name.encode())

    def energies(self):
        return np.array([self.energy(k) for k in ENERGY_NAMES])


def philox(ctr, key):
    L = _port_lib()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.sopo_philox4x32_10(c, k, o)
    return list(o)


def run_many(ports, nsteps, nthreads):
    """Wall seconds for nsteps of every Port on nthreads host threads."""
    L = _port_lib()
    arr = (C.c_void_p * len(ports))(*[p.h.value for p in ports])
    return L.sopo_run_many(arr, len(ports), int(nsteps), int(nthreads))
