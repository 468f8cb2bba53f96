"""SOP systems in the reference's terms, and the seeded synthetic workloads.

A :class:`System` holds what SOP-CPU loads from its four input files
(params.cpp:110-260): bonds ``i j r0``, angles ``i j k a0``, the vdw candidate
list ``i j r type_i type_j`` (native iff ``r < rcut_nat``, params.cpp:197) and
the initial coordinates.  Non-native candidates are implicit: every pair on
different chains, or on one chain with ``|i-j| > 2``, that is not native --
exactly the set a vdw file listing all such pairs describes -- minus the
``exclusions``: pairs of that set a vdw file does not list, which therefore
never interact (params.cpp:186-232).

Values are rounded to the 6 decimals the files carry, so the engine, the
oracle and the reference program read identical doubles.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib

RCUT_NAT_11 = 8.0  # global.cpp:90 (type 1-1)
# rcut_nat[ti][tj] (global.cpp:89-91): a vdw candidate is native iff r < this
RCUT_NAT = np.array([[0.0, 0.0, 0.0], [0.0, 8.0, 11.0], [0.0, 11.0, 14.0]])


def _r6(a):
    """Round to the 6 decimals of the reference's %f text, as atof reads it."""
    return np.array([float("%.6f" % v) for v in np.asarray(a, dtype=np.float64).ravel()],
                    dtype=np.float64).reshape(np.shape(a))


@dataclass
class System:
    xyz: np.ndarray                 # (N,3) float64 initial unc_pos
    bonds: tuple                    # (ib, jb, r0) 0-based
    angles: tuple                   # (ia, ja, ka, a0) 0-based
    natives: tuple                  # (in, jn, rn) 0-based, i<j
    bead_type: np.ndarray = None    # (N,) int, default 1
    chain: np.ndarray = None        # (N,) int, default 0
    params: dict = field(default_factory=dict)  # reference "set" keywords
    exclusions: tuple = None        # (ie, je) 0-based, i<j: implicit candidates
                                    # the vdw file leaves out (never interact)

    @property
    def nbead(self) -> int:
        return int(self.xyz.shape[0])

    def candidate_count(self) -> int:
        n = self.nbead
        if self.chain is None:
            return (n - 2) * (n - 3) // 2 if n > 3 else 0
        ch = np.asarray(self.chain)
        total = n * (n - 1) // 2
        same_close = 0
        for d in (1, 2):
            same_close += int(np.sum(ch[d:] == ch[:-d]))
        return total - same_close


def native_pairs(xyz: np.ndarray, chain=None, cutoff: float = RCUT_NAT_11, min_sep: int = 3,
                 bead_type=None):
    """Pairs (i<j) closer than ``cutoff`` in the native structure, with
    ``|i-j| >= min_sep`` on one chain (natives are intra-chain only).  With
    ``bead_type`` the cutoff of each pair is rcut_nat[ti][tj] instead."""
    n = xyz.shape[0]
    search = cutoff if bead_type is None else float(RCUT_NAT.max())
    try:
        from scipy.spatial import cKDTree
        pairs = np.array(sorted(cKDTree(xyz).query_pairs(search + 1e-3)), dtype=np.int64)
    except ImportError:  # pragma: no cover - scipy is in both images
        d = np.sqrt(((xyz[:, None, :] - xyz[None, :, :]) ** 2).sum(-1))
        ii, jj = np.nonzero(np.triu(d < search + 1e-3, 1))
        pairs = np.stack([ii, jj], 1)
    if pairs.size == 0:
        return (np.zeros(0, np.int32),) * 2 + (np.zeros(0),)
    i, j = pairs[:, 0], pairs[:, 1]
    same = np.ones(len(i), bool) if chain is None else (np.asarray(chain)[i] == np.asarray(chain)[j])
    keep = same & (j - i >= min_sep)
    i, j = i[keep], j[keep]
    r = _r6(np.sqrt(((xyz[j] - xyz[i]) ** 2).sum(1)))
    if bead_type is None:
        keep = r < cutoff
    else:
        t = np.asarray(bead_type, np.int64)
        keep = r < RCUT_NAT[t[i], t[j]]
    order = np.lexsort((j[keep], i[keep]))
    return (i[keep][order].astype(np.int32), j[keep][order].astype(np.int32), r[keep][order])


def system_from_xyz(xyz: np.ndarray, chain=None, params: dict | None = None,
                    bead_type=None) -> System:
    """Topology of the SOP model at a native structure: bonds i,i+1 and angles
    i,i+1,i+2 within each chain, natives at |i-j|>2 within rcut_nat of the
    pair's bead types (8 A for type 1-1, 11 A for 1-2, 14 A for 2-2)."""
    xyz = _r6(xyz)
    n = xyz.shape[0]
    ch = np.zeros(n, np.int32) if chain is None else np.asarray(chain, np.int32)
    ib = np.array([i for i in range(n - 1) if ch[i] == ch[i + 1]], np.int32)
    jb = ib + 1
    r0 = _r6(np.sqrt(((xyz[jb] - xyz[ib]) ** 2).sum(1)))
    ia = np.array([i for i in range(n - 2) if ch[i] == ch[i + 2]], np.int32)
    ja, ka = ia + 1, ia + 2
    a0 = _r6(np.sqrt(((xyz[ka] - xyz[ia]) ** 2).sum(1)))
    typ = np.ones(n, np.int32) if bead_type is None else np.asarray(bead_type, np.int32)
    if typ.shape != (n,) or not np.all((typ == 1) | (typ == 2)):
        raise ValueError("bead types must be 1 or 2, one per bead")
    nat = native_pairs(xyz, None if chain is None else ch,
                       bead_type=None if bead_type is None else typ)
    return System(xyz=xyz, bonds=(ib, jb, r0), angles=(ia, ja, ka, a0), natives=nat,
                  bead_type=typ, chain=None if chain is None else ch,
                  params=dict(params or {}))


def candidate_pairs(system: System):
    """The non-native candidates (i<j, lexicographic order) a vdw file
    listing them explicitly would hold: the implicit set minus the natives
    and the exclusions."""
    n = system.nbead
    ii, jj = np.triu_indices(n, 1)
    if system.chain is None:
        keep = jj - ii > 2
    else:
        ch = np.asarray(system.chain)
        keep = (ch[ii] != ch[jj]) | (jj - ii > 2)
    ii, jj = ii[keep], jj[keep]
    drop = set()
    in_, jn, _ = system.natives
    drop.update(zip(np.asarray(in_).tolist(), np.asarray(jn).tolist()))
    if system.exclusions is not None:
        drop.update(zip(np.asarray(system.exclusions[0]).tolist(),
                        np.asarray(system.exclusions[1]).tolist()))
    if drop:
        key = ii.astype(np.int64) * n + jj
        gone = np.array([a * n + b for a, b in drop], np.int64)
        keep = ~np.isin(key, gone)
        ii, jj = ii[keep], jj[keep]
    return ii.astype(np.int32), jj.astype(np.int32)


def with_exclusions(system: System, fraction: float, seed: int) -> System:
    """A copy of ``system`` whose vdw file leaves out a seeded ``fraction`` of
    the non-native candidates (those pairs then never interact)."""
    ii, jj = candidate_pairs(system)
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(len(ii), int(round(fraction * len(ii))), replace=False))
    out = System(**{k: getattr(system, k) for k in system.__dataclass_fields__})
    out.exclusions = (ii[pick].astype(np.int32), jj[pick].astype(np.int32))
    return out


def synth_chain(seed: int, nbead: int, compact_steps: int = 2000, params=None) -> System:
    """Seeded self-avoiding 3.8 A chain compacted by minimisation
    (sop_synth_chain), with its SOP topology."""
    xyz = _lib.synth_chain(seed, nbead, compact_steps)
    return system_from_xyz(xyz, None, params)


def synth_globule(seed: int, nchain: int, chain_len: int, compact_steps: int = 2000,
                  params=None) -> System:
    xyz = _lib.synth_globule(seed, nchain, chain_len, compact_steps)
    chain = np.repeat(np.arange(nchain, dtype=np.int32), chain_len)
    return system_from_xyz(xyz, chain, params)


# ---- the reference's input files -------------------------------------------

DEFAULT_SCRIPT = [
    ("set", "zeta", "50"),        # config text: zeta=50 then dt=0.05 (order matters)
    ("set", "t_step", "0.05"),
    ("set", "temp", "0.6"),
    ("set", "nstep", "1000"),
    ("set", "nup", "1000"),
    ("set", "cutofftype", "neighborlist"),
    ("set", "nnlup", "10"),
    ("set", "boxl", "500"),
    ("set", "ncell", "62.5"),     # lcell = 8 A
    ("set", "run", "1"),
]


def write_reference_files(system: System, dirpath: str, script=None, run: bool = True) -> str:
    """Write bonds/angles/vdw/init files and a command script in the formats
    params.cpp:110-260 and io.cpp:9-89 read.  Returns the script path."""
    os.makedirs(dirpath, exist_ok=True)
    n = system.nbead
    ib, jb, r0 = system.bonds
    with open(os.path.join(dirpath, "bonds.dat"), "w") as f:
        f.write("nbnd %d\n" % len(ib))
        for a, b, r in zip(ib, jb, r0):
            f.write("%d %d %.6f\n" % (a + 1, b + 1, r))
    ia, ja, ka, a0 = system.angles
    with open(os.path.join(dirpath, "angles.dat"), "w") as f:
        f.write("nang %d\n" % len(ia))
        for a, b, c, r in zip(ia, ja, ka, a0):
            f.write("%d %d %d %.6f\n" % (a + 1, b + 1, c + 1, r))
    in_, jn, rn = system.natives
    nat = {(int(a), int(b)): float(r) for a, b, r in zip(in_, jn, rn)}
    excl = set()
    if system.exclusions is not None:
        excl = set(zip(np.asarray(system.exclusions[0]).tolist(),
                       np.asarray(system.exclusions[1]).tolist()))
    ch = system.chain
    types = system.bead_type if system.bead_type is not None else np.ones(n, np.int32)
    lines = []
    natt = 0
    for i in range(n):
        for j in range(i + 1, n):
            if not ((ch is not None and ch[i] != ch[j]) or j - i > 2):
                continue
            r = nat.get((i, j))
            if r is not None:
                natt += 1
            else:
                if (i, j) in excl:
                    continue  # left out of the file: never interacts
                # any distance at or above rcut_nat keeps the pair non-native
                r = max(RCUT_NAT[types[i], types[j]] + 1.0,
                        float(np.sqrt(((system.xyz[j] - system.xyz[i]) ** 2).sum())))
            lines.append("%d %d %.6f %d %d\n" % (i + 1, j + 1, r, types[i], types[j]))
    with open(os.path.join(dirpath, "vdw.dat"), "w") as f:
        f.write("ncon_att %d ncon_rep %d\n" % (natt, len(lines) - natt))
        f.writelines(lines)
    with open(os.path.join(dirpath, "init.dat"), "w") as f:
        f.write("nbead %d\n" % n)
        for i, (x, y, z) in enumerate(system.xyz):
            f.write("%d %.6f %.6f %.6f\n" % (i + 1, x, y, z))
    cmds = [("load", "bonds", "bonds.dat"), ("load", "angles", "angles.dat"),
            ("load", "vdw", "vdw.dat"), ("load", "init", "init.dat")]
    cmds += list(script if script is not None else DEFAULT_SCRIPT)
    path = os.path.join(dirpath, "input")
    with open(path, "w") as f:
        for c in cmds:
            f.write(" ".join(c) + ";\n")
        if run:
            f.write("run;\n")
    return path


def script_params(script) -> dict:
    """Integrator constants and switches a command script sets, replayed with
    the side effects of set_params (params.cpp:12-101)."""
    p = dict(T=0.6, zeta=0.05, h=2.5e-3, boxl=500.0, ncell=55.0, nnlup=50, nup=1000,
             nstep=5e7, run=1, neighborlist=0, celllist=0, sim_type=1)
    p["halfh"] = p["h"] / 2.0
    _integ(p)
    p["a5"] = p["h"] / p["zeta"]  # params.cpp:392
    p["lcell"] = p["boxl"] / p["ncell"]
    for _, key, *val in script:
        v = val[0] if val else None
        if key == "temp":
            p["T"] = float(v)
        elif key == "nstep":
            p["nstep"] = float(v)
        elif key == "nup":
            p["nup"] = int(v)
        elif key == "run":
            p["run"] = int(v)
        elif key == "cutofftype":
            if v == "neighborlist":
                p["neighborlist"] = 1
            elif v == "celllist":
                p["celllist"] = 1
        elif key == "nnlup":
            p["nnlup"] = int(v)
        elif key == "boxl":
            p["boxl"] = float(v)
        elif key == "ncell":
            p["ncell"] = float(v)
            p["lcell"] = p["boxl"] / p["ncell"]
        elif key == "t_step":
            p["h"] = float(v)
            p["halfh"] = p["h"] / 2.0
            _integ(p)
            p["a5"] = p["h"] / p["zeta"]
        elif key == "zeta":
            p["h"] = 2.5e-3 if p["sim_type"] == 1 else 0.02
            p["zeta"] = float(v)
            h, z, hh = p["h"], p["zeta"], p["halfh"]
            p["a1"] = h * (1.0 - z * hh)
            p["a3"] = (1.0 - h * z / 2.0 + (h * z) * (h * z) / 4.0) / h
            p["a4"] = hh * (1.0 - h * z / 2.0)
            p["a5"] = h / z
        elif key == "dynamics" and v == "underdamped":
            p["sim_type"] = 1
            p["h"] = 2.5e-3
            p["halfh"] = p["h"] / 2.0
            _integ(p)
        elif key == "dynamics" and v == "overdamped":
            p["sim_type"] = 2
            p["h"] = 0.02
            p["a5"] = p["h"] / p["zeta"]
    return p


def _integ(p):
    h, z, hh = p["h"], p["zeta"], p["halfh"]
    p["a1"] = h * (1.0 - z * hh)
    p["a2"] = h * hh
    p["a3"] = (1.0 - h * z / 2.0 + (h * z) * (h * z) / 4.0) / h
    p["a4"] = hh * (1.0 - h * z / 2.0)


# ---- the benchmark workloads -------------------------------------------------

def loguniform_sizes(seed: int, count: int, lo: int, hi: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), count)).round().astype(np.int64)


def mixed_batch(count: int = 512, lo: int = 30, hi: int = 1500, seed: int = 2000,
                compact_steps: int = 2000, synth_many=None):
    """Batched-replica workload: ``count`` chains with log-uniform bead counts
    in [lo, hi] and temperatures uniform in [0.4, 0.9]; replica r is seeded
    ``seed + r``.  Returns (systems, temperatures).  ``synth_many`` replaces
    the engine library's generator with another build of the same source
    (same seeds, same coordinates)."""
    sizes = loguniform_sizes(seed, count, lo, hi)
    temps = np.random.default_rng(seed + 7).uniform(0.4, 0.9, count)
    gen = synth_many or _lib.synth_many
    xyzs = gen([(seed + r, int(n)) for r, n in enumerate(sizes)], compact_steps)
    systems = [system_from_xyz(x) for x in xyzs]
    return systems, temps
