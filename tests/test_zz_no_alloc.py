"""sop_neighbor_list_noalloc: the neighbor list for callers that cannot
allocate device memory (hosts that own all device memory through their own
pool, loops that cannot take the synchronization an allocation may cause).  Every buffer here is allocated by the test
(torch) and handed over as a device pointer; the library itself allocates
nothing for this call.  Its pairs must equal, as integer sets, the list the
engine's own entry points give (sop_update_neighbor_list +
sop_get_pair_list(which=1)) -- on two calls in a row, the second reusing the
shared scratch left behind by the first; for an extended chain near the size
limit whose extent (24,000 A) stretches the FP32 relative positions, also the
oracle's FP64 list; for several chains of bead types 1 and 2.  Rejected
input (non-finite positions, other bead types) reports a negative count.
Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from sop_gb300 import _lib as L
from sop_gb300 import systems as S
from sop_gb300.engine import Engine, make_params

pytestmark = pytest.mark.gpu

MAX_BEADS = 16384  # SOP_NOALLOC_MAX_BEADS
SCRIPT = [("set", "zeta", "50"), ("set", "t_step", "0.05"), ("set", "cutofftype", "neighborlist"),
          ("set", "nnlup", "10"), ("set", "boxl", "2000"), ("set", "run", "1")]


def natives_csr(system):
    n = system.nbead
    per = [[] for _ in range(n)]
    for i, j in zip(system.natives[0], system.natives[1]):
        per[int(i)].append(int(j))
        per[int(j)].append(int(i))
    ptr, idx = [0], []
    for row in per:
        idx.extend(sorted(row))
        ptr.append(len(idx))
    return np.array(ptr, np.int32), np.array(idx if idx else [0], np.int32)


def engine_pairs(system, script=SCRIPT):
    with Engine(0, max_beads=1 << 16, max_replicas=4, max_list_entries=1 << 24) as eng:
        r = eng.add(system, make_params(script))
        ii, jj = eng.pairs(r, 1)
        assert eng.status(r)[0] == 0
    a = np.stack([ii, jj], 1)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def noalloc_call(torch, system, xyz=None, types=None):
    """One call through the C ABI; returns (status, count, sorted pairs)."""
    n = system.nbead
    dev = torch.device("cuda", 0)
    x = system.xyz if xyz is None else xyz
    d_xyz = torch.tensor(np.ascontiguousarray(x).reshape(-1), dtype=torch.float64, device=dev)
    t = system.bead_type if types is None else types
    d_type = torch.tensor(np.asarray(t, np.int32), device=dev) if t is not None else None
    d_chain = (torch.tensor(np.asarray(system.chain, np.int32), device=dev)
               if system.chain is not None else None)
    ptr, idx = natives_csr(system)
    d_ptr = torch.tensor(ptr, device=dev)
    d_idx = torch.tensor(idx, device=dev)
    cap = 64 * n
    pairs = torch.full((2 * cap,), -1, dtype=torch.int32, device=dev)
    count = torch.full((1,), 12345, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = L.lib().sop_neighbor_list_noalloc(
        d_xyz.data_ptr(), n, d_type.data_ptr() if d_type is not None else None,
        d_chain.data_ptr() if d_chain is not None else None, d_ptr.data_ptr(), d_idx.data_ptr(),
        pairs.data_ptr(), cap, count.data_ptr(), None)
    torch.cuda.synchronize()
    c = int(count.item())
    if rc != 0 or c < 0:
        return rc, c, None
    assert c <= cap
    got = pairs[: 2 * c].view(-1, 2).cpu().numpy()
    return rc, c, got[np.lexsort((got[:, 1], got[:, 0]))]


def noalloc_pairs(torch, system):
    rc, c, got = noalloc_call(torch, system)
    assert rc == 0, L.lib().sop_status_string(rc)
    assert c >= 0
    return got


def gpu_torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def extended_chain(n, seed):
    """A helix along x (rise 1.5 A, radius 4 A, 3.8 A bonds) with seeded
    jitter, 1.5 n A long, its start 25,000 A from the origin."""
    i = np.arange(n)
    rise, radius = 1.5, 4.0
    w = 2.0 * np.arcsin(np.sqrt(3.8 ** 2 - rise ** 2) / (2.0 * radius))
    xyz = np.stack([rise * i, radius * np.cos(w * i), radius * np.sin(w * i)], 1)
    xyz = xyz + np.random.default_rng(seed).normal(0.0, 0.3, xyz.shape)
    xyz[:, 0] += 2.5e4
    return S.system_from_xyz(xyz)


def test_noalloc_matches_engine_on_two_calls_in_a_row():
    torch = gpu_torch()
    for seed, n in ((4100, 900), (4200, 2600)):
        system = S.synth_chain(seed, n)
        want = engine_pairs(system)
        got = noalloc_pairs(torch, system)
        assert len(want) > 0
        np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_more_beads_than_its_scratch_holds():
    fake = C.c_void_p(256)  # never dereferenced: the size check comes first
    rc = L.lib().sop_neighbor_list_noalloc(fake, MAX_BEADS + 1, None, None, None, None, fake, 0,
                                           fake, None)
    assert rc == -6  # SOP_ERR_UNSUPPORTED


def test_noalloc_extended_chain_near_the_size_limit():
    """16,000 beads over 24,000 A: the FP32 relative positions carry ~3e-3 A
    of rounding, so the pre-screen and the cell edge must widen with the
    extent.  Equal to the engine's list and to the oracle's FP64 list (the
    reference's decision over the candidates within 13.2 A), twice in a row."""
    torch = gpu_torch()
    from oracle import oracle as O
    system = extended_chain(16000, 4300)
    ext = system.xyz.max(0) - system.xyz.min(0)
    assert ext.max() > 1e4
    script = [c if c[1] != "boxl" else ("set", "boxl", "1000000") for c in SCRIPT]
    want = engine_pairs(system, script)
    port = O.Port()
    port.set_system(system, prune=3.2 * 3.8 + 1.0)
    for _, k, v in script:
        port.command(k, v)
    port.setup(False)
    ii, jj = port.pairs(1)
    oracle = np.stack([ii, jj], 1)
    oracle = oracle[np.lexsort((oracle[:, 1], oracle[:, 0]))]
    assert len(oracle) > 10000
    np.testing.assert_array_equal(want, oracle)
    for _ in range(2):
        np.testing.assert_array_equal(noalloc_pairs(torch, system), oracle)


def test_noalloc_types_and_chains():
    """Eight chains with a seeded mix of bead types 1 and 2 (list cutoffs
    12.16 / 17.28 / 22.4 A): equal to the engine's list."""
    torch = gpu_torch()
    xyz = L.synth_globule(4400, 8, 400)
    chain = np.repeat(np.arange(8, dtype=np.int32), 400)
    types = np.where(np.random.default_rng(4401).random(len(xyz)) < 0.35, 2, 1).astype(np.int32)
    system = S.system_from_xyz(xyz, chain, bead_type=types)
    want = engine_pairs(system)
    assert len(want) > 0
    np.testing.assert_array_equal(noalloc_pairs(torch, system), want)


def test_noalloc_reports_rejected_input():
    """A non-finite position gives count -1, a bead type other than 1 or 2
    gives count -2 (status SOP_OK: the kernels decide), and the next call on
    valid input is exact again."""
    torch = gpu_torch()
    system = S.synth_chain(4500, 300)
    bad = system.xyz.copy()
    bad[17, 1] = np.nan
    rc, c, _ = noalloc_call(torch, system, xyz=bad)
    assert rc == 0 and c == -1
    far = system.xyz.copy()
    far[3, 0] = 2e6
    rc, c, _ = noalloc_call(torch, system, xyz=far)
    assert rc == 0 and c == -1
    types = np.ones(system.nbead, np.int32)
    types[40] = 3
    rc, c, _ = noalloc_call(torch, system, types=types)
    assert rc == 0 and c == -2
    np.testing.assert_array_equal(noalloc_pairs(torch, system), engine_pairs(system))
