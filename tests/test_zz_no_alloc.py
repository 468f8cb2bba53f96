"""sop_neighbor_list_noalloc: the neighbor list for callers that cannot
allocate device memory (hosts that own all device memory through their own
pool, loops that cannot take the synchronization an allocation may cause).  Every buffer here is allocated by the test
(torch) and handed over as a device pointer; the library itself allocates
nothing for this call.  Its pairs must equal, as integer sets, the list the
engine's own entry points give (sop_update_neighbor_list +
sop_get_pair_list(which=1)) -- on two calls in a row, the second reusing the
shared scratch left behind by the first.  Collected last on purpose."""
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


def engine_pairs(system):
    with Engine(0, max_beads=1 << 16, max_replicas=4, max_list_entries=1 << 24) as eng:
        r = eng.add(system, make_params(SCRIPT))
        ii, jj = eng.pairs(r, 1)
    return np.stack([ii, jj], 1)


def noalloc_pairs(torch, system):
    n = system.nbead
    dev = torch.device("cuda", 0)
    xyz = torch.tensor(np.ascontiguousarray(system.xyz).reshape(-1), dtype=torch.float64, device=dev)
    ptr, idx = natives_csr(system)
    d_ptr = torch.tensor(ptr, device=dev)
    d_idx = torch.tensor(idx, device=dev)
    cap = 64 * n
    pairs = torch.full((2 * cap,), -1, dtype=torch.int32, device=dev)
    count = torch.full((1,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = L.lib().sop_neighbor_list_noalloc(xyz.data_ptr(), n, None, None, d_ptr.data_ptr(),
                                           d_idx.data_ptr(), pairs.data_ptr(), cap,
                                           count.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0, L.lib().sop_status_string(rc)
    c = int(count.item())
    assert 0 <= c <= cap
    got = pairs[: 2 * c].view(-1, 2).cpu().numpy()
    return got[np.lexsort((got[:, 1], got[:, 0]))]


def test_noalloc_matches_engine_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
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
