"""The C-ABI library on the CPU: it loads, exports every entry point the
header declares, and its host-side numerics (the double -> float split the
kernels stage positions with, the Philox stream) are exact.  No GPU calls."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from sop_gb300 import _lib as L

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "sop_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sop_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(L.exported_symbols())


@pytest.mark.parametrize("name", ["libsopgpu.so", "libsopgpu_checked.so"])
def test_library_exports_every_declared_symbol(name):
    lib = C.CDLL(os.path.join(os.path.dirname(L.LIB_PATH), name))
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing


def test_version_and_defaults():
    assert b"sm_103a" in L.lib().sop_version()
    p = L.default_params()
    # params.cpp:373-392 defaults, then the a1..a4 of zeta=0.05, h=2.5e-3
    assert (p.T, p.zeta, p.h, p.boxl, p.nnlup, p.nup) == (0.6, 0.05, 2.5e-3, 500.0, 50, 1000)
    h, z = 2.5e-3, 0.05
    assert p.a1 == h * (1.0 - z * (h / 2.0))
    assert p.a3 == (1.0 - h * z / 2.0 + (h * z) * (h * z) / 4.0) / h
    c = L.default_engine_config()
    assert c.lanes_per_bead in (1, 2, 4, 8, 16) and c.block_threads % 32 == 0


@pytest.mark.parametrize("fill,struct", [("sop_engine_config_default", L.EngineConfig),
                                         ("sop_params_default", L.Params)])
def test_struct_bindings_match_the_library(fill, struct):
    """The library's default filler clears its whole struct before setting
    fields, so it writes exactly sizeof(struct) bytes: a binding that is
    shorter than the C struct shows as an overwritten sentinel after it, one
    that is longer as sentinel bytes left inside it (no default holds 0xAB)."""
    n = C.sizeof(struct)
    buf = (C.c_ubyte * (n + 64))(*([0xAB] * (n + 64)))
    getattr(L.lib(), fill)(C.cast(buf, C.POINTER(struct)))
    raw = bytes(buf)
    assert raw[n:] == b"\xab" * 64
    assert 0xAB not in raw[:n]


@pytest.mark.parametrize("name", ["sop_params", "sop_system_desc", "sop_engine_config",
                                  "sop_server_config", "sop_request_result"])
def test_struct_sizes_match_the_library(name):
    assert L.lib().sop_struct_size(name.encode()) == C.sizeof(L.STRUCTS[name])


def test_struct_size_of_other_names():
    assert L.lib().sop_struct_size(b"sop_engine") == -1
    assert L.lib().sop_struct_size(None) == -1


def _split(x):
    hi, lo = C.c_float(), C.c_float()
    L.lib().sop_selftest_split(C.c_double(x), C.byref(hi), C.byref(lo))
    return hi.value, lo.value


def test_split_double_is_nearest_float_pair():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.normal(0, 50, 2000), rng.uniform(-1e4, 1e4, 2000),
                         rng.normal(0, 1e-6, 500), [1.0, -1.0, 0.5, 3.8, 1e-30, 0.0, -0.0,
                                                    np.nextafter(1.0, 2.0), 2.0 - 2.0 ** -30]])
    for x in xs:
        hi, lo = _split(float(x))
        want_hi = np.float32(x)  # round to nearest even
        if abs(x) < 2.0 ** -100:
            assert hi == 0.0 and lo == 0.0
            continue
        assert np.float32(hi) == want_hi, x
        rem = float(x) - float(want_hi)  # exact (Sterbenz)
        if abs(rem) < 2.0 ** -126:  # subnormal remainders flush (documented)
            assert abs(lo) < 2.0 ** -126
            continue
        assert np.float32(lo) == np.float32(rem), x
        # hi + lo recovers x to 2^-48 relative
        assert abs((float(hi) + float(lo)) - x) <= abs(x) * 2.0 ** -47


def test_philox_host_build_matches_oracle():
    rng = np.random.default_rng(2)
    for _ in range(200):
        ctr = [int(v) for v in rng.integers(0, 2 ** 32, 4, dtype=np.uint64)]
        key = [int(v) for v in rng.integers(0, 2 ** 32, 2, dtype=np.uint64)]
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        L.lib().sop_selftest_philox(c, k, o)
        assert list(o) == O.philox(ctr, key)


def test_engine_create_without_gpu_reports_nodev(gpu_available):
    if gpu_available:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    c = L.default_engine_config()
    assert L.lib().sop_engine_create(C.byref(c), C.byref(h)) == -7  # SOP_ERR_NODEV
    assert not h.value


def test_null_arguments_are_rejected():
    lib = L.lib()
    assert lib.sop_engine_create(None, None) == -1
    assert lib.sop_engine_destroy(None) == -1
    assert lib.sop_run(None, 10) == -1
    assert lib.sop_replica_add(None, None, None) == -1
    assert lib.sop_synth_chain(1, 0, 10, None) == -1


def test_synth_is_seeded_and_chain_like():
    a = L.synth_chain(11, 200, 500)
    b = L.synth_chain(11, 200, 500)
    c = L.synth_chain(12, 200, 500)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    bonds = np.linalg.norm(a[1:] - a[:-1], axis=1)
    assert np.all(np.abs(bonds - 3.8) < 0.05)
    d = np.linalg.norm(a[:, None] - a[None], axis=-1)
    iu = np.triu_indices(200, 2)
    assert d[iu].min() > 4.0  # excluded-volume floor


def test_l2_probe_rejects_bad_sizes_before_touching_a_device():
    g = C.c_double(-1.0)
    lib = L.lib()
    assert lib.sop_probe_l2_read(0, 1000, 10, C.byref(g)) == -1        # under 1 MB
    assert lib.sop_probe_l2_read(0, 200 << 20, 10, C.byref(g)) == -1   # over 96 MB
    assert lib.sop_probe_l2_read(0, 32 << 20, 0, C.byref(g)) == -1     # no repetitions
    assert lib.sop_probe_l2_read(0, 32 << 20, 10, None) == -1
