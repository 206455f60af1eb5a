"""avbdg_sort_unique_keys_static: the sort + unique for callers that cannot allocate device memory
(fixed budgets, engines that own the allocator, code running during a stream capture). Its
scratch is a fixed array inside the library instead of a cudaMalloc per call.

Checked through the C ABI against avbdg_sort_unique_keys (the allocating entry point) on two calls
in a row, so a result left behind in the shared array by the first call cannot leak into the
second. The comparison is exact, like every integer check in this suite."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_MAX_KEYS = 1 << 18


def _bind(lib, name):
    fn = getattr(lib, name)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _sorted_unique(fn, keys, bits):
    import torch

    t = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    torch.cuda.synchronize()
    out = ctypes.c_int(-1)
    rc = fn(ctypes.c_void_p(t.data_ptr()), int(keys.size), bits, ctypes.byref(out), None)
    assert rc == 0, rc
    return t.cpu().numpy().view(np.uint64)[: out.value].copy()


def test_static_scratch_sort_matches_allocating_sort(pkg):
    lib = pkg.load_library()
    static_sort = _bind(lib, "avbdg_sort_unique_keys_static")
    alloc_sort = _bind(lib, "avbdg_sort_unique_keys")
    rng = np.random.default_rng(2026)
    # Two calls in a row: a large call fills the shared array, then a smaller one with fewer
    # distinct keys must not see any of it.
    first = rng.integers(0, 1 << 40, size=STATIC_MAX_KEYS, dtype=np.uint64)
    first[::7] = first[3]
    second = rng.choice(rng.integers(0, 1 << 20, size=300, dtype=np.uint64), size=9000).astype(np.uint64)
    for keys, bits in [(first, 40), (second, 20)]:
        got = _sorted_unique(static_sort, keys, bits)
        want = _sorted_unique(alloc_sort, keys, bits)
        assert got.size == want.size and np.array_equal(got, want)
        assert np.array_equal(got, np.unique(keys))


def test_static_scratch_rejects_oversized_input(pkg):
    lib = pkg.load_library()
    static_sort = _bind(lib, "avbdg_sort_unique_keys_static")
    out = ctypes.c_int(-1)
    rc = static_sort(ctypes.c_void_p(16), STATIC_MAX_KEYS + 1, 64, ctypes.byref(out), None)
    assert rc == pkg.capi.ERR_CAPACITY
    err = lib.avbdg_last_error
    err.restype = ctypes.c_char_p
    assert b"262144" in err()
