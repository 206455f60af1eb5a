"""avbdg_sort_unique_keys: sort + unique of 64-bit keys in device memory, checked exactly against
numpy's sort/unique (the reference's pass is radix_std::sort_with_buffer + std::unique)."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fn(pkg):
    lib = pkg.load_library()
    fn = lib.avbdg_sort_unique_keys
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _run(fn, keys, bits):
    import torch

    t = torch.from_numpy(keys.view(np.int64)).cuda()
    out = ctypes.c_int(-1)
    torch.cuda.synchronize()
    rc = fn(ctypes.c_void_p(t.data_ptr()), int(keys.size), bits, ctypes.byref(out), None)
    assert rc == 0
    return t.cpu().numpy().view(np.uint64)[: out.value]


@pytest.mark.parametrize("n,bits,dup", [(1, 64, 1), (7, 8, 1), (5000, 34, 4), (100_000, 40, 2),
                                        (300_000, 64, 1), (4096, 12, 100)])
def test_sort_unique_matches_numpy(pkg, n, bits, dup):
    rng = np.random.default_rng(n + bits)
    base = rng.integers(0, 2 ** min(bits, 63), size=max(1, n // dup), dtype=np.uint64)
    if bits == 64:
        base |= rng.integers(0, 2, size=base.size, dtype=np.uint64) << np.uint64(63)
    keys = rng.choice(base, size=n).astype(np.uint64)
    got = _run(_fn(pkg), keys, bits)
    assert np.array_equal(got, np.unique(keys))


def test_sort_unique_edge_cases(pkg):
    fn = _fn(pkg)
    out = ctypes.c_int(-1)
    assert fn(None, 0, 64, ctypes.byref(out), None) == 0 and out.value == 0
    same = np.full(1000, 42, np.uint64)
    assert np.array_equal(_run(fn, same, 8), np.array([42], np.uint64))
    # Pair keys as the broad phase packs them: (min << 32) | max, already sorted input.
    i = np.arange(2000, dtype=np.uint64)
    pairs = (i << np.uint64(32)) | (i + np.uint64(1))
    assert np.array_equal(_run(fn, pairs, 43), pairs)
    assert fn(None, 10, 64, ctypes.byref(out), None) == pkg.capi.ERR_INVALID
    assert fn(None, 0, 65, ctypes.byref(out), None) == pkg.capi.ERR_INVALID
