"""avbdg_sort_unique_keys_static: the sort + unique for callers that cannot allocate device memory
(fixed budgets, engines that own the allocator, code running while another component captures a
stream). Its scratch is a fixed array inside the library instead of a cudaMalloc per call.

Checked through the C ABI against avbdg_sort_unique_keys (the allocating entry point) on two calls
in a row, so a result left behind in the shared array by the first call cannot leak into the
second. The comparison is exact, like every integer check in this suite. Also checked: a call
leaves the device's free memory unchanged, and it runs beside another stream's capture without
breaking it."""

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


def test_static_call_allocates_nothing(pkg):
    """After a first call (which looks up the array's address and loads the kernels), a full-size
    call leaves the device's free memory exactly where it was."""
    import torch

    lib = pkg.load_library()
    static_sort = _bind(lib, "avbdg_sort_unique_keys_static")
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 1 << 50, size=STATIC_MAX_KEYS, dtype=np.uint64)
    _sorted_unique(static_sort, keys, 50)
    t = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    out = ctypes.c_int(-1)
    assert static_sort(ctypes.c_void_p(t.data_ptr()), int(keys.size), 50, ctypes.byref(out), None) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert np.array_equal(t.cpu().numpy().view(np.uint64)[: out.value], np.unique(keys))


@pytest.mark.parametrize("mode", ["relaxed", "thread_local"])
def test_static_call_beside_a_capture(pkg, mode):
    """Another component captures a CUDA graph on its own stream (in relaxed mode from this
    thread, or in thread-local mode from another thread) while this thread sorts on a separate
    non-blocking stream: the sort is right and the other capture stays valid."""
    import threading

    import torch

    lib = pkg.load_library()
    static_sort = _bind(lib, "avbdg_sort_unique_keys_static")
    rng = np.random.default_rng(11)
    keys = rng.integers(0, 1 << 30, size=50000, dtype=np.uint64)
    _sorted_unique(static_sort, keys, 30)  # first call on this device: before any capture
    t = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    x = torch.zeros(4096, device="cuda")
    capture_stream, sort_stream = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    out = ctypes.c_int(-1)
    rc = []

    def sort():
        rc.append(static_sort(ctypes.c_void_p(t.data_ptr()), int(keys.size), 30, ctypes.byref(out),
                              ctypes.c_void_p(sort_stream.cuda_stream)))

    if mode == "relaxed":
        with torch.cuda.graph(graph, stream=capture_stream, capture_error_mode="relaxed"):
            x.add_(1.0)
            sort()
            x.mul_(3.0)
    else:
        inside, release, captured = threading.Event(), threading.Event(), []

        def capture():
            with torch.cuda.graph(graph, stream=capture_stream, capture_error_mode="thread_local"):
                x.add_(1.0)
                inside.set()
                release.wait(60)
                x.mul_(3.0)
            captured.append(True)

        th = threading.Thread(target=capture)
        th.start()
        assert inside.wait(60)
        sort()
        release.set()
        th.join(60)
        assert captured, "the other thread's capture failed"
    assert rc == [0]
    assert np.array_equal(t.cpu().numpy().view(np.uint64)[: out.value], np.unique(keys))
    graph.replay()
    torch.cuda.synchronize()
    assert torch.all(x == 3.0).item()
