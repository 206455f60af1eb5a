// Standalone sort + unique of 64-bit keys in device memory: the reference's candidate-pair pass
// radix_std::sort_with_buffer followed by std::unique (godot-avbd src/radixsort.hpp:24-83,
// src/avbd/solver_broadphase.cpp:136-137), as a GPU service over a caller-owned key buffer.

#include <cstring>
#include <mutex>
#include <string>

#include "avbdg.h"
#include "prims.cuh"

namespace avbdg {

void setLastError(const std::string &msg); // capi.cu

namespace {

int sortFail(int code, const std::string &msg) {
    setLastError(msg);
    return code;
}

__global__ void uniqueFlagKernel(const uint64_t *keys, int n, int *flags) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void uniqueScatterKernel(const uint64_t *keys, int n, const int *flags, const int *rank, uint64_t *out) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i])
        out[rank[i]] = keys[i];
}

__global__ void copyBackKernel(const uint64_t *src, uint64_t *dst, const int *count) {
    pdlWait();
    pdlTrigger();
    const int n = *count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Scratch of one call: alternate key buffer, radix histograms, flags, ranks, scan blocks, count.
struct SortScratch {
    uint64_t *keysAlt;
    void *radix;
    int *flags;
    int *ranks;
    void *scan;
    int *count;
};

// The sort + unique sequence, enqueued on `stream` with caller-provided scratch.
void enqueueSortUnique(uint64_t *keys, int n, int bits, const SortScratch &s, cudaStream_t stream) {
    radixSortPairs(keys, nullptr, s.keysAlt, nullptr, n, nullptr, 0, bits, s.radix, stream);
    const int grid = divUp(n, 256);
    launchK(uniqueFlagKernel, grid, 256, 0, stream, keys, n, s.flags);
    scanExclusive(s.flags, s.ranks, n, nullptr, s.count, s.scan, stream);
    launchK(uniqueScatterKernel, grid, 256, 0, stream, keys, n, s.flags, s.ranks, s.keysAlt);
    launchK(copyBackKernel, grid < 1184 ? grid : 1184, 256, 0, stream, s.keysAlt, keys, s.count);
}

int checkArgs(uint64_t *keys, int n, int bits, int *uniqueCount) {
    if (!uniqueCount)
        return sortFail(AVBDG_ERR_INVALID, "unique_count must not be NULL");
    if (n < 0 || (n > 0 && !keys))
        return sortFail(AVBDG_ERR_INVALID, "count must be >= 0 and keys non-NULL when count > 0");
    if (bits < 1 || bits > 64)
        return sortFail(AVBDG_ERR_INVALID, "key_bits must be in [1, 64]");
    return AVBDG_OK;
}

// ---- Fixed scratch for callers that cannot allocate ----------------------------------------
//
// Some callers of this library run where device allocation is not available to them: a host
// that hands its physics thread a fixed memory budget and forbids further device allocations,
// a plugin loaded into an engine whose allocator owns all device memory, or code running while
// another component holds a stream in capture (where a cudaMalloc would break the capture).
// They own their key buffer but cannot obtain scratch. For them the sort's scratch is this
// one array in the library's own device image: it exists on every GPU that loads the library
// and stays there until the process exits.
constexpr int kStaticMaxKeys = 1 << 18; // 262,144 keys per call
constexpr size_t kStaticScratchBytes = size_t(9) << 19; // 4.5 MiB
static __device__ __align__(256) unsigned char g_staticSortScratch[kStaticScratchBytes];

// Device address of g_staticSortScratch, per device. In host code the array's name is only a
// host-side stand-in, so the address is looked up once per device, with that device current.
// The cached address lives as long as the device's primary context: cudaDeviceReset ends it
// (with every other device object of this library on that device), and a call made after a
// reset would use a stale address, so the library must not be used on a device after a reset.
constexpr int kMaxDevices = 64;
static void *g_staticScratchAddr[kMaxDevices] = {};
static std::mutex g_staticScratchMutex;

int staticScratchAddress(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return sortFail(AVBDG_ERR_CUDA, "no current CUDA device for the static sort scratch");
    std::lock_guard<std::mutex> lock(g_staticScratchMutex);
    if (!g_staticScratchAddr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_staticSortScratch);
        if (e != cudaSuccess || !p)
            return sortFail(AVBDG_ERR_CUDA, std::string("cudaGetSymbolAddress of the static sort scratch: ") +
                                                cudaGetErrorString(e));
        g_staticScratchAddr[dev] = p;
    }
    *out = g_staticScratchAddr[dev];
    return AVBDG_OK;
}

} // namespace

} // namespace avbdg

extern "C" {

int avbdg_sort_unique_keys_static(uint64_t *d_keys, int count, int key_bits, int *unique_count, void *stream) {
    using namespace avbdg;
    int rc = checkArgs(d_keys, count, key_bits, unique_count);
    if (rc)
        return rc;
    if (count > kStaticMaxKeys)
        return sortFail(AVBDG_ERR_CAPACITY, "avbdg_sort_unique_keys_static takes at most 262144 keys per call; "
                                            "use avbdg_sort_unique_keys for larger inputs");
    if (count == 0) {
        *unique_count = 0;
        return AVBDG_OK;
    }
    const size_t n = static_cast<size_t>(count);
    const size_t offAlt = 0;
    const size_t offRadix = (offAlt + n * sizeof(uint64_t) + 255) & ~size_t(255);
    const size_t offFlags = (offRadix + radixScratchBytes(count) + 255) & ~size_t(255);
    const size_t offRanks = (offFlags + n * sizeof(int) + 255) & ~size_t(255);
    const size_t offScan = (offRanks + n * sizeof(int) + 255) & ~size_t(255);
    const size_t offCount = (offScan + scanScratchBytes(count) + 255) & ~size_t(255);
    if (offCount + 256 > kStaticScratchBytes)
        return sortFail(AVBDG_ERR_CAPACITY, "static sort scratch too small for this count");
    void *addr = nullptr;
    rc = staticScratchAddress(&addr);
    if (rc)
        return rc;
    char *base = static_cast<char *>(addr);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SortScratch s{reinterpret_cast<uint64_t *>(base + offAlt), base + offRadix, reinterpret_cast<int *>(base + offFlags),
                  reinterpret_cast<int *>(base + offRanks), base + offScan, reinterpret_cast<int *>(base + offCount)};
    // The array keeps whatever the previous call left. Every word this call reads is written by
    // it first (the scan's top kernel writes the count before copyBackKernel reads it); the
    // count is cleared as well, defensively.
    cudaMemsetAsync(s.count, 0, sizeof(int), st);
    enqueueSortUnique(d_keys, count, key_bits, s, st);
    const cudaError_t launch = cudaPeekAtLastError();
    int host = 0;
    cudaMemcpyAsync(&host, s.count, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    const cudaError_t bad = e != cudaSuccess ? e : launch;
    if (bad != cudaSuccess) {
        cudaGetLastError(); // the error is reported through the return code
        return sortFail(AVBDG_ERR_CUDA, std::string("static sort: ") + cudaGetErrorString(bad));
    }
    *unique_count = host;
    return AVBDG_OK;
}

int avbdg_sort_unique_keys(uint64_t *d_keys, int count, int key_bits, int *unique_count, void *stream) {
    using namespace avbdg;
    int rc = checkArgs(d_keys, count, key_bits, unique_count);
    if (rc)
        return rc;
    if (count == 0) {
        *unique_count = 0;
        return AVBDG_OK;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = static_cast<size_t>(count);
    const size_t offAlt = 0;
    const size_t offRadix = (offAlt + n * sizeof(uint64_t) + 255) & ~size_t(255);
    const size_t offFlags = (offRadix + radixScratchBytes(count) + 255) & ~size_t(255);
    const size_t offRanks = (offFlags + n * sizeof(int) + 255) & ~size_t(255);
    const size_t offScan = (offRanks + n * sizeof(int) + 255) & ~size_t(255);
    const size_t offCount = (offScan + scanScratchBytes(count) + 255) & ~size_t(255);
    const size_t total = offCount + 256;
    char *base = nullptr;
    if (cudaMalloc(&base, total) != cudaSuccess)
        return sortFail(AVBDG_ERR_CAPACITY, "cudaMalloc of the sort scratch failed");
    SortScratch s{reinterpret_cast<uint64_t *>(base + offAlt), base + offRadix, reinterpret_cast<int *>(base + offFlags),
                  reinterpret_cast<int *>(base + offRanks), base + offScan, reinterpret_cast<int *>(base + offCount)};
    enqueueSortUnique(d_keys, count, key_bits, s, st);
    const cudaError_t launch = cudaPeekAtLastError();
    int host = 0;
    cudaMemcpyAsync(&host, s.count, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(base);
    const cudaError_t bad = e != cudaSuccess ? e : launch;
    if (bad != cudaSuccess) {
        cudaGetLastError();
        return sortFail(AVBDG_ERR_CUDA, std::string("sort: ") + cudaGetErrorString(bad));
    }
    *unique_count = host;
    return AVBDG_OK;
}

} // extern "C"
