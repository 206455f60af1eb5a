// Standalone sort + unique of 64-bit keys in device memory: the reference's candidate-pair pass
// radix_std::sort_with_buffer followed by std::unique (godot-avbd src/radixsort.hpp:24-83,
// src/avbd/solver_broadphase.cpp:136-137), as a GPU service over a caller-owned key buffer.

#include <cstring>
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
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void uniqueScatterKernel(const uint64_t *keys, int n, const int *flags, const int *rank, uint64_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i])
        out[rank[i]] = keys[i];
}

__global__ void copyBackKernel(const uint64_t *src, uint64_t *dst, const int *count) {
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
    uniqueFlagKernel<<<grid, 256, 0, stream>>>(keys, n, s.flags);
    scanExclusive(s.flags, s.ranks, n, nullptr, s.count, s.scan, stream);
    uniqueScatterKernel<<<grid, 256, 0, stream>>>(keys, n, s.flags, s.ranks, s.keysAlt);
    copyBackKernel<<<grid < 1184 ? grid : 1184, 256, 0, stream>>>(s.keysAlt, keys, s.count);
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

} // namespace

} // namespace avbdg

extern "C" {

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
    int host = 0;
    cudaMemcpyAsync(&host, s.count, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(base);
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return sortFail(AVBDG_ERR_CUDA, std::string("sort: ") + cudaGetErrorString(e));
    *unique_count = host;
    return AVBDG_OK;
}

} // extern "C"
