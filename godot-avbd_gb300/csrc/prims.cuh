// Parallel primitives of the step: exclusive scan, stable LSD radix sort, segmented sort.
//
// Every primitive takes its element count from DEVICE memory and sizes its grid from a host
// capacity, so a whole step can run without host round trips (and be captured in a graph).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <utility>
#include <cuda_runtime.h>

namespace avbdg {

// Programmatic dependent launch. The step is a chain of dependent kernels, most of them a few
// microseconds long on small stores, so the gap between one kernel's drain and the next one's
// start is a large part of a step. Every kernel of the library is launched with the programmatic
// stream serialization attribute (launchK) and begins with pdlWait() then pdlTrigger(): the next
// kernel's blocks may be scheduled as soon as every block of the current one has started, and each
// waits in pdlWait() until the kernel before it has completed and its writes are visible. So no
// kernel touches memory before its predecessor is done: the order of the step is unchanged.
// (In a kernel launched without the attribute both are no-ops.)
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdlTrigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// A hint that the line holding `p` will be read soon: it is fetched toward this SM's L1 without
// holding a register or waiting, and the value read later is unchanged.
__device__ __forceinline__ void prefetchL1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// AVBDG_NO_PDL=1: plain stream order between kernels (read once per process).
inline bool pdlEnabled() {
    static const bool on = [] {
        const char *v = std::getenv("AVBDG_NO_PDL");
        return !(v && v[0] == '1');
    }();
    return on;
}

// kernel<<<grid, block, smem, stream>>>(args...) with the programmatic serialization attribute.
template <typename... KArgs, typename... Args>
inline void launchK(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                    Args &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdlEnabled() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Scratch sizes the primitives need for `capacity` elements.
size_t scanScratchBytes(int capacity);
size_t radixScratchBytes(int capacity);

// out[i] = sum(in[0..i)) for i < *d_n; *d_total = sum(in[0..*d_n)) (d_total may be null).
// `in` and `out` may alias.
void scanExclusive(const int *in, int *out, int capacity, const int *d_n, int *d_total, void *scratch,
                   cudaStream_t stream);

// Stable ascending sort of (keys, values) by key bits [beginBit, endBit) for *d_n elements.
// Sorted data ends in keys/values; keysAlt/valuesAlt are the ping-pong buffers.
void radixSortPairs(uint64_t *keys, uint32_t *values, uint64_t *keysAlt, uint32_t *valuesAlt, int capacity,
                    const int *d_n, int beginBit, int endBit, void *scratch, cudaStream_t stream);

// Sorts each segment data[start[s] .. start[s+1]) ascending, for s < *d_segments. Segments up to 32
// entries are sorted by one thread, up to 8192 by one block in shared memory, longer ones by a
// tiled rank sort over several blocks through `tmp` (same capacity as `data`). Values must be
// distinct within a segment. `longList` needs `segCapacity` ints, `longCount` one int.
void segmentedSortU32(uint32_t *data, uint32_t *tmp, const int *start, int segCapacity, const int *d_segments,
                      int *longList, int *longCount, cudaStream_t stream);
void segmentedSortU64(uint64_t *data, uint64_t *tmp, const int *start, int segCapacity, const int *d_segments,
                      int *longList, int *longCount, cudaStream_t stream);

inline int divUp(int a, int b) { return (a + b - 1) / b; }

// Blocks of `block` threads (and `smem` dynamic shared bytes) of `kernel` that are resident on the
// current device at once, capped at `want` (at least 1). Grid-stride kernels over a capacity use it so
// that a mostly empty capacity costs no blocks. Cached per (device, kernel, block, smem).
int residentGrid(const void *kernel, int block, size_t smem, int want);
template <typename K>
inline int residentGrid(K *kernel, int block, int want) {
    return residentGrid(reinterpret_cast<const void *>(kernel), block, 0, want);
}

// True when a launch of `kernel` with `block` threads can run: the block is within the kernel's
// launch bounds (its maxThreadsPerBlock, which the occupancy query does not check) and at least one
// such block fits on an SM (registers and shared memory). A failed query's error is cleared here, so
// the launch checks of a later step do not take it for a failed launch.
template <typename K>
inline bool blockFits(K *kernel, int block) {
    cudaFuncAttributes attr{};
    int n = 0;
    if (cudaFuncGetAttributes(&attr, kernel) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return block <= attr.maxThreadsPerBlock && n > 0;
}

// Kernel attributes the primitives need (large dynamic shared memory); call before any capture.
void preparePrimitives();

// Kernels this library launched from the calling host thread (each launch site increments it).
inline int &launchCount() {
    thread_local int count = 0;
    return count;
}

} // namespace avbdg
