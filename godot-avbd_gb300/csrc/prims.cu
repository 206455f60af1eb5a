// Parallel primitives (see prims.cuh). Counts come from device memory; grids from capacities.

#include "prims.cuh"

#include <mutex>
#include <vector>

namespace avbdg {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kTopThreads = 1024;
// Capacities up to one block's reach are scanned by a single block in one launch (the stores of
// single worlds up to ~2000 bodies): the three-launch form's fixed cost dominates there.
constexpr int kSmallThreads = 1024;
constexpr int kSmallItems = 16;
constexpr int kSmallScanCap = kSmallThreads * kSmallItems;

__device__ __forceinline__ int loadCount(const int *d_n, int capacity) {
    if (!d_n)
        return capacity;
    const int n = *d_n;
    return n < capacity ? n : capacity;
}

// Block-wide exclusive scan of one value per thread; returns the prefix, writes the total.
template <int THREADS>
__device__ __forceinline__ int blockExclusiveScan(int v, int *smemWarp, int &total) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        smemWarp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        constexpr int W = THREADS / 32;
        int s = lane < W ? smemWarp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < W)
            smemWarp[lane] = s;
    }
    __syncthreads();
    const int warpPrefix = warp > 0 ? smemWarp[warp - 1] : 0;
    total = smemWarp[THREADS / 32 - 1];
    __syncthreads();
    return warpPrefix + x - v;
}

__global__ void scanReduceKernel(const int *in, int capacity, const int *d_n, int *blockSums) {
    pdlWait();
    pdlTrigger();
    __shared__ int warpSums[kScanThreads / 32];
    const int n = loadCount(d_n, capacity);
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int i = base + k;
        if (i < n)
            s += in[i];
    }
    int total;
    blockExclusiveScan<kScanThreads>(s, warpSums, total);
    if (threadIdx.x == 0)
        blockSums[blockIdx.x] = total;
}

__global__ void scanTopKernel(int *blockSums, int numBlocks, int *d_total) {
    pdlWait();
    pdlTrigger();
    __shared__ int warpSums[kTopThreads / 32];
    const int per = (numBlocks + kTopThreads - 1) / kTopThreads;
    const int first = threadIdx.x * per;
    int s = 0;
    for (int k = 0; k < per; k++) {
        const int i = first + k;
        if (i < numBlocks)
            s += blockSums[i];
    }
    int total;
    int prefix = blockExclusiveScan<kTopThreads>(s, warpSums, total);
    for (int k = 0; k < per; k++) {
        const int i = first + k;
        if (i < numBlocks) {
            const int v = blockSums[i];
            blockSums[i] = prefix;
            prefix += v;
        }
    }
    if (threadIdx.x == 0 && d_total)
        *d_total = total;
}

// The whole scan in one block: each thread holds kSmallItems consecutive values (read before any
// write, so `in` may alias `out`), exactly the prefixes the three-launch form writes.
__global__ void __launch_bounds__(kSmallThreads) scanSmallKernel(const int *in, int *out, int capacity,
                                                                 const int *d_n, int *d_total) {
    pdlWait();
    pdlTrigger();
    __shared__ int warpSums[kSmallThreads / 32];
    const int n = loadCount(d_n, capacity);
    const int base = threadIdx.x * kSmallItems;
    int v[kSmallItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kSmallItems; k++) {
        const int i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int total;
    int prefix = blockExclusiveScan<kSmallThreads>(s, warpSums, total);
#pragma unroll
    for (int k = 0; k < kSmallItems; k++) {
        const int i = base + k;
        if (i < n)
            out[i] = prefix;
        prefix += v[k];
    }
    if (threadIdx.x == 0 && d_total)
        *d_total = total;
}

__global__ void scanDownKernel(const int *in, int *out, int capacity, const int *d_n, const int *blockSums) {
    pdlWait();
    pdlTrigger();
    __shared__ int warpSums[kScanThreads / 32];
    const int n = loadCount(d_n, capacity);
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int total;
    int prefix = blockExclusiveScan<kScanThreads>(s, warpSums, total) + blockSums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int i = base + k;
        if (i < n)
            out[i] = prefix;
        prefix += v[k];
    }
}

// ---------------------------------------------------------------------------------------------
// Radix sort: 8-bit digits, 256 threads x 8 rounds per tile, stable ranking by warp matching.
// ---------------------------------------------------------------------------------------------

constexpr int kRadixThreads = 256;
constexpr int kRadixRounds = 8;
constexpr int kRadixTile = kRadixThreads * kRadixRounds;
constexpr int kRadixBins = 256;

__global__ void radixHistKernel(const uint64_t *keys, int capacity, const int *d_n, int shift, uint32_t mask,
                                int numBlocks, int *hist) {
    pdlWait();
    pdlTrigger();
    __shared__ int h[kRadixBins];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int n = loadCount(d_n, capacity);
    const int base = blockIdx.x * kRadixTile;
    for (int r = 0; r < kRadixRounds; r++) {
        const int i = base + r * kRadixThreads + threadIdx.x;
        if (i < n)
            atomicAdd(&h[(keys[i] >> shift) & mask], 1);
    }
    __syncthreads();
    hist[threadIdx.x * numBlocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void radixScatterKernel(const uint64_t *keysIn, const uint32_t *valsIn, uint64_t *keysOut,
                                   uint32_t *valsOut, int capacity, const int *d_n, int shift, uint32_t mask,
                                   int numBlocks, const int *offsets) {
    pdlWait();
    pdlTrigger();
    __shared__ int running[kRadixBins];
    __shared__ int warpCount[kRadixThreads / 32][kRadixBins];
    __shared__ int roundTotal[kRadixBins];
    const int n = loadCount(d_n, capacity);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    running[threadIdx.x] = offsets[threadIdx.x * numBlocks + blockIdx.x];
    const int base = blockIdx.x * kRadixTile;
    const uint32_t ltMask = (1u << lane) - 1u;
    for (int r = 0; r < kRadixRounds; r++) {
        for (int w = 0; w < kRadixThreads / 32; w++)
            warpCount[w][threadIdx.x] = 0;
        __syncthreads();
        const int i = base + r * kRadixThreads + threadIdx.x;
        const bool valid = i < n;
        uint64_t key = 0;
        uint32_t val = 0;
        uint32_t d = 0xffffffffu;
        if (valid) {
            key = keysIn[i];
            val = valsIn ? valsIn[i] : 0u;
            d = static_cast<uint32_t>((key >> shift) & mask);
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ltMask);
        if (valid && rank == 0)
            warpCount[warp][d] = __popc(peers);
        __syncthreads();
        {
            int acc = 0;
            for (int w = 0; w < kRadixThreads / 32; w++) {
                const int c = warpCount[w][threadIdx.x];
                warpCount[w][threadIdx.x] = acc;
                acc += c;
            }
            roundTotal[threadIdx.x] = acc;
        }
        __syncthreads();
        if (valid) {
            const int pos = running[d] + warpCount[warp][d] + rank;
            keysOut[pos] = key;
            if (valsOut)
                valsOut[pos] = val;
        }
        __syncthreads();
        running[threadIdx.x] += roundTotal[threadIdx.x];
        __syncthreads();
    }
}

template <typename T>
__global__ void copyKernel(const T *src, T *dst, int capacity, const int *d_n) {
    pdlWait();
    pdlTrigger();
    const int n = loadCount(d_n, capacity);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// ---------------------------------------------------------------------------------------------
// Segmented sort
// ---------------------------------------------------------------------------------------------

constexpr int kSmallSeg = 32;
constexpr int kMidSegThreads = 256;
constexpr int kMidSegCap = 8192;
constexpr int kBigBlocks = 64;
constexpr int kBigTile = 2048;

template <typename T>
__global__ void segSmallKernel(T *data, const int *start, int segCapacity, const int *d_segments, int *longList,
                               int *longCount) {
    pdlWait();
    pdlTrigger();
    const int ns = loadCount(d_segments, segCapacity);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int b = start[s], e = start[s + 1];
        const int len = e - b;
        if (len <= 1)
            continue;
        if (len > kSmallSeg) {
            longList[atomicAdd(longCount, 1)] = s;
            continue;
        }
        for (int i = b + 1; i < e; i++) {
            const T x = data[i];
            int j = i - 1;
            while (j >= b && data[j] > x) {
                data[j + 1] = data[j];
                j--;
            }
            data[j + 1] = x;
        }
    }
}

template <typename T>
__global__ void segMidKernel(T *data, const int *start, const int *longList, const int *longCount) {
    pdlWait();
    pdlTrigger();
    extern __shared__ unsigned char smemRaw[];
    T *buf = reinterpret_cast<T *>(smemRaw);
    const int nl = *longCount;
    for (int k = blockIdx.x; k < nl; k += gridDim.x) {
        const int s = longList[k];
        const int b = start[s], len = start[s + 1] - start[s];
        if (len > kMidSegCap)
            continue;
        for (int i = threadIdx.x; i < len; i += blockDim.x)
            buf[i] = data[b + i];
        __syncthreads();
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            const T x = buf[i];
            int rank = 0;
            for (int j = 0; j < len; j++)
                rank += buf[j] < x ? 1 : 0;
            data[b + rank] = x;
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void segBigCopyKernel(const T *data, T *tmp, const int *start, const int *longList, const int *longCount) {
    pdlWait();
    pdlTrigger();
    const int nl = *longCount;
    for (int k = 0; k < nl; k++) {
        const int s = longList[k];
        const int b = start[s], len = start[s + 1] - start[s];
        if (len <= kMidSegCap)
            continue;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
            tmp[b + i] = data[b + i];
    }
}

template <typename T>
__global__ void segBigRankKernel(T *data, const T *tmp, const int *start, const int *longList, const int *longCount) {
    pdlWait();
    pdlTrigger();
    __shared__ T tile[kBigTile];
    const int nl = *longCount;
    for (int k = 0; k < nl; k++) {
        const int s = longList[k];
        const int b = start[s], len = start[s + 1] - start[s];
        if (len <= kMidSegCap)
            continue;
        for (int i0 = blockIdx.x * blockDim.x; i0 < len; i0 += gridDim.x * blockDim.x) {
            const int i = i0 + threadIdx.x;
            const T x = i < len ? tmp[b + i] : T(0);
            int rank = 0;
            for (int t0 = 0; t0 < len; t0 += kBigTile) {
                __syncthreads();
                for (int j = threadIdx.x; j < kBigTile && t0 + j < len; j += blockDim.x)
                    tile[j] = tmp[b + t0 + j];
                __syncthreads();
                const int tl = len - t0 < kBigTile ? len - t0 : kBigTile;
                if (i < len)
                    for (int j = 0; j < tl; j++)
                        rank += tile[j] < x ? 1 : 0;
            }
            if (i < len)
                data[b + rank] = x;
        }
    }
}

} // namespace

size_t scanScratchBytes(int capacity) {
    const int blocks = divUp(capacity > 0 ? capacity : 1, kScanTile);
    return static_cast<size_t>(blocks) * sizeof(int) + 256;
}

size_t radixScratchBytes(int capacity) {
    const int blocks = divUp(capacity > 0 ? capacity : 1, kRadixTile);
    const int histN = blocks * kRadixBins;
    return static_cast<size_t>(histN) * sizeof(int) + scanScratchBytes(histN) + 256;
}

void scanExclusive(const int *in, int *out, int capacity, const int *d_n, int *d_total, void *scratch,
                   cudaStream_t stream) {
    if (capacity <= kSmallScanCap) {
        ++launchCount(); launchK(scanSmallKernel, 1, kSmallThreads, 0, stream, in, out, capacity, d_n, d_total);
        return;
    }
    const int blocks = divUp(capacity > 0 ? capacity : 1, kScanTile);
    int *blockSums = static_cast<int *>(scratch);
    ++launchCount(); launchK(scanReduceKernel, blocks, kScanThreads, 0, stream, in, capacity, d_n, blockSums);
    ++launchCount(); launchK(scanTopKernel, 1, kTopThreads, 0, stream, blockSums, blocks, d_total);
    ++launchCount(); launchK(scanDownKernel, blocks, kScanThreads, 0, stream, in, out, capacity, d_n, blockSums);
}

void radixSortPairs(uint64_t *keys, uint32_t *values, uint64_t *keysAlt, uint32_t *valuesAlt, int capacity,
                    const int *d_n, int beginBit, int endBit, void *scratch, cudaStream_t stream) {
    const int blocks = divUp(capacity > 0 ? capacity : 1, kRadixTile);
    const int histN = blocks * kRadixBins;
    int *hist = static_cast<int *>(scratch);
    void *scanScratch = reinterpret_cast<char *>(scratch) + static_cast<size_t>(histN) * sizeof(int) + 128;
    uint64_t *kin = keys, *kout = keysAlt;
    uint32_t *vin = values, *vout = valuesAlt;
    int passes = 0;
    for (int bit = beginBit; bit < endBit; bit += 8) {
        const int bits = endBit - bit < 8 ? endBit - bit : 8;
        const uint32_t mask = (1u << bits) - 1u;
        ++launchCount(); launchK(radixHistKernel, blocks, kRadixThreads, 0, stream, kin, capacity, d_n, bit, mask, blocks, hist);
        scanExclusive(hist, hist, histN, nullptr, nullptr, scanScratch, stream);
        ++launchCount(); launchK(radixScatterKernel, blocks, kRadixThreads, 0, stream, kin, vin, kout, vout, capacity, d_n, bit, mask,
                                                                 blocks, hist);
        uint64_t *tk = kin;
        kin = kout;
        kout = tk;
        uint32_t *tv = vin;
        vin = vout;
        vout = tv;
        passes++;
    }
    if (passes & 1) {
        const int grid = divUp(capacity > 0 ? capacity : 1, 256) < 1184 ? divUp(capacity > 0 ? capacity : 1, 256) : 1184;
        ++launchCount(); launchK(copyKernel<uint64_t>, grid, 256, 0, stream, kin, keys, capacity, d_n);
        if (values) {
            ++launchCount();
            launchK(copyKernel<uint32_t>, grid, 256, 0, stream, vin, values, capacity, d_n);
        }
    }
}

template <typename T>
static void segmentedSort(T *data, const int *start, int segCapacity, const int *d_segments, int *longList,
                          int *longCount, T *tmp, cudaStream_t stream) {
    cudaMemsetAsync(longCount, 0, sizeof(int), stream);
    const int grid = divUp(segCapacity > 0 ? segCapacity : 1, 256);
    ++launchCount(); launchK(segSmallKernel<T>, grid < 4096 ? grid : 4096, 256, 0, stream, data, start, segCapacity, d_segments, longList,
                                                                   longCount);
    const size_t smem = kMidSegCap * sizeof(T);
    ++launchCount(); launchK(segMidKernel<T>, 152, kMidSegThreads, smem, stream, data, start, longList, longCount);
    if (tmp) {
        ++launchCount(); launchK(segBigCopyKernel<T>, kBigBlocks, 256, 0, stream, data, tmp, start, longList, longCount);
        ++launchCount(); launchK(segBigRankKernel<T>, kBigBlocks, 256, 0, stream, data, tmp, start, longList, longCount);
    }
}

static bool g_smemConfigured = false;

static void configureSmem();

void preparePrimitives() { configureSmem(); }

int residentGrid(const void *kernel, int block, size_t smem, int want) {
    struct Entry {
        int device;
        const void *kernel;
        int block;
        size_t smem;
        int blocks;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    int blocks = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const Entry &e : cache)
            if (e.device == dev && e.kernel == kernel && e.block == block && e.smem == smem)
                blocks = e.blocks;
        if (blocks == 0) {
            int sms = 0, perSm = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, block, smem);
            blocks = (sms > 0 ? sms : 1) * (perSm > 0 ? perSm : 1);
            cache.push_back(Entry{dev, kernel, block, smem, blocks});
        }
    }
    return want < 1 ? 1 : (want < blocks ? want : blocks);
}

static void configureSmem() {
    if (g_smemConfigured)
        return;
    cudaFuncSetAttribute(segMidKernel<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kMidSegCap * sizeof(uint32_t)));
    cudaFuncSetAttribute(segMidKernel<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kMidSegCap * sizeof(uint64_t)));
    g_smemConfigured = true;
}

void segmentedSortU32(uint32_t *data, uint32_t *tmp, const int *start, int segCapacity, const int *d_segments,
                      int *longList, int *longCount, cudaStream_t stream) {
    configureSmem();
    segmentedSort<uint32_t>(data, start, segCapacity, d_segments, longList, longCount, tmp, stream);
}

void segmentedSortU64(uint64_t *data, uint64_t *tmp, const int *start, int segCapacity, const int *d_segments,
                      int *longList, int *longCount, cudaStream_t stream) {
    configureSmem();
    segmentedSort<uint64_t>(data, start, segCapacity, d_segments, longList, longCount, tmp, stream);
}

} // namespace avbdg
