// Idle sleep, wake-ups and islands (godot-avbd src/avbd/solver_broadphase.cpp:69-81, 139-186;
// solver_solve.cpp:146-361). Runs only when Solver::sleepFrames > 0.
//
// * Broad-phase wake-up (wakeSleeperPair): in sorted pair order, a sleeper whose valid pair has an
//   awake movable partner wakes; a body woken by one pair can wake the sleeper of a later pair, so
//   the order matters. Pairs never mix worlds and each world's pairs are contiguous in key order:
//   the pairs that touch a sleeper are compacted in key order and one thread per world replays
//   them serially, worlds in parallel.
// * Wake pass (selectUpdateBodies): a sleeper with a moving awake neighbour wakes. A body woken
//   here has zero velocity and wakes nobody else, so bodies are independent.
// * Islands (islandSleep): sleep-enabled movable bodies joined by manifolds and forces sleep
//   together once none is awake and all have been still long enough. Components by lock-free
//   union-find (roots are component minima; the result does not depend on the schedule).

#include <climits>

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;

int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }

__device__ __forceinline__ int sleepMode(const Dev &d, int g) { return (d.meta[g].w >> 16) & 0x3; }

__device__ __forceinline__ int2 pairBodies(const Dev &d, int k) {
    const uint64_t key = d.pairs[k];
    return make_int2(d.lpToBody[static_cast<int>(key >> 32)], d.lpToBody[static_cast<int>(key & 0xffffffffu)]);
}

// ---- broad-phase wake-up ----

__global__ void wakeResetKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= d.ctr[C_WORLDS])
        return;
    d.wSleep[2 * w] = INT_MAX; // first compacted pair of the world
    d.wSleep[2 * w + 1] = 0;   // number of them
}

__device__ __forceinline__ bool touchesSleeper(const Dev &d, int k, int2 &ab) {
    if (!d.pairValid[k])
        return false;
    ab = pairBodies(d, k);
    return d.sleep[ab.x].x != 0 || d.sleep[ab.y].x != 0;
}

__global__ void wakeFlagKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ctr[C_PAIRS])
        return;
    int2 ab;
    d.sleepRank[k] = touchesSleeper(d, k, ab) ? 1 : 0;
}

__global__ void wakeScatterKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.ctr[C_PAIRS])
        return;
    int2 ab;
    if (!touchesSleeper(d, k, ab))
        return;
    const int r = d.sleepRank[k];
    d.sleepList[r] = k;
    const int w = d.meta[ab.x].x;
    atomicMin(&d.wSleep[2 * w], r);
    atomicAdd(&d.wSleep[2 * w + 1], 1);
}

// wakeSleeperPair over one world's compacted pairs, in key order.
__global__ void wakeWalkKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= d.ctr[C_WORLDS])
        return;
    const int first = d.wSleep[2 * w], count = d.wSleep[2 * w + 1];
    for (int r = first; r < first + count; r++) {
        const int2 ab = pairBodies(d, d.sleepList[r]);
        const int2 sa = d.sleep[ab.x], sb = d.sleep[ab.y];
        if (sa.x && !sb.x && d.x[ab.y].w > 0.0f)
            d.sleep[ab.x] = make_int2(0, 0);
        else if (sb.x && !sa.x && d.x[ab.x].w > 0.0f)
            d.sleep[ab.y] = make_int2(0, 0);
    }
}

// ---- wake pass over the adjacency ----

__global__ void wakeNeighboursKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.ctr[C_BODIES] || d.meta[g].x < 0 || !d.sleep[g].x || sleepMode(d, g) != 1)
        return;
    for (int e = d.adjStart[g]; e < d.adjStart[g + 1]; e++) {
        const int o = adjInfoOther(d.adjInfo[e]);
        if (o < 0 || !(d.x[o].w > 0.0f) || d.sleep[o].x)
            continue;
        if (length2(xyz(d.v[o])) > p.sleepLin2 || length2(xyz(d.w[o])) > p.sleepAng2) {
            d.sleep[g] = make_int2(0, 0);
            return;
        }
    }
}

// ---- islands ----

__device__ __forceinline__ bool islandMember(const Dev &d, int g) {
    return d.meta[g].x >= 0 && d.x[g].w > 0.0f && sleepMode(d, g) == 1;
}

__global__ void islandInitKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.ctr[C_BODIES])
        return;
    d.island[g] = islandMember(d, g) ? g : -1;
    d.islandAwake[g] = 0;
    d.islandStill[g] = INT_MAX;
}

__device__ __forceinline__ int findRoot(const Dev &d, int x) {
    int p = d.island[x];
    while (p != x) { // path halving; concurrent updates only ever point closer to the root
        const int gp = d.island[p];
        if (gp != p)
            atomicCAS(&d.island[x], p, gp);
        x = p;
        p = d.island[x];
    }
    return x;
}

// Link the larger root under the smaller one; retry when another thread moved a root first.
__device__ __forceinline__ void unite(const Dev &d, int a, int b) {
    if (a < 0 || b < 0 || d.island[a] < 0 || d.island[b] < 0)
        return;
    int ra = findRoot(d, a), rb = findRoot(d, b);
    while (ra != rb) {
        if (ra > rb) {
            const int t = ra;
            ra = rb;
            rb = t;
        }
        const int old = atomicCAS(&d.island[rb], rb, ra);
        if (old == rb)
            return;
        rb = findRoot(d, old);
        ra = findRoot(d, ra);
    }
}

__global__ void islandUnionKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nm = d.ctr[C_LIVE], nf = d.ctr[C_FORCES];
    if (i < nm) {
        const int2 ab = d.live.ab[i];
        unite(d, ab.x, ab.y);
    } else if (i < nm + nf) {
        const int2 ab = d.fAB[i - nm];
        unite(d, ab.x, ab.y);
    }
}

__global__ void islandAggregateKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.ctr[C_BODIES] || d.island[g] < 0)
        return;
    const int r = findRoot(d, g);
    const int2 s = d.sleep[g];
    if (!s.x)
        atomicOr(&d.islandAwake[r], 1);
    atomicMin(&d.islandStill[r], s.y);
}

__global__ void islandApplyKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.ctr[C_BODIES] || d.island[g] < 0)
        return;
    const int r = findRoot(d, g);
    if (d.islandAwake[r] || d.islandStill[r] < p.sleepFrames)
        return;
    const int2 s = d.sleep[g];
    if (!s.x) {
        d.sleep[g] = make_int2(1, s.y);
        const real4 v = d.v[g];
        d.v[g] = mk4(0.0f, 0.0f, 0.0f, v.w);
        d.w[g] = mk4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

} // namespace

void launchSleepWakePairs(const Dev &d, cudaStream_t s) {
    ++launchCount(); launchK(wakeResetKernel, grid(d.WW), kThreads, 0, s, d);
    ++launchCount(); launchK(wakeFlagKernel, grid(d.PP), kThreads, 0, s, d);
    scanExclusive(d.sleepRank, d.sleepRank, d.PP, d.ctr + C_PAIRS, nullptr, d.scanScratch, s);
    ++launchCount(); launchK(wakeScatterKernel, grid(d.PP), kThreads, 0, s, d);
    ++launchCount(); launchK(wakeWalkKernel, grid(d.WW), kThreads, 0, s, d);
}

void launchSleepSelect(const Dev &d, const StepParams &p, cudaStream_t s) {
    ++launchCount(); launchK(wakeNeighboursKernel, grid(d.NB), kThreads, 0, s, d, p);
    ++launchCount(); launchK(islandInitKernel, grid(d.NB), kThreads, 0, s, d);
    ++launchCount(); launchK(islandUnionKernel, grid(d.MM + d.FF), kThreads, 0, s, d);
    ++launchCount(); launchK(islandAggregateKernel, grid(d.NB), kThreads, 0, s, d);
    ++launchCount(); launchK(islandApplyKernel, grid(d.NB), kThreads, 0, s, d, p);
}

} // namespace avbdg
