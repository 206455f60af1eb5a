// Spatial queries of one world (godot-avbd src/avbd/solver_query.cpp): ray picks and box overlap
// collection. The reference scans the body list; here every (ray, body) pair is one thread and the
// nearest hit per ray is an atomic minimum over (distance, list position), so the winner is the
// reference's (the first body in list order among equal distances). Overlap flags are compacted in
// list order.

#include <cfloat>

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ f3 localHalfExtent(const Dev &d, int g) {
    const real4 s = d.size[g];
    const int shape = (d.meta[g].w >> 18) & 0x3;
    return shape == 1 ? f3{s.x, s.x, s.x} : (shape == 2 ? f3{s.x, s.x, s.z * 0.5f} : scale(xyz(s), 0.5f));
}

// The reference's per-body ray test (solver_query.cpp:48-133): distance in units of `dir` or
// +infinity, and the hit point in the body's frame.
__device__ real rayTest(const Dev &d, int g, f3 origin, f3 dir, f3 &local) {
    const real inf = bitsf(0x7f800000);
    const q4 inv = qconj(asq(d.q[g]));
    const f3 o = qrot(inv, sub(origin, xyz(d.x[g])));
    const f3 dd = qrot(inv, dir);
    if (((d.meta[g].w >> 18) & 0x3) == 1) {
        const real r = d.size[g].x;
        const real b = dot(o, dd);
        const real c = length2(o) - r * r;
        const real disc = b * b - c;
        if (disc < 0.0f)
            return inf;
        const real sq = msqrt(disc);
        real t = -b - sq;
        if (t < 0.0f)
            t = -b + sq;
        if (t < 0.0f)
            return inf;
        local = add(o, scale(dd, t));
        return t;
    }
    const f3 half = localHalfExtent(d, g);
    real tEnter = 0.0f, tExit = inf;
    for (int i = 0; i < 3; ++i) {
        const real di = at(dd, i), oi = at(o, i), hi = at(half, i);
        if (mabs(di) < 1.0e-6f) {
            if (oi < -hi || oi > hi)
                return inf;
            continue;
        }
        const real invD = 1.0f / di;
        real t0 = (-hi - oi) * invD;
        real t1 = (hi - oi) * invD;
        if (t0 > t1) {
            const real tmp = t0;
            t0 = t1;
            t1 = tmp;
        }
        tEnter = smax(tEnter, t0);
        tExit = smin(tExit, t1);
        if (tEnter > tExit)
            return inf;
    }
    const real tHit = tEnter >= 0.0f ? tEnter : tExit;
    if (tHit < 0.0f)
        return inf;
    local = add(o, scale(dd, tHit));
    return tHit;
}

__global__ void pickResetKernel(unsigned long long *best, int rays) {
    pdlWait();
    pdlTrigger();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rays)
        best[r] = ~0ull;
}

// Thread per (ray, body); key = (distance bits, list position), distances >= 0 compare as integers
// (-0 counts as +0, as the reference's comparisons do).
__global__ void pickKernel(Dev d, int base, int count, const float *rays, int nRays, unsigned mask,
                           unsigned long long *best) {
    pdlWait();
    pdlTrigger();
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<long long>(nRays) * count)
        return;
    const int r = static_cast<int>(t / count);
    const int g = base + static_cast<int>(t % count);
    if ((static_cast<unsigned>(d.meta[g].y) & mask) == 0)
        return;
    const float *ray = rays + 6 * r;
    f3 local;
    const real dist = rayTest(d, g, f3{ray[0], ray[1], ray[2]}, f3{ray[3], ray[4], ray[5]}, local);
    if (!(dist < bitsf(0x7f800000)))
        return;
    const unsigned bits = static_cast<unsigned>(fbits(dist + 0.0f));
    const unsigned lp = static_cast<unsigned>(listPos(d, g) - base);
    atomicMin(best + r, (static_cast<unsigned long long>(bits) << 32) | lp);
}

__global__ void pickResultKernel(Dev d, int base, int count, const float *rays, int nRays,
                                 const unsigned long long *best, int *outBody, float *outLocal) {
    pdlWait();
    pdlTrigger();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRays)
        return;
    const unsigned long long key = best[r];
    if (key == ~0ull) {
        outBody[r] = -1;
        outLocal[3 * r] = outLocal[3 * r + 1] = outLocal[3 * r + 2] = 0.0f;
        return;
    }
    const int g = base + (count - 1 - static_cast<int>(key & 0xffffffffu)); // list position -> slot
    const float *ray = rays + 6 * r;
    f3 local{0, 0, 0};
    rayTest(d, g, f3{ray[0], ray[1], ray[2]}, f3{ray[3], ray[4], ray[5]}, local);
    outBody[r] = g - base;
    outLocal[3 * r] = local.x;
    outLocal[3 * r + 1] = local.y;
    outLocal[3 * r + 2] = local.z;
}

// Overlap flag per list position of the world (collectAABB's test, solver_query.cpp:154-170).
__global__ void overlapFlagKernel(Dev d, int base, int count, f3 lo, f3 hi, unsigned mask, int *flags) {
    pdlWait();
    pdlTrigger();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count)
        return;
    const int g = base + (count - 1 - p);
    int hit = 0;
    if ((static_cast<unsigned>(d.meta[g].y) & mask) != 0) {
        const m3 rot = qmat(asq(d.q[g]));
        const f3 h = localHalfExtent(d, g);
        const f3 wx{(mabs(rot.c0.x) * h.x + mabs(rot.c1.x) * h.y) + mabs(rot.c2.x) * h.z,
                    (mabs(rot.c0.y) * h.x + mabs(rot.c1.y) * h.y) + mabs(rot.c2.y) * h.z,
                    (mabs(rot.c0.z) * h.x + mabs(rot.c1.z) * h.y) + mabs(rot.c2.z) * h.z};
        const f3 c = xyz(d.x[g]);
        const f3 bmin = sub(c, wx), bmax = add(c, wx);
        hit = !(bmin.x > hi.x || bmin.y > hi.y || bmin.z > hi.z || lo.x > bmax.x || lo.y > bmax.y || lo.z > bmax.z);
    }
    flags[p] = hit;
}

__global__ void overlapScatterKernel(int base, int count, const int *flags, const int *rank, int capacity,
                                     int *out) {
    pdlWait();
    pdlTrigger();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count || !flags[p])
        return;
    if (rank[p] < capacity)
        out[rank[p]] = count - 1 - p; // list position -> creation index
}

} // namespace

void launchPick(const Dev &d, int base, int count, const float *rays, int nRays, unsigned mask,
                unsigned long long *best, int *outBody, float *outLocal, cudaStream_t s) {
    ++launchCount(); launchK(pickResetKernel, divUp(nRays > 0 ? nRays : 1, kThreads), kThreads, 0, s, best, nRays);
    const long long pairs = static_cast<long long>(nRays) * count;
    if (pairs > 0) {
        ++launchCount();
        launchK(pickKernel, static_cast<unsigned>((pairs + kThreads - 1) / kThreads), kThreads, 0, s, d, base, count, rays,
                                                                                              nRays, mask, best);
    }
    ++launchCount();
    launchK(pickResultKernel, divUp(nRays > 0 ? nRays : 1, kThreads), kThreads, 0, s, d, base, count, rays, nRays, best,
                                                                                 outBody, outLocal);
}

void launchCollectAabb(const Dev &d, int base, int count, f3 lo, f3 hi, unsigned mask, int *flags, int *rank,
                       int *total, void *scanScratch, int capacity, int *out, cudaStream_t s) {
    ++launchCount();
    launchK(overlapFlagKernel, divUp(count > 0 ? count : 1, kThreads), kThreads, 0, s, d, base, count, lo, hi, mask, flags);
    scanExclusive(flags, rank, count, nullptr, total, scanScratch, s);
    ++launchCount();
    launchK(overlapScatterKernel, divUp(count > 0 ? count : 1, kThreads), kThreads, 0, s, base, count, flags, rank, capacity,
                                                                                    out);
}

} // namespace avbdg
