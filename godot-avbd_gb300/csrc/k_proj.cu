// Speculative brake and positional projection (godot-avbd src/avbd/solver_projection.cpp:67-281).
//
// The brake is a Gauss-Seidel sweep over manifolds in live order: each braked patch updates its
// bodies' velocities in place and later manifolds see the result. Only manifolds with an open gap
// (some contact with positive separation at the fixed poses) can brake, so the sweep's order only
// matters among them, and a candidate depends on exactly one earlier candidate per movable body:
// the one just before it on that body. The sweep runs as a dataflow inside one cooperative launch:
// every thread takes candidates in increasing live order, waits until the (at most two)
// predecessors have published their velocities, brakes, then publishes its own. Candidates on
// disjoint bodies proceed in parallel and every body sees its candidates in live order, so the
// result equals the serial sweep. The smallest unfinished candidate can always run, so the waits
// end; each is still bounded and reports a timeout instead of hanging. All threads of the
// cooperative launch are resident; everything a candidate reads but the velocities is loaded before
// its wait, so a dependency hop costs only the flag and velocity round trips.
//
// Projection passes are Jacobi: per-manifold patch corrections, then per-body sums in live order
// (the adjacency order), averaged over the manifold count, with the per-world early exit.

#include <cooperative_groups.h>

#include "gridsync.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;
constexpr int kBrakeThreads = 512;

// Movable and in this step's update set (solver_projection.cpp:87, 105-106, 194-195).
__device__ __forceinline__ bool movable(const Dev &d, int g) { return d.x[g].w > 0.0f && inUpdate(d, g); }

__device__ __forceinline__ real angularCompliance(f3 I, f3 axis) {
    real sum = 0.0f;
    if (I.x > 0.0f)
        sum += axis.x * axis.x / I.x;
    if (I.y > 0.0f)
        sum += axis.y * axis.y / I.y;
    if (I.z > 0.0f)
        sum += axis.z * axis.z / I.z;
    return sum;
}

__device__ __forceinline__ f3 angularResponse(f3 I, q4 q, f3 axis) {
    f3 out{0.0f, 0.0f, 0.0f};
    if (I.x > 0.0f)
        out.x = axis.x / I.x;
    if (I.y > 0.0f)
        out.y = axis.y / I.y;
    if (I.z > 0.0f)
        out.z = axis.z / I.z;
    return qrot(q, out);
}

__device__ __forceinline__ void maskLocked(int locks, f3 &v) {
    if (locks) {
        if (locks & 1)
            v.x = 0.0f;
        if (locks & 2)
            v.y = 0.0f;
        if (locks & 4)
            v.z = 0.0f;
    }
}

// projectionActive membership and "can brake" (an open gap at the current poses).
__device__ __forceinline__ void projActiveAt(Dev d, int m) {
    if (m >= d.ctr[C_LIVE])
        return;
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const int n = L.count[m];
    const bool active = n > 0 && (movable(d, ab.x) || movable(d, ab.y));
    uint8_t spec = 0;
    if (active) {
        int *flag = &d.wActive[d.meta[ab.x].x]; // a flag: one store, no atomic traffic on a shared word
        if (*flag == 0)
            *flag = 1;
        const f3 nrm = xyz(L.b0[m]);
        const f3 xa = xyz(d.x[ab.x]), xb = xyz(d.x[ab.y]);
        const q4 qa = asq(d.q[ab.x]), qb = asq(d.q[ab.y]);
        for (int k = 0; k < n; k++) {
            const int ci = cslot(d, m, k);
            const f3 rA = qrot(qa, xyz(L.rA[ci]));
            const f3 rB = qrot(qb, xyz(L.rB[ci]));
            const real gap = dot(nrm, sub(add(xa, rA), add(xb, rB)));
            if (gap > 0.0f) {
                spec = 1;
                break;
            }
        }
    }
    d.mSpec[m] = spec;
    d.mActive[m] = spec;
}

__global__ void projActiveKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x)
        projActiveAt(d, m);
}

// Brake candidates in live order (the scan of their flags gives each one its slot).
__device__ __forceinline__ void specScatterAt(Dev d, const int *flags, const int *rank, int m) {
    if (m >= d.ctr[C_LIVE] || !flags[m])
        return;
    d.specList[rank[m]] = m;
    d.mDone[rank[m]] = 0;
}

__global__ void specScatterKernel(Dev d, const int *flags, const int *rank) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x)
        specScatterAt(d, flags, rank, m);
}

// For each candidate, the preceding candidate on each of its movable bodies (-1 if none), as a
// candidate index, from the body's adjacency (forces first, then manifolds in live order); `rank`
// is the exclusive scan of the candidate flags.
__device__ __forceinline__ void brakePredAt(Dev d, const int *rank, int k) {
    if (k >= d.ctr[C_SPECN])
        return;
    const int m = d.specList[k];
    const int2 ab = d.live.ab[m];
    const int nf = d.ctr[C_FORCES];
    int pred[2] = {-1, -1};
    for (int side = 0; side < 2; side++) {
        const int x = side == 0 ? ab.x : ab.y;
        if (!movable(d, x))
            continue;
        for (int e = d.adjStart[x]; e < d.adjStart[x + 1]; e++) {
            const int seq = static_cast<int>(d.adjSeq[e]);
            if (seq < nf)
                continue;
            const int o = seq - nf;
            if (o >= m)
                break;
            if (d.mSpec[o])
                pred[side] = rank[o];
        }
    }
    d.specPred[k] = make_int2(pred[0], pred[1]);
}

__global__ void brakePredKernel(Dev d, const int *rank) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_SPECN];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        brakePredAt(d, rank, k);
}

__device__ __forceinline__ unsigned loadAcquire(const uint8_t *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u8 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void storeRelease(uint8_t *p, unsigned v) {
    asm volatile("st.release.gpu.global.u8 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool published(const Dev &d, int k) { return k < 0 || loadAcquire(d.mDone + k) != 0; }

// Everything one manifold's brake reads except the velocities: loaded before its wait, so a wait
// is followed only by the velocity reads and the arithmetic.
struct BrakeLoad {
    int a, b, n, locksA, locksB;
    bool moveA, moveB;
    real invMassA, invMassB;
    f3 nrm, IA, IB;
    q4 qa, qb;
    f3 rA[kMaxContacts], rB[kMaxContacts];
    real gap[kMaxContacts];
};

__device__ __forceinline__ void brakeLoad(const Dev &d, int m, BrakeLoad &bl) {
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    bl.a = ab.x;
    bl.b = ab.y;
    const real4 xa4 = d.x[ab.x], xb4 = d.x[ab.y];
    bl.moveA = movable(d, ab.x);
    bl.moveB = movable(d, ab.y);
    bl.invMassA = bl.moveA ? 1.0f / xa4.w : 0.0f;
    bl.invMassB = bl.moveB ? 1.0f / xb4.w : 0.0f;
    bl.nrm = xyz(L.b0[m]);
    bl.qa = asq(d.q[ab.x]);
    bl.qb = asq(d.q[ab.y]);
    bl.IA = xyz(d.moment[ab.x]);
    bl.IB = xyz(d.moment[ab.y]);
    bl.locksA = d.meta[ab.x].w;
    bl.locksB = d.meta[ab.y].w;
    const f3 xa = xyz(xa4), xb = xyz(xb4);
    bl.n = L.count[m];
#pragma unroll
    for (int k = 0; k < kMaxContacts; k++) {
        bl.gap[k] = 0.0f;
        if (k < bl.n) {
            const int ci = cslot(d, m, k);
            bl.rA[k] = qrot(bl.qa, xyz(L.rA[ci]));
            bl.rB[k] = qrot(bl.qb, xyz(L.rB[ci]));
            bl.gap[k] = dot(bl.nrm, sub(add(xa, bl.rA[k]), add(xb, bl.rB[k])));
        }
    }
}

// One manifold of the brake sweep (solver_projection.cpp:98-166) on velocities held by the caller;
// false when no contact braked (velocities untouched).
__device__ __forceinline__ bool brakeSolve(const BrakeLoad &bl, real window, f3 &va, f3 &wa, f3 &vb, f3 &wb) {
    f3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
    real velErr = 0.0f;
    int braked = 0;
#pragma unroll
    for (int k = 0; k < kMaxContacts; k++) {
        if (k >= bl.n || !(bl.gap[k] > 0.0f))
            continue;
        const f3 vAp = add(va, cross(wa, bl.rA[k]));
        const f3 vBp = add(vb, cross(wb, bl.rB[k]));
        const real vn = dot(sub(vAp, vBp), bl.nrm);
        const real target = -bl.gap[k] / window;
        if (vn < target) {
            patchRA = add(patchRA, bl.rA[k]);
            patchRB = add(patchRB, bl.rB[k]);
            velErr += target - vn;
            braked++;
        }
    }
    if (braked == 0)
        return false;
    const real invN = 1.0f / static_cast<real>(braked);
    const f3 tA = bl.moveA ? qrot(qconj(bl.qa), cross(scale(patchRA, invN), bl.nrm)) : f3{0, 0, 0};
    const f3 tB = bl.moveB ? qrot(qconj(bl.qb), cross(scale(patchRB, invN), bl.nrm)) : f3{0, 0, 0};
    const real K = bl.invMassA + bl.invMassB + (bl.moveA ? angularCompliance(bl.IA, tA) : 0.0f) +
                    (bl.moveB ? angularCompliance(bl.IB, tB) : 0.0f);
    const real j = velErr * invN / K;
    if (bl.moveA) {
        f3 dv = scale(bl.nrm, bl.invMassA * j);
        f3 dw = scale(angularResponse(bl.IA, bl.qa, tA), j);
        maskLocked(bl.locksA & 0xff, dv);
        maskLocked((bl.locksA >> 8) & 0xff, dw);
        va = add(va, dv);
        wa = add(wa, dw);
    }
    if (bl.moveB) {
        f3 dv = scale(bl.nrm, bl.invMassB * j);
        f3 dw = scale(angularResponse(bl.IB, bl.qb, tB), j);
        maskLocked(bl.locksB & 0xff, dv);
        maskLocked((bl.locksB >> 8) & 0xff, dw);
        vb = sub(vb, dv);
        wb = sub(wb, dw);
    }
    return true;
}

__global__ void __launch_bounds__(kBrakeThreads) brakeKernel(Dev d, real window) {
    pdlWait();
    pdlTrigger();
    const int ns = d.ctr[C_SPECN];
    const int stride = gridDim.x * blockDim.x;
    volatile int *errors = d.ctr + C_ERRORS;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += stride) {
        const int2 pred = d.specPred[k];
        BrakeLoad bl;
        brakeLoad(d, d.specList[k], bl);
        long long spins = 0;
        while (!(published(d, pred.x) && published(d, pred.y))) {
            if (++spins > d.waitLimit || (*errors & kErrBrakeTimeout)) {
                atomicOr(d.ctr + C_ERRORS, kErrBrakeTimeout);
                return;
            }
            __nanosleep(64);
        }
        const real4 va4 = __ldcg(&d.v[bl.a]), vb4 = __ldcg(&d.v[bl.b]);
        f3 va = xyz(va4), wa = xyz(__ldcg(&d.w[bl.a])), vb = xyz(vb4), wb = xyz(__ldcg(&d.w[bl.b]));
        if (brakeSolve(bl, window, va, wa, vb, wb)) {
            if (bl.moveA) {
                __stcg(&d.v[bl.a], f4(va, va4.w));
                __stcg(&d.w[bl.a], f4(wa, 0.0f));
            }
            if (bl.moveB) {
                __stcg(&d.v[bl.b], f4(vb, vb4.w));
                __stcg(&d.w[bl.b], f4(wb, 0.0f));
            }
        }
        storeRelease(d.mDone + k, 1u); // orders this thread's velocity writes before the flag
    }
}

// ---- positional projection (solver_projection.cpp:169-280) ----

// Returns the patch's mean depth bits for the world's early-exit maximum through `depthBits`
// (left alone when the manifold corrects nothing).
__device__ __forceinline__ void projManifoldAt(Dev d, StepParams p, int m, int &world, int &depthBits) {
    if (m >= d.ctr[C_LIVE])
        return;
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const int a = ab.x, b = ab.y;
    const int w = d.meta[a].x;
    if (d.wStop[w]) // a stopped world's bodies skip the body pass, which reads these entries
        return;
    // The adjacency entries of sides A and B; only bodies with mass have entries (a static side's
    // slot is not written by the adjacency build and is not touched here).
    const int2 slot = d.stampSlot[m];
    const real4 xa4 = d.x[a], xb4 = d.x[b];
    if (xa4.w > 0.0f)
        d.projLin[slot.x].w = 0.0f;
    if (xb4.w > 0.0f)
        d.projLin[slot.y].w = 0.0f;
    const bool moveA = movable(d, a), moveB = movable(d, b);
    const int n = L.count[m];
    if (n == 0 || (!moveA && !moveB))
        return;
    const real invMassA = moveA ? 1.0f / xa4.w : 0.0f;
    const real invMassB = moveB ? 1.0f / xb4.w : 0.0f;
    const f3 nrm = xyz(L.b0[m]);
    const q4 qa = asq(d.q[a]), qb = asq(d.q[b]);
    const f3 xa = xyz(xa4), xb = xyz(xb4);
    const m3 rotA = qmat(qa), rotB = qmat(qb);
    f3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
    real patchDepth = 0.0f;
    int corrected = 0;
    for (int k = 1; k < n; k++) { // the later contacts' arms, requested before the in-order loop
        prefetchL1(&L.rA[cslot(d, m, k)]);
        prefetchL1(&L.rB[cslot(d, m, k)]);
    }
    for (int k = 0; k < n; k++) {
        const int ci = cslot(d, m, k);
        const f3 rA = mul(rotA, xyz(L.rA[ci]));
        const f3 rB = mul(rotB, xyz(L.rB[ci]));
        const real rawDepth = -dot(nrm, sub(add(xa, rA), add(xb, rB)));
        const real depth = rawDepth - p.projSlop;
        if (depth > 0.0f) {
            patchRA = add(patchRA, rA);
            patchRB = add(patchRB, rB);
            patchDepth += depth;
            corrected++;
        }
    }
    if (corrected == 0)
        return;
    const real invN = 1.0f / static_cast<real>(corrected);
    world = w;
    depthBits = fbits(patchDepth * invN); // positive: the bits order like the floats
    const f3 IA = xyz(d.moment[a]), IB = xyz(d.moment[b]);
    const f3 tA = moveA ? qrot(qconj(qa), cross(scale(patchRA, invN), nrm)) : f3{0, 0, 0};
    const f3 tB = moveB ? qrot(qconj(qb), cross(scale(patchRB, invN), nrm)) : f3{0, 0, 0};
    const real K = invMassA + invMassB + (moveA ? angularCompliance(IA, tA) : 0.0f) +
                    (moveB ? angularCompliance(IB, tB) : 0.0f);
    const real dp = p.projBeta * patchDepth * invN / K;
    if (moveA) {
        d.projLin[slot.x] = f4(scale(nrm, invMassA * dp), 1.0f);
        d.projAng[slot.x] = f4(scale(angularResponse(IA, qa, tA), dp), 0.0f);
    }
    if (moveB) {
        d.projLin[slot.y] = f4(scale(nrm, invMassB * dp), -1.0f);
        d.projAng[slot.y] = f4(scale(angularResponse(IB, qb, tB), dp), 0.0f);
    }
}

// Grid-stride in whole warps (every lane runs every pass), so the per-world depth maximum is
// reduced across the warp first and one lane per world and warp does the atomic.
// The manifolds' contributions of one pass, a warp per 32 manifolds: each world's deepest patch is
// reduced across the warp (one atomic per world and warp).
__device__ __forceinline__ void projManifoldPass(const Dev &d, const StepParams &p, int first, int stride) {
    const int n = d.ctr[C_LIVE];
    for (int base = first + (threadIdx.x & ~31); base < n; base += stride) {
        int world = -1, depthBits = 0;
        projManifoldAt(d, p, base + (threadIdx.x & 31), world, depthBits);
        const unsigned peers = __match_any_sync(0xffffffffu, world);
        const int deepest = __reduce_max_sync(peers, depthBits);
        if (world >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1)
            atomicMax(&d.wMaxDepth[world], deepest);
    }
}

// One body's averaged correction of a pass: its contributions in adjacency order, capped, applied.
__device__ __forceinline__ void projBodyAt(const Dev &d, const StepParams &p, int g) {
    // The checks' loads go out together (valid reads of body g), then its world's stop flag.
    const int world = d.meta[g].x;
    const real mass = d.x[g].w;
    const bool updated = inUpdate(d, g);
    if ((world < 0) | !((mass > 0.0f) & updated))
        return;
    if (d.wStop[world])
        return;
    const int nf = d.ctr[C_FORCES];
    f3 sl{0, 0, 0}, sa{0, 0, 0};
    int cnt = 0;
    // Each manifold entry holds the contribution for this body (w: +1 side A, -1 side B, 0 none).
    for (int e = d.adjStart[g]; e < d.adjStart[g + 1]; e++) {
        if (nf > 0 && static_cast<int>(d.adjSeq[e]) < nf)
            continue;
        const real4 cl = d.projLin[e];
        if (cl.w == 0.0f)
            continue;
        const f3 ca = xyz(d.projAng[e]);
        cnt++;
        if (cl.w > 0.0f) {
            sl = add(sl, xyz(cl));
            sa = add(sa, ca);
        } else {
            sl = sub(sl, xyz(cl));
            sa = sub(sa, ca);
        }
    }
    const real invCount = 1.0f / static_cast<real>(cnt > 1 ? cnt : 1);
    f3 dl = scale(sl, invCount);
    f3 da = scale(sa, invCount);
    const int locks = d.meta[g].w;
    maskLocked(locks & 0xff, dl);
    maskLocked((locks >> 8) & 0xff, da);
    const real cap = p.projMaxCorr;
    if (cap > 0.0f) {
        const real moved = length(dl);
        if (moved > cap)
            dl = scale(dl, cap / moved);
        const real turned = length(da);
        if (turned > cap)
            da = scale(da, cap / turned);
    }
    const real4 x4 = d.x[g];
    d.x[g] = f4(add(xyz(x4), dl), x4.w);
    d.q[g] = f4(qintegrate(asq(d.q[g]), da));
}

// The same passes as separate launches, for large stores, where every phase fills the GPU and a
// kernel boundary costs less than a grid barrier of a resident grid.
__global__ void projStartKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int nWorlds = d.ctr[C_WORLDS];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWorlds)
        return;
    d.wStop[w] = d.wActive[w] > 0 ? 0 : 1;
    d.wMaxDepth[w] = 0;
}

__global__ void projManifoldKernel(Dev d, StepParams p) { pdlWait(); pdlTrigger(); projManifoldPass(d, p, blockIdx.x * blockDim.x, gridDim.x * blockDim.x); }

__global__ void projBodyKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < d.ctr[C_BODIES])
        projBodyAt(d, p, g);
}

__global__ void projCheckKernel(Dev d, real tolerance) {
    pdlWait();
    pdlTrigger();
    const int nWorlds = d.ctr[C_WORLDS];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWorlds)
        return;
    if (!d.wStop[w] && bitsf(d.wMaxDepth[w]) <= tolerance)
        d.wStop[w] = 1;
    d.wMaxDepth[w] = 0;
}

// Solver::projectContacts's passes (solver_projection.cpp:169-280) in one cooperative launch: a
// world with no movable manifold is stopped at once (the reference returns early); then each pass
// computes the manifolds' contributions, averages and applies them per body, and stops the worlds
// whose deepest patch is within tolerance, with a grid barrier between these phases (the kernel
// boundaries of the same sequence launched separately).
__global__ void __launch_bounds__(kThreads) projectionKernel(Dev d, StepParams p, real tolerance) {
    pdlWait();
    pdlTrigger();
    const int nWorlds = d.ctr[C_WORLDS];
    const int nBodies = d.ctr[C_BODIES];
    // The grid is sized by the store's capacities; only the blocks this step's counts need take
    // part (every block reads the same counts, which nothing changes during the launch), so a
    // small store's barriers are a block barrier.
    const int items = max(max(d.ctr[C_LIVE], nBodies), nWorlds);
    const unsigned active = static_cast<unsigned>(min(static_cast<int>(gridDim.x), max(1, (items + kThreads - 1) / kThreads)));
    if (blockIdx.x >= active)
        return;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = static_cast<int>(active) * blockDim.x;
    for (int w = tid; w < nWorlds; w += stride) {
        d.wStop[w] = d.wActive[w] > 0 ? 0 : 1;
        d.wMaxDepth[w] = 0;
    }
    for (int it = 0; it < p.projIters; it++) {
        if (!gridSync(d, active))
            return;
        projManifoldPass(d, p, blockIdx.x * blockDim.x, stride);
        if (!gridSync(d, active))
            return;
        for (int g = tid; g < nBodies; g += stride)
            projBodyAt(d, p, g);
        if (!gridSync(d, active))
            return;
        for (int w = tid; w < nWorlds; w += stride) {
            if (!d.wStop[w] && bitsf(d.wMaxDepth[w]) <= tolerance)
                d.wStop[w] = 1;
            d.wMaxDepth[w] = 0;
        }
    }
}

int g_brakeBlocks = 0;

} // namespace

static int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }

int brakeGridBlocks() {
    if (g_brakeBlocks == 0) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, brakeKernel, kBrakeThreads, 0);
        g_brakeBlocks = sms * (perSm < 1 ? 1 : (perSm > 2 ? 2 : perSm));
        if (g_brakeBlocks < 1)
            g_brakeBlocks = 1;
    }
    return g_brakeBlocks;
}

void launchProjActive(const Dev &d, cudaStream_t s) {
    cudaMemsetAsync(d.wActive, 0, sizeof(int) * static_cast<size_t>(d.WW), s);
    ++launchCount(); launchK(projActiveKernel, residentGrid(projActiveKernel, kThreads, grid(d.MM)), kThreads, 0, s, d);
    scanExclusive(d.mActive, d.pairValid, d.MM, d.ctr + C_LIVE, d.ctr + C_SPECN, d.scanScratch, s);
    ++launchCount(); launchK(specScatterKernel, residentGrid(specScatterKernel, kThreads, grid(d.MM)), kThreads, 0, s, d, d.mActive, d.pairValid);
}

// Runs right after launchProjActive, whose scan left each candidate's rank in d.pairValid.
void launchBrake(const Dev &d, real window, cudaStream_t s) {
    ++launchCount(); launchK(brakePredKernel, residentGrid(brakePredKernel, kThreads, grid(d.MM)), kThreads, 0, s, d, d.pairValid);
    Dev dd = d;
    real win = window;
    void *args[] = {&dd, &win};
    // No more blocks than the store's manifolds can fill (the list is a subset of them).
    const int want = divUp(d.MM > 0 ? d.MM : 1, kBrakeThreads), most = brakeGridBlocks();
    ++launchCount();
    cudaLaunchCooperativeKernel(reinterpret_cast<void *>(brakeKernel), dim3(want < most ? want : most),
                                dim3(kBrakeThreads), args, 0, s);
}

static int g_projBlocks = 0;

static int projGridMax() {
    if (g_projBlocks == 0) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, projectionKernel, kThreads, 0);
        g_projBlocks = sms * (perSm < 1 ? 1 : perSm);
    }
    return g_projBlocks;
}

int projectionGridBlocks() { return projGridMax(); }

// Stores whose manifold and body capacities fit in one resident wave take the cooperative form (its
// grid barriers cost less than kernel boundaries when each phase is a few blocks); larger stores
// launch the phases separately.
void launchProjection(const Dev &d, const StepParams &p, cudaStream_t s) {
    const int need = grid(d.MM > d.NB ? d.MM : d.NB);
    const int most = projGridMax();
    if (need > most) {
        const real tol0 = smax(p.projSlop * 0.01f, 1.0e-6f);
        ++launchCount(); launchK(projStartKernel, grid(d.WW), kThreads, 0, s, d);
        for (int it = 0; it < p.projIters; it++) {
            ++launchCount(); launchK(projManifoldKernel, residentGrid(projManifoldKernel, kThreads, grid(d.MM)), kThreads, 0, s, d, p);
            ++launchCount(); launchK(projBodyKernel, grid(d.NB), kThreads, 0, s, d, p);
            ++launchCount(); launchK(projCheckKernel, grid(d.WW), kThreads, 0, s, d, tol0);
        }
        return;
    }
    const int blocks = need;
    cudaMemsetAsync(d.gridBar, 0, sizeof(unsigned), s);
    Dev dd = d;
    StepParams pp = p;
    real tol = smax(p.projSlop * 0.01f, 1.0e-6f);
    void *args[] = {&dd, &pp, &tol};
    ++launchCount();
    cudaLaunchCooperativeKernel(reinterpret_cast<void *>(projectionKernel), dim3(blocks), dim3(kThreads), args, 0, s);
}

} // namespace avbdg
