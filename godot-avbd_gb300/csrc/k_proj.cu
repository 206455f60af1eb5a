// Speculative brake and positional projection (godot-avbd src/avbd/solver_projection.cpp:67-281).
//
// The brake is a Gauss-Seidel sweep over manifolds in live order: each braked patch updates its
// bodies' velocities in place and later manifolds see the result. Only manifolds with an open gap
// (some contact with positive separation at the fixed poses) can brake, so the sweep's order only
// matters among them. A manifold runs once every earlier such manifold on one of its movable
// bodies is done; ready manifolds never share a movable body, so each round runs them in
// parallel and the result equals the serial sweep. Rounds are separated by a grid barrier inside
// one cooperative launch; every wait is bounded and reports a timeout instead of hanging.
//
// Projection passes are Jacobi: per-manifold patch corrections, then per-body sums in live order
// (the adjacency order), averaged over the manifold count, with the per-world early exit.

#include <cooperative_groups.h>

#include "grid_sync.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;
constexpr int kBrakeThreads = 512;

__device__ __forceinline__ bool movable(const Dev &d, int g) { return d.x[g].w > 0.0f; }

__device__ __forceinline__ float angularCompliance(f3 I, f3 axis) {
    float sum = 0.0f;
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
__global__ void projActiveKernel(Dev d) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= d.ctr[C_LIVE])
        return;
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const int n = L.count[m];
    const bool active = n > 0 && (movable(d, ab.x) || movable(d, ab.y));
    uint8_t spec = 0;
    if (active) {
        atomicAdd(&d.wActive[d.meta[ab.x].x], 1);
        const f3 nrm = xyz(L.b0[m]);
        const f3 xa = xyz(d.x[ab.x]), xb = xyz(d.x[ab.y]);
        const q4 qa = asq(d.q[ab.x]), qb = asq(d.q[ab.y]);
        for (int k = 0; k < n; k++) {
            const int ci = m * kMaxContacts + k;
            const f3 rA = qrot(qa, xyz(L.rA[ci]));
            const f3 rB = qrot(qb, xyz(L.rB[ci]));
            const float gap = dot(nrm, sub(add(xa, rA), add(xb, rB)));
            if (gap > 0.0f) {
                spec = 1;
                break;
            }
        }
    }
    d.mSpec[m] = spec;
    d.mDone[m] = spec ? 0 : 1;
    d.mActive[m] = spec;
}

// Brake candidates in live order (the scan of their flags gives each one its slot).
__global__ void specScatterKernel(Dev d, const int *flags, const int *rank) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m == 0)
        d.ctr[C_SPEC] = d.ctr[C_SPECN];
    if (m >= d.ctr[C_LIVE] || !flags[m])
        return;
    d.specList[rank[m]] = m;
}

// Is manifold m the earliest unfinished braking candidate on each of its movable bodies?
__device__ bool brakeReady(const Dev &d, int m, int2 ab, int nf) {
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
            if (__ldcg(&d.mSpec[o]) && !__ldcg(&d.mDone[o]))
                return false;
        }
    }
    return true;
}

// One manifold of the brake sweep (solver_projection.cpp:98-166).
__device__ void brakeManifold(const Dev &d, int m, float window) {
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const int a = ab.x, b = ab.y;
    const float4 xa4 = d.x[a], xb4 = d.x[b];
    const bool moveA = xa4.w > 0.0f, moveB = xb4.w > 0.0f;
    const float invMassA = moveA ? 1.0f / xa4.w : 0.0f;
    const float invMassB = moveB ? 1.0f / xb4.w : 0.0f;
    const f3 nrm = xyz(L.b0[m]);
    const q4 qa = asq(d.q[a]), qb = asq(d.q[b]);
    const f3 xa = xyz(xa4), xb = xyz(xb4);
    const f3 va = xyz(__ldcg(&d.v[a])), wa = xyz(__ldcg(&d.w[a]));
    const f3 vb = xyz(__ldcg(&d.v[b])), wb = xyz(__ldcg(&d.w[b]));
    f3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
    float velErr = 0.0f;
    int braked = 0;
    const int n = L.count[m];
    for (int k = 0; k < n; k++) {
        const int ci = m * kMaxContacts + k;
        const f3 rA = qrot(qa, xyz(L.rA[ci]));
        const f3 rB = qrot(qb, xyz(L.rB[ci]));
        const float gap = dot(nrm, sub(add(xa, rA), add(xb, rB)));
        if (!(gap > 0.0f))
            continue;
        const f3 vAp = add(va, cross(wa, rA));
        const f3 vBp = add(vb, cross(wb, rB));
        const float vn = dot(sub(vAp, vBp), nrm);
        const float target = -gap / window;
        if (vn < target) {
            patchRA = add(patchRA, rA);
            patchRB = add(patchRB, rB);
            velErr += target - vn;
            braked++;
        }
    }
    if (braked == 0)
        return;
    const float invN = 1.0f / static_cast<float>(braked);
    const f3 IA = xyz(d.moment[a]), IB = xyz(d.moment[b]);
    const f3 tA = moveA ? qrot(qconj(qa), cross(scale(patchRA, invN), nrm)) : f3{0, 0, 0};
    const f3 tB = moveB ? qrot(qconj(qb), cross(scale(patchRB, invN), nrm)) : f3{0, 0, 0};
    const float K = invMassA + invMassB + (moveA ? angularCompliance(IA, tA) : 0.0f) +
                    (moveB ? angularCompliance(IB, tB) : 0.0f);
    const float j = velErr * invN / K;
    if (moveA) {
        const int locks = d.meta[a].w;
        f3 dv = scale(nrm, invMassA * j);
        f3 dw = scale(angularResponse(IA, qa, tA), j);
        maskLocked(locks & 0xff, dv);
        maskLocked((locks >> 8) & 0xff, dw);
        const float4 v4 = __ldcg(&d.v[a]);
        __stcg(&d.v[a], f4(add(xyz(v4), dv), v4.w));
        __stcg(&d.w[a], f4(add(wa, dw), 0.0f));
    }
    if (moveB) {
        const int locks = d.meta[b].w;
        f3 dv = scale(nrm, invMassB * j);
        f3 dw = scale(angularResponse(IB, qb, tB), j);
        maskLocked(locks & 0xff, dv);
        maskLocked((locks >> 8) & 0xff, dw);
        const float4 v4 = __ldcg(&d.v[b]);
        __stcg(&d.v[b], f4(sub(xyz(v4), dv), v4.w));
        __stcg(&d.w[b], f4(sub(wb, dw), 0.0f));
    }
}

__global__ void __launch_bounds__(kBrakeThreads) brakeKernel(Dev d, float window, unsigned *bar) {
    const int ns = d.ctr[C_SPECN];
    const int nf = d.ctr[C_FORCES];
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    volatile int *remaining = d.ctr + C_SPEC;
    for (int round = 0; round <= ns; round++) {
        if (*remaining == 0)
            break;
        // Phase 1: mark the ready manifolds (mSpec = 2).
        for (int k = tid; k < ns; k += stride) {
            const int m = d.specList[k];
            if (__ldcg(&d.mDone[m]))
                continue;
            if (brakeReady(d, m, d.live.ab[m], nf))
                d.mSpec[m] = 2;
        }
        if (!gridBarrier(bar, d.ctr + C_ERRORS, kErrBrakeTimeout))
            return;
        // Phase 2: run them; they touch disjoint movable bodies.
        for (int k = tid; k < ns; k += stride) {
            const int m = d.specList[k];
            if (__ldcg(&d.mSpec[m]) != 2)
                continue;
            brakeManifold(d, m, window);
            __stcg(&d.mSpec[m], static_cast<uint8_t>(1));
            __stcg(&d.mDone[m], static_cast<uint8_t>(1));
            atomicSub(d.ctr + C_SPEC, 1);
        }
        if (!gridBarrier(bar, d.ctr + C_ERRORS, kErrBrakeTimeout))
            return;
    }
}

// ---- positional projection (solver_projection.cpp:169-280) ----

__global__ void projManifoldKernel(Dev d, StepParams p) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= d.ctr[C_LIVE])
        return;
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const int a = ab.x, b = ab.y;
    const int w = d.meta[a].x;
    d.projLin[2 * m].w = 0.0f;
    d.projLin[2 * m + 1].w = 0.0f;
    if (d.wStop[w])
        return;
    const float4 xa4 = d.x[a], xb4 = d.x[b];
    const bool moveA = xa4.w > 0.0f, moveB = xb4.w > 0.0f;
    const int n = L.count[m];
    if (n == 0 || (!moveA && !moveB))
        return;
    const float invMassA = moveA ? 1.0f / xa4.w : 0.0f;
    const float invMassB = moveB ? 1.0f / xb4.w : 0.0f;
    const f3 nrm = xyz(L.b0[m]);
    const q4 qa = asq(d.q[a]), qb = asq(d.q[b]);
    const f3 xa = xyz(xa4), xb = xyz(xb4);
    const m3 rotA = qmat(qa), rotB = qmat(qb);
    f3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
    float patchDepth = 0.0f;
    int corrected = 0;
    for (int k = 0; k < n; k++) {
        const int ci = m * kMaxContacts + k;
        const f3 rA = mul(rotA, xyz(L.rA[ci]));
        const f3 rB = mul(rotB, xyz(L.rB[ci]));
        const float rawDepth = -dot(nrm, sub(add(xa, rA), add(xb, rB)));
        const float depth = rawDepth - p.projSlop;
        if (depth > 0.0f) {
            patchRA = add(patchRA, rA);
            patchRB = add(patchRB, rB);
            patchDepth += depth;
            corrected++;
        }
    }
    if (corrected == 0)
        return;
    const float invN = 1.0f / static_cast<float>(corrected);
    atomicMax(&d.wMaxDepth[w], __float_as_int(patchDepth * invN));
    const f3 IA = xyz(d.moment[a]), IB = xyz(d.moment[b]);
    const f3 tA = moveA ? qrot(qconj(qa), cross(scale(patchRA, invN), nrm)) : f3{0, 0, 0};
    const f3 tB = moveB ? qrot(qconj(qb), cross(scale(patchRB, invN), nrm)) : f3{0, 0, 0};
    const float K = invMassA + invMassB + (moveA ? angularCompliance(IA, tA) : 0.0f) +
                    (moveB ? angularCompliance(IB, tB) : 0.0f);
    const float dp = p.projBeta * patchDepth * invN / K;
    if (moveA) {
        d.projLin[2 * m] = f4(scale(nrm, invMassA * dp), 1.0f);
        d.projAng[2 * m] = f4(scale(angularResponse(IA, qa, tA), dp), 0.0f);
    }
    if (moveB) {
        d.projLin[2 * m + 1] = f4(scale(nrm, invMassB * dp), 1.0f);
        d.projAng[2 * m + 1] = f4(scale(angularResponse(IB, qb, tB), dp), 0.0f);
    }
}

__global__ void projBodyKernel(Dev d, int nBodies, StepParams p) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nBodies || d.meta[g].x < 0 || !movable(d, g))
        return;
    if (d.wStop[d.meta[g].x])
        return;
    const int nf = d.ctr[C_FORCES];
    f3 sl{0, 0, 0}, sa{0, 0, 0};
    int cnt = 0;
    for (int e = d.adjStart[g]; e < d.adjStart[g + 1]; e++) {
        const int seq = static_cast<int>(d.adjSeq[e]);
        if (seq < nf)
            continue;
        const int m = seq - nf;
        const int side = d.live.ab[m].x == g ? 0 : 1;
        const float4 cl = d.projLin[2 * m + side];
        if (cl.w == 0.0f)
            continue;
        const f3 ca = xyz(d.projAng[2 * m + side]);
        cnt++;
        if (side == 0) {
            sl = add(sl, xyz(cl));
            sa = add(sa, ca);
        } else {
            sl = sub(sl, xyz(cl));
            sa = sub(sa, ca);
        }
    }
    const float invCount = 1.0f / static_cast<float>(cnt > 1 ? cnt : 1);
    f3 dl = scale(sl, invCount);
    f3 da = scale(sa, invCount);
    const int locks = d.meta[g].w;
    maskLocked(locks & 0xff, dl);
    maskLocked((locks >> 8) & 0xff, da);
    const float cap = p.projMaxCorr;
    if (cap > 0.0f) {
        const float moved = length(dl);
        if (moved > cap)
            dl = scale(dl, cap / moved);
        const float turned = length(da);
        if (turned > cap)
            da = scale(da, cap / turned);
    }
    const float4 x4 = d.x[g];
    d.x[g] = f4(add(xyz(x4), dl), x4.w);
    d.q[g] = f4(qintegrate(asq(d.q[g]), da));
}

__global__ void projCheckKernel(Dev d, int nWorlds, float tolerance) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWorlds)
        return;
    if (!d.wStop[w] && __int_as_float(d.wMaxDepth[w]) <= tolerance)
        d.wStop[w] = 1;
    d.wMaxDepth[w] = 0;
}

// Worlds with no movable manifold skip the whole projection (the reference returns early).
__global__ void projStartKernel(Dev d, int nWorlds) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nWorlds)
        return;
    d.wStop[w] = d.wActive[w] > 0 ? 0 : 1;
    d.wMaxDepth[w] = 0;
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

void launchProjActive(const Dev &d, int nWorlds, cudaStream_t s) {
    cudaMemsetAsync(d.wActive, 0, sizeof(int) * static_cast<size_t>(nWorlds), s);
    ++launchCount(); projActiveKernel<<<grid(d.MM), kThreads, 0, s>>>(d);
    scanExclusive(d.mActive, d.pairValid, d.MM, d.ctr + C_LIVE, d.ctr + C_SPECN, d.scanScratch, s);
    ++launchCount(); specScatterKernel<<<grid(d.MM), kThreads, 0, s>>>(d, d.mActive, d.pairValid);
}

void launchBrake(const Dev &d, int, float window, cudaStream_t s) {
    unsigned *bar = reinterpret_cast<unsigned *>(d.barrier);
    cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
    Dev dd = d;
    float win = window;
    void *args[] = {&dd, &win, &bar};
    ++launchCount();
    cudaLaunchCooperativeKernel(reinterpret_cast<void *>(brakeKernel), dim3(brakeGridBlocks()), dim3(kBrakeThreads),
                                args, 0, s);
}

void launchProjection(const Dev &d, int nBodies, int nWorlds, const StepParams &p, cudaStream_t s) {
    ++launchCount(); projStartKernel<<<grid(nWorlds), kThreads, 0, s>>>(d, nWorlds);
    const float tol = smax(p.projSlop * 0.01f, 1.0e-6f);
    for (int it = 0; it < p.projIters; it++) {
        ++launchCount(); projManifoldKernel<<<grid(d.MM), kThreads, 0, s>>>(d, p);
        ++launchCount(); projBodyKernel<<<grid(nBodies), kThreads, 0, s>>>(d, nBodies, p);
        ++launchCount(); projCheckKernel<<<grid(nWorlds), kThreads, 0, s>>>(d, nWorlds, tol);
    }
}

} // namespace avbdg
