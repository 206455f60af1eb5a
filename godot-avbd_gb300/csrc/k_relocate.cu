// Removal of whole worlds from a store (the served form evicts finished requests every tick).
//
// The surviving worlds keep their order and move down so that body slots stay dense: world w's
// range [base, base + count) becomes [newBase, newBase + count). Everything that names a body slot
// is rewritten through one slot map: the per-body state, the live manifolds (kept in live order by
// the same stable compaction a step uses, so every world's live order is unchanged) and the force
// list (stable, so every world's force order is unchanged). A world's results therefore do not
// depend on which other worlds share the store, or where its range sits.

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;

int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }

// remap[2w] = new world id (-1 = removed), remap[2w + 1] = new base slot.
__global__ void slotMapKernel(Dev d, int n, const int *remap, int *slotMap) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    const int w = d.meta[g].x;
    const int nid = remap[2 * w];
    slotMap[g] = nid < 0 ? -1 : remap[2 * w + 1] + (g - d.wBase[w]);
}

template <typename T>
__global__ void scatterKernel(const T *src, T *dst, const int *slotMap, int n) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    const int t = slotMap[g];
    if (t >= 0)
        dst[t] = src[g];
}

__global__ void metaScatterKernel(const int4 *src, int4 *dst, const int *slotMap, const int *remap, int n) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    const int t = slotMap[g];
    if (t < 0)
        return;
    int4 m = src[g];
    m.x = remap[2 * m.x];
    dst[t] = m;
}

// Live manifolds -> stage with rewritten bodies; mActive marks the survivors for the stable
// compaction back into live order.
__global__ void manifoldRelocateKernel(Dev d, const int *slotMap) {
    pdlWait();
    pdlTrigger();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= d.ctr[C_CAND])
        return;
    const ManifoldBuf L = d.live;
    const ManifoldBuf S = d.stage;
    const int2 ab = L.ab[m];
    const int na = slotMap[ab.x];
    d.mActive[m] = na >= 0 ? 1 : 0;
    if (na < 0)
        return;
    S.ab[m] = make_int2(na, slotMap[ab.y]);
    S.b0[m] = L.b0[m];
    S.b1[m] = L.b1[m];
    S.b2[m] = L.b2[m];
    const int cnt = L.count[m];
    const int2 dorm = L.dormant[m];
    S.count[m] = cnt;
    S.dormant[m] = dorm;
    const int kept = cnt > 0 ? cnt : dorm.y;
    for (int c = 0; c < kept; c++) {
        const int i = cslot(d, m, c);
        S.key[i] = L.key[i];
        S.rA[i] = L.rA[i];
        S.rB[i] = L.rB[i];
        S.C0[i] = L.C0[i];
        S.k[i] = L.k[i];
        S.lam[i] = L.lam[i];
        if (d.ARM) {
            S.armA[i] = L.armA[i];
            S.armB[i] = L.armB[i];
        }
    }
    if (d.ARM) {
        S.armFlag[m] = L.armFlag[m];
        S.capA[m] = L.capA[m];
        S.capB[m] = L.capB[m];
    }
}

// Force b is always a body of the force's world (a may be the static world anchor, -1).
__global__ void forceFlagKernel(Dev d, int nf, const int *slotMap, int2 *abOut) {
    pdlWait();
    pdlTrigger();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf)
        return;
    const int2 ab = d.fAB[f];
    const int nb = slotMap[ab.y];
    d.fKeep[f] = nb >= 0 ? 1 : 0;
    abOut[f] = make_int2(ab.x >= 0 ? slotMap[ab.x] : -1, nb);
}

template <typename T>
__global__ void compactKernel(const T *src, T *dst, const int *keep, const int *rank, int n) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && keep[i])
        dst[rank[i]] = src[i];
}

// Strided records (kExtF4 float4 per force) follow their force.
__global__ void compactExtKernel(const real4 *src, real4 *dst, const int *keep, const int *rank, int n) {
    pdlWait();
    pdlTrigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kExtF4)
        return;
    const int f = i / kExtF4;
    if (keep[f])
        dst[static_cast<size_t>(rank[f]) * kExtF4 + i % kExtF4] = src[i];
}

// List position -> body of every world's range, from the (new) world table.
__global__ void listPosKernel(Dev d, int n) {
    pdlWait();
    pdlTrigger();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n)
        return;
    const int w = d.meta[p].x;
    d.lpToBody[p] = 2 * d.wBase[w] + d.wCount[w] - 1 - p;
}

template <typename T>
void moveArray(T *arr, T *tmp, const int *slotMap, int nOld, int nNew, cudaStream_t s) {
    ++launchCount(); launchK(scatterKernel<T>, grid(nOld), kThreads, 0, s, arr, tmp, slotMap, nOld);
    if (nNew > 0)
        cudaMemcpyAsync(arr, tmp, sizeof(T) * static_cast<size_t>(nNew), cudaMemcpyDeviceToDevice, s);
}

// The survivors form a prefix of tmp; all n slots are copied back (the tail is dead), so the call
// needs no host read of the surviving count.
template <typename T>
void compactArray(T *arr, T *tmp, const int *keep, const int *rank, int n, cudaStream_t s) {
    ++launchCount(); launchK(compactKernel<T>, grid(n), kThreads, 0, s, arr, tmp, keep, rank, n);
    cudaMemcpyAsync(arr, tmp, sizeof(T) * static_cast<size_t>(n), cudaMemcpyDeviceToDevice, s);
}

} // namespace

void launchRelocateWorlds(const Dev &d, int nOld, int nNew, int nForces, const int *remap, cudaStream_t s) {
    int *slotMap = d.relocInt;
    ++launchCount(); launchK(slotMapKernel, grid(nOld), kThreads, 0, s, d, nOld, remap, slotMap);

    // Bodies, through a staging array (slots only move down, so an in-place move would race).
    real4 *tmp4 = d.relocF4;
    for (real4 *arr : {d.x, d.q, d.x0, d.q0, d.xi, d.qi, d.v, d.w, d.vprev, d.size, d.moment})
        moveArray(arr, tmp4, slotMap, nOld, nNew, s);
    moveArray(d.sleep, reinterpret_cast<int2 *>(tmp4), slotMap, nOld, nNew, s);
    int4 *tmpMeta = reinterpret_cast<int4 *>(tmp4);
    ++launchCount(); launchK(metaScatterKernel, grid(nOld), kThreads, 0, s, d.meta, tmpMeta, slotMap, remap, nOld);
    if (nNew > 0)
        cudaMemcpyAsync(d.meta, tmpMeta, sizeof(int4) * static_cast<size_t>(nNew), cudaMemcpyDeviceToDevice, s);

    // Live manifolds: stage with new body slots, then the step's stable compaction into live.
    cudaMemcpyAsync(d.ctr + C_CAND, d.ctr + C_LIVE, sizeof(int), cudaMemcpyDeviceToDevice, s);
    ++launchCount(); launchK(manifoldRelocateKernel, grid(d.MM), kThreads, 0, s, d, slotMap);
    launchManifoldCompact(d, s);

    // Forces: flags + exclusive rank, then a stable scatter of every field.
    if (nForces > 0) {
        // relocF4 holds max(NB, FF * kExtF4) float4: room for two int2 arrays of FF entries.
        int2 *abNew = reinterpret_cast<int2 *>(tmp4);
        int *rank = d.relocInt + d.NB;
        ++launchCount(); launchK(forceFlagKernel, grid(nForces), kThreads, 0, s, d, nForces, slotMap, abNew);
        scanExclusive(d.fKeep, rank, d.FF, d.ctr + C_FORCES, d.ctr + C_TMP, d.scanScratch, s);
        int2 *abTmp = reinterpret_cast<int2 *>(tmp4) + d.FF;
        ++launchCount(); launchK(compactKernel<int2>, grid(nForces), kThreads, 0, s, abNew, abTmp, d.fKeep, rank, nForces);
        cudaMemcpyAsync(d.fAB, abTmp, sizeof(int2) * static_cast<size_t>(nForces), cudaMemcpyDeviceToDevice, s);
        for (real4 *arr : {d.fRA, d.fRB, d.fC0L, d.fC0A, d.fKL, d.fKA, d.fLL, d.fLA, d.fPar})
            compactArray(arr, tmp4, d.fKeep, rank, nForces, s);
        int *tmpI = reinterpret_cast<int *>(tmp4);
        compactArray(d.fKind, tmpI, d.fKeep, rank, nForces, s);
        compactArray(d.fBroken, tmpI, d.fKeep, rank, nForces, s);
        // Generic-joint records (relocF4 holds FF * kExtF4 float4).
        real4 *extTmp = d.relocF4;
        ++launchCount();
        launchK(compactExtKernel, grid(nForces * kExtF4), kThreads, 0, s, d.fExt, extTmp, d.fKeep, rank, nForces);
        cudaMemcpyAsync(d.fExt, extTmp, sizeof(real4) * static_cast<size_t>(nForces) * kExtF4,
                        cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(d.ctr + C_FORCES, d.ctr + C_TMP, sizeof(int), cudaMemcpyDeviceToDevice, s);
    }
}

void launchListPositions(const Dev &d, int nBodies, cudaStream_t s) {
    if (nBodies > 0) {
        ++launchCount(); launchK(listPosKernel, grid(nBodies), kThreads, 0, s, d, nBodies);
    }
}

} // namespace avbdg
