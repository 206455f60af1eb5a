// Manifold store maintenance and the constraint adjacency (godot-avbd src/avbd/manifold.cpp,
// src/avbd/solver_solve.cpp:31-105, src/avbd/joint.cpp:62-78).
//
// Live manifolds are kept densely in live order; a step appends the newly acquired ones, runs the
// narrow phase and warm start for every candidate into a staging buffer, and compacts the
// survivors back in order (the reference's stable compaction of `live`). Slot recycling is an
// allocation detail of the reference that never reaches its arithmetic, so it has no equivalent.

#include <cmath>

#include "forces.cuh"
#include "kernels.cuh"
#include "narrow.cuh"
#include "narrow_round.cuh"
#include "prims.cuh"

namespace avbdg {

// Cylinder rim directions (narrow_round.cuh), uploaded once by prepareNarrowPhase.
__constant__ narrow::RimTable c_rim;

namespace {

constexpr int kThreads = 256;

// ---- adjacency (ForceAdjacency::build, manifold.cpp:123-166) ----
// Entry sequence numbers: forces in list order (0 .. F-1, newest first), then manifolds in live
// order (F + m). Only dynamic bodies carry lists: static bodies are never solved or coloured, and
// a pair query always has a dynamic side.

__global__ void adjCountKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int nf = d.ctr[C_FORCES];
    const int nm = d.ctr[C_LIVE];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int2 ab;
    if (i < nf)
        ab = d.fAB[i];
    else if (i - nf < nm)
        ab = d.live.ab[i - nf];
    else
        return;
    if (ab.x >= 0 && d.x[ab.x].w > 0.0f)
        atomicAdd(&d.adjStart[ab.x], 1);
    if (ab.y >= 0 && d.x[ab.y].w > 0.0f)
        atomicAdd(&d.adjStart[ab.y], 1);
}

__global__ void adjFillKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int nf = d.ctr[C_FORCES];
    const int nm = d.ctr[C_LIVE];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int2 ab;
    uint32_t seq;
    if (i < nf) {
        ab = d.fAB[i];
        seq = static_cast<uint32_t>(nf - 1 - i);
    } else if (i - nf < nm) {
        ab = d.live.ab[i - nf];
        seq = static_cast<uint32_t>(i);
    } else {
        return;
    }
    if (ab.x >= 0 && d.x[ab.x].w > 0.0f)
        d.adjSeq[d.adjStart[ab.x] + atomicAdd(&d.adjFill[ab.x], 1)] = seq;
    if (ab.y >= 0 && d.x[ab.y].w > 0.0f)
        d.adjSeq[d.adjStart[ab.y] + atomicAdd(&d.adjFill[ab.y], 1)] = seq;
}

// Each entry's other body and side, once per adjacency build, so the per-round passes need no
// load of the force's or manifold's body pair to find them; and each manifold side's entry, where
// its block stamp is stored, so a body's stamps lie contiguous in its adjacency range.
__global__ void adjInfoKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    const int nf = d.ctr[C_FORCES];
    for (int e = d.adjStart[g]; e < d.adjStart[g + 1]; e++) {
        const int seq = static_cast<int>(d.adjSeq[e]);
        const int2 ab = seq < nf ? d.fAB[nf - 1 - seq] : d.live.ab[seq - nf];
        const int side = ab.x == g ? 0 : 1;
        const int other = side == 0 ? ab.y : ab.x;
        d.adjInfo[e] = (other >= 0 ? other : kNoBody) | static_cast<int>(static_cast<unsigned>(side) << 31);
        if (seq >= nf)
            reinterpret_cast<int *>(d.stampSlot)[2 * (seq - nf) + side] = e;
    }
}

__global__ void adjTotalKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    if (d.ctr[C_ADJ] > 2 * (d.FF + d.MM))
        atomicOr(&d.ctr[C_ERRORS], kErrAdjacency);
}

// ---- manifold initialize (ManifoldStore::initialize, manifold.cpp:237-435) ----

// mul(basis, v) with the basis stored as rows.
__device__ __forceinline__ f3 basisMul(f3 r0, f3 r1, f3 r2, f3 v) {
    return f3{(r0.x * v.x + r0.y * v.y) + r0.z * v.z, (r1.x * v.x + r1.y * v.y) + r1.z * v.z,
              (r2.x * v.x + r2.y * v.y) + r2.z * v.z};
}

// ROUND: the store holds spheres or cylinders, whose sampled paths need kilobytes of local memory
// per thread; box-only stores run the variant without them.
template <bool ROUND>
__device__ __forceinline__ void manifoldInitAt(Dev d, StepParams p, int i) {
    if (i >= d.ctr[C_CAND])
        return;
    const ManifoldBuf L = d.live;
    const ManifoldBuf S = d.stage;
    const int2 ab = L.ab[i];
    const int a = ab.x, b = ab.y;
    const real4 xa4 = d.x[a], xb4 = d.x[b];
    const int sleepA = d.sleep[a].x, sleepB = d.sleep[b].x; // loaded with the poses, not after them
    const bool dynA = xa4.w > 0.0f, dynB = xb4.w > 0.0f;
    const bool awakeA = dynA & (sleepA == 0), awakeB = dynB & (sleepB == 0);
    int oldN = L.count[i];
    const int2 dorm = L.dormant[i];
    S.ab[i] = ab;
    if (!awakeA && !awakeB) {
        // Frozen: every input is parked, the state is kept verbatim.
        S.b0[i] = L.b0[i];
        S.b1[i] = L.b1[i];
        S.b2[i] = L.b2[i];
        S.count[i] = oldN;
        S.dormant[i] = dorm;
        const int kept = oldN > 0 ? oldN : dorm.y; // a parked manifold keeps its saved contacts
        for (int k = 0; k < kept; k++) {
            S.key[cslot(d, i, k)] = L.key[cslot(d, i, k)];
            S.rA[cslot(d, i, k)] = L.rA[cslot(d, i, k)];
            S.rB[cslot(d, i, k)] = L.rB[cslot(d, i, k)];
            S.C0[cslot(d, i, k)] = L.C0[cslot(d, i, k)];
            S.k[cslot(d, i, k)] = L.k[cslot(d, i, k)];
            S.lam[cslot(d, i, k)] = L.lam[cslot(d, i, k)];
        }
        if (d.ARM) { // frozen manifolds keep their captured arms (initialize does not run)
            S.armFlag[i] = L.armFlag[i];
            S.capA[i] = L.capA[i];
            S.capB[i] = L.capB[i];
            for (int k = 0; k < kept; k++) {
                S.armA[cslot(d, i, k)] = L.armA[cslot(d, i, k)];
                S.armB[cslot(d, i, k)] = L.armB[cslot(d, i, k)];
            }
        }
        d.mActive[i] = 1;
        return;
    }
    if (d.ARM)
        S.armFlag[i] = 0; // a new contact set drops the cached arms (manifold.cpp:245-246)
    // Grace revival (manifold.cpp:249-253): a dormant manifold matches against its saved contacts.
    if (oldN == 0 && dorm.y > 0)
        oldN = dorm.y;
    // The old contacts are read after the separating-axis test; their lines are requested now.
    for (int j = 0; j < oldN; j++) {
        const int cj = cslot(d, i, j);
        prefetchL1(&L.key[cj]);
        prefetchL1(&L.rA[cj]);
        prefetchL1(&L.rB[cj]);
        prefetchL1(&L.C0[cj]);
        prefetchL1(&L.k[cj]);
        prefetchL1(&L.lam[cj]);
    }
    const f3 xa = xyz(xa4), xb = xyz(xb4);
    const q4 qa = asq(d.q[a]), qb = asq(d.q[b]);
    const real4 ma4 = d.moment[a], mb4 = d.moment[b];
    const real mu = msqrt(ma4.w * mb4.w);

    // Speculative margin (Manifold::collide, collide.cpp:1100-1120).
    real margin = p.specMargin;
    if (margin > 0.0f) {
        const real horizon = p.collisionDt;
        const real4 va4 = d.v[a], vb4 = d.v[b];
        const real gA = dynA ? va4.w : 0.0f;
        const real gB = dynB ? vb4.w : 0.0f;
        const f3 disp = add(scale(sub(xyz(va4), xyz(vb4)), horizon), f3{0, 0, (gA - gB) * horizon * horizon});
        const real ra = d.size[a].w, rb = d.size[b].w;
        margin += length(disp) + (ra * length(xyz(d.w[a])) + rb * length(xyz(d.w[b]))) * horizon;
    }
    NContact nc[kMaxContacts];
    m3 basis = mcols(xyz(L.b0[i]), xyz(L.b1[i]), xyz(L.b2[i])); // rows kept when the SAT fails early
    basis = transpose(basis);
    const int shapeA = (d.meta[a].w >> 18) & 0x3, shapeB = (d.meta[b].w >> 18) & 0x3;
    const int n = (!ROUND || (shapeA == 0 && shapeB == 0))
                          ? collideBoxes(xa, qa, scale(xyz(d.size[a]), 0.5f), xb, qb, scale(xyz(d.size[b]), 0.5f),
                                         margin, nc, basis)
                          : collideRound(shapeA, xa, qa, xyz(d.size[a]), shapeB, xb, qb, xyz(d.size[b]), margin,
                                         c_rim, nc, basis);
    const f3 r0 = mrow(basis, 0), r1 = mrow(basis, 1), r2 = mrow(basis, 2);

    f3 newK[kMaxContacts], newLam[kMaxContacts];
    real newBeta[kMaxContacts], prevErr[kMaxContacts];
    int newStick[kMaxContacts];
    for (int c = 0; c < kMaxContacts; c++) {
        newK[c] = f3{0, 0, 0};
        newLam[c] = f3{0, 0, 0};
        newStick[c] = 0;
        newBeta[c] = 1.0f;
        prevErr[c] = -1.0f;
    }
    // The old contacts' feature keys, loaded once (registers; unused slots never match).
    int oldKey[kMaxContacts];
#pragma unroll
    for (int j = 0; j < kMaxContacts; j++)
        oldKey[j] = j < oldN ? L.key[cslot(d, i, j)] : 0;
    for (int c = 0; c < n; c++) {
        // The first old contact with the same key (the reference's linear search).
        int j = -1;
#pragma unroll
        for (int t = kMaxContacts - 1; t >= 0; t--)
            if (t < oldN && oldKey[t] == nc[c].key)
                j = t;
        if (j >= 0) {
            const f3 newRA = nc[c].rA, newRB = nc[c].rB;
            const real4 oRA = L.rA[cslot(d, i, j)], oRB = L.rB[cslot(d, i, j)];
            const real4 oLam = L.lam[cslot(d, i, j)];
            nc[c].rA = xyz(oRA);
            nc[c].rB = xyz(oRB);
            prevErr[c] = smax(0.0f, COLLISION_MARGIN - L.C0[cslot(d, i, j)].x);
            newK[c] = xyz(L.k[cslot(d, i, j)]);
            newLam[c] = xyz(oLam);
            const int oldStick = oLam.w != 0.0f;
            newStick[c] = oldStick;
            newBeta[c] = oRA.w;
            if (!oldStick) {
                nc[c].rA = newRA;
                nc[c].rB = newRB;
            } else {
                const f3 oldA = add(xa, qrot(qa, xyz(oRA)));
                const f3 oldB = add(xb, qrot(qb, xyz(oRB)));
                const f3 nA = add(xa, qrot(qa, newRA));
                const f3 nB = add(xb, qrot(qb, newRB));
                const real drift = smax(length(sub(oldA, nA)), length(sub(oldB, nB)));
                if (drift > p.stickDriftHeal) {
                    nc[c].rA = newRA;
                    nc[c].rB = newRB;
                    newStick[c] = 0;
                    newLam[c] = f3{newLam[c].x, 0.0f, 0.0f};
                }
            }
        }
    }
    // Fresh contacts seed their penalty when grace is on (manifold.cpp:339-347).
    if (p.graceTicks > 0)
        for (int c = 0; c < n; c++)
            if (prevErr[c] < 0.0f)
                newK[c] = f3{p.graceSeed, p.graceSeed, p.graceSeed};
    S.b0[i] = f4(r0, mu);
    S.b1[i] = f4(r1, 0.0f);
    S.b2[i] = f4(r2, 0.0f);
    S.count[i] = n;
    if (n == 0) {
        // Grace dormancy (manifold.cpp:359-378): parked, not reaped, within the grace ticks; the
        // saved contacts keep their state except force and stick.
        if (p.graceTicks > 0 && dorm.x < p.graceTicks) {
            for (int j = 0; j < oldN; j++) {
                S.key[cslot(d, i, j)] = L.key[cslot(d, i, j)];
                S.rA[cslot(d, i, j)] = L.rA[cslot(d, i, j)];
                S.rB[cslot(d, i, j)] = L.rB[cslot(d, i, j)];
                S.C0[cslot(d, i, j)] = L.C0[cslot(d, i, j)];
                S.k[cslot(d, i, j)] = L.k[cslot(d, i, j)];
                S.lam[cslot(d, i, j)] = mk4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            S.dormant[i] = make_int2(dorm.x + 1, oldN);
            d.mActive[i] = 1;
            return;
        }
        S.dormant[i] = make_int2(0, 0);
        d.mActive[i] = 0;
        return;
    }
    S.dormant[i] = make_int2(0, dorm.y);
    for (int c = 0; c < n; c++) {
        const f3 rA = nc[c].rA, rB = nc[c].rB;
        const f3 pA = add(xa, qrot(qa, rA));
        const f3 pB = add(xb, qrot(qb, rB));
        f3 C0 = add(basisMul(r0, r1, r2, sub(pA, pB)), f3{COLLISION_MARGIN, 0, 0});
        if (C0.x < -p.maxPen)
            C0.x = -p.maxPen;
        real beta = 1.0f;
        if (p.adaptiveBeta && prevErr[c] >= 0.0f) {
            const real err = smax(0.0f, COLLISION_MARGIN - C0.x);
            const real fl = p.adaptiveFloor;
            real sc = newBeta[c];
            if (err <= fl)
                sc = smax(sc * 0.5f, 1.0f);
            else if (prevErr[c] <= fl)
                sc = smin(sc * 2.0f, ADAPTIVE_BETA_MAX);
            else if (err > 0.5f * prevErr[c])
                sc = smin(sc * 2.0f, ADAPTIVE_BETA_MAX);
            else if (err < 0.1f * prevErr[c])
                sc = smax(sc * 0.5f, 1.0f);
            beta = sc;
        }
        f3 lam = newLam[c];
        int stick = newStick[c];
        if (C0.x > kReleaseAbove) {
            lam = f3{0, 0, 0};
            stick = 0;
        }
        lam = scale(scale(lam, p.alpha), p.gamma);
        const f3 k = lclampv(scale(newK[c], p.gamma), PENALTY_MIN, PENALTY_MAX);
        S.key[cslot(d, i, c)] = nc[c].key;
        S.rA[cslot(d, i, c)] = f4(rA, beta);
        S.rB[cslot(d, i, c)] = f4(rB, 0.0f);
        S.C0[cslot(d, i, c)] = f4(C0, 0.0f);
        S.k[cslot(d, i, c)] = f4(k, 0.0f);
        S.lam[cslot(d, i, c)] = f4(lam, stick ? 1.0f : 0.0f);
    }
    d.mActive[i] = n > 0 ? 1 : 0;
}

template <bool ROUND>
__global__ void manifoldInitKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_CAND];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        manifoldInitAt<ROUND>(d, p, i);
}

// One thread per contact slot (8 per candidate, slot-major like the arrays), so the copies of the
// contact arrays coalesce; the slot-0 thread also moves the manifold's own record. Grid-stride.
// Index type T: 32-bit where the slot count fits (the usual case; its division is far cheaper).
template <typename T>
__device__ __forceinline__ void manifoldCompactRun(const Dev &d, const int *flags, const int *rank, int cand) {
    const T slots = static_cast<T>(cand) * kMaxContacts;
    const T stride = static_cast<T>(gridDim.x) * blockDim.x;
    const ManifoldBuf L = d.live;
    const ManifoldBuf S = d.stage;
    for (T t = static_cast<T>(blockIdx.x) * blockDim.x + threadIdx.x; t < slots; t += stride) {
        const int c = static_cast<int>(t / static_cast<T>(cand));
        const int i = static_cast<int>(t - static_cast<T>(c) * static_cast<T>(cand));
        if (!flags[i])
            continue;
        const int r = rank[i];
        const int n = S.count[i];
        const int2 dorm = S.dormant[i];
        if (c == 0) {
            L.ab[r] = S.ab[i];
            L.b0[r] = S.b0[i];
            L.b1[r] = S.b1[i];
            L.b2[r] = S.b2[i];
            L.count[r] = n;
            L.dormant[r] = dorm;
            if (d.ARM) {
                L.armFlag[r] = S.armFlag[i];
                L.capA[r] = S.capA[i];
                L.capB[r] = S.capB[i];
            }
        }
        const int kept = n > 0 ? n : dorm.y; // a parked manifold keeps its saved contacts
        if (c >= kept)
            continue;
        const int si = cslot(d, i, c), di = cslot(d, r, c);
        L.key[di] = S.key[si];
        L.rA[di] = S.rA[si];
        L.rB[di] = S.rB[si];
        L.C0[di] = S.C0[si];
        L.k[di] = S.k[si];
        L.lam[di] = S.lam[si];
        if (d.ARM) {
            L.armA[di] = S.armA[si];
            L.armB[di] = S.armB[si];
        }
    }
}

__global__ void manifoldCompactKernel(Dev d, const int *flags, const int *rank) {
    pdlWait();
    pdlTrigger();
    const int cand = d.ctr[C_CAND];
    const unsigned long long span = static_cast<unsigned long long>(cand) * kMaxContacts +
                                    static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    if (span < 0xffffffffull)
        manifoldCompactRun<unsigned>(d, flags, rank, cand);
    else
        manifoldCompactRun<unsigned long long>(d, flags, rank, cand);
}

// ---- rebase (ManifoldStore::rebase, manifold.cpp:448-461) ----
__device__ __forceinline__ void rebaseAt(Dev d, StepParams p, int m) {
    if (m >= d.ctr[C_LIVE])
        return;
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const f3 xa = xyz(d.x[ab.x]), xb = xyz(d.x[ab.y]);
    const q4 qa = asq(d.q[ab.x]), qb = asq(d.q[ab.y]);
    const f3 r0 = xyz(L.b0[m]), r1 = xyz(L.b1[m]), r2 = xyz(L.b2[m]);
    const int n = L.count[m];
    for (int c = 0; c < n; c++) {
        const int ci = cslot(d, m, c);
        const f3 pA = add(xa, qrot(qa, xyz(L.rA[ci])));
        const f3 pB = add(xb, qrot(qb, xyz(L.rB[ci])));
        f3 C0 = add(basisMul(r0, r1, r2, sub(pA, pB)), f3{COLLISION_MARGIN, 0, 0});
        if (C0.x < -p.maxPen)
            C0.x = -p.maxPen;
        L.C0[ci] = f4(C0, 0.0f);
    }
}

__global__ void rebaseKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x)
        rebaseAt(d, p, m);
}

// ---- forces: Joint::initialize (joint.cpp:62-78) and reaping of broken joints ----

__device__ __forceinline__ f3 jointLinError(const Dev &d, int f) {
    const int2 ab = d.fAB[f];
    const f3 rA = xyz(d.fRA[f]), rB = xyz(d.fRB[f]);
    const f3 pa = ab.x >= 0 ? add(xyz(d.x[ab.x]), qrot(asq(d.q[ab.x]), rA)) : rA;
    return sub(pa, add(xyz(d.x[ab.y]), qrot(asq(d.q[ab.y]), rB)));
}

__device__ __forceinline__ f3 jointAngError(const Dev &d, int f) {
    const int2 ab = d.fAB[f];
    const q4 qa = ab.x >= 0 ? asq(d.q[ab.x]) : q4{0.0f, 0.0f, 0.0f, 1.0f};
    return scale(qdiff(qa, asq(d.q[ab.y])), d.fPar[f].w);
}

__device__ __forceinline__ f3 warmPenalty(f3 k, real gamma, real stiffness) {
    return f3{smin(sclamp(k.x * gamma, PENALTY_MIN, PENALTY_MAX), stiffness),
              smin(sclamp(k.y * gamma, PENALTY_MIN, PENALTY_MAX), stiffness),
              smin(sclamp(k.z * gamma, PENALTY_MIN, PENALTY_MAX), stiffness)};
}

__global__ void forceInitKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    const int nf = d.ctr[C_FORCES];
    if (f >= nf)
        return;
    const int kind = d.fKind[f];
    if (kind == kForceGeneric)
        genericInit(d, p, f);
    if (kind != kForceBall) { // IgnoreCollision, Spring, GenericJoint: never reaped
        d.fKeep[f] = 1;
        return;
    }
    const real4 par = d.fPar[f];
    d.fC0L[f] = f4(jointLinError(d, f), 0.0f);
    d.fC0A[f] = f4(jointAngError(d, f), 0.0f);
    d.fLL[f] = f4(scale(scale(xyz(d.fLL[f]), p.alpha), p.gamma), 0.0f);
    d.fLA[f] = f4(scale(scale(xyz(d.fLA[f]), p.alpha), p.gamma), 0.0f);
    d.fKL[f] = f4(warmPenalty(xyz(d.fKL[f]), p.gamma, par.x), 0.0f);
    d.fKA[f] = f4(warmPenalty(xyz(d.fKA[f]), p.gamma, par.y), 0.0f);
    const int keep = d.fBroken[f] ? 0 : 1;
    d.fKeep[f] = keep;
    if (!keep)
        atomicOr(&d.ctr[C_TMP], 1);
}

// Stable in-place compaction of the force list (reaping is rare; one thread walks it in order).
__global__ void forceCompactKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    if (!d.ctr[C_TMP])
        return;
    const int nf = d.ctr[C_FORCES];
    int w = 0;
    for (int f = 0; f < nf; f++) {
        if (!d.fKeep[f])
            continue;
        if (w != f) {
            d.fAB[w] = d.fAB[f];
            d.fRA[w] = d.fRA[f];
            d.fRB[w] = d.fRB[f];
            d.fC0L[w] = d.fC0L[f];
            d.fC0A[w] = d.fC0A[f];
            d.fKL[w] = d.fKL[f];
            d.fKA[w] = d.fKA[f];
            d.fLL[w] = d.fLL[f];
            d.fLA[w] = d.fLA[f];
            d.fPar[w] = d.fPar[f];
            d.fKind[w] = d.fKind[f];
            d.fBroken[w] = d.fBroken[f];
            for (int k = 0; k < kExtF4; k++)
                d.fExt[static_cast<size_t>(w) * kExtF4 + k] = d.fExt[static_cast<size_t>(f) * kExtF4 + k];
        }
        w++;
    }
    d.ctr[C_FORCES] = w;
}

} // namespace

static int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }

// cos/sin of 2 pi * (5 i mod 8) / 8 with the C library, exactly as collide.cpp:739-753 builds them.
void prepareNarrowPhase() {
    narrow::RimTable t{};
    for (int i = 0; i < narrow::kRimSamples; ++i) {
        const int step = i * 5 % narrow::kRimSamples;
        const real a = 6.28318530718f * (real)step / (real)narrow::kRimSamples;
        t.c[i] = std::cos(a);
        t.s[i] = std::sin(a);
    }
    cudaMemcpyToSymbol(c_rim, &t, sizeof(t));
}

void launchAdjacency(const Dev &d, cudaStream_t s) {
    cudaMemsetAsync(d.adjStart, 0, sizeof(int) * static_cast<size_t>(d.NB + 1), s);
    cudaMemsetAsync(d.adjFill, 0, sizeof(int) * static_cast<size_t>(d.NB), s);
    ++launchCount(); launchK(adjCountKernel, grid(d.FF + d.MM), kThreads, 0, s, d);
    // Slots past the last body count zero, so scanning the whole capacity gives the same starts.
    scanExclusive(d.adjStart, d.adjStart, d.NB + 1, nullptr, d.ctr + C_ADJ, d.scanScratch, s);
    ++launchCount(); launchK(adjTotalKernel, 1, 1, 0, s, d);
    ++launchCount(); launchK(adjFillKernel, grid(d.FF + d.MM), kThreads, 0, s, d);
    segmentedSortU32(d.adjSeq, d.adjTmp, d.adjStart, d.NB, d.ctr + C_BODIES, d.longList, d.ctr + C_LONG, s);
    ++launchCount(); launchK(adjInfoKernel, grid(d.NB), kThreads, 0, s, d);
}

bool narrowBlockFits(int block) {
    return blockFits(manifoldInitKernel<false>, block) && blockFits(manifoldInitKernel<true>, block);
}

void launchManifoldInit(const Dev &d, const StepParams &p, bool round, int block, cudaStream_t s) {
    ++launchCount();
    if (round)
        launchK(manifoldInitKernel<true>, divUp(d.MM, block), block, 0, s, d, p);
    else
        launchK(manifoldInitKernel<false>, divUp(d.MM, block), block, 0, s, d, p);
}

void launchManifoldCompact(const Dev &d, cudaStream_t s) {
    scanExclusive(d.mActive, d.pairValid, d.MM, d.ctr + C_CAND, d.ctr + C_LIVE, d.scanScratch, s);
    ++launchCount();
    const int blocks = residentGrid(reinterpret_cast<const void *>(manifoldCompactKernel), kThreads, 0,
                                    divUp(d.MM * kMaxContacts, kThreads));
    launchK(manifoldCompactKernel, blocks, kThreads, 0, s, d, d.mActive, d.pairValid);
}

void launchRebase(const Dev &d, const StepParams &p, cudaStream_t s) {
    ++launchCount(); launchK(rebaseKernel, residentGrid(rebaseKernel, kThreads, grid(d.MM)), kThreads, 0, s, d, p);
}

void launchForceInit(const Dev &d, const StepParams &p, bool forces, cudaStream_t s) {
    if (!forces)
        return;
    cudaMemsetAsync(d.ctr + C_TMP, 0, sizeof(int), s);
    ++launchCount(); launchK(forceInitKernel, grid(d.FF), kThreads, 0, s, d, p);
    ++launchCount(); launchK(forceCompactKernel, 1, 1, 0, s, d);
}

} // namespace avbdg
