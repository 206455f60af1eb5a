// Broad phase: swept AABBs, Morton codes, Karras LBVH per world, refit, candidate pairs, exact
// filter and manifold acquisition (godot-avbd src/avbd/solver_broadphase.cpp:85-186,
// src/avbd/bvh_broadphase.cpp:19-292, src/avbd/rigid.cpp:83-106).
//
// The reference builds its tree by pairwise merging of Morton-sorted leaves and walks it
// serially; the candidate set it produces is "every leaf pair whose closed swept AABBs overlap",
// which does not depend on the tree's shape. Here each world gets a Karras radix tree over the
// same (code, list index) order, every body walks it in parallel and emits its partners with a
// larger list index, and per-body segments are sorted, so the sorted key list equals the
// reference's sorted, de-duplicated sweepPairs bit for bit.

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;
constexpr int kStack = 128;

__device__ __forceinline__ int orderedInt(real f) {
    const int i = fbits(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ real orderedFloat(int i) { return bitsf(i >= 0 ? i : i ^ 0x7fffffff); }

// Swept AABB (solver_broadphase.cpp:103-122) over the tight box bound (rigid.cpp:83-106).
__global__ void aabbKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0)
        return;
    const real4 x4 = d.x[g];
    const real4 v4 = d.v[g];
    const real4 s4 = d.size[g];
    const m3 rot = qmat(asq(d.q[g]));
    // aabbHalfExtent (rigid.cpp:83-106): sphere (r, r, r), cylinder (r, r, h/2), box size/2.
    const int shape = (d.meta[g].w >> 18) & 0x3;
    const f3 h = shape == 1 ? f3{s4.x, s4.x, s4.x} : (shape == 2 ? f3{s4.x, s4.x, s4.z * 0.5f} : scale(xyz(s4), 0.5f));
    const f3 tight{(mabs(rot.c0.x) * h.x + mabs(rot.c1.x) * h.y) + mabs(rot.c2.x) * h.z,
                   (mabs(rot.c0.y) * h.x + mabs(rot.c1.y) * h.y) + mabs(rot.c2.y) * h.z,
                   (mabs(rot.c0.z) * h.x + mabs(rot.c1.z) * h.y) + mabs(rot.c2.z) * h.z};
    const real cdt = p.collisionDt;
    f3 disp = scale(xyz(v4), cdt);
    if (x4.w > 0)
        disp = add(disp, f3{0, 0, v4.w * cdt * cdt});
    const real rotSweep = s4.w * length(xyz(d.w[g])) * cdt;
    const real grow = rotSweep + p.specMargin;
    const f3 c = add(xyz(x4), scale(disp, 0.5f));
    const f3 half = add(add(tight, scale(vabs(disp), 0.5f)), f3{grow, grow, grow});
    d.aabbC[g] = f4(c, 0.0f);
    d.aabbH[g] = f4(half, 0.0f);
}

// ---- Morton codes (bvh_broadphase.cpp:19-36, 70-85) ----

__global__ void boundsResetKernel(Dev d, int *wBounds) {
    pdlWait();
    pdlTrigger();
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= d.ctr[C_WORLDS])
        return;
    for (int k = 0; k < 3; k++) {
        wBounds[6 * w + k] = 0x7fffffff;          // lo (ordered)
        wBounds[6 * w + 3 + k] = (int)0x80000000; // hi (ordered)
    }
}

// Per-world min/max of the AABB centres. Lanes of a warp reduce per world first (worlds are slot
// ranges, so a warp mostly holds one), and one lane per world and warp does the atomics: a single
// large world would otherwise serialise six atomics per body on six addresses.
__global__ void boundsKernel(Dev d, int *wBounds) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = g < n ? d.meta[g].x : -1;
    int v[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, static_cast<int>(0x80000000), static_cast<int>(0x80000000),
                static_cast<int>(0x80000000)};
    if (w >= 0) {
        const real4 c = d.aabbC[g];
        v[0] = v[3] = orderedInt(c.x);
        v[1] = v[4] = orderedInt(c.y);
        v[2] = v[5] = orderedInt(c.z);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, w);
    int r[6];
    for (int k = 0; k < 3; k++) {
        r[k] = __reduce_min_sync(peers, v[k]);
        r[k + 3] = __reduce_max_sync(peers, v[k + 3]);
    }
    if (w < 0 || (threadIdx.x & 31) != __ffs(peers) - 1)
        return;
    for (int k = 0; k < 3; k++) {
        atomicMin(&wBounds[6 * w + k], r[k]);
        atomicMax(&wBounds[6 * w + 3 + k], r[k + 3]);
    }
}

__device__ __forceinline__ uint64_t expandBits21(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10cfcfcfcfcfcfcfull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__device__ __forceinline__ uint32_t quantise(real v, real lo, real scaleF) {
    return static_cast<uint32_t>(sclamp((v - lo) * scaleF, 0.0f, 2097151.0f));
}

// Code per body; keys/values laid out by list position for the stable (code, list index) sort.
__global__ void mortonKernel(Dev d, const int *wBounds) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0)
        return;
    const int w = d.meta[g].x;
    const real lox = orderedFloat(wBounds[6 * w + 0]), loy = orderedFloat(wBounds[6 * w + 1]),
                loz = orderedFloat(wBounds[6 * w + 2]);
    const real hix = orderedFloat(wBounds[6 * w + 3]), hiy = orderedFloat(wBounds[6 * w + 4]),
                hiz = orderedFloat(wBounds[6 * w + 5]);
    const f3 ext{hix - lox, hiy - loy, hiz - loz};
    real e = ext.x;
    if (e < ext.y)
        e = ext.y;
    if (e < ext.z)
        e = ext.z;
    if (e < 1.0e-6f)
        e = 1.0e-6f;
    const real sc = 2097151.0f / e;
    const real4 c = d.aabbC[g];
    // The reference quantises all three axes against lo.x (bvh_broadphase.cpp:85): kept for the
    // code and order dumps. Where a scene does not extend from lo.x in y and z, that clamps whole
    // regions to one code and degrades the tree, so the tree is built from codes with each axis's
    // own origin. The candidate pairs do not depend on the tree's shape.
    d.codes[g] = expandBits21(quantise(c.x, lox, sc)) | (expandBits21(quantise(c.y, lox, sc)) << 1) |
                 (expandBits21(quantise(c.z, lox, sc)) << 2);
    const uint64_t code = expandBits21(quantise(c.x, lox, sc)) | (expandBits21(quantise(c.y, loy, sc)) << 1) |
                          (expandBits21(quantise(c.z, loz, sc)) << 2);
    d.treeCodes[g] = code;
    const int lp = listPos(d, g);
    d.sortK[lp] = code;
    d.sortV[lp] = static_cast<uint32_t>(lp);
}

// Slots without a body keep key ~0 and map to themselves in list-position space.
__global__ void mortonResetKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    d.sortK[i] = ~0ull;
    d.sortV[i] = static_cast<uint32_t>(i);
}

// Second key: the world's first slot (a free slot keys on its own position), so after the stable
// sort world w's leaves occupy sorted positions [wBase, wBase + wCount).
__global__ void worldKeyKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int lp = static_cast<int>(d.sortV[i]);
    const int g = d.lpToBody[lp];
    d.sortK[i] = static_cast<uint64_t>(g >= 0 ? d.wBase[d.meta[g].x] : lp);
}

__global__ void leafKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    d.leafBody[i] = d.lpToBody[d.sortV[i]];
}

// Longest common prefix of the augmented keys (code, list position) within one world segment.
__device__ __forceinline__ int deltaKey(const Dev &d, int s, int n, int i, int j) {
    if (j < 0 || j >= n)
        return -1;
    const uint64_t ci = d.treeCodes[d.leafBody[s + i]];
    const uint64_t cj = d.treeCodes[d.leafBody[s + j]];
    if (ci != cj)
        return __clzll(static_cast<long long>(ci ^ cj));
    return 64 + __clz(static_cast<int>(d.sortV[s + i] ^ d.sortV[s + j]));
}

constexpr int kLeafBit = 0x40000000;

// Karras (2012) radix tree: internal node i of a world spans a key range and splits at the
// highest differing bit.
__global__ void karrasKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n)
        return;
    const int g = d.leafBody[p];
    if (g < 0)
        return;
    const int w = d.meta[g].x;
    const int s = d.wBase[w];
    const int cnt = d.wCount[w];
    const int i = p - s;
    if (i == 0)
        d.nodeParent[s] = -1;
    if (cnt < 2 || i >= cnt - 1)
        return;
    const int dir = (deltaKey(d, s, cnt, i, i + 1) - deltaKey(d, s, cnt, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = deltaKey(d, s, cnt, i, i - dir);
    int lmax = 2;
    while (deltaKey(d, s, cnt, i, i + lmax * dir) > dmin)
        lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (deltaKey(d, s, cnt, i, i + (l + t) * dir) > dmin)
            l += t;
    const int j = i + l * dir;
    const int dnode = deltaKey(d, s, cnt, i, j);
    int sp = 0;
    for (int div = 2;; div <<= 1) {
        const int t = (l + div - 1) / div;
        if (deltaKey(d, s, cnt, i, i + (sp + t) * dir) > dnode)
            sp += t;
        if (t <= 1)
            break;
    }
    const int gamma = i + sp * dir + (dir < 0 ? -1 : 0);
    const int lo = i < j ? i : j;
    const int hi = i < j ? j : i;
    int left, right;
    if (lo == gamma) {
        left = kLeafBit | (s + gamma);
        d.leafParent[s + gamma] = s + i;
    } else {
        left = s + gamma;
        d.nodeParent[s + gamma] = s + i;
    }
    if (hi == gamma + 1) {
        right = kLeafBit | (s + gamma + 1);
        d.leafParent[s + gamma + 1] = s + i;
    } else {
        right = s + gamma + 1;
        d.nodeParent[s + gamma + 1] = s + i;
    }
    d.nodeL[s + i] = left;
    d.nodeR[s + i] = right;
}

__device__ __forceinline__ void childBounds(const Dev &d, int c, real4 &mn, real4 &mx) {
    if (c & kLeafBit) {
        const int b = d.leafBody[c & ~kLeafBit];
        const real4 cc = d.aabbC[b];
        const real4 hh = d.aabbH[b];
        mn = mk4(cc.x - hh.x, cc.y - hh.y, cc.z - hh.z, 0.0f);
        mx = mk4(cc.x + hh.x, cc.y + hh.y, cc.z + hh.z, 0.0f);
    } else {
        mn = __ldcg(&d.nodeMin[c]);
        mx = __ldcg(&d.nodeMax[c]);
    }
}

// Arrival count at a node, acquire-release at GPU scope: it releases this thread's earlier bound
// writes to the node's other child thread and acquires that thread's, in one instruction instead of
// a fence on each side of a relaxed add.
__device__ __forceinline__ int arriveAcqRel(int *flag) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(flag) : "memory");
    return old;
}

// Bottom-up refit: the second child to arrive at a node computes its bounds. The arriving thread
// carries the box and largest list position of the child it comes from (the values it stored, or a
// leaf's c -/+ h) and loads only the other child's; the node's topology is read with the arrival.
// The bounds are combined as (left, right) in the same order as always.
__global__ void refitKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n)
        return;
    const int g = d.leafBody[p];
    if (g < 0)
        return;
    const int w = d.meta[g].x;
    if (d.wCount[w] < 2)
        return;
    int child = p | kLeafBit;
    real4 cMin, cMax;
    childBounds(d, child, cMin, cMax);
    int cLp = static_cast<int>(d.sortV[p]);
    int node = d.leafParent[p];
    while (node >= 0) {
        const int l = d.nodeL[node], r = d.nodeR[node], parent = d.nodeParent[node];
        if (arriveAcqRel(&d.nodeFlag[node]) == 0)
            return;
        const bool fromLeft = l == child;
        const int other = fromLeft ? r : l;
        real4 oMin, oMax;
        childBounds(d, other, oMin, oMax);
        const int oLp = (other & kLeafBit) ? static_cast<int>(d.sortV[other & ~kLeafBit]) : __ldcg(&d.nodeMaxLp[other]);
        const real4 a0 = fromLeft ? cMin : oMin, a1 = fromLeft ? cMax : oMax;
        const real4 b0 = fromLeft ? oMin : cMin, b1 = fromLeft ? oMax : cMax;
        const int ml = fromLeft ? cLp : oLp, mr = fromLeft ? oLp : cLp;
        const real4 nMin = mk4(mmin2(a0.x, b0.x), mmin2(a0.y, b0.y), mmin2(a0.z, b0.z), 0.0f);
        const real4 nMax = mk4(mmax2(a1.x, b1.x), mmax2(a1.y, b1.y), mmax2(a1.z, b1.z), 0.0f);
        __stcg(&d.nodeMin[node], nMin);
        __stcg(&d.nodeMax[node], nMax);
        __stcg(&d.nodeMaxLp[node], ml > mr ? ml : mr);
        real4 *kids = d.nodeKids + 4 * static_cast<size_t>(node);
        __stcg(kids, a0);
        __stcg(kids + 1, a1);
        __stcg(kids + 2, b0);
        __stcg(kids + 3, b1);
        __stcg(&d.nodeLink[node], make_int4(l, r, ml, mr));
        child = node;
        cMin = nMin;
        cMax = nMax;
        cLp = ml > mr ? ml : mr;
        node = parent;
    }
}

__device__ __forceinline__ bool overlapClosed(f3 aMin, f3 aMax, f3 bMin, f3 bMax) {
    return !(bMin.x > aMax.x || bMin.y > aMax.y || bMin.z > aMax.z || aMin.x > bMax.x || aMin.y > bMax.y ||
             aMin.z > bMax.z);
}

// Walk the world's tree with body g's box for partners with a larger list position.
// COUNT: threads take bodies in tree (Morton) order, so a warp's walks follow nearby paths; each
// counts its partners and keeps the first kPairStash of them, and a body with more is listed for
// a second walk. EMIT (that second walk): the listed bodies write their partners into their
// segments. Pair keys are (lpA << 32 | lpB); the segmented sort orders each segment afterwards.
template <bool EMIT>
__global__ void traverseKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = EMIT ? d.ctr[C_PAIRSPILL] : d.ctr[C_BODIES];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int g = EMIT ? d.pairSpill[i] : d.leafBody[i];
    if (g < 0)
        return;
    const int w = d.meta[g].x;
    if (w < 0)
        return;
    const int cnt = d.wCount[w];
    const int lpA = listPos(d, g);
    int out = EMIT ? d.pairStart[lpA] : 0;
    int found = 0;
    int *stash = d.pairStash + static_cast<size_t>(lpA) * kPairStash;
    if (cnt >= 2) {
        const real4 c4 = d.aabbC[g], h4 = d.aabbH[g];
        const f3 aMin{c4.x - h4.x, c4.y - h4.y, c4.z - h4.z};
        const f3 aMax{c4.x + h4.x, c4.y + h4.y, c4.z + h4.z};
        int stack[kStack];
        int sp = 0;
        // The next node to visit stays in a register; only a second child to visit goes on the stack.
        int node = d.wBase[w];
        while (node >= 0) {
            int next = -1;
            // One visit reads the node's record: both children, their boxes and list positions
            // (a leaf's box is c -/+ h of its body, the floats the test below used to compute).
            const int4 link = d.nodeLink[node];
            const real4 *kidBox = d.nodeKids + 4 * static_cast<size_t>(node);
            const real4 boxes[4] = {kidBox[0], kidBox[1], kidBox[2], kidBox[3]};
            const int kids[2] = {link.x, link.y};
            const int kidLp[2] = {link.z, link.w};
            for (int k = 0; k < 2; k++) {
                const int c = kids[k];
                const real4 mn = boxes[2 * k], mx = boxes[2 * k + 1];
                if (c & kLeafBit) {
                    const int lpB = kidLp[k];
                    if (lpB <= lpA)
                        continue;
                    const f3 bMin{mn.x, mn.y, mn.z};
                    const f3 bMax{mx.x, mx.y, mx.z};
                    if (overlapClosed(aMin, aMax, bMin, bMax)) {
                        if (EMIT) {
                            if (out < d.PP)
                                d.pairs[out] = (static_cast<uint64_t>(lpA) << 32) | static_cast<uint32_t>(lpB);
                            out++;
                        } else if (found < kPairStash) {
                            stash[found] = lpB;
                        }
                        found++;
                    }
                } else {
                    if (kidLp[k] <= lpA)
                        continue; // every leaf below was emitted by a partner with a smaller position
                    if (overlapClosed(aMin, aMax, f3{mn.x, mn.y, mn.z}, f3{mx.x, mx.y, mx.z})) {
                        if (next < 0)
                            next = c;
                        else if (sp < kStack)
                            stack[sp++] = c;
                        else
                            atomicOr(&d.ctr[C_ERRORS], kErrPairs);
                    }
                }
            }
            node = next >= 0 ? next : (sp > 0 ? stack[--sp] : -1);
        }
    }
    if (!EMIT) {
        d.pairStart[lpA] = found;
        if (found > kPairStash)
            d.pairSpill[atomicAdd(&d.ctr[C_PAIRSPILL], 1)] = g;
    }
}

// The same partner search without the tree, for stores whose worlds are all small: body g tests
// every body of its world with a larger list position (a smaller slot: lp = 2 base + count - 1 -
// slot) with the traversal's own closed-box test, and hands on the same count, stash and spill list
// (EMIT: the same second pass for bodies with more than kPairStash partners), so the pair set and
// everything after it are the traversal's. Threads take bodies in slot order; the threads of one
// world read the same candidate on each iteration (one broadcast load).
template <bool EMIT>
__global__ void bruteKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = EMIT ? d.ctr[C_PAIRSPILL] : d.ctr[C_BODIES];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int g = EMIT ? d.pairSpill[i] : i;
    const int w = d.meta[g].x;
    if (w < 0)
        return;
    const int base = d.wBase[w], cnt = d.wCount[w];
    const int lpA = 2 * base + cnt - 1 - g;
    int out = EMIT ? d.pairStart[lpA] : 0;
    int found = 0;
    int *stash = d.pairStash + static_cast<size_t>(lpA) * kPairStash;
    if (cnt >= 2) {
        const real4 c4 = d.aabbC[g], h4 = d.aabbH[g];
        const f3 aMin{c4.x - h4.x, c4.y - h4.y, c4.z - h4.z};
        const f3 aMax{c4.x + h4.x, c4.y + h4.y, c4.z + h4.z};
#pragma unroll 4
        for (int b = base; b < g; b++) {
            const real4 bc = d.aabbC[b], bh = d.aabbH[b];
            const f3 bMin{bc.x - bh.x, bc.y - bh.y, bc.z - bh.z};
            const f3 bMax{bc.x + bh.x, bc.y + bh.y, bc.z + bh.z};
            if (overlapClosed(aMin, aMax, bMin, bMax)) {
                const int lpB = 2 * base + cnt - 1 - b;
                if (EMIT) {
                    if (out < d.PP)
                        d.pairs[out] = (static_cast<uint64_t>(lpA) << 32) | static_cast<uint32_t>(lpB);
                    out++;
                } else if (found < kPairStash) {
                    stash[found] = lpB;
                }
                found++;
            }
        }
    }
    if (!EMIT) {
        d.pairStart[lpA] = found;
        if (found > kPairStash)
            d.pairSpill[atomicAdd(&d.ctr[C_PAIRSPILL], 1)] = g;
    }
}

// Stashed partners into their body's segment (bodies with more partners are walked again).
__global__ void pairStashKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int lpA = blockIdx.x * blockDim.x + threadIdx.x;
    if (lpA >= n)
        return;
    const int start = d.pairStart[lpA], found = d.pairStart[lpA + 1] - start;
    if (found > kPairStash)
        return;
    const int *stash = d.pairStash + static_cast<size_t>(lpA) * kPairStash;
    for (int j = 0; j < found; j++)
        if (start + j < d.PP)
            d.pairs[start + j] = (static_cast<uint64_t>(lpA) << 32) | static_cast<uint32_t>(stash[j]);
}

__global__ void pairTotalKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    int t = d.ctr[C_TMP];
    if (t > d.PP) {
        atomicOr(&d.ctr[C_ERRORS], kErrPairs);
        t = d.PP;
    }
    d.ctr[C_PAIRS] = t;
}

// pairOverlaps (solver_broadphase.cpp:30-65): bounds, layer/mask, not constrained, not both static.
__device__ __forceinline__ void filterAt(Dev d, int k) {
    const int np = d.ctr[C_PAIRS];
    if (k >= np)
        return;
    const uint64_t key = d.pairs[k];
    const int a = d.lpToBody[static_cast<int>(key >> 32)];
    const int b = d.lpToBody[static_cast<int>(key & 0xffffffffu)];
    const real4 ac = d.aabbC[a], ah = d.aabbH[a], bc = d.aabbC[b], bh = d.aabbH[b];
    const bool bounds = overlapClosed(f3{ac.x - ah.x, ac.y - ah.y, ac.z - ah.z}, f3{ac.x + ah.x, ac.y + ah.y, ac.z + ah.z},
                                      f3{bc.x - bh.x, bc.y - bh.y, bc.z - bh.z}, f3{bc.x + bh.x, bc.y + bh.y, bc.z + bh.z});
    const int4 ma = d.meta[a], mb = d.meta[b];
    const bool layers = ((static_cast<uint32_t>(ma.y) & static_cast<uint32_t>(mb.z)) != 0) ||
                        ((static_cast<uint32_t>(mb.y) & static_cast<uint32_t>(ma.z)) != 0);
    const bool dynA = d.x[a].w > 0.0f, dynB = d.x[b].w > 0.0f;
    const bool bothStatic = !dynA && !dynB;
    bool constrained = false;
    if (!bothStatic) {
        // The relation is symmetric; only dynamic bodies carry adjacency lists.
        const int xb = dynA ? a : b;
        const int yb = dynA ? b : a;
        for (int e = d.adjStart[xb]; e < d.adjStart[xb + 1]; e++)
            if (adjInfoOther(d.adjInfo[e]) == yb) {
                constrained = true;
                break;
            }
    }
    d.pairValid[k] = (bounds && layers && !constrained && !bothStatic) ? 1 : 0;
}

__global__ void filterKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_PAIRS];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        filterAt(d, k);
}

__device__ __forceinline__ void acquireAt(Dev d, const int *flags, const int *rank, int k) {
    const int np = d.ctr[C_PAIRS];
    if (k >= np || !flags[k])
        return;
    const int m = d.ctr[C_LIVE] + rank[k];
    if (m >= d.MM)
        return;
    const uint64_t key = d.pairs[k];
    d.live.ab[m] = make_int2(d.lpToBody[static_cast<int>(key >> 32)], d.lpToBody[static_cast<int>(key & 0xffffffffu)]);
    d.live.count[m] = 0;
    d.live.dormant[m] = make_int2(0, 0);
}

__global__ void acquireKernel(Dev d, const int *flags, const int *rank) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_PAIRS];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        acquireAt(d, flags, rank, k);
}

__global__ void candTotalKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    int c = d.ctr[C_LIVE] + d.ctr[C_TMP];
    if (c > d.MM) {
        atomicOr(&d.ctr[C_ERRORS], kErrManifolds);
        c = d.MM;
    }
    d.ctr[C_CAND] = c;
}

} // namespace

static int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }

void launchAabb(const Dev &d, const StepParams &p, cudaStream_t s) {
    ++launchCount(); launchK(aabbKernel, grid(d.NB), kThreads, 0, s, d, p);
}

void launchRebuildTree(const Dev &d, bool multiWorld, cudaStream_t s) {
    const int *nb = d.ctr + C_BODIES;
    ++launchCount(); launchK(boundsResetKernel, grid(d.WW), kThreads, 0, s, d, d.wBounds);
    ++launchCount(); launchK(boundsKernel, grid(d.NB), kThreads, 0, s, d, d.wBounds);
    ++launchCount(); launchK(mortonResetKernel, grid(d.NB), kThreads, 0, s, d);
    ++launchCount(); launchK(mortonKernel, grid(d.NB), kThreads, 0, s, d, d.wBounds);
    radixSortPairs(d.sortK, d.sortV, d.sortKAlt, d.sortVAlt, d.NB, nb, 0, 63, d.radixScratch, s);
    if (multiWorld) {
        int bits = 1; // world bases are below the slot capacity
        while ((1 << bits) < d.NB + 1)
            bits++;
        ++launchCount(); launchK(worldKeyKernel, grid(d.NB), kThreads, 0, s, d);
        radixSortPairs(d.sortK, d.sortV, d.sortKAlt, d.sortVAlt, d.NB, nb, 0, bits, d.radixScratch, s);
    }
    ++launchCount(); launchK(leafKernel, grid(d.NB), kThreads, 0, s, d);
    ++launchCount(); launchK(karrasKernel, grid(d.NB), kThreads, 0, s, d);
}

void launchRefit(const Dev &d, cudaStream_t s) {
    cudaMemsetAsync(d.nodeFlag, 0, sizeof(int) * static_cast<size_t>(d.NB), s);
    ++launchCount(); launchK(refitKernel, grid(d.NB), kThreads, 0, s, d);
}

bool traverseBlockFits(int block) {
    return blockFits(traverseKernel<false>, block) && blockFits(traverseKernel<true>, block) &&
           blockFits(bruteKernel<false>, block) && blockFits(bruteKernel<true>, block);
}

void launchPairs(const Dev &d, int block, bool brute, cudaStream_t s) {
    cudaMemsetAsync(d.pairStart, 0, sizeof(int) * static_cast<size_t>(d.NB + 1), s);
    cudaMemsetAsync(d.ctr + C_PAIRSPILL, 0, sizeof(int), s);
    ++launchCount();
    if (brute)
        launchK(bruteKernel<false>, divUp(d.NB, block), block, 0, s, d);
    else
        launchK(traverseKernel<false>, divUp(d.NB, block), block, 0, s, d);
    scanExclusive(d.pairStart, d.pairStart, d.NB + 1, nullptr, d.ctr + C_TMP, d.scanScratch, s);
    ++launchCount(); launchK(pairTotalKernel, 1, 1, 0, s, d);
    ++launchCount(); launchK(pairStashKernel, divUp(d.NB, kThreads), kThreads, 0, s, d);
    ++launchCount();
    if (brute)
        launchK(bruteKernel<true>, divUp(d.NB, block), block, 0, s, d);
    else
        launchK(traverseKernel<true>, divUp(d.NB, block), block, 0, s, d);
    segmentedSortU64(d.pairs, d.pairsTmp, d.pairStart, d.NB, d.ctr + C_BODIES, d.longList, d.ctr + C_LONG, s);
}

void launchFilterAcquire(const Dev &d, cudaStream_t s) {
    ++launchCount(); launchK(filterKernel, residentGrid(filterKernel, kThreads, grid(d.PP)), kThreads, 0, s, d);
    scanExclusive(d.pairValid, d.mActive, d.PP, d.ctr + C_PAIRS, d.ctr + C_TMP, d.scanScratch, s);
    ++launchCount(); launchK(acquireKernel, residentGrid(acquireKernel, kThreads, grid(d.PP)), kThreads, 0, s, d, d.pairValid, d.mActive);
    ++launchCount(); launchK(candTotalKernel, 1, 1, 0, s, d);
}

} // namespace avbdg
