// Update set, colouring and the substep (godot-avbd src/avbd/solver_solve.cpp,
// src/avbd/solver_step.cpp:79-105,195-316, src/avbd/manifold.cpp:465-671, src/avbd/joint.cpp,
// src/avbd/types.hpp:147-201, src/avbd/maths.h:156-343).
//
// Primal, block-Jacobi ("overflow") bodies: the reference computes each round's per-contact force
// cache once per manifold (preCompute), then every overflow body stamps its incident manifolds
// from that cache in adjacency order and solves its 6x6 block against the round's pose snapshot.
// Here one kernel per manifold computes the dual update AND, from the same poses, the next
// round's per-side block contributions ("stamps"); one kernel per body then sums its stamps in
// adjacency order, solves the LDL^T in registers and applies the relaxed delta. Both steps keep
// the reference's operation order, so the result is bit-identical.
//
// Coloured (Gauss-Seidel) bodies recompute their manifold terms from the current poses at every
// touch; the reference's "first touch uses the dual's cache" rule yields the same floats.

#include "forces.cuh"
#include "gridsync.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

constexpr int kThreads = 256;
constexpr int kSolveThreads = 128;
constexpr int kQueueThreads = 128; // items per round-queue tile

__device__ __forceinline__ int divUpDev(int a, int b) { return (a + b - 1) / b; }

struct Blk {
    m3 lin, ang, crs;
    f3 rl, ra;
};

// Block::Block (types.hpp:157-172).
__device__ __forceinline__ Blk makeBlock(real mass, f3 moment, real dtSq, f3 x, f3 xi, q4 q, q4 qi) {
    Blk b;
    const f3 mo = divs(f3{mass, mass, mass}, dtSq);
    b.lin = mdiag(mo.x, mo.y, mo.z);
    b.crs = mzero();
    b.rl = cmul(mo, sub(x, xi));
    const m3 rot = qmat(q);
    const m3 iw = mul(rot, mul(mdiag(moment.x, moment.y, moment.z), transpose(rot)));
    b.ang = mdivs(iw, dtSq);
    b.ra = mul(b.ang, qdiff(q, qi));
    return b;
}

// ---- 6x6 solves (maths.h:156-343) ----

__device__ bool ldlt6(const real a[6][6], const real b[6], real x[6]) {
    real l[6][6];
    real dd[6];
#pragma unroll
    for (int j = 0; j < 6; j++) {
        real dj = a[j][j];
#pragma unroll
        for (int s = 0; s < j; s++)
            dj -= l[j][s] * l[j][s] * dd[s];
        if (!(dj > 1.0e-12f))
            return false;
        dd[j] = dj;
        l[j][j] = 1.0f;
#pragma unroll
        for (int i = j + 1; i < 6; i++) {
            real lij = a[i][j];
#pragma unroll
            for (int s = 0; s < j; s++)
                lij -= l[i][s] * l[j][s] * dd[s];
            l[i][j] = lij / dd[j];
        }
    }
    real z[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        real v = b[i];
#pragma unroll
        for (int s = 0; s < i; s++)
            v -= l[i][s] * z[s];
        z[i] = v;
    }
#pragma unroll
    for (int i = 0; i < 6; i++)
        x[i] = z[i] / dd[i];
#pragma unroll
    for (int i = 5; i >= 0; i--) {
        real v = x[i];
#pragma unroll
        for (int s = i + 1; s < 6; s++)
            v -= l[s][i] * x[s];
        x[i] = v;
    }
    real worst = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; i++)
        worst = smax(worst, mabs(x[i]));
    return isfinite(worst) && worst < 1.0e1f;
}

__device__ __forceinline__ bool ldlt6Pivoted(const real aIn[6][6], const real b[6], real x[6]) {
    real a[6][6];
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++)
            a[r][c] = aIn[r][c];
    real dd[6] = {0, 0, 0, 0, 0, 0};
    int t[6] = {0, 1, 2, 3, 4, 5};
    bool foundZero = false;
    for (int k = 0; k < 6; k++) {
        int j = k;
        real best = mabs(a[k][k]);
        for (int i = k + 1; i < 6; i++) {
            const real cand = mabs(a[i][i]);
            if (cand > best) {
                best = cand;
                j = i;
            }
        }
        t[k] = j;
        if (j != k) {
            for (int c = 0; c < 6; c++) {
                const real tmp = a[k][c];
                a[k][c] = a[j][c];
                a[j][c] = tmp;
            }
            for (int r = 0; r < 6; r++) {
                const real tmp = a[r][k];
                a[r][k] = a[r][j];
                a[r][j] = tmp;
            }
        }
        if (k > 0) {
            real temp[6] = {0, 0, 0, 0, 0, 0};
            for (int i = 0; i < k; i++)
                temp[i] = dd[i] * a[k][i];
            real prod[6] = {0, 0, 0, 0, 0, 0};
            for (int i = 0; i < k; i++)
                prod[i] = a[k][i] * temp[i];
            real dotv;
            switch (k) {
            case 1: dotv = prod[0]; break;
            case 2: dotv = prod[0] + prod[1]; break;
            case 3: dotv = (prod[0] + prod[1]) + prod[2]; break;
            case 4: dotv = (prod[0] + prod[2]) + (prod[1] + prod[3]); break;
            default: dotv = ((prod[0] + prod[2]) + (prod[1] + prod[3])) + prod[4]; break;
            }
            a[k][k] -= dotv;
            for (int i = 0; i < k; i++) {
                const real ti = temp[i];
                for (int r = k + 1; r < 6; r++)
                    a[r][k] -= a[r][i] * ti;
            }
        }
        const real pivot = a[k][k];
        const bool valid = mabs(pivot) > 0.0f;
        if (!valid) {
            for (int r = k + 1; r < 6; r++)
                if (a[r][k] != 0.0f)
                    return false;
            foundZero = true;
        } else if (foundZero) {
            return false;
        }
        if (valid)
            for (int r = k + 1; r < 6; r++)
                a[r][k] /= pivot;
        dd[k] = pivot;
    }
    for (int i = 0; i < 6; i++)
        x[i] = b[i];
    for (int k = 0; k < 6; k++) {
        const real tmp = x[k];
        x[k] = x[t[k]];
        x[t[k]] = tmp;
    }
    for (int jj = 0; jj < 5; jj++) {
        const real v = x[jj];
        if (v != 0.0f)
            for (int i = jj + 1; i < 6; i++)
                x[i] -= a[i][jj] * v;
    }
    const real tolerance = 1.17549435e-38f; // FLT_MIN
    for (int i = 0; i < 6; i++)
        x[i] = mabs(dd[i]) > tolerance ? x[i] / dd[i] : 0.0f;
    for (int jj = 5; jj >= 1; jj--) {
        const real v = x[jj];
        if (v != 0.0f)
            for (int i = jj - 1; i >= 0; i--)
                x[i] -= a[jj][i] * v;
    }
    for (int k = 5; k >= 0; k--) {
        const real tmp = x[k];
        x[k] = x[t[k]];
        x[t[k]] = tmp;
    }
    real worst = 0.0f;
    for (int i = 0; i < 6; i++)
        worst = smax(worst, mabs(x[i]));
    return isfinite(worst) && worst < 1.0e1f;
}

// The 6x6 system of Block::solveDelta (types.hpp:176-197): a = [lin crs^T; crs ang], b = -rhs.
__device__ __forceinline__ void blockSystem(const Blk &k, real a[6][6], real b[6]) {
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            a[r][c] = mat(k.lin, c, r);
            a[r + 3][c + 3] = mat(k.ang, c, r);
            a[r + 3][c] = mat(k.crs, c, r);
            a[r][c + 3] = mat(k.crs, r, c);
        }
    b[0] = -k.rl.x;
    b[1] = -k.rl.y;
    b[2] = -k.rl.z;
    b[3] = -k.ra.x;
    b[4] = -k.ra.y;
    b[5] = -k.ra.z;
}

struct Delta {
    f3 dl, da;
    bool ok;
};

// solve()'s pivoted fallback, out of line: the block travels by value, so the fast path's matrix
// never needs an address and stays in registers.
__device__ __noinline__ Delta solvePivoted(Blk k) {
    real a[6][6], b[6], x[6];
    blockSystem(k, a, b);
    Delta r;
    r.ok = ldlt6Pivoted(a, b, x);
    r.dl = f3{x[0], x[1], x[2]};
    r.da = f3{x[3], x[4], x[5]};
    return r;
}

// Block::solveDelta's plain LDLT; false when solve() would fall back.
__device__ __forceinline__ bool solveBlockFast(const Blk &k, f3 &dl, f3 &da) {
    real a[6][6], b[6], x[6];
    blockSystem(k, a, b);
    if (!ldlt6(a, b, x))
        return false;
    dl = f3{x[0], x[1], x[2]};
    da = f3{x[3], x[4], x[5]};
    return true;
}

// Block::solveDelta with solve()'s fallback chain: plain LDLT, pivoted LDLT, then no step.
__device__ __forceinline__ void solveBlock(const Blk &k, f3 &dl, f3 &da) {
    if (solveBlockFast(k, dl, da))
        return;
    const Delta r = solvePivoted(k);
    if (r.ok) {
        dl = r.dl;
        da = r.da;
        return;
    }
    dl = f3{0, 0, 0};
    da = f3{0, 0, 0};
}

// ---- contact terms (manifold.cpp:196-234, 465-570, 583-671) ----

__device__ __forceinline__ void basisHessianD(f3 b0, f3 b1, f3 b2, f3 k, real S[6]) {
    const real b0x2 = b0.x * b0.x, b0y2 = b0.y * b0.y, b0z2 = b0.z * b0.z;
    const real b0xy = b0.x * b0.y, b0xz = b0.x * b0.z, b0yz = b0.y * b0.z;
    const real b1x2 = b1.x * b1.x, b1y2 = b1.y * b1.y, b1z2 = b1.z * b1.z;
    const real b1xy = b1.x * b1.y, b1xz = b1.x * b1.z, b1yz = b1.y * b1.z;
    const real b2x2 = b2.x * b2.x, b2y2 = b2.y * b2.y, b2z2 = b2.z * b2.z;
    const real b2xy = b2.x * b2.y, b2xz = b2.x * b2.z, b2yz = b2.y * b2.z;
    S[0] = k.x * b0x2 + k.y * b1x2 + k.z * b2x2;
    S[1] = k.x * b0xy + k.y * b1xy + k.z * b2xy;
    S[2] = k.x * b0xz + k.y * b1xz + k.z * b2xz;
    S[3] = k.x * b0y2 + k.y * b1y2 + k.z * b2y2;
    S[4] = k.x * b0yz + k.y * b1yz + k.z * b2yz;
    S[5] = k.x * b0z2 + k.y * b1z2 + k.z * b2z2;
}

__device__ __forceinline__ f3 basisMulD(f3 r0, f3 r1, f3 r2, f3 v) {
    return f3{(r0.x * v.x + r0.y * v.y) + r0.z * v.z, (r1.x * v.x + r1.y * v.y) + r1.z * v.z,
              (r2.x * v.x + r2.y * v.y) + r2.z * v.z};
}

struct Cone {
    real bounds, scale;
};

__device__ __forceinline__ Cone clampForce(f3 &F, real mu) {
    F.x = smin(F.x, 0.0f);
    const real bounds = mabs(F.x) * mu;
    const real fs = length2d(F.y, F.z);
    if (fs > bounds && fs > 0) {
        F.y = F.y * (bounds / fs);
        F.z = F.z * (bounds / fs);
    }
    return Cone{bounds, fs};
}

// A symmetric 3x3 sum kept as its unique entries (00, 01, 02, 11, 12, 22). Every term added to it
// is symmetric, so the full matrix's two off-diagonal copies would take the same adds in the same
// order; the stamp record stores only these six.
struct Sym3 {
    real v[6];
};

__device__ __forceinline__ Sym3 symZero() { return Sym3{{0, 0, 0, 0, 0, 0}}; }

__device__ __forceinline__ void symAdd(Sym3 &a, const real t[6]) {
    for (int i = 0; i < 6; i++)
        a.v[i] = a.v[i] + t[i];
}

// Per-side accumulators of stampCached.
struct SideAcc {
    Sym3 ang;
    m3 crs;
    f3 rhsAng;
};
struct SharedAcc {
    Sym3 lin;
    f3 rhsLin;
};

// One contact's terms of one side's stamp: the unique entries of the angular block (h00, h01, h02,
// h11, h12, h22), the cross block r x S and the angular right-hand side r x fw.
struct SideTerms {
    real h[6];
    m3 rs;
    f3 rc;
};

__device__ __forceinline__ SideTerms sideTerms(const real S[6], f3 r, f3 fw) {
    const real s00 = S[0], s01 = S[1], s02 = S[2], s11 = S[3], s12 = S[4], s22 = S[5];
    const m3 Sm = mcols(f3{s00, s01, s02}, f3{s01, s11, s12}, f3{s02, s12, s22});
    SideTerms t;
    t.rs = mcols(cross(r, Sm.c0), cross(r, Sm.c1), cross(r, Sm.c2));
    const real rx2 = r.x * r.x, ry2 = r.y * r.y, rz2 = r.z * r.z;
    const real rxy = r.x * r.y, rxz = r.x * r.z, ryz = r.y * r.z;
    t.h[0] = s11 * rz2 - 2.0f * s12 * ryz + s22 * ry2;
    t.h[1] = s12 * rxz + s02 * ryz - s22 * rxy - s01 * rz2;
    t.h[2] = s12 * rxy + s01 * ryz - s11 * rxz - s02 * ry2;
    t.h[3] = s22 * rx2 - 2.0f * s02 * rxz + s00 * rz2;
    t.h[4] = s02 * rxy + s01 * rxz - s00 * ryz - s12 * rx2;
    t.h[5] = s00 * ry2 - 2.0f * s01 * rxy + s11 * rx2;
    t.rc = cross(r, fw);
    return t;
}

__device__ __forceinline__ void stampContact(const real S[6], f3 r, f3 fw, SideAcc &acc) {
    const SideTerms t = sideTerms(S, r, fw);
    const real *h = t.h;
    symAdd(acc.ang, h);
    acc.crs = madd(acc.crs, t.rs);
    acc.rhsAng = add(acc.rhsAng, t.rc);
}

__device__ __forceinline__ void stampShared(const real S[6], f3 fw, SharedAcc &acc) {
    symAdd(acc.lin, S);
    acc.rhsLin = add(acc.rhsLin, fw);
}

__device__ __forceinline__ void zeroAcc(SideAcc &a) {
    a.ang = symZero();
    a.crs = mzero();
    a.rhsAng = f3{0, 0, 0};
}

// One stamp record, loaded whole before it is added.
struct StampRec {
    real4 s0, s1, s2, s3, s4, s5, s6;
};

// Stamps are read-only while bodies solve: the read-only path.
__device__ __forceinline__ StampRec loadStamp(const real4 *src) {
    return StampRec{__ldg(src), __ldg(src + 1), __ldg(src + 2), __ldg(src + 3), __ldg(src + 4), __ldg(src + 5),
                    __ldg(src + 6)};
}

// block += stamp (full 3x3 adds, as the reference adds its accumulators).
__device__ __forceinline__ void addStamp(Blk &b, const StampRec &r) {
    const real4 s0 = r.s0, s1 = r.s1, s2 = r.s2, s3 = r.s3, s4 = r.s4, s5 = r.s5, s6 = r.s6;
    const m3 lin = mcols(f3{s0.x, s0.y, s0.z}, f3{s0.y, s0.w, s1.x}, f3{s0.z, s1.x, s1.y});
    const m3 ang = mcols(f3{s2.y, s2.z, s2.w}, f3{s2.z, s3.x, s3.y}, f3{s2.w, s3.y, s3.z});
    const m3 crs = mcols(f3{s4.z, s4.w, s5.x}, f3{s5.y, s5.z, s5.w}, f3{s6.x, s6.y, s6.z});
    b.lin = madd(b.lin, lin);
    b.ang = madd(b.ang, ang);
    b.crs = madd(b.crs, crs);
    b.rl = add(b.rl, f3{s1.z, s1.w, s2.x});
    b.ra = add(b.ra, f3{s3.w, s4.x, s4.y});
}

// The same record through ordinary (coherent) loads, for a kernel that also writes the stamps.
__device__ __forceinline__ StampRec loadStampCoherent(const real4 *src) {
    return StampRec{src[0], src[1], src[2], src[3], src[4], src[5], src[6]};
}

template <bool RO = true>
__device__ __forceinline__ StampRec loadStampAs(const real4 *src) {
    return RO ? loadStamp(src) : loadStampCoherent(src);
}

__device__ __forceinline__ void addStamp(Blk &b, const real4 *src) { addStamp(b, loadStamp(src)); }

struct Pose {
    f3 x, dLin, dAng;
    q4 q;
    m3 rot;
};

__device__ __forceinline__ Pose loadPose(const Dev &d, int g) {
    Pose p;
    const real4 x4 = d.x[g];
    p.x = xyz(x4);
    p.q = asq(d.q[g]);
    p.dLin = sub(p.x, xyz(d.x0[g]));
    p.dAng = qdiff(p.q, asq(d.q0[g]));
    p.rot = qmat(p.q);
    return p;
}

// loadPose through the read-only path, for kernels that write no pose.
__device__ __forceinline__ Pose loadPoseRO(const Dev &d, int g) {
    Pose p;
    const real4 x4 = __ldg(&d.x[g]);
    p.x = xyz(x4);
    p.q = asq(__ldg(&d.q[g]));
    p.dLin = sub(p.x, xyz(__ldg(&d.x0[g])));
    p.dAng = qdiff(p.q, asq(__ldg(&d.q0[g])));
    p.rot = qmat(p.q);
    return p;
}

// Force the round's primal sees for contact c (preCompute, manifold.cpp:483-499).
__device__ __forceinline__ f3 contactError(const StepParams &p, f3 C0, f3 bracket, f3 r0, f3 r1, f3 r2) {
    const bool separated = p.specMargin > 0.0f && C0.x > kReleaseAbove;
    return add(scale(C0, separated ? 1.0f : p.oneMinusAlpha), basisMulD(r0, r1, r2, bracket));
}

enum : int { kSideA = 1, kSideB = 2 };

// Stamp record: lin (6 unique), rhsLin (signed), ang (6 unique), rhsAng (signed), cross (9).
__device__ __forceinline__ void storeStamp(real4 *dst, const SharedAcc &sh, const SideAcc &sd, real side) {
    const f3 rl = scale(sh.rhsLin, side);
    const f3 ra = scale(sd.rhsAng, side);
    dst[0] = mk4(sh.lin.v[0], sh.lin.v[1], sh.lin.v[2], sh.lin.v[3]);
    dst[1] = mk4(sh.lin.v[4], sh.lin.v[5], rl.x, rl.y);
    dst[2] = mk4(rl.z, sd.ang.v[0], sd.ang.v[1], sd.ang.v[2]);
    dst[3] = mk4(sd.ang.v[3], sd.ang.v[4], sd.ang.v[5], ra.x);
    dst[4] = mk4(ra.y, ra.z, sd.crs.c0.x, sd.crs.c0.y);
    dst[5] = mk4(sd.crs.c0.z, sd.crs.c1.x, sd.crs.c1.y, sd.crs.c1.z);
    dst[6] = mk4(sd.crs.c2.x, sd.crs.c2.y, sd.crs.c2.z, 0.0f);
}

// Stamps of manifold m for the requested sides, from the current poses and penalties.
__device__ void computeStamps(const Dev &d, const StepParams &p, int m, int sides) {
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const Pose A = loadPose(d, ab.x), B = loadPose(d, ab.y);
    const real4 b04 = L.b0[m];
    const f3 r0 = xyz(b04), r1 = xyz(L.b1[m]), r2 = xyz(L.b2[m]);
    const real mu = b04.w;
    const int n = L.count[m];
    SharedAcc sh;
    sh.lin = symZero();
    sh.rhsLin = f3{0, 0, 0};
    SideAcc sa, sb;
    zeroAcc(sa);
    zeroAcc(sb);
    for (int c = 1; c < n; c++) { // the later contacts' lines, requested before the in-order loop
        const int ci = cslot(d, m, c);
        prefetchL1(&L.rA[ci]);
        prefetchL1(&L.rB[ci]);
        prefetchL1(&L.C0[ci]);
        prefetchL1(&L.k[ci]);
        prefetchL1(&L.lam[ci]);
    }
    for (int c = 0; c < n; c++) {
        const int ci = cslot(d, m, c);
        const f3 rAw = mul(A.rot, xyz(L.rA[ci]));
        const f3 rBw = mul(B.rot, xyz(L.rB[ci]));
        if (p.armCache) { // preCompute refreshes the cached world arms (manifold.cpp:486-487)
            L.armA[ci] = f4(rAw, 0.0f);
            L.armB[ci] = f4(rBw, 0.0f);
        }
        const f3 bracket = sub(add(sub(A.dLin, B.dLin), cross(A.dAng, rAw)), cross(B.dAng, rBw));
        const f3 C = contactError(p, xyz(L.C0[ci]), bracket, r0, r1, r2);
        const f3 k = xyz(L.k[ci]);
        f3 F = add(cmul(k, C), xyz(L.lam[ci]));
        clampForce(F, mu);
        real S[6];
        basisHessianD(r0, r1, r2, k, S);
        const f3 fw = add(add(scale(r0, F.x), scale(r1, F.y)), scale(r2, F.z));
        stampShared(S, fw, sh);
        if (sides & kSideA)
            stampContact(S, rAw, fw, sa);
        if (sides & kSideB)
            stampContact(S, rBw, fw, sb);
    }
    const int2 slot = d.stampSlot[m];
    if (sides & kSideA)
        storeStamp(d.stamps + static_cast<size_t>(slot.x) * kStampF4, sh, sa, 1.0f);
    if (sides & kSideB)
        storeStamp(d.stamps + static_cast<size_t>(slot.y) * kStampF4, sh, sb, -1.0f);
}

// The flags of a manifold's two bodies the dual reads before its poses (awake: mass and not
// asleep; in the update set; colour), loaded together: each is a word or a byte of a valid body, so
// none waits for another to decide whether it is needed.
struct PairFlags {
    bool awakeA, awakeB;
    int sides;    // overflow sides that take stamps (kSideA | kSideB)
    bool touches; // a coloured body touches the manifold
};

template <bool STAMPS>
__device__ __forceinline__ PairFlags loadPairFlags(const Dev &d, int2 ab) {
    const real wA = d.x[ab.x].w, wB = d.x[ab.y].w;
    const int sA = d.sleep[ab.x].x, sB = d.sleep[ab.y].x;
    PairFlags f;
    f.awakeA = (wA > 0.0f) & (sA == 0);
    f.awakeB = (wB > 0.0f) & (sB == 0);
    f.sides = 0;
    f.touches = false;
    if (STAMPS) { // overflow sides take stamps; a coloured side means the colour passes recompute it
        // (the colour is read whether or not the body is in the update set, and used only if it is)
        const bool dynA = d.upd[ab.x] != 0, dynB = d.upd[ab.y] != 0;
        const uint8_t cA = d.colour[ab.x], cB = d.colour[ab.y];
        f.touches = (dynA & (cA < kOverflowColour)) | (dynB & (cB < kOverflowColour));
        f.sides = ((dynA & (cA == kOverflowColour)) ? kSideA : 0) | ((dynB & (cB == kOverflowColour)) ? kSideB : 0);
    }
    return f;
}

__device__ __forceinline__ void stampsAt(Dev d, StepParams p, int mixedOnly, int m) {
    if (m >= d.ctr[C_LIVE])
        return;
    const PairFlags flags = loadPairFlags<true>(d, d.live.ab[m]); // the awake fields are not used here
    if (!flags.sides || flags.touches != (mixedOnly != 0))
        return;
    computeStamps(d, p, m, flags.sides);
}

__global__ void stampsKernel(Dev d, StepParams p, int mixedOnly) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x)
        stampsAt(d, p, mixedOnly, m);
}

// Dual pass (ManifoldStore::updateDual, manifold.cpp:583-671) and, with STAMPS, the next round's
// stamps (the reference's phase-A recompute of each force, manifold.cpp:655-659, from the same
// floats). One thread per manifold, grid-stride over the live ones.
// ARM: the arm cache is on (compiled out otherwise, so the common path keeps its code).
// One manifold's dual pass (and, with STAMPS, its next-round stamps): the body of dualKernel's loop,
// also run by the tile queue of the round loop.
// RO: poses are read-only for the whole launch (read-only cache path); false inside the round-loop
// tile queue, which writes them in the same launch.
template <bool STAMPS, bool ARM, bool RO = true>
__device__ __forceinline__ void dualAt(const Dev &d, const StepParams &p, real decay, int m) {
    const ManifoldBuf L = d.live;
    const int2 ab = __ldg(&L.ab[m]);
    const PairFlags flags = loadPairFlags<STAMPS>(d, ab);
    if (!flags.awakeA && !flags.awakeB)
        return; // frozen (manifold.cpp:168-172)
    int sides = flags.sides;
    if (flags.touches)
        sides = 0; // recomputed after the colour passes
    const Pose A = RO ? loadPoseRO(d, ab.x) : loadPose(d, ab.x), B = RO ? loadPoseRO(d, ab.y) : loadPose(d, ab.y);
    const real4 b04 = __ldg(&L.b0[m]);
    const f3 r0 = xyz(b04), r1 = xyz(__ldg(&L.b1[m])), r2 = xyz(__ldg(&L.b2[m]));
    const real mu = b04.w;
    const int n = __ldg(&L.count[m]);
    // Drift-gated arm reuse (manifold.cpp:600-608): under the rotation threshold the cached
    // world arms stand in for the current ones.
    bool driftUsable = false;
    if (ARM) {
        const f3 dA = sub(A.rot.c0, xyz(L.capA[m])), dB = sub(B.rot.c0, xyz(L.capB[m]));
        driftUsable = L.armFlag[m] != 0 && length2(dA) <= p.armRebuild2 && length2(dB) <= p.armRebuild2;
    }
    SharedAcc sh;
    sh.lin = symZero();
    sh.rhsLin = f3{0, 0, 0};
    SideAcc sa, sb;
    zeroAcc(sa);
    zeroAcc(sb);
    // The later contacts' inputs are requested now; the loop below reads them in order.
    for (int c = 1; c < n; c++) {
        const int ci = cslot(d, m, c);
        prefetchL1(&L.rA[ci]);
        prefetchL1(&L.rB[ci]);
        prefetchL1(&L.C0[ci]);
        prefetchL1(&L.k[ci]);
        prefetchL1(&L.lam[ci]);
    }
    for (int c = 0; c < n; c++) {
        const int ci = cslot(d, m, c);
        const real4 rA4 = __ldg(&L.rA[ci]);
        f3 rAw, rBw;
        if (driftUsable) {
            rAw = xyz(L.armA[ci]);
            rBw = xyz(L.armB[ci]);
        } else {
            rAw = mul(A.rot, xyz(rA4));
            rBw = mul(B.rot, xyz(__ldg(&L.rB[ci])));
            if (ARM) {
                L.armA[ci] = f4(rAw, 0.0f);
                L.armB[ci] = f4(rBw, 0.0f);
            }
        }
        const f3 bracket = sub(add(sub(A.dLin, B.dLin), cross(A.dAng, rAw)), cross(B.dAng, rBw));
        const f3 C = contactError(p, xyz(__ldg(&L.C0[ci])), bracket, r0, r1, r2);
        f3 k = xyz(L.k[ci]);
        if (decay < 1.0f)
            k = lclampv(scale(k, decay), PENALTY_MIN, PENALTY_MAX);
        const real4 lam4 = L.lam[ci];
        real stick = lam4.w;
        f3 F = add(cmul(k, C), xyz(lam4));
        const Cone cone = clampForce(F, mu);
        const f3 lam = F;
        const real beta = p.betaLin * rA4.w;
        if (F.x < 0)
            k.x = smin(k.x + beta * mabs(C.x), PENALTY_MAX);
        if (cone.scale <= cone.bounds) {
            k.y = smin(k.y + beta * mabs(C.y), PENALTY_MAX);
            k.z = smin(k.z + beta * mabs(C.z), PENALTY_MAX);
            stick = length2d(C.y, C.z) < STICK_THRESH ? 1.0f : 0.0f;
        }
        L.k[ci] = f4(k, 0.0f);
        L.lam[ci] = f4(lam, stick);
        if (STAMPS && sides) {
            // These are the next round's overflow phase A (solver_step.cpp:236-248): it always
            // precomputes with fresh arms at this pose and stores them, whatever the dual used.
            f3 rAs = rAw, rBs = rBw, Cs = C;
            if (ARM) {
                if (driftUsable) {
                    rAs = mul(A.rot, xyz(rA4));
                    rBs = mul(B.rot, xyz(L.rB[ci]));
                    const f3 bracketF = sub(add(sub(A.dLin, B.dLin), cross(A.dAng, rAs)), cross(B.dAng, rBs));
                    Cs = contactError(p, xyz(L.C0[ci]), bracketF, r0, r1, r2);
                }
                L.armA[ci] = f4(rAs, 0.0f);
                L.armB[ci] = f4(rBs, 0.0f);
            }
            f3 Fn = add(cmul(k, Cs), lam);
            clampForce(Fn, mu);
            real S[6];
            basisHessianD(r0, r1, r2, k, S);
            const f3 fw = add(add(scale(r0, Fn.x), scale(r1, Fn.y)), scale(r2, Fn.z));
            stampShared(S, fw, sh);
            if (sides & kSideA)
                stampContact(S, rAs, fw, sa);
            if (sides & kSideB)
                stampContact(S, rBs, fw, sb);
        }
    }
    if (sides) {
        const int2 slot = d.stampSlot[m];
        if (sides & kSideA)
            storeStamp(d.stamps + static_cast<size_t>(slot.x) * kStampF4, sh, sa, 1.0f);
        if (sides & kSideB)
            storeStamp(d.stamps + static_cast<size_t>(slot.y) * kStampF4, sh, sb, -1.0f);
    }
    if (ARM && !driftUsable) { // capture (manifold.cpp:662-667)
        L.capA[m] = f4(A.rot.c0, 0.0f);
        L.capB[m] = f4(B.rot.c0, 0.0f);
        L.armFlag[m] = 1;
    }
}

template <bool STAMPS, bool ARM>
__global__ void __launch_bounds__(512) dualKernel(Dev d, StepParams p, real decay) { pdlWait(); pdlTrigger(); // 512: largest tuned block
    const int live = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < live; m += gridDim.x * blockDim.x)
        dualAt<STAMPS, ARM>(d, p, decay, m);
}

// ---- joints (joint.cpp:80-230) ----

__device__ __forceinline__ f3 jointLin(const Dev &d, int f) {
    const int2 ab = d.fAB[f];
    const f3 rA = xyz(d.fRA[f]), rB = xyz(d.fRB[f]);
    const f3 pa = ab.x >= 0 ? add(xyz(d.x[ab.x]), qrot(asq(d.q[ab.x]), rA)) : rA;
    return sub(pa, add(xyz(d.x[ab.y]), qrot(asq(d.q[ab.y]), rB)));
}

__device__ __forceinline__ f3 jointAng(const Dev &d, int f) {
    const int2 ab = d.fAB[f];
    const q4 qa = ab.x >= 0 ? asq(d.q[ab.x]) : q4{0.0f, 0.0f, 0.0f, 1.0f};
    return scale(qdiff(qa, asq(d.q[ab.y])), d.fPar[f].w);
}

__device__ __forceinline__ m3 geometricStiffness(int k, f3 v) {
    const real vk = at(v, k);
    m3 m = mdiag(-vk, -vk, -vk);
    f3 ck = col(m, k);
    ck = f3{ck.x + v.x, ck.y + v.y, ck.z + v.z};
    if (k == 0)
        m.c0 = ck;
    else if (k == 1)
        m.c1 = ck;
    else
        m.c2 = ck;
    return m;
}

__device__ void ballStamp(const Dev &d, const StepParams &p, int f, int body, Blk &blk) {
    const int2 ab = d.fAB[f];
    const bool isA = body == ab.x;
    const real4 par = d.fPar[f];
    const f3 kl = xyz(d.fKL[f]);
    if (length2(kl) > 0) {
        const m3 K = mdiag(kl.x, kl.y, kl.z);
        f3 C = jointLin(d, f);
        if (isinf(par.x))
            C = sub(C, scale(xyz(d.fC0L[f]), p.alpha));
        const f3 F = add(mul(K, C), xyz(d.fLL[f]));
        const m3 I = mdiag(1, 1, 1);
        const m3 jLin = isA ? I : mneg(I);
        f3 r;
        if (isA)
            r = neg(qrot(asq(d.q[ab.x]), xyz(d.fRA[f])));
        else
            r = qrot(asq(d.q[ab.y]), xyz(d.fRB[f]));
        const m3 jAng = mcols(f3{0, r.z, -r.y}, f3{-r.z, 0, r.x}, f3{r.y, -r.x, 0});
        const m3 jLinT = transpose(jLin);
        const m3 jAngT = transpose(jAng);
        const m3 jAngTk = mul(jAngT, K);
        blk.lin = madd(blk.lin, mul(mul(jLinT, K), jLin));
        blk.ang = madd(blk.ang, mul(jAngTk, jAng));
        blk.crs = madd(blk.crs, mul(jAngTk, jLin));
        const f3 rr = isA ? qrot(asq(d.q[ab.x]), xyz(d.fRA[f])) : neg(qrot(asq(d.q[ab.y]), xyz(d.fRB[f])));
        const m3 H = madd(madd(mscale(geometricStiffness(0, rr), F.x), mscale(geometricStiffness(1, rr), F.y)),
                          mscale(geometricStiffness(2, rr), F.z));
        blk.ang = madd(blk.ang, mdiag(H.c0.x, H.c1.y, H.c2.z));
        blk.rl = add(blk.rl, mul(jLinT, F));
        blk.ra = add(blk.ra, mul(jAngT, F));
    }
    const f3 ka = xyz(d.fKA[f]);
    if (length2(ka) > 0) {
        const m3 K = mdiag(ka.x, ka.y, ka.z);
        f3 C = jointAng(d, f);
        if (isinf(par.y))
            C = sub(C, scale(xyz(d.fC0A[f]), p.alpha));
        const f3 F = add(mul(K, C), xyz(d.fLA[f]));
        const m3 base = isA ? mdiag(1, 1, 1) : mcols(f3{0, 0, 0}, f3{0, -1, 0}, f3{0, 0, -1});
        const m3 jAng = mscale(base, par.w);
        blk.ang = madd(blk.ang, mul(mul(transpose(jAng), K), jAng));
        blk.ra = add(blk.ra, mul(transpose(jAng), F));
    }
}

// A non-manifold force's stamp into body `body`'s block (Force::updatePrimal by kind).
// Not inlined: forces are rare next to manifolds, and inlining all kinds would raise the
// register count of every body pass.
__device__ __noinline__ void jointStamp(const Dev &d, const StepParams &p, int f, int body, Blk &blk) {
    const int kind = d.fKind[f];
    if (kind == kForceBall)
        ballStamp(d, p, f, body, blk);
    else if (kind == kForceSpring)
        springStamp(d, f, body, blk);
    else if (kind == kForceGeneric)
        genericStamp(d, p, f, body, blk);
}

__global__ void forceDualKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.ctr[C_FORCES])
        return;
    if (d.fKind[f] == kForceGeneric) {
        genericDual(d, p, f);
        return;
    }
    if (d.fKind[f] != kForceBall)
        return;
    const real4 par = d.fPar[f];
    f3 kl = xyz(d.fKL[f]), ka = xyz(d.fKA[f]);
    f3 ll = xyz(d.fLL[f]), la = xyz(d.fLA[f]);
    if (length2(kl) > 0) {
        const m3 K = mdiag(kl.x, kl.y, kl.z);
        f3 C = jointLin(d, f);
        if (isinf(par.x)) {
            C = sub(C, scale(xyz(d.fC0L[f]), p.alpha));
            ll = add(mul(K, C), ll);
        }
        const f3 cap = lminv(f3{par.x, par.x, par.x}, f3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
        kl = lminv(add(kl, scale(vabs(C), p.betaLin)), cap);
    }
    if (length2(ka) > 0) {
        const m3 K = mdiag(ka.x, ka.y, ka.z);
        f3 C = jointAng(d, f);
        if (isinf(par.y)) {
            C = sub(C, scale(xyz(d.fC0A[f]), p.alpha));
            la = add(mul(K, C), la);
        }
        const f3 cap = lminv(f3{par.y, par.y, par.y}, f3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
        ka = lminv(add(ka, scale(vabs(C), p.betaAng)), cap);
    }
    if (length2(la) > par.z * par.z) {
        kl = ka = ll = la = f3{0, 0, 0};
        d.fBroken[f] = 1;
    }
    d.fKL[f] = f4(kl, 0.0f);
    d.fKA[f] = f4(ka, 0.0f);
    d.fLL[f] = f4(ll, 0.0f);
    d.fLA[f] = f4(la, 0.0f);
}

// ---- per-body passes ----

__device__ __forceinline__ int nForcesDev(const Dev &d) { return d.ctr[C_FORCES]; }

// Body g has a force (joint or spring) among its adjacency entries; forces come first in a body's
// entries, so its first entry decides.
__device__ __forceinline__ bool bodyHasForce(const Dev &d, int g, int nf) {
    const int e0 = d.adjStart[g];
    return nf > 0 && e0 < d.adjStart[g + 1] && static_cast<int>(d.adjSeq[e0]) < nf;
}

// One side of manifold m recomputed for coloured body g from the current poses (the same floats
// as stampsKernel for that side, with the arms the colour pass may reuse), as a stamp record. The
// record's adds (addStamp) are the ones of summing the side's accumulators into the block: its
// symmetric blocks are summed entry by entry in the same order on both sides of the diagonal, so
// their unique entries carry every value, and its right-hand sides are stored already signed.
__device__ __forceinline__ StampRec recomputeSide(const Dev &d, const StepParams &p, int g, int m, int side,
                                                  int armsFromDual) {
    const ManifoldBuf L = d.live;
    const int2 ab = L.ab[m];
    const Pose A = loadPose(d, ab.x), B = loadPose(d, ab.y);
    const real4 b04 = L.b0[m];
    const f3 r0 = xyz(b04), r1 = xyz(L.b1[m]), r2 = xyz(L.b2[m]);
    const int n = L.count[m];
    bool cached = false;
    if (p.armCache && armsFromDual) {
        const int o = side == 0 ? ab.y : ab.x;
        cached = !(inUpdate(d, o) && d.colour[o] < d.colour[g]);
    }
    SharedAcc sh;
    sh.lin = symZero();
    sh.rhsLin = f3{0, 0, 0};
    SideAcc sd;
    zeroAcc(sd);
    for (int c = 0; c < n; c++) {
        const int ci = cslot(d, m, c);
        f3 rAw, rBw;
        if (cached) {
            rAw = xyz(L.armA[ci]);
            rBw = xyz(L.armB[ci]);
        } else {
            rAw = mul(A.rot, xyz(L.rA[ci]));
            rBw = mul(B.rot, xyz(L.rB[ci]));
            if (p.armCache) {
                L.armA[ci] = f4(rAw, 0.0f);
                L.armB[ci] = f4(rBw, 0.0f);
            }
        }
        const f3 bracket = sub(add(sub(A.dLin, B.dLin), cross(A.dAng, rAw)), cross(B.dAng, rBw));
        const f3 C = contactError(p, xyz(L.C0[ci]), bracket, r0, r1, r2);
        const f3 k = xyz(L.k[ci]);
        f3 F = add(cmul(k, C), xyz(L.lam[ci]));
        clampForce(F, b04.w);
        real S[6];
        basisHessianD(r0, r1, r2, k, S);
        const f3 fw = add(add(scale(r0, F.x), scale(r1, F.y)), scale(r2, F.z));
        stampShared(S, fw, sh);
        stampContact(S, side == 0 ? rAw : rBw, fw, sd);
    }
    real4 rec[kStampF4];
    storeStamp(rec, sh, sd, side == 0 ? 1.0f : -1.0f);
    return StampRec{rec[0], rec[1], rec[2], rec[3], rec[4], rec[5], rec[6]};
}

// Assemble body g's block from its adjacency; manifold terms from stamps (Jacobi) or recomputed
// from the current poses (Gauss-Seidel).
// Without FORCES (a store with no non-manifold force) the force branch is compiled out, so the
// body passes keep their registers in registers.
// With RECOMPUTE (coloured Gauss-Seidel, ManifoldStore::updatePrimal, manifold.cpp:572-581) and the
// arm cache on, the first touch of a manifold after a dual pass (`armsFromDual`: rounds after the
// first) consumes that dual's cache, so it uses the cached world arms; the other touches precompute
// with fresh arms and store them. The first touch is the body whose partner has not been solved
// this round (not coloured, or coloured later).
// RO: the stamps are read-only for the whole launch (read-only cache path); false inside the
// round-loop tile queue, which writes them in the same launch.
template <bool RECOMPUTE, bool FORCES = true, bool RO = true>
__device__ __forceinline__ void assemble(const Dev &d, const StepParams &p, int g, Blk &blk, int armsFromDual = 0) {
    const int nf = nForcesDev(d);
    const int e1 = d.adjStart[g + 1];
    if (!RECOMPUTE && !bodyHasForce(d, g, nf)) {
        // Every entry is a manifold stamped for this body, stored at the entry itself; two records
        // are loaded before either is added (the sums keep the entry order), and the records after
        // the first pair are requested before any of them.
        int e = d.adjStart[g];
        for (int f = e + 2; f < e1; f++) {
            prefetchL1(d.stamps + static_cast<size_t>(f) * kStampF4);
            prefetchL1(d.stamps + static_cast<size_t>(f) * kStampF4 + kStampF4 - 1);
        }
        for (; e + 1 < e1; e += 2) {
            const StampRec r0 = loadStampAs<RO>(d.stamps + static_cast<size_t>(e) * kStampF4);
            const StampRec r1 = loadStampAs<RO>(d.stamps + static_cast<size_t>(e + 1) * kStampF4);
            addStamp(blk, r0);
            addStamp(blk, r1);
        }
        if (e < e1)
            addStamp(blk, loadStampAs<RO>(d.stamps + static_cast<size_t>(e) * kStampF4));
        return;
    }
    for (int e = d.adjStart[g]; e < e1; e++) {
        const int seq = static_cast<int>(d.adjSeq[e]);
        if (seq < nf) {
            if (FORCES)
                jointStamp(d, p, nf - 1 - seq, g, blk);
            continue;
        }
        const int m = seq - nf;
        const int side = adjInfoSide(__ldg(&d.adjInfo[e]));
        if (RECOMPUTE) {
            addStamp(blk, recomputeSide(d, p, g, m, side, armsFromDual));
        } else {
            addStamp(blk, loadStampAs<RO>(d.stamps + static_cast<size_t>(e) * kStampF4));
        }
    }
}

__device__ __forceinline__ Blk bodyBlock(const Dev &d, const StepParams &p, int g) {
    const real4 x4 = d.x[g];
    return makeBlock(x4.w, xyz(d.moment[g]), p.dtSq, xyz(x4), xyz(d.xi[g]), asq(d.q[g]), asq(d.qi[g]));
}

// One coloured body's Gauss-Seidel update (solver_step.cpp:209-229).
__device__ __forceinline__ void colourPassAt(const Dev &d, const StepParams &p, int colour, int k, int armsFromDual) {
    const int g = d.colourList[colour * d.NB + k];
    Blk blk = bodyBlock(d, p, g);
    assemble<true>(d, p, g, blk, armsFromDual);
    f3 dl, da;
    solveBlock(blk, dl, da);
    const real4 x4 = d.x[g];
    d.x[g] = f4(add(xyz(x4), dl), x4.w);
    d.q[g] = f4(qintegrate(asq(d.q[g]), da));
}

// One round's colour passes in one cooperative launch: colours in order, each a grid-stride loop
// over its list, a grid barrier after each but the last non-empty one. Every block reads the same
// counts (nothing writes them during the sweep), so all blocks skip the same empty colours.
__global__ void __launch_bounds__(kSolveThreads) colourSweepKernel(Dev d, StepParams p, int armsFromDual) {
    pdlWait();
    pdlTrigger();
    int last = -1;
    for (int c = 0; c < kMaxColours; c++)
        if (d.colourCount[c] > 0)
            last = c;
    const int stride = gridDim.x * blockDim.x;
    for (int c = 0; c <= last; c++) {
        const int cnt = d.colourCount[c];
        if (cnt == 0)
            continue;
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride)
            colourPassAt(d, p, c, k, armsFromDual);
        if (c < last && !gridSync(d))
            return;
    }
}

// An overflow body's step: in place, or (a body with a force, in a store with forces) into
// dLin/dAng for overflowApplyKernel.
__device__ __forceinline__ void applyOverflow(const Dev &d, const StepParams &p, int g, int inPlace, f3 dl, f3 da) {
    if (inPlace) {
        const real4 x4 = d.x[g];
        d.x[g] = f4(add(xyz(x4), scale(dl, p.jacobiRelax)), x4.w);
        d.q[g] = f4(qintegrate(asq(d.q[g]), scale(da, p.jacobiRelax)));
    } else {
        d.dLin[g] = f4(dl, 0.0f);
        d.dAng[g] = f4(da, 0.0f);
    }
}

// solve()'s pivoted fallback for a body whose plain LDLT failed, out of line so the common path
// keeps its registers; the kernel's parameters are grid constants, so the call passes their
// addresses without copying them. The block is assembled again (the same floats: it reads the
// stamps, this body's own pose, which it has not written yet, and for a body with a force its
// partners' poses, which defer their updates to the apply pass).
template <bool FORCES, bool RO = true>
__device__ __noinline__ void fallbackSolve(const Dev &d, const StepParams &p, int g, int inPlace) {
    Blk blk = bodyBlock(d, p, g);
    assemble<false, FORCES, RO>(d, p, g, blk);
    const Delta r = solvePivoted(blk);
    applyOverflow(d, p, g, inPlace, r.ok ? r.dl : f3{0, 0, 0}, r.ok ? r.da : f3{0, 0, 0});
}

// One overflow body's block-Jacobi solve (the body of overflowSolveKernel), also run by the
// round-loop tile queue (RO false there: the stamps are written in the same launch).
// inPlace 0 (a store with forces): a body with a force of its own leaves its update to the apply
// pass, because its force terms read its partners' poses, which must stay at the round's start
// (every partner has the same force, so it defers too); any other body reads only its own pose and
// its stamps, so it updates in place with the same floats.
template <bool FORCES, bool RO = true>
__device__ __forceinline__ void solveAt(const Dev &d, const StepParams &p, int g, int inPlace) {
    // The three checks' loads go out together (non-short-circuit: all three are valid reads).
    const int world = d.meta[g].x;
    const bool updated = d.upd[g] != 0;
    const uint8_t colour = d.colour[g];
    if ((world < 0) | !updated | (colour != kOverflowColour))
        return;
    if (!inPlace && !bodyHasForce(d, g, nForcesDev(d)))
        inPlace = 1;
    Blk blk = bodyBlock(d, p, g);
    assemble<false, FORCES, RO>(d, p, g, blk);
    f3 dl, da;
    if (!solveBlockFast(blk, dl, da)) {
        fallbackSolve<FORCES, RO>(d, p, g, inPlace);
        return;
    }
    applyOverflow(d, p, g, inPlace, dl, da);
}

#ifdef AVBDG_FP64
#define AVBDG_SOLVE_BOUNDS __launch_bounds__(kSolveThreads)
#else
#define AVBDG_SOLVE_BOUNDS __launch_bounds__(kSolveThreads, 8) // 64 registers: 8 blocks an SM
#endif
// Overflow bodies are walked in slot order (coalesced body loads); the overflow colour has no list.
template <bool FORCES>
__global__ void AVBDG_SOLVE_BOUNDS
        overflowSolveKernel(const __grid_constant__ Dev d, const __grid_constant__ StepParams p, int inPlace) {
    pdlWait();
    pdlTrigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < d.ctr[C_BODIES])
        solveAt<FORCES>(d, p, g, inPlace);
}

// ---- the round loop as one persistent launch over a tile queue ----
//
// In a store without forces or coloured bodies, round r's body solve in world w needs only the
// stamps round r-1's dual wrote for w, and round r's dual needs only that round's solves in w;
// worlds never read each other. One launch runs all the rounds: tiles (round, phase, world, chunk)
// are handed out in that order by one counter, a tile waits (bounded by waitLimit) until its world
// has completed the previous phase, runs one item per thread and counts itself done; the last
// chunk of a phase advances the world's stage. Every tile a tile waits for was handed out earlier
// to a block that is running (cooperative launch), so the waits end. Worlds move through their
// rounds independently instead of every world waiting at each kernel boundary. The per-item work
// is the separate kernels' (solveAt, dualAt, with coherent loads), so the results are the same.
__device__ __forceinline__ int worldOfTile(const int *pre, int nWorlds, int t) {
    int lo = 0, hi = nWorlds - 1; // the largest w with pre[w] <= t (every world has a chunk)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <bool ARM>
__global__ void __launch_bounds__(kQueueThreads, 4) roundQueueKernel(Dev d, StepParams p, QueueRounds qr) {
    pdlWait();
    pdlTrigger();
    __shared__ int sTile, sOk;
    const int nWorlds = d.ctr[C_WORLDS];
    const int ts = d.ctr[C_QSOLVE], td = d.ctr[C_QDUAL];
    const int perRound = ts + td;
    const int total = qr.rounds * perRound;
    const int *sPre = d.qPre, *dPre = d.qPre + (d.WW + 1);
    volatile int *errors = d.ctr + C_ERRORS;
    for (;;) {
        if (threadIdx.x == 0)
            sTile = static_cast<int>(atomicAdd(d.qTicket, 1u));
        __syncthreads();
        const int t = sTile;
        __syncthreads();
        if (t >= total)
            return;
        const int r = t / perRound;
        int u = t - r * perRound;
        const bool solve = u < ts;
        if (!solve)
            u -= ts;
        const int *pre = solve ? sPre : dPre;
        const int w = worldOfTile(pre, nWorlds, u);
        const int chunk = u - pre[w];
        const int q = 2 * r + (solve ? 0 : 1); // phases of world w completed before this tile may run
        if (threadIdx.x == 0) {
            sOk = 1;
            long long spins = 0;
            while (static_cast<int>(ldAcquireU32(reinterpret_cast<const unsigned *>(d.qStage + w))) < q) {
                if (++spins > d.waitLimit || (*errors & kErrQueueTimeout)) {
                    atomicOr(d.ctr + C_ERRORS, kErrQueueTimeout);
                    sOk = 0;
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
        }
        __syncthreads();
        if (!sOk)
            return;
        if (solve) {
            const int g = d.wBase[w] + chunk * kQueueThreads + threadIdx.x;
            if (((qr.newtonMask >> r) & 1u) && g < d.wBase[w] + d.wCount[w])
                solveAt<false, false>(d, p, g, 1);
        } else {
            const int k = d.wManStart[w] + chunk * kQueueThreads + threadIdx.x;
            if (k < d.wManStart[w + 1]) {
                const int m = d.wManList[k];
                if ((qr.stampMask >> r) & 1u)
                    dualAt<true, ARM, false>(d, p, qr.decay[r], m);
                else
                    dualAt<false, ARM, false>(d, p, qr.decay[r], m);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence(); // the tile's writes before its count
            if (atomicAdd(d.qDone + w, 1) + 1 == pre[w + 1] - pre[w]) {
                d.qDone[w] = 0;
                __threadfence();
                stReleaseU32(reinterpret_cast<unsigned *>(d.qStage + w), static_cast<unsigned>(q + 1));
            }
        }
    }
}

// Each live manifold into its world's group (the order inside a group does not matter: every
// manifold's dual reads and writes only its own state and its bodies' stamp entries).
__global__ void worldManCountKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x)
        atomicAdd(&d.wManStart[d.meta[d.live.ab[m].x].x], 1);
}

__global__ void worldManFillKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_LIVE];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        const int w = d.meta[d.live.ab[m].x].x;
        d.wManList[d.wManStart[w] + atomicAdd(&d.wManFill[w], 1)] = m;
    }
}

// Chunks of each world's solve and dual phases (at least one each, so every phase of every world
// has a tile that advances its stage), zero past the last world; the stages start at zero.
__global__ void queueChunksKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int nWorlds = d.ctr[C_WORLDS];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w > d.WW)
        return;
    int cs = 0, cd = 0;
    if (w < nWorlds) {
        cs = divUpDev(d.wCount[w], kQueueThreads);
        cd = divUpDev(d.wManStart[w + 1] - d.wManStart[w], kQueueThreads);
        cs = cs > 0 ? cs : 1;
        cd = cd > 0 ? cd : 1;
        d.qStage[w] = 0;
        d.qDone[w] = 0;
    }
    d.qPre[w] = cs;
    d.qPre[d.WW + 1 + w] = cd;
}

__global__ void overflowApplyKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0 || !inUpdate(d, g) || d.colour[g] != kOverflowColour ||
        !bodyHasForce(d, g, nForcesDev(d)))
        return; // bodies without a force were updated in place by the solve
    const real4 x4 = d.x[g];
    d.x[g] = f4(add(xyz(x4), scale(xyz(d.dLin[g]), p.jacobiRelax)), x4.w);
    d.q[g] = f4(qintegrate(asq(d.q[g]), scale(xyz(d.dAng[g]), p.jacobiRelax)));
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

// Solver::warmstartBody (solver_solve.cpp:109-142).
__global__ void warmstartKernel(Dev d, StepParams p) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0)
        return;
    const int locks = d.meta[g].w;
    const int lockLin = locks & 0xff, lockAng = (locks >> 8) & 0xff;
    const real4 x4 = d.x[g];
    const real4 v4 = d.v[g];
    const real mass = x4.w;
    f3 v = xyz(v4), w = xyz(d.w[g]);
    maskLocked(lockLin, v);
    maskLocked(lockAng, w);
    const real dt = p.dt;
    const real gr = (lockLin & 0x4) ? 0.0f : v4.w;
    const f3 x = xyz(x4);
    const q4 q = asq(d.q[g]);
    f3 xi = add(x, scale(v, dt));
    if (mass > 0)
        xi = add(xi, scale(f3{0, 0, gr}, dt * dt));
    const q4 qi = qintegrate(q, scale(w, dt));
    const f3 accel = divs(sub(v, xyz(d.vprev[g])), dt);
    const real accelExt = accel.z * mcopysign(1.0f, gr);
    real weight = sclamp(accelExt / mabs(gr), 0.0f, 1.0f);
    if (!isfinite(weight))
        weight = 0.0f;
    d.xi[g] = f4(xi, 0.0f);
    d.qi[g] = f4(qi);
    d.x0[g] = f4(x, 0.0f);
    d.q0[g] = f4(q);
    d.v[g] = f4(v, v4.w);
    d.w[g] = f4(w, 0.0f);
    if (mass > 0) {
        d.x[g] = f4(add(add(x, scale(v, dt)), scale(f3{0, 0, gr}, weight * dt * dt)), mass);
        d.q[g] = f4(qintegrate(q, scale(w, dt)));
    }
}

// Solver::finishBody (solver_solve.cpp:146-176), idle sleep disabled.
__global__ void finishKernel(Dev d, StepParams p, int idle) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0)
        return;
    const int locks = d.meta[g].w;
    const real4 x4 = d.x[g];
    const real4 v4 = d.v[g];
    d.vprev[g] = f4(xyz(v4), 0.0f);
    f3 v = xyz(v4), w = xyz(d.w[g]);
    const int2 s = d.sleep[g];
    if (x4.w > 0 && !s.x) {
        v = divs(sub(xyz(x4), xyz(d.x0[g])), p.dt);
        w = divs(qdiff(asq(d.q[g]), asq(d.q0[g])), p.dt);
    }
    maskLocked(locks & 0xff, v);
    maskLocked((locks >> 8) & 0xff, w);
    // Idle detection on the tick's last substep (sleep mode 1 only).
    if (idle && p.sleepFrames > 0 && x4.w > 0 && !s.x && ((locks >> 16) & 0x3) == 1) {
        const int still = (length2(v) < p.sleepLin2 && length2(w) < p.sleepAng2) ? s.y + 1 : 0;
        if (still >= p.sleepFrames) {
            d.sleep[g] = make_int2(1, still);
            v = f3{0, 0, 0};
            w = f3{0, 0, 0};
        } else {
            d.sleep[g] = make_int2(0, still);
        }
    }
    d.v[g] = f4(v, v4.w);
    d.w[g] = f4(w, 0.0f);
}

// ---- update set and colouring (solver_solve.cpp:263-424) ----

__global__ void contactOnlyInitKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n)
        return;
    d.contactOnly[g] = 1;
    // The update set (solver_solve.cpp:296-339): movable bodies, minus idle sleepers (mode 1) and
    // untouched, motionless bodies that start asleep (mode 2); a mode-2 sleeper otherwise wakes.
    const bool dyn = d.meta[g].x >= 0 && d.x[g].w > 0.0f;
    bool update = dyn;
    if (dyn) {
        const int mode = (d.meta[g].w >> 16) & 0x3;
        const int2 s = d.sleep[g];
        if (mode == 1) {
            update = s.x == 0;
        } else if (mode == 2) {
            if (!s.x && length2(xyz(d.v[g])) == 0.0f && d.adjStart[g] == d.adjStart[g + 1])
                update = false;
            else if (s.x)
                d.sleep[g] = make_int2(0, s.y);
        }
    }
    d.upd[g] = update ? 1 : 0;
    d.colour[g] = update ? kUncoloured : (dyn ? kNotUpdated : kOverflowColour);
}

__global__ void contactOnlyMarkKernel(Dev d) {
    pdlWait();
    pdlTrigger();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.ctr[C_FORCES])
        return;
    const int2 ab = d.fAB[f];
    if (ab.x >= 0)
        d.contactOnly[ab.x] = 0;
    if (ab.y >= 0)
        d.contactOnly[ab.y] = 0;
    d.wColour[d.meta[ab.y].x] = 1;
}

// One Jones-Plassmann attempt with list-order priority: a body is coloured once every earlier
// (lower list position) neighbour in the update set is, with the smallest colour none of them
// uses (the sequential greedy of colourGraph, reproduced exactly). A body still waiting counts
// itself in *waiting.
__device__ __forceinline__ unsigned loadColour(const uint8_t *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u8 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void publishColour(uint8_t *p, unsigned v) {
    asm volatile("st.release.gpu.global.u8 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int kColourThreads = 512;

// Greedy colouring (solver_solve.cpp:365-424) as a dataflow in one cooperative launch: bodies are
// taken in increasing list position; each waits until its earlier dynamic neighbours have
// published their colours, takes the smallest colour none of them has (or the overflow colour)
// and publishes it. That is the sequential greedy assignment; the body with the smallest
// uncoloured list position can always proceed, so the waits end (each is bounded anyway).
// Worlds that no force touches hold only contact-only bodies, which go to the overflow colour
// whatever their greedy colour, so they are not coloured at all (unless every body is coloured).
__global__ void __launch_bounds__(kColourThreads) colourFlowKernel(Dev d, int everyWorld) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int stride = gridDim.x * blockDim.x;
    volatile int *errors = d.ctr + C_ERRORS;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
        const int g = d.lpToBody[p];
        if (g < 0 || d.meta[g].x < 0 || !inUpdate(d, g))
            continue;
        if (!everyWorld && !d.wColour[d.meta[g].x]) {
            publishColour(d.colour + g, kOverflowColour);
            continue;
        }
        unsigned used = 0;
        for (int e = d.adjStart[g]; e < d.adjStart[g + 1]; e++) {
            const int h = adjInfoOther(d.adjInfo[e]);
            if (h < 0 || !inUpdate(d, h) || listPos(d, h) >= p)
                continue;
            unsigned c;
            long long spins = 0;
            while ((c = loadColour(d.colour + h)) == kUncoloured) {
                if (++spins > d.waitLimit || (*errors & kErrColourTimeout)) {
                    atomicOr(d.ctr + C_ERRORS, kErrColourTimeout);
                    return;
                }
                __nanosleep(64);
            }
            if (c < kMaxColours)
                used |= 1u << c;
        }
        unsigned c = kOverflowColour;
        for (int k = 0; k < kMaxColours; k++)
            if (!(used & (1u << k))) {
                c = static_cast<unsigned>(k);
                break;
            }
        publishColour(d.colour + g, c);
    }
}

__global__ void colourListKernel(Dev d, int contactOnlyOverflow) {
    pdlWait();
    pdlTrigger();
    const int n = d.ctr[C_BODIES];
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n || d.meta[g].x < 0 || !inUpdate(d, g))
        return;
    uint8_t c = d.colour[g];
    if (contactOnlyOverflow && d.contactOnly[g])
        c = kOverflowColour;
    if (c > kOverflowColour) // left uncoloured by a colouring that timed out (the step reports it)
        c = kOverflowColour;
    d.colour[g] = c;
    // One atomic per warp and colour (the overflow colour is counted, not listed).
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, static_cast<int>(c));
    const int leader = __ffs(peers) - 1;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader)
        base = atomicAdd(&d.colourCount[c], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (c < kOverflowColour)
        d.colourList[c * d.NB + base + __popc(peers & ((1u << lane) - 1u))] = g;
}

} // namespace

static int grid(int n) { return divUp(n > 0 ? n : 1, kThreads); }
static int queueGridMax();

void launchContactOnly(const Dev &d, cudaStream_t s) {
    cudaMemsetAsync(d.wColour, 0, sizeof(int) * static_cast<size_t>(d.WW), s);
    ++launchCount(); launchK(contactOnlyInitKernel, grid(d.NB), kThreads, 0, s, d);
    ++launchCount(); launchK(contactOnlyMarkKernel, grid(d.FF), kThreads, 0, s, d);
}

static int g_colourBlocks = 0;

int colourGridBlocks() {
    if (g_colourBlocks == 0) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, colourFlowKernel, kColourThreads, 0);
        g_colourBlocks = sms * (perSm < 1 ? 1 : (perSm > 2 ? 2 : perSm));
        if (g_colourBlocks < 1)
            g_colourBlocks = 1;
    }
    return g_colourBlocks;
}

bool dualBlockFits(int block) {
    return blockFits(dualKernel<false, false>, block) && blockFits(dualKernel<true, false>, block) &&
           blockFits(dualKernel<false, true>, block) && blockFits(dualKernel<true, true>, block);
}

bool solveBlockFits(int block) {
    return blockFits(overflowSolveKernel<false>, block) && blockFits(overflowSolveKernel<true>, block);
}

static int g_sweepBlocks = 0;

static int sweepGridMax() {
    if (g_sweepBlocks == 0) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, colourSweepKernel, kSolveThreads, 0);
        g_sweepBlocks = sms * (perSm < 1 ? 1 : perSm);
    }
    return g_sweepBlocks;
}

void prepareKernels() {
    sweepGridMax();
    queueGridMax();
    projectionGridBlocks();
    preparePrimitives();
    prepareNarrowPhase();
    brakeGridBlocks();
    colourGridBlocks();
}

void launchColour(const Dev &d, bool needGreedy, bool everyWorld, cudaStream_t s) {
    if (!needGreedy)
        return;
    // No more blocks than the store's bodies can fill.
    const int want = divUp(d.NB > 0 ? d.NB : 1, kColourThreads), most = colourGridBlocks();
    Dev dd = d;
    int every = everyWorld ? 1 : 0;
    void *args[] = {&dd, &every};
    ++launchCount();
    cudaLaunchCooperativeKernel(reinterpret_cast<void *>(colourFlowKernel), dim3(want < most ? want : most),
                                dim3(kColourThreads), args, 0, s);
}

void launchColourLists(const Dev &d, int contactOnlyOverflow, cudaStream_t s) {
    cudaMemsetAsync(d.colourCount, 0, sizeof(int) * (kMaxColours + 1), s);
    ++launchCount(); launchK(colourListKernel, grid(d.NB), kThreads, 0, s, d, contactOnlyOverflow);
}

void launchWarmstartBodies(const Dev &d, const StepParams &p, cudaStream_t s) {
    ++launchCount(); launchK(warmstartKernel, grid(d.NB), kThreads, 0, s, d, p);
}

void launchFinishBodies(const Dev &d, const StepParams &p, bool idle, cudaStream_t s) {
    ++launchCount(); launchK(finishKernel, grid(d.NB), kThreads, 0, s, d, p, idle ? 1 : 0);
}

void launchStamps(const Dev &d, const StepParams &p, bool mixedOnly, cudaStream_t s) {
    ++launchCount(); launchK(stampsKernel, residentGrid(stampsKernel, kThreads, grid(d.MM)), kThreads, 0, s, d, p, mixedOnly ? 1 : 0);
}

void launchColourSweep(const Dev &d, const StepParams &p, bool armsFromDual, cudaStream_t s) {
    // With contact-only bodies in the overflow colour, a coloured body has a force of its own and a
    // force touches at most two bodies, so the grid (and its barrier) scales with the forces.
    const int bound = p.contactOnlyOverflow && d.FF < d.NB / 2 ? 2 * d.FF : d.NB;
    const int want = divUp(bound > 0 ? bound : 1, kSolveThreads), most = sweepGridMax();
    const int blocks = want < most ? want : most;
    cudaMemsetAsync(d.gridBar, 0, sizeof(unsigned), s);
    Dev dd = d;
    StepParams pp = p;
    int arms = armsFromDual ? 1 : 0;
    void *args[] = {&dd, &pp, &arms};
    ++launchCount();
    cudaLaunchCooperativeKernel(reinterpret_cast<void *>(colourSweepKernel), dim3(blocks), dim3(kSolveThreads),
                                args, 0, s);
}

void launchOverflowSolve(const Dev &d, const StepParams &p, bool inPlace, bool forces, int block, cudaStream_t s) {
    ++launchCount();
    if (forces)
        launchK(overflowSolveKernel<true>, divUp(d.NB, block), block, 0, s, d, p, inPlace ? 1 : 0);
    else
        launchK(overflowSolveKernel<false>, divUp(d.NB, block), block, 0, s, d, p, inPlace ? 1 : 0);
}

static int g_queueBlocks = 0;

static int queueGridMax() {
    if (g_queueBlocks == 0) {
        int dev = 0, sms = 0, perSm = 0, perSmArm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, roundQueueKernel<false>, kQueueThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSmArm, roundQueueKernel<true>, kQueueThreads, 0);
        perSm = perSm < perSmArm ? perSm : perSmArm;
        g_queueBlocks = sms * (perSm < 1 ? 1 : perSm);
    }
    return g_queueBlocks;
}

void launchRoundQueue(const Dev &d, const StepParams &p, const QueueRounds &qr, cudaStream_t s) {
    const int cap = static_cast<int>(static_cast<size_t>(d.WW) + 1);
    cudaMemsetAsync(d.wManStart, 0, sizeof(int) * static_cast<size_t>(cap), s);
    cudaMemsetAsync(d.wManFill, 0, sizeof(int) * static_cast<size_t>(d.WW), s);
    ++launchCount(); launchK(worldManCountKernel, residentGrid(worldManCountKernel, kThreads, grid(d.MM)), kThreads, 0, s, d);
    scanExclusive(d.wManStart, d.wManStart, cap, nullptr, nullptr, d.scanScratch, s);
    ++launchCount(); launchK(worldManFillKernel, residentGrid(worldManFillKernel, kThreads, grid(d.MM)), kThreads, 0, s, d);
    ++launchCount(); launchK(queueChunksKernel, divUp(cap, kThreads), kThreads, 0, s, d);
    scanExclusive(d.qPre, d.qPre, cap, nullptr, d.ctr + C_QSOLVE, d.scanScratch, s);
    scanExclusive(d.qPre + cap, d.qPre + cap, cap, nullptr, d.ctr + C_QDUAL, d.scanScratch, s);
    cudaMemsetAsync(d.qTicket, 0, sizeof(unsigned), s);
    Dev dd = d;
    StepParams pp = p;
    QueueRounds q = qr;
    void *args[] = {&dd, &pp, &q};
    ++launchCount();
    cudaLaunchCooperativeKernel(p.armCache ? reinterpret_cast<void *>(roundQueueKernel<true>)
                                           : reinterpret_cast<void *>(roundQueueKernel<false>),
                                dim3(queueGridMax()), dim3(kQueueThreads), args, 0, s);
}

void launchOverflowApply(const Dev &d, const StepParams &p, cudaStream_t s) {
    ++launchCount();
    launchK(overflowApplyKernel, grid(d.NB), kThreads, 0, s, d, p);
}

template <bool STAMPS, bool ARM>
static void dualLaunch(const Dev &d, const StepParams &p, real decay, int block, cudaStream_t s) {
    const int blocks = residentGrid(dualKernel<STAMPS, ARM>, block, divUp(d.MM, block));
    launchK(dualKernel<STAMPS, ARM>, blocks, block, 0, s, d, p, decay);
}

void launchDual(const Dev &d, const StepParams &p, bool stamps, real decay, int block, cudaStream_t s) {
    ++launchCount();
    if (p.armCache)
        stamps ? dualLaunch<true, true>(d, p, decay, block, s) : dualLaunch<false, true>(d, p, decay, block, s);
    else
        stamps ? dualLaunch<true, false>(d, p, decay, block, s) : dualLaunch<false, false>(d, p, decay, block, s);
}

void launchForceDual(const Dev &d, const StepParams &p, bool forces, cudaStream_t s) {
    if (!forces)
        return;
    ++launchCount(); launchK(forceDualKernel, grid(d.FF), kThreads, 0, s, d, p);
}

} // namespace avbdg
