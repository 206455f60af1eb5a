// Box-box narrow phase with a speculative margin (godot-avbd src/avbd/collide.cpp:27-490,
// 1001-1098): SAT over 15 axes with a 3x3 frame table and an edge bias, Sutherland-Hodgman clip
// of the incident face against the reference face's side planes, up to eight contacts with
// feature keys. One thread per manifold; operation order follows the reference so the contact
// set is bit-identical.
#pragma once

#include <cfloat>

#include "dmath.cuh"

namespace avbdg {

struct NContact {
    int key;
    f3 rA, rB;
};

namespace narrow {

constexpr int kMaxPoly = 16;
constexpr real kSatEps = 1.0e-6f;
constexpr real kPlaneEps = 1.0e-5f;
constexpr real kMergeSq = 1.0e-6f;
enum { kFaceA = 0, kFaceB = 1, kEdge = 2 };

struct Obb {
    f3 c;
    q4 q;
    f3 h;
    f3 ax[3];
};

struct Sat {
    int type, ia, ib;
    real sep;
    f3 nAB;
    bool valid;
};

__device__ __forceinline__ real hv(const f3 &h, int i) { return at(h, i); }

__device__ inline f3 support(const Obb &b, f3 dir) {
    const real sx = dot(dir, b.ax[0]) >= 0.0f ? 1.0f : -1.0f;
    const real sy = dot(dir, b.ax[1]) >= 0.0f ? 1.0f : -1.0f;
    const real sz = dot(dir, b.ax[2]) >= 0.0f ? 1.0f : -1.0f;
    return add(add(add(b.c, scale(b.ax[0], b.h.x * sx)), scale(b.ax[1], b.h.y * sy)), scale(b.ax[2], b.h.z * sz));
}

__device__ inline void faceAxes(const Obb &b, int k, f3 &u, f3 &v, real &eu, real &ev) {
    if (k == 0) {
        u = b.ax[1]; v = b.ax[2]; eu = b.h.y; ev = b.h.z;
    } else if (k == 1) {
        u = b.ax[0]; v = b.ax[2]; eu = b.h.x; ev = b.h.z;
    } else {
        u = b.ax[0]; v = b.ax[1]; eu = b.h.x; ev = b.h.y;
    }
}

__device__ inline int clip(const f3 *in, int inCount, f3 n, real off, f3 *out) {
    if (inCount <= 0)
        return 0;
    int oc = 0;
    f3 a = in[inCount - 1];
    real da = dot(n, a) - off;
    for (int i = 0; i < inCount; ++i) {
        const f3 b = in[i];
        const real db = dot(n, b) - off;
        const bool aIn = da <= kPlaneEps;
        const bool bIn = db <= kPlaneEps;
        if (aIn != bIn) {
            real t = 0.0f;
            const real denom = da - db;
            if (mabs(denom) > kSatEps)
                t = sclamp(da / denom, 0.0f, 1.0f);
            if (oc < kMaxPoly)
                out[oc++] = add(a, scale(sub(b, a), t));
        }
        if (bIn && oc < kMaxPoly)
            out[oc++] = b;
        a = b;
        da = db;
    }
    return oc;
}

struct Sink {
    f3 cA, cB;
    q4 qA, qB;
    NContact *out;
    int n;
    f3 mid[8];

    // addContact (collide.cpp:208-233): false when merged into an earlier contact or full.
    __device__ bool addc(f3 xA, f3 xB, int key) {
        const f3 m = scale(add(xA, xB), 0.5f);
        for (int i = 0; i < n; ++i)
            if (length2(sub(m, mid[i])) < kMergeSq)
                return false;
        if (n >= 8)
            return false;
        out[n].key = key;
        out[n].rA = qrot(qconj(qA), sub(xA, cA));
        out[n].rB = qrot(qconj(qB), sub(xB, cB));
        mid[n] = m;
        ++n;
        return true;
    }
};

__device__ inline bool faceA(const Obb &A, const Obb &B, f3 dA, const m3 &m, int i, real margin, Sat &best) {
    const real sep = mabs(at(dA, i)) -
            (((hv(A.h, i) + B.h.x * mabs(mat(m, 0, i))) + B.h.y * mabs(mat(m, 1, i))) + B.h.z * mabs(mat(m, 2, i)));
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.sep) {
        best.valid = true;
        best.type = kFaceA;
        best.ia = i;
        best.ib = -1;
        best.sep = sep;
        best.nAB = scale(A.ax[i], at(dA, i) < 0.0f ? -1.0f : 1.0f);
    }
    return true;
}

__device__ inline bool faceB(const Obb &A, const Obb &B, f3 dB, const m3 &m, int j, real margin, Sat &best) {
    const real sep = mabs(at(dB, j)) -
            (((hv(B.h, j) + A.h.x * mabs(mat(m, j, 0))) + A.h.y * mabs(mat(m, j, 1))) + A.h.z * mabs(mat(m, j, 2)));
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.sep) {
        best.valid = true;
        best.type = kFaceB;
        best.ia = -1;
        best.ib = j;
        best.sep = sep;
        best.nAB = scale(B.ax[j], at(dB, j) < 0.0f ? -1.0f : 1.0f);
    }
    return true;
}

__device__ inline bool edge(const Obb &A, const Obb &B, f3 delta, f3 axis, const m3 &m, int i, int j, real margin,
                            Sat &best) {
    const real lenSq = length2(axis);
    if (lenSq < kSatEps)
        return true;
    const real invLen = 1.0f / msqrt(lenSq);
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    const real rA = (hv(A.h, i1) * mabs(mat(m, j, i2)) + hv(A.h, i2) * mabs(mat(m, j, i1))) * invLen;
    const real rB = (hv(B.h, j1) * mabs(mat(m, j2, i)) + hv(B.h, j2) * mabs(mat(m, j1, i))) * invLen;
    const real sd = dot(delta, axis) * invLen;
    const real sep = mabs(sd) - (rA + rB);
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.sep) {
        best.valid = true;
        best.type = kEdge;
        best.ia = i;
        best.ib = j;
        best.sep = sep;
        best.nAB = scale(axis, sd < 0.0f ? -invLen : invLen);
    }
    return true;
}

__device__ inline void supportEdge(const Obb &b, int k, f3 dir, f3 &e0, f3 &e1) {
    const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
    const real s1 = dot(dir, b.ax[k1]) >= 0.0f ? 1.0f : -1.0f;
    const real s2 = dot(dir, b.ax[k2]) >= 0.0f ? 1.0f : -1.0f;
    const f3 ec = add(add(b.c, scale(b.ax[k1], hv(b.h, k1) * s1)), scale(b.ax[k2], hv(b.h, k2) * s2));
    e0 = sub(ec, scale(b.ax[k], hv(b.h, k)));
    e1 = add(ec, scale(b.ax[k], hv(b.h, k)));
}

__device__ inline void closestSegments(f3 p0, f3 p1, f3 q0, f3 q1, f3 &c0, f3 &c1) {
    const f3 d1 = sub(p1, p0);
    const f3 d2 = sub(q1, q0);
    const f3 r = sub(p0, q0);
    const real a = dot(d1, d1);
    const real e = dot(d2, d2);
    const real f = dot(d2, r);
    real s = 0.0f, t = 0.0f;
    if (a <= kSatEps && e <= kSatEps) {
        c0 = p0;
        c1 = q0;
        return;
    }
    if (a <= kSatEps) {
        t = sclamp(f / e, 0.0f, 1.0f);
    } else {
        const real c = dot(d1, r);
        if (e <= kSatEps) {
            s = sclamp(-c / a, 0.0f, 1.0f);
        } else {
            const real b = dot(d1, d2);
            const real denom = a * e - b * b;
            if (mabs(denom) > kSatEps)
                s = sclamp((b * f - c * e) / denom, 0.0f, 1.0f);
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = sclamp(-c / a, 0.0f, 1.0f);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = sclamp((b - c) / a, 0.0f, 1.0f);
            }
        }
    }
    c0 = add(p0, scale(d1, s));
    c1 = add(q0, scale(d2, t));
}

__device__ inline int faceManifold(const Obb &A, const Obb &B, bool refIsA, int refAxis, f3 nAB, real margin,
                                   NContact *out) {
    const Obb &ref = refIsA ? A : B;
    const Obb &inc = refIsA ? B : A;
    const f3 outward = refIsA ? nAB : neg(nAB);
    const real rs = dot(outward, ref.ax[refAxis]) >= 0.0f ? 1.0f : -1.0f;
    const f3 rn = scale(ref.ax[refAxis], rs);
    const f3 rc = add(ref.c, scale(rn, hv(ref.h, refAxis)));
    f3 ru, rv;
    real reu, rev;
    faceAxes(ref, refAxis, ru, rv, reu, rev);
    int incAxis = 0;
    {
        real best = -FLT_MAX;
        for (int i = 0; i < 3; ++i) {
            const real dd = mabs(dot(inc.ax[i], rn));
            if (dd > best) {
                best = dd;
                incAxis = i;
            }
        }
    }
    f3 c0[kMaxPoly], c1[kMaxPoly];
    {
        const real sg = dot(inc.ax[incAxis], rn) > 0.0f ? -1.0f : 1.0f;
        const f3 fn = scale(inc.ax[incAxis], sg);
        const f3 fc = add(inc.c, scale(fn, hv(inc.h, incAxis)));
        f3 u, v;
        real eu, ev;
        faceAxes(inc, incAxis, u, v, eu, ev);
        c0[0] = add(add(fc, scale(u, eu)), scale(v, ev));
        c0[1] = add(sub(fc, scale(u, eu)), scale(v, ev));
        c0[2] = sub(sub(fc, scale(u, eu)), scale(v, ev));
        c0[3] = sub(add(fc, scale(u, eu)), scale(v, ev));
    }
    int cnt = 4;
    cnt = clip(c0, cnt, ru, dot(ru, rc) + reu, c1);
    if (!cnt)
        return 0;
    const f3 nu = neg(ru);
    cnt = clip(c1, cnt, nu, dot(nu, rc) + reu, c0);
    if (!cnt)
        return 0;
    cnt = clip(c0, cnt, rv, dot(rv, rc) + rev, c1);
    if (!cnt)
        return 0;
    const f3 nv = neg(rv);
    cnt = clip(c1, cnt, nv, dot(nv, rc) + rev, c0);
    if (!cnt)
        return 0;
    Sink sink;
    sink.cA = A.c;
    sink.cB = B.c;
    sink.qA = A.q;
    sink.qB = B.q;
    sink.out = out;
    sink.n = 0;
    int prefix = (refIsA ? kFaceA : kFaceB) << 24;
    prefix |= (refAxis & 0xFF) << 16;
    prefix |= (incAxis & 0xFF) << 8;
    const real accept = smax(margin, kPlaneEps);
    for (int i = 0; i < cnt && sink.n < 8; ++i) {
        const f3 p = c0[i];
        const real dist = dot(sub(p, rc), rn);
        if (dist > accept)
            continue;
        const f3 pr = sub(p, scale(rn, dist));
        sink.addc(refIsA ? pr : p, refIsA ? p : pr, prefix | (i & 0xFF));
    }
    if (!sink.n) {
        const f3 xA = support(A, nAB);
        f3 xB = support(B, neg(nAB));
        xB = sub(xA, scale(nAB, dot(sub(xA, xB), nAB)));
        sink.addc(xA, xB, prefix);
    }
    return sink.n;
}

__device__ inline int edgeContact(const Obb &A, const Obb &B, int axA, int axB, f3 nAB, NContact *out) {
    f3 a0, a1, b0, b1;
    supportEdge(A, axA, nAB, a0, a1);
    supportEdge(B, axB, neg(nAB), b0, b1);
    f3 xA, xB;
    closestSegments(a0, a1, b0, b1, xA, xB);
    Sink sink;
    sink.cA = A.c;
    sink.cB = B.c;
    sink.qA = A.q;
    sink.qB = B.q;
    sink.out = out;
    sink.n = 0;
    const int key = (kEdge << 24) | ((axA & 0xFF) << 8) | (axB & 0xFF);
    sink.addc(xA, xB, key);
    if (!sink.n) {
        xA = support(A, nAB);
        xB = support(B, neg(nAB));
        sink.addc(xA, xB, key);
    }
    return sink.n;
}

__device__ inline Obb makeObb(f3 c, q4 q, f3 h) {
    Obb o;
    o.c = c;
    o.q = q;
    o.h = h;
    o.ax[0] = qrot(q, f3{1.0f, 0.0f, 0.0f});
    o.ax[1] = qrot(q, f3{0.0f, 1.0f, 0.0f});
    o.ax[2] = qrot(q, f3{0.0f, 0.0f, 1.0f});
    return o;
}

} // namespace narrow

// Returns the contact count (0 = separated beyond the margin); `basis` is written only when the
// SAT finds no separating axis, as in the reference.
__device__ inline int collideBoxes(f3 ca, q4 qa, f3 ha, f3 cb, q4 qb, f3 hb, real margin, NContact *out, m3 &basis) {
    using namespace narrow;
    const Obb A = makeObb(ca, qa, ha);
    const Obb B = makeObb(cb, qb, hb);
    const f3 delta = sub(B.c, A.c);
    m3 m;
    // m[j][i] = axisA_i . axisB_j (column j, row i).
    m.c0 = f3{dot(A.ax[0], B.ax[0]), dot(A.ax[1], B.ax[0]), dot(A.ax[2], B.ax[0])};
    m.c1 = f3{dot(A.ax[0], B.ax[1]), dot(A.ax[1], B.ax[1]), dot(A.ax[2], B.ax[1])};
    m.c2 = f3{dot(A.ax[0], B.ax[2]), dot(A.ax[1], B.ax[2]), dot(A.ax[2], B.ax[2])};
    const f3 dA{dot(delta, A.ax[0]), dot(delta, A.ax[1]), dot(delta, A.ax[2])};
    const f3 dB{dot(delta, B.ax[0]), dot(delta, B.ax[1]), dot(delta, B.ax[2])};
    Sat bf{0, -1, -1, -FLT_MAX, f3{0, 0, 0}, false};
    Sat be{0, -1, -1, -FLT_MAX, f3{0, 0, 0}, false};
    for (int i = 0; i < 3; ++i)
        if (!faceA(A, B, dA, m, i, margin, bf))
            return 0;
    for (int j = 0; j < 3; ++j)
        if (!faceB(A, B, dB, m, j, margin, bf))
            return 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (!edge(A, B, delta, cross(A.ax[i], B.ax[j]), m, i, j, margin, be))
                return 0;
    if (!bf.valid)
        return 0;
    Sat best = bf;
    if (be.valid && 0.95f * be.sep > bf.sep + 0.01f)
        best = be;
    basis = orthonormal(neg(best.nAB));
    if (best.type == kEdge)
        return edgeContact(A, B, best.ia, best.ib, best.nAB, out);
    if (best.type == kFaceA)
        return faceManifold(A, B, true, best.ia, best.nAB, margin, out);
    return faceManifold(A, B, false, best.ib, best.nAB, margin, out);
}

} // namespace avbdg
