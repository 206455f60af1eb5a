// Oracle: serial CPU restatement of the reference AVBD step (test infrastructure only).
// Each function names the reference lines it restates; expression order follows them exactly,
// because the parity bar is bit equality (compile with -ffp-contract=off).

#include "avbd_oracle.hpp"

#include <algorithm>
#include <climits>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

namespace {

constexpr float kReleaseAbove = COLLISION_MARGIN + CONTACT_RELEASE_GAP;
constexpr uint8_t kArmsCached = 1;
constexpr uint8_t kPrimalCacheReady = 2;

} // namespace

// ------------------------------------------------------------------------------------------
// 6x6 block and its solvers (src/avbd/types.hpp:147-201, src/avbd/maths.h:156-343)
// ------------------------------------------------------------------------------------------

struct Block {
    M3 lhsLin, lhsAng, lhsCross;
    V3 rhsLin, rhsAng;
};

typedef float Mat6[6][6];

// Unpivoted LDL^T with the sanity test |x| < 10 (maths.h:156-198).
static bool ldlt6(const Mat6 &a, const float b[6], float x[6]) {
    float l[6][6] = {};
    float d[6] = {};
    for (int j = 0; j < 6; j++) {
        float dj = a[j][j];
        for (int s = 0; s < j; s++)
            dj -= l[j][s] * l[j][s] * d[s];
        if (!(dj > 1.0e-12f))
            return false;
        d[j] = dj;
        l[j][j] = 1.0f;
        for (int i = j + 1; i < 6; i++) {
            float lij = a[i][j];
            for (int s = 0; s < j; s++)
                lij -= l[i][s] * l[j][s] * d[s];
            l[i][j] = lij / d[j];
        }
    }
    float z[6] = {};
    for (int i = 0; i < 6; i++) {
        float v = b[i];
        for (int s = 0; s < i; s++)
            v -= l[i][s] * z[s];
        z[i] = v;
    }
    for (int i = 0; i < 6; i++)
        x[i] = z[i] / d[i];
    for (int i = 5; i >= 0; i--) {
        float v = x[i];
        for (int s = i + 1; s < 6; s++)
            v -= l[s][i] * x[s];
        x[i] = v;
    }
    float worst = 0.0f;
    for (int i = 0; i < 6; i++)
        worst = smax(worst, std::fabs(x[i]));
    return std::isfinite(worst) && worst < 1.0e1f;
}

// Pivoted LDL^T (maths.h:202-307): largest-diagonal pivoting, Eigen's reduction pairing.
static bool ldlt6Pivoted(const Mat6 &aIn, const float b[6], float x[6]) {
    float a[6][6];
    std::memcpy(a, aIn, sizeof(a));
    float d[6] = {};
    int t[6] = {0, 1, 2, 3, 4, 5};
    bool foundZeroPivot = false;
    for (int k = 0; k < 6; k++) {
        int j = k;
        float best = std::fabs(a[k][k]);
        for (int i = k + 1; i < 6; i++) {
            const float cand = std::fabs(a[i][i]);
            if (cand > best) {
                best = cand;
                j = i;
            }
        }
        t[k] = j;
        if (j != k) {
            for (int c = 0; c < 6; c++)
                std::swap(a[k][c], a[j][c]);
            for (int r = 0; r < 6; r++)
                std::swap(a[r][k], a[r][j]);
        }
        if (k > 0) {
            float temp[6] = {};
            for (int i = 0; i < k; i++)
                temp[i] = d[i] * a[k][i];
            float prod[6] = {};
            for (int i = 0; i < k; i++)
                prod[i] = a[k][i] * temp[i];
            float dotv;
            switch (k) {
            case 1: dotv = prod[0]; break;
            case 2: dotv = prod[0] + prod[1]; break;
            case 3: dotv = (prod[0] + prod[1]) + prod[2]; break;
            case 4: dotv = (prod[0] + prod[2]) + (prod[1] + prod[3]); break;
            default: dotv = ((prod[0] + prod[2]) + (prod[1] + prod[3])) + prod[4]; break;
            }
            a[k][k] -= dotv;
            for (int i = 0; i < k; i++) {
                const float ti = temp[i];
                for (int r = k + 1; r < 6; r++)
                    a[r][k] -= a[r][i] * ti;
            }
        }
        const float pivot = a[k][k];
        const bool valid = std::fabs(pivot) > 0.0f;
        if (!valid) {
            for (int r = k + 1; r < 6; r++)
                if (a[r][k] != 0.0f)
                    return false;
            foundZeroPivot = true;
        } else if (foundZeroPivot) {
            return false;
        }
        if (valid)
            for (int r = k + 1; r < 6; r++)
                a[r][k] /= pivot;
        d[k] = pivot;
    }
    for (int i = 0; i < 6; i++)
        x[i] = b[i];
    for (int k = 0; k < 6; k++)
        std::swap(x[k], x[t[k]]);
    for (int jj = 0; jj < 5; jj++) {
        const float v = x[jj];
        if (v != 0.0f)
            for (int i = jj + 1; i < 6; i++)
                x[i] -= a[i][jj] * v;
    }
    const float tolerance = std::numeric_limits<float>::min();
    for (int i = 0; i < 6; i++)
        x[i] = std::fabs(d[i]) > tolerance ? x[i] / d[i] : 0.0f;
    for (int jj = 5; jj >= 1; jj--) {
        const float v = x[jj];
        if (v != 0.0f)
            for (int i = jj - 1; i >= 0; i--)
                x[i] -= a[jj][i] * v;
    }
    for (int k = 5; k >= 0; k--)
        std::swap(x[k], x[t[k]]);
    float worst = 0.0f;
    for (int i = 0; i < 6; i++)
        worst = smax(worst, std::fabs(x[i]));
    return std::isfinite(worst) && worst < 1.0e1f;
}

static void assemble(const Block &blk, Mat6 &a) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            a[r][c] = blk.lhsLin.c[c][r];
            a[r + 3][c + 3] = blk.lhsAng.c[c][r];
            a[r + 3][c] = blk.lhsCross.c[c][r];
            a[r][c + 3] = blk.lhsCross.c[r][c];
        }
}

// Block::solveDelta (types.hpp:176-197) and its fallback solve() (maths.h:315-343).
static void solveDelta(const Block &blk, V3 &dLin, V3 &dAng) {
    Mat6 a;
    assemble(blk, a);
    const float b[6] = {-blk.rhsLin.x, -blk.rhsLin.y, -blk.rhsLin.z,
                        -blk.rhsAng.x, -blk.rhsAng.y, -blk.rhsAng.z};
    float x[6] = {};
    if (ldlt6(a, b, x)) {
        dLin = V3{x[0], x[1], x[2]};
        dAng = V3{x[3], x[4], x[5]};
        return;
    }
    // solve(lhsLin, lhsAng, lhsCross, -rhsLin, -rhsAng): same matrix and right-hand side.
    float y[6] = {};
    if (ldlt6(a, b, y) || ldlt6Pivoted(a, b, y)) {
        dLin = V3{y[0], y[1], y[2]};
        dAng = V3{y[3], y[4], y[5]};
        return;
    }
    dLin = V3{0, 0, 0};
    dAng = V3{0, 0, 0};
}

// Block::Block (types.hpp:157-172).
static Block makeBlock(const Body &b, float dtSq) {
    Block blk;
    const V3 mo = V3{b.mass, b.mass, b.mass} / dtSq;
    blk.lhsLin = mdiag(mo.x, mo.y, mo.z);
    blk.lhsCross = mzero();
    blk.rhsLin = cmul(mo, b.x - b.xi);
    const M3 rot = qmat(b.q);
    const M3 inertiaWorld = mul(rot, mul(mdiag(b.moment.x, b.moment.y, b.moment.z), transpose(rot)));
    blk.lhsAng = inertiaWorld / dtSq;
    blk.rhsAng = mul(blk.lhsAng, qdiff(b.q, b.qi));
    return blk;
}

// ------------------------------------------------------------------------------------------
// Box-box narrow phase (src/avbd/collide.cpp:27-490, 1001-1098)
// ------------------------------------------------------------------------------------------

namespace {

constexpr int kMaxPolyVerts = 16;
constexpr float kSatAxisEps = 1.0e-6f;
constexpr float kPlaneEps = 1.0e-5f;
constexpr float kMergeDistSq = 1.0e-6f;
enum { kAxisFaceA = 0, kAxisFaceB = 1, kAxisEdge = 2 };

struct Obb {
    V3 center;
    Q4 rot;
    V3 half;
    V3 axis[3];
};

struct Sat {
    int type = 0, ia = -1, ib = -1;
    float separation = -FLT_MAX;
    V3 normalAB{0, 0, 0};
    bool valid = false;
};

struct Face {
    int axis;
    V3 normal, center, u, v;
    float eu, ev;
};

Obb makeObb(V3 c, Q4 q, V3 h) {
    Obb o;
    o.center = c;
    o.rot = q;
    o.half = h;
    o.axis[0] = qrot(q, V3{1.0f, 0.0f, 0.0f});
    o.axis[1] = qrot(q, V3{0.0f, 1.0f, 0.0f});
    o.axis[2] = qrot(q, V3{0.0f, 0.0f, 1.0f});
    return o;
}

V3 supportPoint(const Obb &b, V3 dir) {
    const float sx = dot(dir, b.axis[0]) >= 0.0f ? 1.0f : -1.0f;
    const float sy = dot(dir, b.axis[1]) >= 0.0f ? 1.0f : -1.0f;
    const float sz = dot(dir, b.axis[2]) >= 0.0f ? 1.0f : -1.0f;
    return ((b.center + b.axis[0] * (b.half.x * sx)) + b.axis[1] * (b.half.y * sy)) +
           b.axis[2] * (b.half.z * sz);
}

void faceAxes(const Obb &b, int k, V3 &u, V3 &v, float &eu, float &ev) {
    if (k == 0) {
        u = b.axis[1]; v = b.axis[2]; eu = b.half.y; ev = b.half.z;
    } else if (k == 1) {
        u = b.axis[0]; v = b.axis[2]; eu = b.half.x; ev = b.half.z;
    } else {
        u = b.axis[0]; v = b.axis[1]; eu = b.half.x; ev = b.half.y;
    }
}

int clipPolygon(const V3 *in, int inCount, V3 n, float offset, V3 *out) {
    if (inCount <= 0)
        return 0;
    int outCount = 0;
    V3 a = in[inCount - 1];
    float da = dot(n, a) - offset;
    for (int i = 0; i < inCount; ++i) {
        const V3 b = in[i];
        const float db = dot(n, b) - offset;
        const bool aIn = da <= kPlaneEps;
        const bool bIn = db <= kPlaneEps;
        if (aIn != bIn) {
            float t = 0.0f;
            const float denom = da - db;
            if (std::fabs(denom) > kSatAxisEps)
                t = sclamp(da / denom, 0.0f, 1.0f);
            if (outCount < kMaxPolyVerts)
                out[outCount++] = a + (b - a) * t;
        }
        if (bIn && outCount < kMaxPolyVerts)
            out[outCount++] = b;
        a = b;
        da = db;
    }
    return outCount;
}

struct ContactSink {
    const Obb &A, &B;
    Contact *out;
    int count = 0;
    V3 mid[kMaxContacts];
    // addContact (collide.cpp:208-233).
    bool add(V3 xA, V3 xB, int key) {
        const V3 m = (xA + xB) * 0.5f;
        for (int i = 0; i < count; ++i) {
            const V3 d = m - mid[i];
            if (length2(d) < kMergeDistSq)
                return false;
        }
        if (count >= kMaxContacts)
            return false;
        Contact &c = out[count];
        c.key = key;
        c.rA = qrot(qconj(A.rot), xA - A.center);
        c.rB = qrot(qconj(B.rot), xB - B.center);
        mid[count] = m;
        ++count;
        return true;
    }
};

bool testFaceA(const Obb &A, const Obb &B, V3 dA, const M3 &m, int i, float margin, Sat &best) {
    const float sep = std::fabs(dA[i]) -
            (((A.half[i] + B.half.x * std::fabs(m.c[0][i])) + B.half.y * std::fabs(m.c[1][i])) +
             B.half.z * std::fabs(m.c[2][i]));
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.separation) {
        best.valid = true;
        best.type = kAxisFaceA;
        best.ia = i;
        best.ib = -1;
        best.separation = sep;
        best.normalAB = A.axis[i] * (dA[i] < 0.0f ? -1.0f : 1.0f);
    }
    return true;
}

bool testFaceB(const Obb &A, const Obb &B, V3 dB, const M3 &m, int j, float margin, Sat &best) {
    const float sep = std::fabs(dB[j]) -
            (((B.half[j] + A.half.x * std::fabs(m.c[j][0])) + A.half.y * std::fabs(m.c[j][1])) +
             A.half.z * std::fabs(m.c[j][2]));
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.separation) {
        best.valid = true;
        best.type = kAxisFaceB;
        best.ia = -1;
        best.ib = j;
        best.separation = sep;
        best.normalAB = B.axis[j] * (dB[j] < 0.0f ? -1.0f : 1.0f);
    }
    return true;
}

bool testEdge(const Obb &A, const Obb &B, V3 delta, V3 axis, const M3 &m, int i, int j, float margin,
        Sat &best) {
    const float lenSq = length2(axis);
    if (lenSq < kSatAxisEps)
        return true;
    const float invLen = 1.0f / std::sqrt(lenSq);
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
    const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    const float rA = (A.half[i1] * std::fabs(m.c[j][i2]) + A.half[i2] * std::fabs(m.c[j][i1])) * invLen;
    const float rB = (B.half[j1] * std::fabs(m.c[j2][i]) + B.half[j2] * std::fabs(m.c[j1][i])) * invLen;
    const float signedDist = dot(delta, axis) * invLen;
    const float sep = std::fabs(signedDist) - (rA + rB);
    if (sep > margin)
        return false;
    if (!best.valid || sep > best.separation) {
        best.valid = true;
        best.type = kAxisEdge;
        best.ia = i;
        best.ib = j;
        best.separation = sep;
        best.normalAB = axis * (signedDist < 0.0f ? -invLen : invLen);
    }
    return true;
}

void supportEdge(const Obb &b, int k, V3 dir, V3 &e0, V3 &e1) {
    const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
    const float s1 = dot(dir, b.axis[k1]) >= 0.0f ? 1.0f : -1.0f;
    const float s2 = dot(dir, b.axis[k2]) >= 0.0f ? 1.0f : -1.0f;
    const V3 ec = (b.center + b.axis[k1] * (b.half[k1] * s1)) + b.axis[k2] * (b.half[k2] * s2);
    e0 = ec - b.axis[k] * b.half[k];
    e1 = ec + b.axis[k] * b.half[k];
}

void closestOnSegments(V3 p0, V3 p1, V3 q0, V3 q1, V3 &c0, V3 &c1) {
    const V3 d1 = p1 - p0;
    const V3 d2 = q1 - q0;
    const V3 r = p0 - q0;
    const float a = dot(d1, d1);
    const float e = dot(d2, d2);
    const float f = dot(d2, r);
    float s = 0.0f, t = 0.0f;
    if (a <= kSatAxisEps && e <= kSatAxisEps) {
        c0 = p0;
        c1 = q0;
        return;
    }
    if (a <= kSatAxisEps) {
        t = sclamp(f / e, 0.0f, 1.0f);
    } else {
        const float c = dot(d1, r);
        if (e <= kSatAxisEps) {
            s = sclamp(-c / a, 0.0f, 1.0f);
        } else {
            const float b = dot(d1, d2);
            const float denom = a * e - b * b;
            if (std::fabs(denom) > kSatAxisEps)
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
    c0 = p0 + d1 * s;
    c1 = q0 + d2 * t;
}

int faceManifold(const Obb &A, const Obb &B, bool refIsA, int refAxis, V3 normalAB, float margin,
        Contact *out) {
    const Obb &ref = refIsA ? A : B;
    const Obb &inc = refIsA ? B : A;
    const V3 outward = refIsA ? normalAB : -normalAB;
    Face rf;
    {
        const float sign = dot(outward, ref.axis[refAxis]) >= 0.0f ? 1.0f : -1.0f;
        rf.axis = refAxis;
        rf.normal = ref.axis[refAxis] * sign;
        rf.center = ref.center + rf.normal * ref.half[refAxis];
        faceAxes(ref, refAxis, rf.u, rf.v, rf.eu, rf.ev);
    }
    int incAxis = 0;
    {
        float best = -FLT_MAX;
        for (int i = 0; i < 3; ++i) {
            const float d = std::fabs(dot(inc.axis[i], rf.normal));
            if (d > best) {
                best = d;
                incAxis = i;
            }
        }
    }
    V3 clip0[kMaxPolyVerts], clip1[kMaxPolyVerts];
    {
        const float sign = dot(inc.axis[incAxis], rf.normal) > 0.0f ? -1.0f : 1.0f;
        const V3 fn = inc.axis[incAxis] * sign;
        const V3 fc = inc.center + fn * inc.half[incAxis];
        V3 u, v;
        float eu, ev;
        faceAxes(inc, incAxis, u, v, eu, ev);
        clip0[0] = (fc + u * eu) + v * ev;
        clip0[1] = (fc - u * eu) + v * ev;
        clip0[2] = (fc - u * eu) - v * ev;
        clip0[3] = (fc + u * eu) - v * ev;
    }
    int count = 4;
    const V3 n0 = rf.u;
    count = clipPolygon(clip0, count, n0, dot(n0, rf.center) + rf.eu, clip1);
    if (!count)
        return 0;
    const V3 n1 = -rf.u;
    count = clipPolygon(clip1, count, n1, dot(n1, rf.center) + rf.eu, clip0);
    if (!count)
        return 0;
    const V3 n2 = rf.v;
    count = clipPolygon(clip0, count, n2, dot(n2, rf.center) + rf.ev, clip1);
    if (!count)
        return 0;
    const V3 n3 = -rf.v;
    count = clipPolygon(clip1, count, n3, dot(n3, rf.center) + rf.ev, clip0);
    if (!count)
        return 0;

    ContactSink sink{A, B, out, 0, {}};
    int prefix = (refIsA ? kAxisFaceA : kAxisFaceB) << 24;
    prefix |= (refAxis & 0xFF) << 16;
    prefix |= (incAxis & 0xFF) << 8;
    const float accept = smax(margin, kPlaneEps);
    for (int i = 0; i < count && sink.count < kMaxContacts; ++i) {
        const V3 p = clip0[i];
        const float dist = dot(p - rf.center, rf.normal);
        if (dist > accept)
            continue;
        const V3 pr = p - rf.normal * dist;
        sink.add(refIsA ? pr : p, refIsA ? p : pr, prefix | (i & 0xFF));
    }
    if (!sink.count) {
        const V3 xA = supportPoint(A, normalAB);
        V3 xB = supportPoint(B, -normalAB);
        xB = xA - normalAB * dot(xA - xB, normalAB);
        sink.add(xA, xB, prefix);
    }
    return sink.count;
}

int edgeContact(const Obb &A, const Obb &B, int axisA, int axisB, V3 normalAB, Contact *out) {
    V3 a0, a1, b0, b1;
    supportEdge(A, axisA, normalAB, a0, a1);
    supportEdge(B, axisB, -normalAB, b0, b1);
    V3 xA, xB;
    closestOnSegments(a0, a1, b0, b1, xA, xB);
    ContactSink sink{A, B, out, 0, {}};
    const int key = (kAxisEdge << 24) | ((axisA & 0xFF) << 8) | (axisB & 0xFF);
    sink.add(xA, xB, key);
    if (!sink.count) {
        xA = supportPoint(A, normalAB);
        xB = supportPoint(B, -normalAB);
        sink.add(xA, xB, key);
    }
    return sink.count;
}

} // namespace

int collideBoxes(V3 ca, Q4 qa, V3 ha, V3 cb, Q4 qb, V3 hb, float margin, Contact *out, M3 &basis) {
    const Obb A = makeObb(ca, qa, ha);
    const Obb B = makeObb(cb, qb, hb);
    const V3 delta = B.center - A.center;
    M3 m;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            m.c[j][i] = dot(A.axis[i], B.axis[j]);
    const V3 dA{dot(delta, A.axis[0]), dot(delta, A.axis[1]), dot(delta, A.axis[2])};
    const V3 dB{dot(delta, B.axis[0]), dot(delta, B.axis[1]), dot(delta, B.axis[2])};
    Sat bestFace, bestEdge;
    for (int i = 0; i < 3; ++i)
        if (!testFaceA(A, B, dA, m, i, margin, bestFace))
            return 0;
    for (int j = 0; j < 3; ++j)
        if (!testFaceB(A, B, dB, m, j, margin, bestFace))
            return 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (!testEdge(A, B, delta, cross(A.axis[i], B.axis[j]), m, i, j, margin, bestEdge))
                return 0;
    if (!bestFace.valid)
        return 0;
    Sat best = bestFace;
    if (bestEdge.valid && 0.95f * bestEdge.separation > bestFace.separation + 0.01f)
        best = bestEdge;
    basis = orthonormal(-best.normalAB);
    if (best.type == kAxisEdge)
        return edgeContact(A, B, best.ia, best.ib, best.normalAB, out);
    if (best.type == kAxisFaceA)
        return faceManifold(A, B, true, best.ia, best.normalAB, margin, out);
    return faceManifold(A, B, false, best.ib, best.normalAB, margin, out);
}

// ------------------------------------------------------------------------------------------
// Bodies and forces
// ------------------------------------------------------------------------------------------

// Rigid::Rigid for boxes (src/avbd/rigid.cpp:22-72).
int World::addBody(const avbdg_body_desc &d) {
    Body b;
    b.size = V3{d.size[0], d.size[1], d.size[2]};
    b.shape = d.shape;
    b.friction = d.friction;
    b.gravity = P.gravity;
    b.x = V3{d.position[0], d.position[1], d.position[2]};
    b.q = Q4{d.orientation[0], d.orientation[1], d.orientation[2], d.orientation[3]};
    b.v = V3{d.velocity[0], d.velocity[1], d.velocity[2]};
    b.vprev = b.v;
    b.w = V3{d.angular_velocity[0], d.angular_velocity[1], d.angular_velocity[2]};
    b.layer = d.collision_layer;
    b.mask = d.collision_mask;
    b.lockLin = static_cast<uint8_t>(d.axis_lock_linear);
    b.lockAng = static_cast<uint8_t>(d.axis_lock_angular);
    b.sleepMode = static_cast<int>(d.sleep_mode);
    // Mass properties and bounding radius per shape (rigid.cpp:34-72).
    if (b.shape == 1) {
        const float r = b.size.x;
        b.mass = (4.0f / 3.0f) * 3.14159265358979f * r * r * r * d.density;
        const float i = 0.4f * b.mass * r * r;
        b.moment = V3{i, i, i};
        b.radius = r;
    } else if (b.shape == 2) {
        const float r = b.size.x, h = b.size.z;
        b.mass = 3.14159265358979f * r * r * h * d.density;
        const float axial = 0.5f * b.mass * r * r;
        const float radial = b.mass * (3.0f * r * r + h * h) / 12.0f;
        b.moment = V3{radial, radial, axial};
        b.radius = std::sqrt(dot(V3{r, h * 0.5f, r}, V3{r, h * 0.5f, r}));
    } else {
        b.mass = b.size.x * b.size.y * b.size.z * d.density;
        b.moment = V3{(b.size.y * b.size.y + b.size.z * b.size.z) / 12.0f * b.mass,
                      (b.size.x * b.size.x + b.size.z * b.size.z) / 12.0f * b.mass,
                      (b.size.x * b.size.x + b.size.y * b.size.y) / 12.0f * b.mass};
        b.radius = std::sqrt(dot(b.size * 0.5f, b.size * 0.5f));
    }
    bodies.push_back(b);
    treeBodies = -1;
    return static_cast<int>(bodies.size()) - 1;
}

// Joint::Joint (src/avbd/joint.cpp:28-40); the new force becomes the list head.
void World::addJoint(int a, int b, V3 rA, V3 rB, float kLin, float kAng, float fracture) {
    Force f;
    f.kind = kJoint;
    f.a = a;
    f.b = b;
    f.rA = rA;
    f.rB = rB;
    f.stiffLin = kLin;
    f.stiffAng = kAng;
    f.fracture = fracture;
    const V3 sa = a >= 0 ? bodies[a].size : V3{0, 0, 0};
    f.torqueArm = length2(sa + bodies[b].size);
    forces.insert(forces.begin(), f);
}

void World::addIgnore(int a, int b) {
    Force f;
    f.kind = kIgnore;
    f.a = a;
    f.b = b;
    forces.insert(forces.begin(), f);
}

V3 World::jointLin(const Force &f) const {
    const Body &B = bodies[f.b];
    const V3 pa = f.a >= 0 ? bodies[f.a].x + qrot(bodies[f.a].q, f.rA) : f.rA;
    return pa - (B.x + qrot(B.q, f.rB));
}

V3 World::jointAng(const Force &f) const {
    const Q4 qa = f.a >= 0 ? bodies[f.a].q : Q4{0.0f, 0.0f, 0.0f, 1.0f};
    return qdiff(qa, bodies[f.b].q) * f.torqueArm;
}

static V3 warmPenalty(V3 p, float gamma, float k) {
    return V3{smin(sclamp(p.x * gamma, PENALTY_MIN, PENALTY_MAX), k),
              smin(sclamp(p.y * gamma, PENALTY_MIN, PENALTY_MAX), k),
              smin(sclamp(p.z * gamma, PENALTY_MIN, PENALTY_MAX), k)};
}

// Joint::initialize (joint.cpp:62-78).
bool World::jointInitialize(Force &f) {
    if (f.kind != kJoint)
        return true;
    f.C0Lin = jointLin(f);
    f.C0Ang = jointAng(f);
    f.lamLin = f.lamLin * P.alpha * P.gamma;
    f.lamAng = f.lamAng * P.alpha * P.gamma;
    f.kLin = warmPenalty(f.kLin, P.gamma, f.stiffLin);
    f.kAng = warmPenalty(f.kAng, P.gamma, f.stiffAng);
    return !f.broken;
}

static M3 geometricStiffness(int k, V3 v) {
    M3 m = mdiag(-v[k], -v[k], -v[k]);
    m.c[k][0] += v[0];
    m.c[k][1] += v[1];
    m.c[k][2] += v[2];
    return m;
}

// Joint::updatePrimal (joint.cpp:80-160).
void World::jointUpdatePrimal(const Force &f, int body, Block &blk) const {
    if (f.kind != kJoint)
        return;
    const float alpha = P.alpha;
    const bool isA = body == f.a;
    if (length2(f.kLin) > 0) {
        const M3 K = mdiag(f.kLin.x, f.kLin.y, f.kLin.z);
        V3 C = jointLin(f);
        if (std::isinf(f.stiffLin))
            C -= f.C0Lin * alpha;
        const V3 F = mul(K, C) + f.lamLin;
        const M3 I = mdiag(1, 1, 1);
        const M3 jLin = isA ? I : -I;
        M3 jAng;
        if (isA) {
            const V3 r = -qrot(bodies[f.a].q, f.rA);
            jAng = mcols(V3{0, r.z, -r.y}, V3{-r.z, 0, r.x}, V3{r.y, -r.x, 0});
        } else {
            const V3 r = qrot(bodies[f.b].q, f.rB);
            jAng = mcols(V3{0, r.z, -r.y}, V3{-r.z, 0, r.x}, V3{r.y, -r.x, 0});
        }
        const M3 jLinT = transpose(jLin);
        const M3 jAngT = transpose(jAng);
        const M3 jAngTk = mul(jAngT, K);
        blk.lhsLin += mul(mul(jLinT, K), jLin);
        blk.lhsAng += mul(jAngTk, jAng);
        blk.lhsCross += mul(jAngTk, jLin);
        const V3 r = isA ? qrot(bodies[f.a].q, f.rA) : -qrot(bodies[f.b].q, f.rB);
        const M3 H = (geometricStiffness(0, r) * F[0] + geometricStiffness(1, r) * F[1]) +
                     geometricStiffness(2, r) * F[2];
        blk.lhsAng += mdiag(H.c[0][0], H.c[1][1], H.c[2][2]);
        blk.rhsLin += mul(jLinT, F);
        blk.rhsAng += mul(jAngT, F);
    }
    if (length2(f.kAng) > 0) {
        const M3 K = mdiag(f.kAng.x, f.kAng.y, f.kAng.z);
        V3 C = jointAng(f);
        if (std::isinf(f.stiffAng))
            C -= f.C0Ang * alpha;
        const V3 F = mul(K, C) + f.lamAng;
        const M3 base = isA ? mdiag(1, 1, 1) : mcols(V3{0, 0, 0}, V3{0, -1, 0}, V3{0, 0, -1});
        const M3 jAng = base * f.torqueArm;
        blk.lhsAng += mul(mul(transpose(jAng), K), jAng);
        blk.rhsAng += mul(transpose(jAng), F);
    }
}

// Joint::updateDual (joint.cpp:171-230).
void World::jointUpdateDual(Force &f) {
    if (f.kind != kJoint)
        return;
    const float alpha = P.alpha;
    if (length2(f.kLin) > 0) {
        const M3 K = mdiag(f.kLin.x, f.kLin.y, f.kLin.z);
        V3 C = jointLin(f);
        if (std::isinf(f.stiffLin)) {
            C -= f.C0Lin * alpha;
            f.lamLin = mul(K, C) + f.lamLin;
        }
        const V3 cap = lminv(V3{f.stiffLin, f.stiffLin, f.stiffLin}, V3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
        f.kLin = lminv(f.kLin + vabs(C) * P.beta_lin, cap);
    }
    if (length2(f.kAng) > 0) {
        const M3 K = mdiag(f.kAng.x, f.kAng.y, f.kAng.z);
        V3 C = jointAng(f);
        if (std::isinf(f.stiffAng)) {
            C -= f.C0Ang * alpha;
            f.lamAng = mul(K, C) + f.lamAng;
        }
        const V3 cap = lminv(V3{f.stiffAng, f.stiffAng, f.stiffAng}, V3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
        f.kAng = lminv(f.kAng + vabs(C) * P.beta_ang, cap);
    }
    if (length2(f.lamAng) > f.fracture * f.fracture) {
        f.kLin = f.kAng = f.lamLin = f.lamAng = V3{0, 0, 0};
        f.broken = true;
    }
}

// Spring::Spring (spring.cpp:16-27): a negative rest length is the anchors' current distance.
void World::addSpring(int a, int b, V3 rA, V3 rB, float stiffness, float rest) {
    Force f;
    f.kind = kSpring;
    f.a = a;
    f.b = b;
    f.rA = rA;
    f.rB = rB;
    f.springK = stiffness;
    if (rest < 0.0f) {
        const Body &A = bodies[a], &B = bodies[b];
        rest = length((A.x + qrot(A.q, rA)) - (B.x + qrot(B.q, rB)));
    }
    f.rest = rest;
    forces.insert(forces.begin(), f);
}

// GenericJoint::GenericJoint (generic_joint.cpp:24-30): its zero is the creation arrangement.
void World::addGeneric(int a, int b, V3 rA, V3 rB, const Axis axes[6]) {
    Force f;
    f.kind = kGeneric;
    f.a = a;
    f.b = b;
    f.rA = rA;
    f.rB = rB;
    for (int i = 0; i < 6; i++)
        f.axis[i] = axes[i];
    f.restQ = qmul(qconj(frameOrientation(f)), bodies[b].q);
    forces.insert(forces.begin(), f);
}

static M3 outerprod(V3 a, V3 b) { return mcols(a * b.x, a * b.y, a * b.z); }

// Spring::updatePrimal (spring.cpp:31-70).
void World::springUpdatePrimal(const Force &f, int body, Block &blk) const {
    const Body &A = bodies[f.a], &B = bodies[f.b];
    const V3 pA = A.x + qrot(A.q, f.rA);
    const V3 pB = B.x + qrot(B.q, f.rB);
    const V3 d = pA - pB;
    const float dLen = length(d);
    if (dLen <= 1.0e-6f)
        return;
    const V3 n = d / dLen;
    const float C = dLen - f.rest;
    const float force = f.springK * C;
    V3 jLin, jAng;
    if (body == f.a) {
        const V3 r = qrot(A.q, f.rA);
        jLin = n;
        jAng = cross(r, n);
    } else {
        const V3 r = qrot(B.q, f.rB);
        jLin = -n;
        jAng = -cross(r, n);
    }
    const V3 F = jLin * force;
    const V3 tau = jAng * force;
    const M3 kll = outerprod(jLin, jLin) * f.springK;
    const M3 kla = outerprod(jAng, jLin) * f.springK;
    const M3 kaa = outerprod(jAng, jAng) * f.springK;
    blk.lhsLin += kll;
    blk.lhsAng += kaa;
    blk.lhsCross += kla;
    blk.rhsLin += F;
    blk.rhsAng += tau;
}

static V3 unitAxis(int i) { return i == 0 ? V3{1, 0, 0} : (i == 1 ? V3{0, 1, 0} : V3{0, 0, 1}); }
static float qcomp(Q4 q, int i) { return i == 0 ? q.x : (i == 1 ? q.y : (i == 2 ? q.z : q.w)); }
static float v3comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
// maths.h qinv: conj(q) / qlength2(q).
static Q4 qinvm(Q4 q) {
    const float l = qlength2(q);
    return Q4{-q.x / l, -q.y / l, -q.z / l, q.w / l};
}

Q4 World::frameOrientation(const Force &f) const {
    return f.a >= 0 ? bodies[f.a].q : Q4{0.0f, 0.0f, 0.0f, 1.0f};
}

// qrot(conj(qA), anchorA - anchorB) (generic_joint.cpp:37-45, 100-104).
V3 World::genericOffset(const Force &f) const {
    const V3 anchorA = f.a >= 0 ? bodies[f.a].x + qrot(bodies[f.a].q, f.rA) : f.rA;
    const Body &B = bodies[f.b];
    const V3 anchorB = B.x + qrot(B.q, f.rB);
    return qrot(qconj(frameOrientation(f)), anchorA - anchorB);
}

// Swing-twist measurement (generic_joint.cpp:49-98): each non-locked axis takes its twist
// (2 atan2(v.n, w)), the locked axes read the remaining swing.
void World::genericAngles(const Force &f, float out[3]) const {
    const Q4 qA = frameOrientation(f);
    const Q4 relativeNow = qmul(qconj(qA), qnormalize(bodies[f.b].q));
    Q4 dev = qmul(qnormalize(f.restQ), qconj(relativeNow));
    for (int i = 0; i < 3; i++) {
        if (f.axis[3 + i].mode == kLocked)
            continue;
        const float proj = dot(V3{dev.x, dev.y, dev.z}, unitAxis(i));
        const Q4 twist{dev.x * proj, dev.y * proj, dev.z * proj, dev.w};
        if (std::sqrt(qlength2(twist)) <= 1.0e-12f) {
            out[i] = 0.0f;
            continue;
        }
        out[i] = 2.0f * std::atan2(proj, dev.w);
        dev = qmul(qnormalize(dev), qinvm(twist));
    }
    for (int i = 0; i < 3; i++)
        if (f.axis[3 + i].mode == kLocked)
            out[i] = qcomp(dev, i) * 2.0f;
}

// GenericJoint::penaltyLimit (generic_joint.cpp:198-222).
float World::penaltyLimit(int body, V3 axis, bool angular) const {
    const Body &b = bodies[body];
    float effective;
    if (angular) {
        const V3 local = qrot(qconj(b.q), axis);
        effective = local.x * local.x * b.moment.x + local.y * local.y * b.moment.y + local.z * local.z * b.moment.z;
    } else {
        effective = b.mass;
    }
    if (effective <= 0.0f)
        return PENALTY_MAX;
    const float limit = effective * 0.25f * 0.25f / (P.dt * P.dt);
    return smin(limit, PENALTY_MAX);
}

// GenericJoint::initialize (generic_joint.cpp:224-245).
void World::genericInitialize(Force &f) {
    float ang[3];
    genericAngles(f, ang);
    const V3 offset = genericOffset(f);
    for (int i = 0; i < 3; i++) {
        f.axis[i].initial = v3comp(offset, i);
        f.axis[3 + i].initial = ang[i];
        for (int k = 0; k < 2; k++) {
            Axis &ax = f.axis[3 * k + i];
            ax.lambda = ax.lambda * (P.alpha * P.gamma);
            ax.penalty = sclamp(ax.penalty * P.gamma, PENALTY_MIN, PENALTY_MAX);
        }
    }
}

// axisConstraint + axisForce (generic_joint.cpp:120-168).
static bool axisForce(const Axis &ax, float value, float alpha, float &C, float &F) {
    if (ax.mode == kLocked) {
        C = value;
    } else if (ax.mode == kLimited) {
        if (value > ax.upper)
            C = value - ax.upper;
        else if (value < ax.lower)
            C = value - ax.lower;
        else
            return false;
    } else {
        return false;
    }
    if (ax.mode == kLocked)
        C -= ax.initial * alpha;
    float force = ax.penalty * C + ax.lambda;
    if (ax.mode == kLimited)
        force = C > 0.0f ? smax(force, 0.0f) : smin(force, 0.0f);
    F = force;
    return true;
}

// GenericJoint::stampAxis (generic_joint.cpp:170-196).
static void stampAxis(Block &blk, const Axis &ax, float value, float alpha, V3 jLin, V3 jAng, float rate) {
    float C, F;
    if (axisForce(ax, value, alpha, C, F)) {
        blk.lhsLin += outerprod(jLin, jLin) * ax.penalty;
        blk.lhsAng += outerprod(jAng, jAng) * ax.penalty;
        blk.lhsCross += outerprod(jAng, jLin) * ax.penalty;
        blk.rhsLin += jLin * F;
        blk.rhsAng += jAng * F;
    }
    if (ax.springK > 0.0f) {
        const float Cs = value - ax.springEq;
        const float Fs = ax.springK * Cs - ax.springDamp * rate;
        blk.lhsLin += outerprod(jLin, jLin) * ax.springK;
        blk.lhsAng += outerprod(jAng, jAng) * ax.springK;
        blk.lhsCross += outerprod(jAng, jLin) * ax.springK;
        blk.rhsLin += jLin * Fs;
        blk.rhsAng += jAng * Fs;
    }
}

// GenericJoint::updatePrimal (generic_joint.cpp:247-287).
void World::genericUpdatePrimal(const Force &f, int body, Block &blk) const {
    const Q4 qA = frameOrientation(f);
    const Body &B = bodies[f.b];
    const V3 rAWorld = qrot(qA, f.rA);
    const V3 rBWorld = qrot(B.q, f.rB);
    const V3 offset = genericOffset(f);
    float ang[3];
    genericAngles(f, ang);
    const bool isA = body == f.a;
    const float sign = isA ? 1.0f : -1.0f;
    const V3 arm = isA ? rAWorld : rBWorld;
    const V3 vA = f.a >= 0 ? bodies[f.a].v + cross(bodies[f.a].w, rAWorld) : V3{0, 0, 0};
    const V3 vB = B.v + cross(B.w, rBWorld);
    const V3 relV = vA - vB;
    const V3 wA = f.a >= 0 ? bodies[f.a].w : V3{0, 0, 0};
    const V3 wB = B.w;
    for (int i = 0; i < 3; i++) {
        const V3 axis = qrot(qA, unitAxis(i));
        const V3 jLin = axis * sign;
        const V3 jAng = cross(arm, jLin);
        stampAxis(blk, f.axis[i], v3comp(offset, i), P.alpha, jLin, jAng, dot(relV, axis));
        stampAxis(blk, f.axis[3 + i], ang[i], P.alpha, V3{0, 0, 0}, axis * sign, dot(wA - wB, axis));
    }
}

// GenericJoint::updateDual (generic_joint.cpp:289-319).
void World::genericUpdateDual(Force &f) {
    float ang[3];
    genericAngles(f, ang);
    const V3 offset = genericOffset(f);
    for (int i = 0; i < 3; i++) {
        const float values[2] = {v3comp(offset, i), ang[i]};
        const float betas[2] = {P.beta_lin, P.beta_ang};
        for (int k = 0; k < 2; k++) {
            Axis &ax = f.axis[3 * k + i];
            float C, F;
            if (!axisForce(ax, values[k], P.alpha, C, F)) {
                if (ax.mode == kLimited)
                    ax.lambda = 0.0f;
                continue;
            }
            ax.lambda = F;
            const V3 dir = qrot(frameOrientation(f), unitAxis(i));
            float cap = penaltyLimit(f.b, dir, k == 1);
            if (f.a >= 0)
                cap = smin(cap, penaltyLimit(f.a, dir, k == 1));
            ax.penalty = sclamp(ax.penalty + std::fabs(C) * betas[k], 0.0f, cap);
        }
    }
}

void World::forceUpdatePrimal(const Force &f, int body, Block &blk) const {
    if (f.kind == kJoint)
        jointUpdatePrimal(f, body, blk);
    else if (f.kind == kSpring)
        springUpdatePrimal(f, body, blk);
    else if (f.kind == kGeneric)
        genericUpdatePrimal(f, body, blk);
}

void World::forceUpdateDual(Force &f) {
    if (f.kind == kJoint)
        jointUpdateDual(f);
    else if (f.kind == kGeneric)
        genericUpdateDual(f);
}

// ------------------------------------------------------------------------------------------
// Manifolds (src/avbd/manifold.cpp)
// ------------------------------------------------------------------------------------------

static void basisHessian(const M3 &basis, V3 k, float S[6]) {
    const V3 b0 = mrow(basis, 0), b1 = mrow(basis, 1), b2 = mrow(basis, 2);
    const float b0x2 = b0.x * b0.x, b0y2 = b0.y * b0.y, b0z2 = b0.z * b0.z;
    const float b0xy = b0.x * b0.y, b0xz = b0.x * b0.z, b0yz = b0.y * b0.z;
    const float b1x2 = b1.x * b1.x, b1y2 = b1.y * b1.y, b1z2 = b1.z * b1.z;
    const float b1xy = b1.x * b1.y, b1xz = b1.x * b1.z, b1yz = b1.y * b1.z;
    const float b2x2 = b2.x * b2.x, b2y2 = b2.y * b2.y, b2z2 = b2.z * b2.z;
    const float b2xy = b2.x * b2.y, b2xz = b2.x * b2.z, b2yz = b2.y * b2.z;
    S[0] = k.x * b0x2 + k.y * b1x2 + k.z * b2x2;
    S[1] = k.x * b0xy + k.y * b1xy + k.z * b2xy;
    S[2] = k.x * b0xz + k.y * b1xz + k.z * b2xz;
    S[3] = k.x * b0y2 + k.y * b1y2 + k.z * b2y2;
    S[4] = k.x * b0yz + k.y * b1yz + k.z * b2yz;
    S[5] = k.x * b0z2 + k.y * b1z2 + k.z * b2z2;
}

static V3 constraintError(V3 c0, V3 bracket, const M3 &basis, float oneMinusAlpha, bool speculative) {
    const bool separated = speculative && c0.x > kReleaseAbove;
    return c0 * (separated ? 1.0f : oneMinusAlpha) + mul(basis, bracket);
}

struct Cone {
    float bounds, scale;
};

static Cone clampForce(V3 &F, float mu) {
    F.x = smin(F.x, 0.0f);
    const float bounds = std::fabs(F.x) * mu;
    const float fs = length2d(F.y, F.z);
    if (fs > bounds && fs > 0) {
        F.y *= bounds / fs;
        F.z *= bounds / fs;
    }
    return {bounds, fs};
}

// Manifold::collide (collide.cpp:1100-1120).
// ---- Spheres and cylinders (collide.cpp:493-999): closest points, cylinder surface samples ----

namespace {

constexpr int kRimSamples = 8, kAxialSamples = 3;
constexpr int kMaxCylSamples = 2 * (kRimSamples + 1) + kRimSamples * (kAxialSamples - 1);
constexpr int kMaxCandidates = 2 * kMaxCylSamples + 8;
constexpr uint32_t kAxisCylSample = 3, kAxisCylCorner = 4;

struct Shape {
    int type; // 0 box, 1 sphere, 2 cylinder
    V3 center;
    Q4 rot;
    V3 half;
    float radius, halfHeight;
    V3 axis;
};

Shape makeShape(const Body &b) {
    return Shape{b.shape, b.x, b.q, b.size * 0.5f, b.size.x, b.size.z * 0.5f, qrot(b.q, V3{0, 0, 1})};
}

// Rim directions, a coprime stride around the circle (collide.cpp:731-753).
struct RimTrig {
    float c[kRimSamples], s[kRimSamples];
    RimTrig() {
        for (int i = 0; i < kRimSamples; ++i) {
            const int step = i * 5 % kRimSamples;
            const float a = 6.28318530718f * (float)step / (float)kRimSamples;
            c[i] = std::cos(a);
            s[i] = std::sin(a);
        }
    }
};
const RimTrig &rimTrig() {
    static const RimTrig t;
    return t;
}

bool pointInBox(const Shape &box, V3 p, V3 &push, float &depth) {
    const V3 local = qrot(qconj(box.rot), p - box.center);
    float best = FLT_MAX;
    int axis = 0;
    float sign = 1.0f;
    for (int i = 0; i < 3; ++i) {
        const float d = box.half[i] - std::fabs(local[i]);
        if (d <= 0.0f)
            return false;
        if (d < best) {
            best = d;
            axis = i;
            sign = local[i] >= 0.0f ? 1.0f : -1.0f;
        }
    }
    V3 lp{0, 0, 0};
    lp[axis] = sign;
    push = qrot(box.rot, lp);
    depth = best;
    return true;
}

bool pointNearBox(const Shape &box, V3 p, float margin, V3 &push, float &depth) {
    const V3 local = qrot(qconj(box.rot), p - box.center);
    bool outside = false;
    for (int i = 0; i < 3; ++i)
        if (std::fabs(local[i]) >= box.half[i]) {
            outside = true;
            break;
        }
    if (!outside)
        return false;
    const V3 cl{sclamp(local.x, -box.half.x, box.half.x), sclamp(local.y, -box.half.y, box.half.y),
                sclamp(local.z, -box.half.z, box.half.z)};
    const V3 d = local - cl;
    const float gap = length(d);
    if (gap > margin || gap <= 1.0e-9f)
        return false;
    push = qrot(box.rot, d / gap);
    depth = -gap;
    return true;
}

V3 closestPointOnCylinder(const Shape &cyl, V3 p, V3 &outward, float &distance) {
    const V3 local = qrot(qconj(cyl.rot), p - cyl.center);
    const float t = sclamp(local.z, -cyl.halfHeight, cyl.halfHeight);
    const float lenSq = (0.0f + local.x * local.x) + local.y * local.y; // linalg length2 of (x, y)
    V3 closest{0, 0, t};
    if (lenSq > cyl.radius * cyl.radius) {
        const float scale = cyl.radius / std::sqrt(lenSq);
        closest.x = local.x * scale;
        closest.y = local.y * scale;
    } else if (lenSq > 1.0e-12f) {
        closest.x = local.x;
        closest.y = local.y;
    } else {
        closest.x = cyl.radius;
    }
    const V3 onCyl = qrot(cyl.rot, closest) + cyl.center;
    const V3 d = p - onCyl;
    distance = length(d);
    outward = distance > 1.0e-9f ? d / distance : qrot(cyl.rot, V3{1, 0, 0});
    return onCyl;
}

bool pointInCylinder(const Shape &cyl, V3 p, V3 &push, float &surface) {
    const V3 local = qrot(qconj(cyl.rot), p - cyl.center);
    const float radialSq = local.x * local.x + local.y * local.y;
    if (radialSq >= cyl.radius * cyl.radius || std::fabs(local.z) >= cyl.halfHeight)
        return false;
    const float radialDepth = cyl.radius - std::sqrt(radialSq);
    const float capDepth = cyl.halfHeight - std::fabs(local.z);
    V3 pl{0, 0, 0};
    if (capDepth < radialDepth) {
        pl.z = local.z >= 0.0f ? 1.0f : -1.0f;
        surface = capDepth;
    } else {
        const float len = std::sqrt(radialSq);
        if (len > 1.0e-6f) {
            pl.x = local.x / len;
            pl.y = local.y / len;
        } else {
            pl.x = 1.0f;
        }
        surface = radialDepth;
    }
    push = qrot(cyl.rot, pl);
    return true;
}

bool pointNearCylinder(const Shape &cyl, V3 p, float margin, V3 &push, float &depth) {
    const V3 local = qrot(qconj(cyl.rot), p - cyl.center);
    const float radialSq = local.x * local.x + local.y * local.y;
    if (radialSq < cyl.radius * cyl.radius && std::fabs(local.z) < cyl.halfHeight)
        return false;
    V3 outward;
    float distance;
    closestPointOnCylinder(cyl, p, outward, distance);
    if (distance > margin)
        return false;
    push = outward;
    depth = -distance;
    return true;
}

bool sampleInsideBox(const Shape &box, V3 p, float margin, V3 &push, float &depth) {
    return pointInBox(box, p, push, depth) || (margin > 0.0f && pointNearBox(box, p, margin, push, depth));
}

bool sampleInsideCylinder(const Shape &cyl, V3 p, float margin, V3 &push, float &depth) {
    return pointInCylinder(cyl, p, push, depth) || (margin > 0.0f && pointNearCylinder(cyl, p, margin, push, depth));
}

void cylinderSamples(const Shape &cyl, V3 *out, int &count) {
    count = 0;
    const V3 x = qrot(cyl.rot, V3{1, 0, 0});
    const V3 y = qrot(cyl.rot, V3{0, 1, 0});
    const RimTrig &trig = rimTrig();
    for (int end = -1; end <= 1; end += 2) {
        const V3 cap = cyl.center + cyl.axis * (cyl.halfHeight * (float)end);
        out[count++] = cap;
        for (int i = 0; i < kRimSamples; ++i)
            out[count++] = cap + (x * trig.c[i] + y * trig.s[i]) * cyl.radius;
    }
    for (int ring = 1; ring < kAxialSamples; ++ring) {
        const float t = -cyl.halfHeight + 2.0f * cyl.halfHeight * (float)ring / (float)kAxialSamples;
        const V3 rc = cyl.center + cyl.axis * t;
        for (int i = 0; i < kRimSamples; ++i)
            out[count++] = rc + (x * trig.c[i] + y * trig.s[i]) * cyl.radius;
    }
}

struct Candidate {
    V3 xA, xB, normal;
    float depth;
    uint32_t feature;
};

// Deepest first, stable (equal depths keep their order); emission stops at the first contact the
// sink refuses (collide.cpp:699-729).
void emitRanked(const Candidate *cand, int n, ContactSink &sink) {
    int order[kMaxCandidates];
    for (int i = 0; i < n; ++i) {
        int j = i;
        while (j > 0 && cand[order[j - 1]].depth < cand[i].depth) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = i;
    }
    const int emit = std::min(n, kMaxContacts);
    for (int i = 0; i < emit; ++i)
        if (!sink.add(cand[order[i]].xA, cand[order[i]].xB, static_cast<int>(cand[order[i]].feature)))
            break;
}

int collideSphereSphere(const Shape &a, const Shape &b, float margin, ContactSink &sink, M3 &basis) {
    const V3 d = b.center - a.center;
    const float distSq = length2(d);
    const float sumPlus = a.radius + b.radius + margin;
    if (distSq >= sumPlus * sumPlus)
        return 0;
    const float dist = std::sqrt(distSq);
    const V3 n = dist > 1.0e-6f ? d / dist : V3{0, 0, 1};
    basis = orthonormal(-n);
    sink.add(a.center + n * a.radius, b.center - n * b.radius, 1);
    return sink.count;
}

int collideSphereBox(const Shape &a, const Shape &b, bool sphereIsA, float margin, ContactSink &sink, M3 &basis) {
    const Shape &sphere = sphereIsA ? a : b;
    const Shape &box = sphereIsA ? b : a;
    const V3 local = qrot(qconj(box.rot), sphere.center - box.center);
    const V3 cl{sclamp(local.x, -box.half.x, box.half.x), sclamp(local.y, -box.half.y, box.half.y),
                sclamp(local.z, -box.half.z, box.half.z)};
    const V3 closest = qrot(box.rot, cl) + box.center;
    const V3 d = sphere.center - closest;
    const float distSq = length2(d);
    const float radPlus = sphere.radius + margin;
    if (distSq >= radPlus * radPlus)
        return 0;
    const float dist = std::sqrt(distSq);
    V3 n;
    if (dist > 1.0e-6f) {
        n = d / dist;
    } else {
        float depth;
        if (!pointInBox(box, sphere.center, n, depth))
            return 0;
    }
    basis = orthonormal(-(sphereIsA ? -n : n));
    const V3 onSphere = sphere.center - n * sphere.radius;
    sink.add(sphereIsA ? onSphere : closest, sphereIsA ? closest : onSphere, 1);
    return sink.count;
}

int collideSphereCylinder(const Shape &a, const Shape &b, bool sphereIsA, float margin, ContactSink &sink,
                          M3 &basis) {
    const Shape &sphere = sphereIsA ? a : b;
    const Shape &cyl = sphereIsA ? b : a;
    V3 outward;
    float distance;
    const V3 onCyl = closestPointOnCylinder(cyl, sphere.center, outward, distance);
    if (distance >= sphere.radius + margin)
        return 0;
    basis = orthonormal(-(sphereIsA ? -outward : outward));
    const V3 onSphere = sphere.center - outward * sphere.radius;
    sink.add(sphereIsA ? onSphere : onCyl, sphereIsA ? onCyl : onSphere, 1);
    return sink.count;
}

int collideCylinderBox(const Shape &a, const Shape &b, bool cylIsA, float margin, ContactSink &sink, M3 &basis) {
    const Shape &cyl = cylIsA ? a : b;
    const Shape &box = cylIsA ? b : a;
    Candidate cand[kMaxCandidates];
    int nc = 0;
    V3 normalAB{0, 0, 0};
    V3 samples[kMaxCylSamples];
    int ns = 0;
    cylinderSamples(cyl, samples, ns);
    for (int i = 0; i < ns && nc < kMaxCandidates; ++i) {
        V3 push;
        float depth;
        if (!sampleInsideBox(box, samples[i], margin, push, depth))
            continue;
        Candidate &c = cand[nc++];
        c.xA = cylIsA ? samples[i] : samples[i] + push * depth;
        c.xB = cylIsA ? samples[i] + push * depth : samples[i];
        c.normal = cylIsA ? -push : push;
        c.depth = depth;
        c.feature = (kAxisCylSample << 24) | ((cylIsA ? 1u : 0u) << 20) | static_cast<uint32_t>(i);
        normalAB += c.normal;
    }
    for (int corner = 0; corner < 8 && nc < kMaxCandidates; ++corner) {
        const V3 cl{(corner & 1) ? box.half.x : -box.half.x, (corner & 2) ? box.half.y : -box.half.y,
                    (corner & 4) ? box.half.z : -box.half.z};
        const V3 cw = qrot(box.rot, cl) + box.center;
        V3 push;
        float surf;
        if (!sampleInsideCylinder(cyl, cw, margin, push, surf))
            continue;
        Candidate &c = cand[nc++];
        c.xA = cylIsA ? cw + push * surf : cw;
        c.xB = cylIsA ? cw : cw + push * surf;
        c.normal = cylIsA ? push : -push;
        c.depth = surf;
        c.feature = (kAxisCylCorner << 24) | ((cylIsA ? 0u : 1u) << 20) | static_cast<uint32_t>(corner);
        normalAB += c.normal;
    }
    if (!nc)
        return 0;
    basis = orthonormal(-(length2(normalAB) > 1.0e-12f ? normalize(normalAB) : cyl.axis));
    emitRanked(cand, nc, sink);
    return sink.count;
}

int collideCylinderCylinder(const Shape &a, const Shape &b, float margin, ContactSink &sink, M3 &basis) {
    Candidate cand[kMaxCandidates];
    int nc = 0;
    V3 normalAB{0, 0, 0};
    V3 samples[kMaxCylSamples];
    const Shape *pair[2] = {&a, &b};
    for (int pass = 0; pass < 2; ++pass) {
        const Shape &from = *pair[pass];
        const Shape &into = *pair[pass == 0 ? 1 : 0];
        const bool fromIsA = pass == 0;
        int ns = 0;
        cylinderSamples(from, samples, ns);
        for (int i = 0; i < ns && nc < kMaxCandidates; ++i) {
            V3 push;
            float surf;
            if (!sampleInsideCylinder(into, samples[i], margin, push, surf))
                continue;
            Candidate &c = cand[nc++];
            c.xA = fromIsA ? samples[i] : samples[i] + push * surf;
            c.xB = fromIsA ? samples[i] + push * surf : samples[i];
            c.normal = fromIsA ? -push : push;
            c.depth = surf;
            c.feature = (kAxisCylSample << 24) | ((fromIsA ? 1u : 0u) << 20) | static_cast<uint32_t>(i);
            normalAB += c.normal;
        }
    }
    if (!nc)
        return 0;
    basis = orthonormal(-(length2(normalAB) > 1.0e-12f ? normalize(normalAB) : a.axis));
    emitRanked(cand, nc, sink);
    return sink.count;
}

// collideShapes' dispatch for pairs with a sphere or cylinder (collide.cpp:1001-1027).
int collideRound(const Body &A, const Body &B, float margin, Contact *out, M3 &basis) {
    const Shape a = makeShape(A), b = makeShape(B);
    const Obb oa{a.center, a.rot, a.half, {}}, ob{b.center, b.rot, b.half, {}};
    ContactSink sink{oa, ob, out, 0, {}};
    if (a.type == 1 && b.type == 1)
        return collideSphereSphere(a, b, margin, sink, basis);
    if (a.type == 1 || b.type == 1) {
        const bool sphereIsA = a.type == 1;
        if (a.type == 2 || b.type == 2)
            return collideSphereCylinder(a, b, sphereIsA, margin, sink, basis);
        return collideSphereBox(a, b, sphereIsA, margin, sink, basis);
    }
    if (a.type == 2 && b.type == 2)
        return collideCylinderCylinder(a, b, margin, sink, basis);
    return collideCylinderBox(a, b, a.type == 2, margin, sink, basis);
}

} // namespace

int World::collide(const Body &A, const Body &B, Contact *out, M3 &basis) const {
    float margin = P.speculative_margin;
    if (margin > 0.0f) {
        const float horizon = collisionDt;
        const float gA = A.mass > 0.0f ? A.gravity : 0.0f;
        const float gB = B.mass > 0.0f ? B.gravity : 0.0f;
        const V3 disp = (A.v - B.v) * horizon + V3{0, 0, (gA - gB) * horizon * horizon};
        margin += length(disp) + (A.radius * length(A.w) + B.radius * length(B.w)) * horizon;
    }
    if (A.shape != 0 || B.shape != 0)
        return collideRound(A, B, margin, out, basis);
    return collideBoxes(A.x, A.q, A.size * 0.5f, B.x, B.q, B.size * 0.5f, margin, out, basis);
}

// ManifoldStore::initialize (manifold.cpp:237-435), contact grace disabled.
bool World::manifoldInitialize(Manifold &m) {
    const Body &A = bodies[m.a];
    const Body &B = bodies[m.b];
    m.mu = std::sqrt(A.friction * B.friction);
    m.flags = 0;
    // Grace revival (manifold.cpp:249-253): a dormant manifold re-enters with its saved contacts.
    if (m.n == 0 && m.dormantSaved > 0)
        m.n = m.dormantSaved;
    const int liveCount = m.n;
    Contact nc[kMaxContacts];
    const int n = collide(A, B, nc, m.basis);
    V3 newK[kMaxContacts], newLam[kMaxContacts];
    uint8_t newStick[kMaxContacts];
    float newBeta[kMaxContacts], prevErr[kMaxContacts];
    for (int i = 0; i < kMaxContacts; i++) {
        newK[i] = newLam[i] = V3{0, 0, 0};
        newStick[i] = 0;
        newBeta[i] = 1.0f;
        prevErr[i] = -1.0f;
    }
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < m.n; j++) {
            const Contact &old = m.c[j];
            if (nc[i].key != old.key)
                continue;
            const V3 newRA = nc[i].rA, newRB = nc[i].rB;
            nc[i].key = old.key;
            nc[i].rA = old.rA;
            nc[i].rB = old.rB;
            prevErr[i] = smax(0.0f, COLLISION_MARGIN - old.C0.x);
            newK[i] = old.k;
            newLam[i] = old.lam;
            newStick[i] = old.stick;
            newBeta[i] = old.betaScale;
            if (!old.stick) {
                nc[i].rA = newRA;
                nc[i].rB = newRB;
            } else {
                const V3 oldA = A.x + qrot(A.q, old.rA);
                const V3 oldB = B.x + qrot(B.q, old.rB);
                const V3 nA = A.x + qrot(A.q, newRA);
                const V3 nB = B.x + qrot(B.q, newRB);
                const float drift = smax(length(oldA - nA), length(oldB - nB));
                if (drift > P.stick_drift_heal) {
                    nc[i].rA = newRA;
                    nc[i].rB = newRB;
                    newStick[i] = 0;
                    newLam[i] = V3{newLam[i].x, 0.0f, 0.0f};
                }
            }
            break;
        }
    }
    // Fresh contacts seed their penalty when grace is on (manifold.cpp:339-347).
    if (P.contact_grace_ticks > 0) {
        const float seed = smax(PENALTY_MIN, 0.05f * P.beta_lin);
        for (int i = 0; i < n; i++)
            if (prevErr[i] < 0.0f)
                newK[i] = V3{seed, seed, seed};
    }
    m.n = n;
    for (int i = 0; i < n; i++) {
        Contact &c = m.c[i];
        c.key = nc[i].key;
        c.rA = nc[i].rA;
        c.rB = nc[i].rB;
        c.k = newK[i];
        c.lam = newLam[i];
        c.stick = newStick[i];
        c.betaScale = newBeta[i];
    }
    // Grace dormancy (manifold.cpp:359-378): park without contacts, force dropped, state kept.
    if (m.n == 0) {
        if (P.contact_grace_ticks > 0 && m.dormantTicks < P.contact_grace_ticks) {
            for (int i = 0; i < liveCount; i++) {
                m.c[i].lam = V3{0, 0, 0};
                m.c[i].stick = 0;
            }
            m.dormantTicks++;
            m.dormantSaved = liveCount;
            return false;
        }
        m.dormantSaved = 0;
    }
    m.dormantTicks = 0;
    for (int i = 0; i < n; i++) {
        Contact &c = m.c[i];
        const V3 xA = A.x + qrot(A.q, c.rA);
        const V3 xB = B.x + qrot(B.q, c.rB);
        c.C0 = mul(m.basis, xA - xB) + V3{COLLISION_MARGIN, 0, 0};
        if (c.C0.x < -P.max_penetration)
            c.C0.x = -P.max_penetration;
        if (P.adaptive_beta && prevErr[i] >= 0.0f) {
            const float err = smax(0.0f, COLLISION_MARGIN - c.C0.x);
            const float fl = P.adaptive_beta_error_floor;
            float scale = newBeta[i];
            if (err <= fl)
                scale = smax(scale * 0.5f, 1.0f);
            else if (prevErr[i] <= fl)
                scale = smin(scale * 2.0f, ADAPTIVE_BETA_MAX);
            else if (err > 0.5f * prevErr[i])
                scale = smin(scale * 2.0f, ADAPTIVE_BETA_MAX);
            else if (err < 0.1f * prevErr[i])
                scale = smax(scale * 0.5f, 1.0f);
            c.betaScale = scale;
        } else {
            c.betaScale = 1.0f;
        }
        if (c.C0.x > kReleaseAbove) {
            c.lam = V3{0, 0, 0};
            c.stick = 0;
        }
        c.lam = c.lam * P.alpha * P.gamma;
        c.k = lclampv(c.k * P.gamma, V3{PENALTY_MIN, PENALTY_MIN, PENALTY_MIN},
                      V3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
        basisHessian(m.basis, c.k, c.S);
    }
    return m.n > 0;
}

bool World::frozen(const Manifold &m) const {
    const auto awake = [](const Body &b) { return b.mass > 0.0f && !b.sleeping; };
    return !awake(bodies[m.a]) && !awake(bodies[m.b]);
}

void World::decayPenalty(Manifold &m, float decay) {
    for (int i = 0; i < m.n; i++)
        m.c[i].k = lclampv(m.c[i].k * decay, V3{PENALTY_MIN, PENALTY_MIN, PENALTY_MIN},
                           V3{PENALTY_MAX, PENALTY_MAX, PENALTY_MAX});
}

// ManifoldStore::rebase (manifold.cpp:448-461).
void World::rebase(Manifold &m) {
    const Body &A = bodies[m.a];
    const Body &B = bodies[m.b];
    for (int i = 0; i < m.n; i++) {
        Contact &c = m.c[i];
        const V3 xA = A.x + qrot(A.q, c.rA);
        const V3 xB = B.x + qrot(B.q, c.rB);
        c.C0 = mul(m.basis, xA - xB) + V3{COLLISION_MARGIN, 0, 0};
        if (c.C0.x < -P.max_penetration)
            c.C0.x = -P.max_penetration;
    }
    m.flags = static_cast<uint8_t>(m.flags & ~kPrimalCacheReady);
}

// ManifoldStore::preCompute (manifold.cpp:465-501).
void World::preCompute(Manifold &m) {
    const Body &A = bodies[m.a];
    const Body &B = bodies[m.b];
    const V3 dqALin = A.x - A.x0;
    const V3 dqAAng = qdiff(A.q, A.q0);
    const V3 dqBLin = B.x - B.x0;
    const V3 dqBAng = qdiff(B.q, B.q0);
    const M3 rotA = qmat(A.q);
    const M3 rotB = qmat(B.q);
    const bool spec = P.speculative_margin > 0.0f;
    for (int i = 0; i < m.n; i++) {
        Contact &c = m.c[i];
        const V3 rA = mul(rotA, c.rA);
        const V3 rB = mul(rotB, c.rB);
        c.rAW = rA;
        c.rBW = rB;
        const V3 bracket = ((dqALin - dqBLin) + cross(dqAAng, rA)) - cross(dqBAng, rB);
        const V3 C = constraintError(c.C0, bracket, m.basis, 1 - P.alpha, spec);
        V3 F = cmul(c.k, C) + c.lam;
        clampForce(F, m.mu);
        c.F = F;
    }
    m.flags = static_cast<uint8_t>(m.flags | kPrimalCacheReady);
}

// ManifoldStore::stampCached (manifold.cpp:503-570).
void World::stampCached(const Manifold &m, int body, Block &blk) const {
    const bool fromA = body == m.a;
    const float side = fromA ? 1.0f : -1.0f;
    const V3 b0 = mrow(m.basis, 0), b1 = mrow(m.basis, 1), b2 = mrow(m.basis, 2);
    M3 accLin = mzero(), accAng = mzero(), accCross = mzero();
    V3 accRhsLin{0, 0, 0}, accRhsAng{0, 0, 0};
    for (int i = 0; i < m.n; i++) {
        const Contact &c = m.c[i];
        const V3 F = c.F;
        const V3 r = fromA ? c.rAW : c.rBW;
        const float s00 = c.S[0], s01 = c.S[1], s02 = c.S[2], s11 = c.S[3], s12 = c.S[4], s22 = c.S[5];
        const M3 S = mcols(V3{s00, s01, s02}, V3{s01, s11, s12}, V3{s02, s12, s22});
        const M3 RS = mcols(cross(r, S.c[0]), cross(r, S.c[1]), cross(r, S.c[2]));
        const float rx2 = r.x * r.x, ry2 = r.y * r.y, rz2 = r.z * r.z;
        const float rxy = r.x * r.y, rxz = r.x * r.z, ryz = r.y * r.z;
        const float h00 = s11 * rz2 - 2.0f * s12 * ryz + s22 * ry2;
        const float h11 = s22 * rx2 - 2.0f * s02 * rxz + s00 * rz2;
        const float h22 = s00 * ry2 - 2.0f * s01 * rxy + s11 * rx2;
        const float h01 = s12 * rxz + s02 * ryz - s22 * rxy - s01 * rz2;
        const float h02 = s12 * rxy + s01 * ryz - s11 * rxz - s02 * ry2;
        const float h12 = s02 * rxy + s01 * rxz - s00 * ryz - s12 * rx2;
        const V3 fw = b0 * F.x + b1 * F.y + b2 * F.z;
        const V3 fwAng = cross(r, fw);
        accLin += S;
        accAng += mcols(V3{h00, h01, h02}, V3{h01, h11, h12}, V3{h02, h12, h22});
        accCross += RS;
        accRhsLin += fw;
        accRhsAng += fwAng;
    }
    blk.lhsLin += accLin;
    blk.lhsAng += accAng;
    blk.lhsCross += accCross;
    blk.rhsLin += accRhsLin * side;
    blk.rhsAng += accRhsAng * side;
}

// ManifoldStore::updatePrimal (manifold.cpp:572-581).
void World::manifoldUpdatePrimal(Manifold &m, int body, Block &blk) {
    if ((m.flags & kPrimalCacheReady) == 0)
        preCompute(m);
    stampCached(m, body, blk);
    m.flags = static_cast<uint8_t>(m.flags & ~kPrimalCacheReady);
}

// ManifoldStore::updateDual (manifold.cpp:583-671), with the drift-gated arm cache
// (jacobianRebuildDistance, :600-608, 662-667).
void World::manifoldUpdateDual(Manifold &m) {
    const Body &A = bodies[m.a];
    const Body &B = bodies[m.b];
    const V3 dqALin = A.x - A.x0;
    const V3 dqAAng = qdiff(A.q, A.q0);
    const V3 dqBLin = B.x - B.x0;
    const V3 dqBAng = qdiff(B.q, B.q0);
    const M3 rotA = qmat(A.q);
    const M3 rotB = qmat(B.q);
    const bool cacheable = P.jacobian_rebuild_distance > 0.0f;
    const float rebuild2 = P.jacobian_rebuild_distance * P.jacobian_rebuild_distance;
    const V3 dA = rotA.c[0] - m.rotACap;
    const V3 dB = rotB.c[0] - m.rotBCap;
    const bool driftUsable = cacheable && (m.flags & kArmsCached) != 0 && length2(dA) <= rebuild2 &&
                             length2(dB) <= rebuild2;
    const bool spec = P.speculative_margin > 0.0f;
    for (int i = 0; i < m.n; i++) {
        Contact &c = m.c[i];
        V3 rA, rB;
        if (driftUsable) {
            rA = c.rAW;
            rB = c.rBW;
        } else {
            rA = mul(rotA, c.rA);
            rB = mul(rotB, c.rB);
            c.rAW = rA;
            c.rBW = rB;
        }
        const V3 bracket = ((dqALin - dqBLin) + cross(dqAAng, rA)) - cross(dqBAng, rB);
        const V3 C = constraintError(c.C0, bracket, m.basis, 1 - P.alpha, spec);
        V3 F = cmul(c.k, C) + c.lam;
        const Cone cone = clampForce(F, m.mu);
        c.lam = F;
        const float beta = P.beta_lin * c.betaScale;
        if (F.x < 0)
            c.k.x = smin(c.k.x + beta * std::fabs(C.x), PENALTY_MAX);
        if (cone.scale <= cone.bounds) {
            c.k.y = smin(c.k.y + beta * std::fabs(C.y), PENALTY_MAX);
            c.k.z = smin(c.k.z + beta * std::fabs(C.z), PENALTY_MAX);
            c.stick = length2d(C.y, C.z) < STICK_THRESH;
        }
        basisHessian(m.basis, c.k, c.S);
        V3 fNext = cmul(c.k, C) + c.lam;
        clampForce(fNext, m.mu);
        c.F = fNext;
    }
    if (!driftUsable && cacheable) {
        m.rotACap = rotA.c[0];
        m.rotBCap = rotB.c[0];
        m.flags = static_cast<uint8_t>(m.flags | kArmsCached);
    }
    m.flags = static_cast<uint8_t>(m.flags | kPrimalCacheReady);
}

// ------------------------------------------------------------------------------------------
// Step phases
// ------------------------------------------------------------------------------------------

// ForceAdjacency::build (manifold.cpp:123-166): per list index, forces in list order, then
// manifolds in live order.
void World::buildAdjacency() {
    const int n = count();
    adjStart.assign(n + 1, 0);
    for (const Force &f : forces) {
        if (f.a >= 0)
            adjStart[listIndex(f.a) + 1]++;
        if (f.b >= 0)
            adjStart[listIndex(f.b) + 1]++;
    }
    for (const Manifold &m : live) {
        adjStart[listIndex(m.a) + 1]++;
        adjStart[listIndex(m.b) + 1]++;
    }
    for (int i = 0; i < n; i++)
        adjStart[i + 1] += adjStart[i];
    adjRefs.assign(adjStart[n], Ref{false, 0});
    std::vector<int> cursor(adjStart.begin(), adjStart.begin() + n);
    for (int fi = 0; fi < (int)forces.size(); fi++) {
        const Force &f = forces[fi];
        if (f.a >= 0)
            adjRefs[cursor[listIndex(f.a)]++] = Ref{false, fi};
        if (f.b >= 0)
            adjRefs[cursor[listIndex(f.b)]++] = Ref{false, fi};
    }
    for (int mi = 0; mi < (int)live.size(); mi++) {
        adjRefs[cursor[listIndex(live[mi].a)]++] = Ref{true, mi};
        adjRefs[cursor[listIndex(live[mi].b)]++] = Ref{true, mi};
    }
}

// otherBody (solver_internal.hpp:46-66): -1 = none / world.
int World::otherBody(const Ref &r, int body) const {
    int a, b;
    if (r.manifold) {
        a = live[r.index].a;
        b = live[r.index].b;
    } else {
        a = forces[r.index].a;
        b = forces[r.index].b;
    }
    if (a == body)
        return b;
    if (b == body)
        return a;
    return -1;
}

// pairConstrained (solver_internal.hpp:70-86), grace disabled.
bool World::pairConstrained(int a, int b) const {
    const int li = listIndex(a);
    for (int k = adjStart[li]; k < adjStart[li + 1]; k++)
        if (otherBody(adjRefs[k], a) == b)
            return true;
    return false;
}

namespace {

uint64_t expandBits21(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10cfcfcfcfcfcfcfull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

uint32_t quantise(float v, float lo, float scale) {
    return static_cast<uint32_t>(sclamp((v - lo) * scale, 0.0f, 2097151.0f));
}

struct Node {
    V3 mn, mx;
    int left, right; // left < 0: leaf, right = body list index
};

} // namespace

// Solver::broadPhase (solver_broadphase.cpp:85-186) with the LBVH of bvh_broadphase.cpp:61-292.
void World::broadPhase() {
    const int n = count();
    buildAdjacency();
    if (n < 2) {
        codes.clear();
        order.clear();
        pairs.clear();
        return;
    }
    aabbCenter.resize(n);
    aabbHalf.resize(n);
    const float cdt = collisionDt;
    for (int i = 0; i < n; i++) {
        const Body &b = bodies[idAt(i)];
        const M3 rot = qmat(b.q);
        // aabbHalfExtent (rigid.cpp:83-106): sphere (r, r, r), cylinder (r, r, h/2), box size/2.
        const V3 h = b.shape == 1 ? V3{b.size.x, b.size.x, b.size.x}
                                  : (b.shape == 2 ? V3{b.size.x, b.size.x, b.size.z * 0.5f} : b.size * 0.5f);
        const V3 tight{(std::fabs(rot.c[0][0]) * h.x + std::fabs(rot.c[1][0]) * h.y) + std::fabs(rot.c[2][0]) * h.z,
                       (std::fabs(rot.c[0][1]) * h.x + std::fabs(rot.c[1][1]) * h.y) + std::fabs(rot.c[2][1]) * h.z,
                       (std::fabs(rot.c[0][2]) * h.x + std::fabs(rot.c[1][2]) * h.y) + std::fabs(rot.c[2][2]) * h.z};
        V3 disp = b.v * cdt;
        if (b.mass > 0)
            disp += V3{0, 0, b.gravity * cdt * cdt};
        const float rotSweep = b.radius * length(b.w) * cdt;
        const float grow = rotSweep + P.speculative_margin;
        aabbCenter[i] = b.x + disp * 0.5f;
        aabbHalf[i] = (tight + vabs(disp) * 0.5f) + V3{grow, grow, grow};
    }

    // Morton codes over AABB centres; lo.x is the origin of all three axes (bvh_broadphase.cpp:85).
    V3 lo{FLT_MAX, FLT_MAX, FLT_MAX};
    V3 hi{std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(),
          std::numeric_limits<float>::lowest()};
    for (int i = 0; i < n; i++) {
        const V3 c = aabbCenter[i];
        lo = V3{smin(lo.x, c.x), smin(lo.y, c.y), smin(lo.z, c.z)};
        hi = V3{smax(hi.x, c.x), smax(hi.y, c.y), smax(hi.z, c.z)};
    }
    const V3 ext = hi - lo;
    float ex = ext.x;
    if (ex < ext.y)
        ex = ext.y;
    if (ex < ext.z)
        ex = ext.z;
    if (ex < 1.0e-6f)
        ex = 1.0e-6f;
    const float scale = 2097151.0f / ex;
    // The reference refreshes its codes and order only when it rebuilds the tree: the body set
    // changed or 16 refits have passed (bvh_broadphase.cpp:186-203). The candidate set does not
    // depend on the tree, so the oracle walks a fresh tree every step but keeps the reference's
    // code/order schedule for the diagnostic dumps.
    if (treeBodies != n || treeAge >= 16) {
        codes.resize(n);
        for (int i = 0; i < n; i++) {
            const V3 c = aabbCenter[i];
            codes[i] = expandBits21(quantise(c.x, lo.x, scale)) | (expandBits21(quantise(c.y, lo.x, scale)) << 1) |
                       (expandBits21(quantise(c.z, lo.x, scale)) << 2);
        }
        order.resize(n);
        for (int i = 0; i < n; i++)
            order[i] = i;
        std::sort(order.begin(), order.end(), [this](int a, int b) {
            if (codes[a] != codes[b])
                return codes[a] < codes[b];
            return a < b;
        });
        treeBodies = n;
        treeAge = 0;
    } else {
        treeAge++;
    }

    // Pairwise bottom-up merge of the sorted leaves, bounds by min/max of the children.
    std::vector<Node> nodes;
    nodes.reserve(2 * n);
    std::vector<int> level;
    for (int i = 0; i < n; i++) {
        const int b = order[i];
        nodes.push_back(Node{aabbCenter[b] - aabbHalf[b], aabbCenter[b] + aabbHalf[b], -1, b});
        level.push_back(static_cast<int>(nodes.size()) - 1);
    }
    while (level.size() > 1) {
        std::vector<int> next;
        for (size_t i = 0; i + 1 < level.size(); i += 2) {
            const Node &a = nodes[level[i]];
            const Node &b = nodes[level[i + 1]];
            Node p{V3{smin(a.mn.x, b.mn.x), smin(a.mn.y, b.mn.y), smin(a.mn.z, b.mn.z)},
                   V3{smax(a.mx.x, b.mx.x), smax(a.mx.y, b.mx.y), smax(a.mx.z, b.mx.z)}, level[i], level[i + 1]};
            nodes.push_back(p);
            next.push_back(static_cast<int>(nodes.size()) - 1);
        }
        if (level.size() % 2 == 1)
            next.push_back(level.back());
        level.swap(next);
    }
    const int root = level[0];
    const auto overlaps = [&nodes](int a, int b) {
        const Node &x = nodes[a];
        const Node &y = nodes[b];
        return !(y.mn.x > x.mx.x || y.mx.x < x.mn.x || y.mn.y > x.mx.y || y.mx.y < x.mn.y ||
                 y.mn.z > x.mx.z || y.mx.z < x.mn.z);
    };
    pairs.clear();
    std::vector<std::pair<int, int>> stack;
    stack.push_back({root, root});
    const auto push = [&](int a, int b) {
        if (a == b) {
            if (nodes[a].left >= 0)
                stack.push_back({a, b});
            return;
        }
        if (overlaps(a, b))
            stack.push_back({a, b});
    };
    while (!stack.empty()) {
        const auto ab = stack.back();
        stack.pop_back();
        const int a = ab.first, b = ab.second;
        if (a == b) {
            push(nodes[a].left, nodes[a].left);
            push(nodes[a].left, nodes[a].right);
            push(nodes[a].right, nodes[a].right);
            continue;
        }
        const bool aLeaf = nodes[a].left < 0, bLeaf = nodes[b].left < 0;
        if (aLeaf && bLeaf) {
            const uint64_t i = static_cast<uint32_t>(nodes[a].right), j = static_cast<uint32_t>(nodes[b].right);
            pairs.push_back(i < j ? (i << 32) | j : (j << 32) | i);
        } else if (aLeaf) {
            push(a, nodes[b].left);
            push(a, nodes[b].right);
        } else if (bLeaf) {
            push(nodes[a].left, b);
            push(nodes[a].right, b);
        } else {
            push(nodes[a].left, nodes[b].left);
            push(nodes[a].left, nodes[b].right);
            push(nodes[a].right, nodes[b].left);
            push(nodes[a].right, nodes[b].right);
        }
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());

    // Exact filter (pairOverlaps, solver_broadphase.cpp:30-65) then serial acquisition in key order.
    std::vector<uint8_t> valid(pairs.size(), 0);
    for (size_t k = 0; k < pairs.size(); k++) {
        const int i = static_cast<int>(pairs[k] >> 32);
        const int j = static_cast<int>(pairs[k] & 0xffffffffu);
        const int ia = idAt(i), ib = idAt(j);
        const Body &A = bodies[ia];
        const Body &B = bodies[ib];
        const V3 aMin = aabbCenter[i] - aabbHalf[i], aMax = aabbCenter[i] + aabbHalf[i];
        const V3 bMin = aabbCenter[j] - aabbHalf[j], bMax = aabbCenter[j] + aabbHalf[j];
        const bool bounds = !(bMin.x > aMax.x || bMin.y > aMax.y || bMin.z > aMax.z || aMin.x > bMax.x ||
                              aMin.y > bMax.y || aMin.z > bMax.z);
        const bool layers = ((A.layer & B.mask) != 0) || ((B.layer & A.mask) != 0);
        const bool bothStatic = A.mass <= 0.0f && B.mass <= 0.0f;
        valid[k] = bounds && layers && !pairConstrained(ia, ib) && !bothStatic;
    }
    for (size_t k = 0; k < pairs.size(); k++) {
        if (!valid[k])
            continue;
        const int ia = idAt(static_cast<int>(pairs[k] >> 32));
        const int ib = idAt(static_cast<int>(pairs[k] & 0xffffffffu));
        // wakeSleeperPair (solver_broadphase.cpp:69-81), in pair order: a body woken by an earlier
        // pair wakes the sleepers of later pairs.
        Body &A = bodies[ia], &B = bodies[ib];
        if (A.sleeping && !B.sleeping && B.mass > 0.0f) {
            A.sleeping = false;
            A.stillFrames = 0;
        } else if (B.sleeping && !A.sleeping && A.mass > 0.0f) {
            B.sleeping = false;
            B.stillFrames = 0;
        }
        bool exists = false;
        const int li = listIndex(ia);
        for (int r = adjStart[li]; r < adjStart[li + 1]; r++)
            if (adjRefs[r].manifold && otherBody(adjRefs[r], ia) == ib) {
                exists = true;
                break;
            }
        if (exists)
            continue;
        Manifold m;
        m.a = ia;
        m.b = ib;
        live.push_back(m);
    }
}

// Solver::warmstartForces (solver_solve.cpp:31-105), grace disabled.
int World::warmstartForces() {
    std::vector<Force> kept;
    kept.reserve(forces.size());
    for (Force &f : forces)
        if (f.kind == kGeneric ? (genericInitialize(f), true) : jointInitialize(f))
            kept.push_back(f);
    forces.swap(kept);
    // Independent per manifold (the reference dispatches this loop to its pool too); the stable
    // compaction stays serial.
    const int nm = static_cast<int>(live.size());
    std::vector<uint8_t> active(nm);
#pragma omp parallel for schedule(dynamic, 64) if (parallel())
    for (int i = 0; i < nm; i++)
        active[i] = frozen(live[i]) || manifoldInitialize(live[i]);
    std::vector<Manifold> keptM;
    keptM.reserve(live.size());
    for (int i = 0; i < nm; i++)
        if (active[i] || (P.contact_grace_ticks > 0 && live[i].dormantTicks > 0))
            keptM.push_back(live[i]);
    live.swap(keptM);
    buildAdjacency();
    return static_cast<int>(forces.size());
}

// Solver::islandSleep (solver_solve.cpp:179-250): sleep-enabled movable bodies joined by
// manifolds and forces sleep together once every member passed idle detection.
void World::islandSleep() {
    std::vector<int> members;
    for (int li = 0; li < count(); li++) {
        const int id = idAt(li);
        if (bodies[id].mass > 0 && bodies[id].sleepMode == 1)
            members.push_back(id);
    }
    const int n = static_cast<int>(members.size());
    if (n < 2)
        return;
    std::vector<int> parent(n), slot(bodies.size(), -1);
    for (int i = 0; i < n; i++) {
        parent[i] = i;
        slot[members[i]] = i;
    }
    const auto find = [&parent](int x) {
        while (parent[x] != x)
            x = parent[x] = parent[parent[x]];
        return x;
    };
    const auto join = [&](int a, int b) {
        if (a < 0 || b < 0 || slot[a] < 0 || slot[b] < 0)
            return;
        parent[find(slot[a])] = find(slot[b]);
    };
    for (const Manifold &m : live)
        join(m.a, m.b);
    for (const Force &f : forces)
        join(f.a, f.b);
    std::vector<char> awake(n, 0);
    std::vector<int> still(n, INT_MAX);
    for (int i = 0; i < n; i++) {
        const int r = find(i);
        if (!bodies[members[i]].sleeping)
            awake[r] = 1;
        still[r] = std::min(still[r], bodies[members[i]].stillFrames);
    }
    for (int i = 0; i < n; i++) {
        const int r = find(i);
        if (awake[r] || still[r] < P.sleep_frames)
            continue;
        Body &b = bodies[members[i]];
        if (!b.sleeping) {
            b.sleeping = true;
            b.v = V3{0, 0, 0};
            b.w = V3{0, 0, 0};
        }
    }
}

// Solver::selectUpdateBodies (solver_solve.cpp:263-361).
void World::selectUpdateBodies() {
    if (P.sleep_frames > 0) {
        // Wake a sleeper touched (manifold or force) by a moving awake body; a body woken here has
        // zero velocity, so the order does not matter.
        const float lin2 = P.sleep_linear_threshold * P.sleep_linear_threshold;
        const float ang2 = P.sleep_angular_threshold * P.sleep_angular_threshold;
        for (int li = 0; li < count(); li++) {
            Body &b = bodies[idAt(li)];
            if (!b.sleeping || b.sleepMode != 1)
                continue;
            for (int r = adjStart[li]; r < adjStart[li + 1]; r++) {
                const int o = otherBody(adjRefs[r], idAt(li));
                if (o < 0)
                    continue;
                const Body &other = bodies[o];
                if (other.mass > 0 && !other.sleeping && (length2(other.v) > lin2 || length2(other.w) > ang2)) {
                    b.sleeping = false;
                    b.stillFrames = 0;
                    break;
                }
            }
        }
        islandSleep();
    }
    updateOrder.clear();
    for (int li = 0; li < count(); li++) {
        const int id = idAt(li);
        Body &b = bodies[id];
        b.inUpdate = false;
        b.updateIndex = -1;
        b.contactOnly = true;
        if (b.mass > 0) {
            bool update = true;
            if (b.sleepMode == 1) {
                if (b.sleeping)
                    update = false;
            } else if (b.sleepMode == 2) {
                if (!b.sleeping && length2(b.v) == 0.0f && adjStart[li] == adjStart[li + 1])
                    update = false;
                else
                    b.sleeping = false;
            }
            if (update) {
                b.updateIndex = static_cast<int>(updateOrder.size());
                updateOrder.push_back(id);
                b.inUpdate = true;
            }
        }
    }
    for (const Force &f : forces) {
        if (f.a >= 0)
            bodies[f.a].contactOnly = false;
        if (f.b >= 0)
            bodies[f.b].contactOnly = false;
    }
    colourGraph();
}

// Solver::colourGraph (solver_solve.cpp:365-424).
void World::colourGraph() {
    const int n = static_cast<int>(updateOrder.size());
    colour.assign(n, kOverflowColour);
    colourOrder.clear();
    overflowOrder.clear();
    for (int i = 0; i < n; i++) {
        const int id = updateOrder[i];
        uint8_t used[kMaxColours] = {};
        const int li = listIndex(id);
        for (int r = adjStart[li]; r < adjStart[li + 1]; r++) {
            const int other = otherBody(adjRefs[r], id);
            if (other < 0 || bodies[other].updateIndex < 0 || bodies[other].updateIndex >= i)
                continue;
            const uint8_t c = colour[bodies[other].updateIndex];
            if (c < kMaxColours)
                used[c] = 1;
        }
        uint8_t col = kOverflowColour;
        for (int c = 0; c < kMaxColours; c++)
            if (!used[c]) {
                col = static_cast<uint8_t>(c);
                break;
            }
        colour[i] = col;
    }
    colourBegins.assign(kMaxColours + 1, 0);
    for (int i = 0; i < n; i++) {
        if (P.contact_only_overflow && bodies[updateOrder[i]].contactOnly) {
            colour[i] = kOverflowColour;
            overflowOrder.push_back(i);
        }
        if (colour[i] != kOverflowColour)
            colourBegins[colour[i] + 1]++;
    }
    for (int c = 0; c < kMaxColours; c++)
        colourBegins[c + 1] += colourBegins[c];
    colourOrder.assign(n - overflowOrder.size(), 0);
    int cursor[kMaxColours];
    for (int c = 0; c < kMaxColours; c++)
        cursor[c] = colourBegins[c];
    for (int i = 0; i < n; i++)
        if (colour[i] < kMaxColours)
            colourOrder[cursor[colour[i]]++] = i;
    colourCount = 0;
    for (int c = 0; c < kMaxColours; c++)
        if (colourBegins[c + 1] > colourBegins[c])
            colourCount = c + 1;
    overflowCount = static_cast<int>(overflowOrder.size());
}

static void maskLocked(uint8_t locks, V3 &v) {
    if (locks)
        for (int k = 0; k < 3; ++k)
            if (locks & (1 << k))
                v[k] = 0.0f;
}

// Solver::warmstartBody (solver_solve.cpp:109-142).
void World::warmstartBody(Body &b) {
    const float dt = P.dt;
    maskLocked(b.lockLin, b.v);
    maskLocked(b.lockAng, b.w);
    const float g = (b.lockLin & 0x4) ? 0.0f : b.gravity;
    b.xi = b.x + b.v * dt;
    if (b.mass > 0)
        b.xi += V3{0, 0, g} * (dt * dt);
    b.qi = qintegrate(b.q, b.w * dt);
    const V3 accel = (b.v - b.vprev) / dt;
    const float accelExt = accel.z * std::copysign(1.0f, g);
    float weight = sclamp(accelExt / std::fabs(g), 0.0f, 1.0f);
    if (!std::isfinite(weight))
        weight = 0.0f;
    b.x0 = b.x;
    b.q0 = b.q;
    if (b.mass > 0) {
        b.x = b.x + b.v * dt + V3{0, 0, g} * (weight * dt * dt);
        b.q = qintegrate(b.q, b.w * dt);
    }
}

// Solver::finishBody (solver_solve.cpp:146-176).
void World::finishBody(Body &b, bool idleDetection) {
    const float dt = P.dt;
    b.vprev = b.v;
    if (b.mass > 0 && !b.sleeping) {
        b.v = (b.x - b.x0) / dt;
        b.w = qdiff(b.q, b.q0) / dt;
    }
    maskLocked(b.lockLin, b.v);
    maskLocked(b.lockAng, b.w);
    if (idleDetection && P.sleep_frames > 0 && b.mass > 0 && !b.sleeping && b.sleepMode == 1) {
        if (length2(b.v) < P.sleep_linear_threshold * P.sleep_linear_threshold &&
            length2(b.w) < P.sleep_angular_threshold * P.sleep_angular_threshold)
            ++b.stillFrames;
        else
            b.stillFrames = 0;
        if (b.stillFrames >= P.sleep_frames) {
            b.sleeping = true;
            b.v = V3{0, 0, 0};
            b.w = V3{0, 0, 0};
        }
    }
}

// Solver::iterateBody (solver_step.cpp:195-316) as the single-participant region.
void World::iterate(int rounds, int forceCount) {
    const float dtSq = P.dt * P.dt;
    const float alpha = P.alpha;
    const int newtonRounds =
            std::clamp(static_cast<int>(std::ceil(P.newton_ratio * static_cast<float>(rounds))), 1, rounds);
    std::vector<V3> dLin(updateOrder.size()), dAng(updateOrder.size());
    float prevResidual = 0.0f; // solver_step.cpp:88
    for (int it = 0; it < rounds; it++) {
        const bool newton = it < newtonRounds;
        for (int c = 0; newton && c < colourCount; c++) {
            // Bodies of one colour share no force: independent.
#pragma omp parallel for schedule(dynamic, 16) if (parallel())
            for (int k = colourBegins[c]; k < colourBegins[c + 1]; k++) {
                const int id = updateOrder[colourOrder[k]];
                Body &body = bodies[id];
                Block blk = makeBlock(body, dtSq);
                const int li = listIndex(id);
                for (int r = adjStart[li]; r < adjStart[li + 1]; r++) {
                    const Ref &ref = adjRefs[r];
                    if (ref.manifold)
                        manifoldUpdatePrimal(live[ref.index], id, blk);
                    else
                        forceUpdatePrimal(forces[ref.index], id, blk);
                }
                V3 dl, da;
                solveDelta(blk, dl, da);
                body.x = body.x + dl;
                body.q = qintegrate(body.q, da);
            }
        }
        const int ovf = newton ? overflowCount : 0;
        if (ovf > 0) {
            const int nm = static_cast<int>(live.size());
#pragma omp parallel for schedule(dynamic, 64) if (parallel())
            for (int mi = 0; mi < nm; mi++) {
                Manifold &m = live[mi];
                const Body &A = bodies[m.a];
                const Body &B = bodies[m.b];
                const bool aIn = A.inUpdate && colour[A.updateIndex] == kOverflowColour;
                const bool bIn = B.inUpdate && colour[B.updateIndex] == kOverflowColour;
                if (!aIn && !bIn)
                    continue;
                preCompute(m);
            }
#pragma omp parallel for schedule(dynamic, 16) if (parallel())
            for (int k = 0; k < ovf; k++) {
                const int i = overflowOrder[k];
                const int id = updateOrder[i];
                Block blk = makeBlock(bodies[id], dtSq);
                const int li = listIndex(id);
                for (int r = adjStart[li]; r < adjStart[li + 1]; r++) {
                    const Ref &ref = adjRefs[r];
                    if (ref.manifold)
                        stampCached(live[ref.index], id, blk);
                    else
                        forceUpdatePrimal(forces[ref.index], id, blk);
                }
                solveDelta(blk, dLin[i], dAng[i]);
            }
#pragma omp parallel for schedule(static) if (parallel())
            for (int k = 0; k < ovf; k++) {
                const int i = overflowOrder[k];
                Body &body = bodies[updateOrder[i]];
                body.x = body.x + dLin[i] * P.jacobi_relaxation;
                body.q = qintegrate(body.q, dAng[i] * P.jacobi_relaxation);
            }
        }
        const float decay = newton ? 1.0f : P.stiffness_decay;
        const int nm = static_cast<int>(live.size());
#pragma omp parallel for schedule(dynamic, 64) if (parallel())
        for (int mi = 0; mi < nm; mi++) {
            Manifold &m = live[mi];
            if (frozen(m))
                continue;
            if (decay < 1.0f)
                decayPenalty(m, decay);
            manifoldUpdateDual(m);
        }
#pragma omp parallel for schedule(static) if (parallel())
        for (int f = 0; f < forceCount; f++)
            forceUpdateDual(forces[f]);
        (void)alpha;
        // Convergence probe (solver_step.cpp:301-314, ManifoldStore::accumulatePenetration,
        // manifold.cpp:673-691): mean normal penetration of the step-start errors, in live order.
        if (P.convergence_threshold > 0.0f && it + 1 < rounds) {
            const bool spec = P.speculative_margin > 0.0f;
            float total = 0.0f;
            int cnt = 0;
            for (const Manifold &m : live)
                for (int i = 0; i < m.n; i++) {
                    if (spec && m.c[i].C0.x > 0.0f)
                        continue;
                    const float pen = -m.c[i].C0.x;
                    if (pen > 0.0f) {
                        total += pen;
                        cnt++;
                    }
                }
            const float residual = cnt > 0 ? total / static_cast<float>(cnt) : 0.0f;
            const bool converged = prevResidual - residual < P.convergence_threshold;
            prevResidual = residual;
            if (converged)
                break;
        }
    }
}

void World::runSubstep(int forceCount, int rounds, bool idleDetection) {
    const int n = count();
#pragma omp parallel for schedule(static) if (parallel())
    for (int li = 0; li < n; li++)
        warmstartBody(bodies[idAt(li)]);
    iterate(rounds, forceCount);
#pragma omp parallel for schedule(static) if (parallel())
    for (int li = 0; li < n; li++)
        finishBody(bodies[idAt(li)], idleDetection);
}

static float angularCompliance(const Body &b, V3 axis) {
    float sum = 0.0f;
    for (int k = 0; k < 3; k++)
        if (b.moment[k] > 0.0f)
            sum += axis[k] * axis[k] / b.moment[k];
    return sum;
}

static V3 angularResponse(const Body &b, V3 axis) {
    V3 out{0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; k++)
        if (b.moment[k] > 0.0f)
            out[k] = axis[k] / b.moment[k];
    return qrot(b.q, out);
}

// Solver::projectContacts (solver_projection.cpp:67-281).
void World::projectContacts(bool projectPositions, float brakeWindow) {
    if (live.empty())
        return;
    const float slop = P.projection_slop;
    const float beta = P.projection_beta;
    const float cap = P.projection_max_correction;
    const float window = brakeWindow > 0.0f ? brakeWindow : collisionDt;
    std::vector<int> active;
    for (int mi = 0; mi < (int)live.size(); mi++) {
        const Manifold &m = live[mi];
        if (m.n == 0)
            continue;
        const Body &A = bodies[m.a];
        const Body &B = bodies[m.b];
        if (!(A.mass > 0.0f && A.inUpdate) && !(B.mass > 0.0f && B.inUpdate))
            continue;
        active.push_back(mi);
    }
    if (active.empty())
        return;
    if (P.speculative_margin > 0.0f) {
        for (int mi : active) {
            const Manifold &m = live[mi];
            Body &A = bodies[m.a];
            Body &B = bodies[m.b];
            const bool moveA = A.mass > 0.0f && A.inUpdate;
            const bool moveB = B.mass > 0.0f && B.inUpdate;
            const float invMassA = moveA ? 1.0f / A.mass : 0.0f;
            const float invMassB = moveB ? 1.0f / B.mass : 0.0f;
            const V3 n = mrow(m.basis, 0);
            V3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
            float velErr = 0.0f;
            int braked = 0;
            for (int k = 0; k < m.n; k++) {
                const V3 rA = qrot(A.q, m.c[k].rA);
                const V3 rB = qrot(B.q, m.c[k].rB);
                const float gap = dot(n, (A.x + rA) - (B.x + rB));
                if (!(gap > 0.0f))
                    continue;
                const V3 vAp = A.v + cross(A.w, rA);
                const V3 vBp = B.v + cross(B.w, rB);
                const float vn = dot(vAp - vBp, n);
                const float target = -gap / window;
                if (vn < target) {
                    patchRA += rA;
                    patchRB += rB;
                    velErr += target - vn;
                    braked++;
                }
            }
            if (braked == 0)
                continue;
            const float invN = 1.0f / braked;
            const V3 tA = moveA ? qrot(qconj(A.q), cross(patchRA * invN, n)) : V3{0, 0, 0};
            const V3 tB = moveB ? qrot(qconj(B.q), cross(patchRB * invN, n)) : V3{0, 0, 0};
            const float K = invMassA + invMassB + (moveA ? angularCompliance(A, tA) : 0.0f) +
                            (moveB ? angularCompliance(B, tB) : 0.0f);
            const float j = velErr * invN / K;
            if (moveA) {
                V3 dv = n * (invMassA * j);
                V3 dw = angularResponse(A, tA) * j;
                maskLocked(A.lockLin, dv);
                maskLocked(A.lockAng, dw);
                A.v += dv;
                A.w += dw;
            }
            if (moveB) {
                V3 dv = n * (invMassB * j);
                V3 dw = angularResponse(B, tB) * j;
                maskLocked(B.lockLin, dv);
                maskLocked(B.lockAng, dw);
                B.v -= dv;
                B.w -= dw;
            }
        }
    }
    if (!projectPositions || P.projection_iterations <= 0)
        return;
    const size_t nu = updateOrder.size();
    std::vector<V3> pLin(nu), pAng(nu);
    std::vector<int> pCount(nu);
    const float depthTol = smax(slop * 0.01f, 1.0e-6f);
    for (int iter = 0; iter < P.projection_iterations; iter++) {
        std::fill(pCount.begin(), pCount.end(), 0);
        std::fill(pLin.begin(), pLin.end(), V3{0, 0, 0});
        std::fill(pAng.begin(), pAng.end(), V3{0, 0, 0});
        float maxDepth = 0.0f;
        for (int mi : active) {
            const Manifold &m = live[mi];
            const Body &A = bodies[m.a];
            const Body &B = bodies[m.b];
            const bool moveA = A.mass > 0.0f && A.inUpdate;
            const bool moveB = B.mass > 0.0f && B.inUpdate;
            const float invMassA = moveA ? 1.0f / A.mass : 0.0f;
            const float invMassB = moveB ? 1.0f / B.mass : 0.0f;
            const V3 n = mrow(m.basis, 0);
            V3 patchRA{0, 0, 0}, patchRB{0, 0, 0};
            float patchDepth = 0.0f;
            int corrected = 0;
            const M3 rotA = qmat(A.q);
            const M3 rotB = qmat(B.q);
            for (int k = 0; k < m.n; k++) {
                const V3 rA = mul(rotA, m.c[k].rA);
                const V3 rB = mul(rotB, m.c[k].rB);
                const float rawDepth = -dot(n, (A.x + rA) - (B.x + rB));
                const float depth = rawDepth - slop;
                if (depth > 0.0f) {
                    patchRA += rA;
                    patchRB += rB;
                    patchDepth += depth;
                    corrected++;
                }
            }
            if (corrected == 0)
                continue;
            const float invN = 1.0f / corrected;
            maxDepth = smax(maxDepth, patchDepth * invN);
            const V3 tA = moveA ? qrot(qconj(A.q), cross(patchRA * invN, n)) : V3{0, 0, 0};
            const V3 tB = moveB ? qrot(qconj(B.q), cross(patchRB * invN, n)) : V3{0, 0, 0};
            const float K = invMassA + invMassB + (moveA ? angularCompliance(A, tA) : 0.0f) +
                            (moveB ? angularCompliance(B, tB) : 0.0f);
            const float dp = beta * patchDepth * invN / K;
            if (moveA) {
                const int i = A.updateIndex;
                pCount[i]++;
                pLin[i] += n * (invMassA * dp);
                pAng[i] += angularResponse(A, tA) * dp;
            }
            if (moveB) {
                const int i = B.updateIndex;
                pCount[i]++;
                pLin[i] -= n * (invMassB * dp);
                pAng[i] -= angularResponse(B, tB) * dp;
            }
        }
        for (size_t i = 0; i < nu; i++) {
            Body &body = bodies[updateOrder[i]];
            const float invCount = 1.0f / std::max(pCount[i], 1);
            V3 dl = pLin[i] * invCount;
            V3 da = pAng[i] * invCount;
            maskLocked(body.lockLin, dl);
            maskLocked(body.lockAng, da);
            if (cap > 0.0f) {
                const float moved = length(dl);
                if (moved > cap)
                    dl = dl * (cap / moved);
                const float turned = length(da);
                if (turned > cap)
                    da = da * (cap / turned);
            }
            body.x = body.x + dl;
            body.q = qintegrate(body.q, da);
        }
        if (maxDepth <= depthTol)
            break;
    }
}

static void setThreads(int threads) {
#ifdef _OPENMP
    if (threads > 1)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

// Solver::step (solver_step.cpp:44-75).
void World::step() {
    setThreads(P.threads);
    collisionDt = P.dt;
    broadPhase();
    const int forceCount = warmstartForces();
    selectUpdateBodies();
    projectContacts(false, 0.0f);
    runSubstep(forceCount, P.iterations, true);
    projectContacts(P.position_projection != 0, 0.0f);
    for (Manifold &m : live)
        rebase(m);
    steps++;
}

// Solver::stepInterleaved (solver_step.cpp:109-160).
void World::stepInterleaved(int substeps, int roundsPerSubstep) {
    if (substeps <= 1) {
        step();
        return;
    }
    collisionDt = P.dt * substeps;
    broadPhase();
    const int forceCount = warmstartForces();
    selectUpdateBodies();
    const int rounds = roundsPerSubstep > 0 ? std::max(1, roundsPerSubstep)
                                            : std::max(2, (P.iterations + substeps - 1) / substeps);
    for (int sub = 0; sub < substeps; ++sub) {
        if (sub > 0)
            for (Manifold &m : live)
                rebase(m);
        projectContacts(false, P.dt * (substeps - sub));
        runSubstep(forceCount, rounds, sub + 1 == substeps);
    }
    projectContacts(P.position_projection != 0, collisionDt);
    for (Manifold &m : live)
        rebase(m);
    steps++;
}

static V3 localHalfExtent(const Body &b) {
    if (b.shape == 1)
        return V3{b.size.x, b.size.x, b.size.x};
    if (b.shape == 2)
        return V3{b.size.x, b.size.x, b.size.z * 0.5f};
    return b.size * 0.5f;
}

// Solver::pick (solver_query.cpp:24-152): exact ray tests per body in list order.
int World::pick(V3 origin, V3 dir, uint32_t mask, V3 &local) const {
    const float eps = 1.0e-6f;
    float bestT = std::numeric_limits<float>::infinity();
    int best = -1;
    V3 bestLocal{0, 0, 0};
    for (int li = 0; li < count(); li++) {
        const int id = idAt(li);
        const Body &b = bodies[id];
        if ((b.layer & mask) == 0)
            continue;
        const Q4 inv = qconj(b.q);
        const V3 o = qrot(inv, origin - b.x);
        const V3 d = qrot(inv, dir);
        if (b.shape == 1) {
            const float r = b.size.x;
            const float bb = dot(o, d);
            const float c = length2(o) - r * r;
            const float disc = bb * bb - c;
            if (disc < 0.0f)
                continue;
            const float sq = std::sqrt(disc);
            float t = -bb - sq;
            if (t < 0.0f)
                t = -bb + sq;
            if (t < 0.0f || t >= bestT)
                continue;
            bestT = t;
            best = id;
            bestLocal = o + d * t;
            continue;
        }
        const V3 half = localHalfExtent(b);
        float tEnter = 0.0f, tExit = std::numeric_limits<float>::infinity();
        bool hit = true;
        for (int i = 0; i < 3; ++i) {
            if (std::fabs(d[i]) < eps) {
                if (o[i] < -half[i] || o[i] > half[i]) {
                    hit = false;
                    break;
                }
                continue;
            }
            const float invD = 1.0f / d[i];
            float t0 = (-half[i] - o[i]) * invD;
            float t1 = (half[i] - o[i]) * invD;
            if (t0 > t1) {
                const float tmp = t0;
                t0 = t1;
                t1 = tmp;
            }
            tEnter = smax(tEnter, t0);
            tExit = smin(tExit, t1);
            if (tEnter > tExit) {
                hit = false;
                break;
            }
        }
        if (!hit)
            continue;
        const float tHit = tEnter >= 0.0f ? tEnter : tExit;
        if (tHit < 0.0f)
            continue;
        if (tHit < bestT) {
            bestT = tHit;
            best = id;
            bestLocal = o + d * tHit;
        }
    }
    if (best >= 0)
        local = bestLocal;
    return best;
}

// Solver::collectAABB (solver_query.cpp:154-170): tight bounds (aabbHalfExtent) about each centre.
void World::collectAABB(V3 lo, V3 hi, uint32_t mask, std::vector<int> &out) const {
    for (int li = 0; li < count(); li++) {
        const int id = idAt(li);
        const Body &b = bodies[id];
        if ((b.layer & mask) == 0)
            continue;
        const M3 rot = qmat(b.q);
        const V3 h = localHalfExtent(b);
        const V3 wx{(std::fabs(rot.c[0][0]) * h.x + std::fabs(rot.c[1][0]) * h.y) + std::fabs(rot.c[2][0]) * h.z,
                    (std::fabs(rot.c[0][1]) * h.x + std::fabs(rot.c[1][1]) * h.y) + std::fabs(rot.c[2][1]) * h.z,
                    (std::fabs(rot.c[0][2]) * h.x + std::fabs(rot.c[1][2]) * h.y) + std::fabs(rot.c[2][2]) * h.z};
        const V3 bmin = b.x - wx, bmax = b.x + wx;
        if (!(bmin.x > hi.x || bmin.y > hi.y || bmin.z > hi.z || lo.x > bmax.x || lo.y > bmax.y || lo.z > bmax.z))
            out.push_back(id);
    }
}

// state_digest (test/core_test.cpp:133-149).
uint64_t World::digest() const {
    uint64_t h = 1469598103934665603ull;
    const auto mix = [&h](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; i++) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    for (int li = 0; li < count(); li++) {
        const Body &b = bodies[idAt(li)];
        const float s[13] = {b.x.x, b.x.y, b.x.z, b.q.x, b.q.y, b.q.z, b.q.w,
                             b.v.x, b.v.y, b.v.z, b.w.x, b.w.y, b.w.z};
        mix(s, sizeof(s));
    }
    return h;
}

} // namespace oracle
