// Scalar float math of the oracle (test infrastructure).
//
// Every operation restates the reference's arithmetic with its exact rounding order, so that the
// oracle reproduces the reference bit for bit when compiled with -ffp-contract=off:
//   - linalg.h 2.2 conventions (src/avbd/linalg.h): column-major 3x3 (m[col][row]); dot(a,b) is
//     a left fold starting at 0 (:365-402,501); mat*vec sums scaled columns left to right
//     (:534-537); component min/max/clamp are `a<b ? ...` selections (:155-157).
//   - maths.h (src/avbd/maths.h:48-152): Eigen-order qrot, qmat, qmul, qlength2, the rotation
//     vector `quat - quat` and the integrator `quat + float3`.
//   - std::min/max/clamp selections as libstdc++ defines them.
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle {

struct V3 {
    float x, y, z;
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct Q4 {
    float x, y, z, w;
};
// Column-major 3x3: c[col][row].
struct M3 {
    V3 c[3];
    float at(int row, int col) const { return c[col][row]; }
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline V3 cmul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 cdiv(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
inline V3 &operator-=(V3 &a, V3 b) { a = a - b; return a; }
inline V3 vabs(V3 a) { return V3{std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }

// linalg dot: fold(+, 0, a*b).
inline float dot(V3 a, V3 b) {
    const float px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    float s = 0.0f;
    s = s + px;
    s = s + py;
    s = s + pz;
    return s;
}
inline float length2(V3 a) { return dot(a, a); }
inline float length(V3 a) { return std::sqrt(length2(a)); }
inline V3 normalize(V3 a) { return a / length(a); }
// linalg length of a float2 {a, b}.
inline float length2d(float a, float b) {
    const float pa = a * a, pb = b * b;
    float s = 0.0f;
    s = s + pa;
    s = s + pb;
    return std::sqrt(s);
}
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Selections.
inline float lmin(float a, float b) { return a < b ? a : b; }             // linalg min
inline float lmax(float a, float b) { return a < b ? b : a; }             // linalg max
inline float lclamp(float x, float l, float h) { return x < l ? l : (x < h ? x : h); }
inline float smin(float a, float b) { return b < a ? b : a; }             // std::min
inline float smax(float a, float b) { return a < b ? b : a; }             // std::max
inline float sclamp(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }
inline V3 lminv(V3 a, V3 b) { return V3{lmin(a.x, b.x), lmin(a.y, b.y), lmin(a.z, b.z)}; }
inline V3 lclampv(V3 x, V3 l, V3 h) {
    return V3{lclamp(x.x, l.x, h.x), lclamp(x.y, l.y, h.y), lclamp(x.z, l.z, h.z)};
}

// Matrices.
inline M3 mcols(V3 c0, V3 c1, V3 c2) { return M3{{c0, c1, c2}}; }
inline M3 mzero() { return mcols(V3{0, 0, 0}, V3{0, 0, 0}, V3{0, 0, 0}); }
inline M3 mdiag(float a, float b, float c) { return mcols(V3{a, 0, 0}, V3{0, b, 0}, V3{0, 0, c}); }
inline V3 mrow(const M3 &m, int r) { return V3{m.c[0][r], m.c[1][r], m.c[2][r]}; }
inline M3 transpose(const M3 &m) { return mcols(mrow(m, 0), mrow(m, 1), mrow(m, 2)); }
inline V3 mul(const M3 &a, V3 b) { return (a.c[0] * b.x + a.c[1] * b.y) + a.c[2] * b.z; }
inline M3 mul(const M3 &a, const M3 &b) { return mcols(mul(a, b.c[0]), mul(a, b.c[1]), mul(a, b.c[2])); }
inline M3 operator+(const M3 &a, const M3 &b) { return mcols(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
inline M3 &operator+=(M3 &a, const M3 &b) { a = a + b; return a; }
inline M3 operator*(const M3 &a, float s) { return mcols(a.c[0] * s, a.c[1] * s, a.c[2] * s); }
inline M3 operator/(const M3 &a, float s) { return mcols(a.c[0] / s, a.c[1] / s, a.c[2] / s); }
inline M3 operator-(const M3 &a) { return mcols(-a.c[0], -a.c[1], -a.c[2]); }

// Quaternions (maths.h:48-152).
inline float qlength2(Q4 q) { return (q.x * q.x + q.z * q.z) + (q.y * q.y + q.w * q.w); }
inline Q4 qnormalize(Q4 q) {
    const float z = qlength2(q);
    if (z > 0.0f) {
        const float s = std::sqrt(z);
        return Q4{q.x / s, q.y / s, q.z / s, q.w / s};
    }
    return q;
}
inline Q4 qconj(Q4 q) { return Q4{-q.x, -q.y, -q.z, q.w}; }
inline Q4 qmul(Q4 a, Q4 b) {
    return Q4{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z,
              a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x,
              a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
inline V3 qrot(Q4 q, V3 v) {
    const V3 z{q.x, q.y, q.z};
    V3 uv = cross(z, v);
    uv = uv + uv;
    return (v + uv * q.w) + cross(z, uv);
}
inline M3 qmat(Q4 q) {
    const float tx = 2.0f * q.x, ty = 2.0f * q.y, tz = 2.0f * q.z;
    const float twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const float txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const float tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    return mcols(V3{1.0f - (tyy + tzz), txy + twz, txz - twy},
                 V3{txy - twz, 1.0f - (txx + tzz), tyz + twx},
                 V3{txz + twy, tyz - twx, 1.0f - (txx + tyy)});
}
// Rotation vector from b to a: 2 * vec(a * conj(b)).
inline V3 qdiff(Q4 a, Q4 b) {
    const Q4 d = qmul(a, qconj(b));
    return V3{d.x * 2.0f, d.y * 2.0f, d.z * 2.0f};
}
// First-order integration of a rotation vector.
inline Q4 qintegrate(Q4 a, V3 b) {
    const Q4 omega{b.x, b.y, b.z, 0.0f};
    const Q4 p = qmul(omega, a);
    return qnormalize(Q4{a.x + p.x * 0.5f, a.y + p.y * 0.5f, a.z + p.z * 0.5f, a.w + p.w * 0.5f});
}

// Right-handed frame with `n` as its first row (maths.h:108-116).
inline M3 orthonormal(V3 n) {
    V3 t1 = std::fabs(n.x) > std::fabs(n.z) ? V3{-n.y, n.x, 0} : V3{0, -n.z, n.y};
    t1 = normalize(t1);
    const V3 t2 = cross(n, t1);
    return transpose(mcols(n, t1, t2));
}

} // namespace oracle
