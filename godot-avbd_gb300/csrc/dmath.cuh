// Device float math with the reference solver's exact rounding order.
//
// The step is reproduced bit for bit only if every operation rounds as in the reference
// (compiled there with -ffp-contract=off). This file is therefore built with --fmad=false and
// IEEE division and square root, and each helper spells out its operation order:
//   - linalg.h 2.2 (godot-avbd src/avbd/linalg.h): column-major 3x3, dot() as a left fold that
//     starts at 0 (:365-402,501), mat*vec as a left-to-right sum of scaled columns (:534-537),
//     min/max/clamp as `a<b ? ...` selections (:155-157);
//   - maths.h (src/avbd/maths.h:48-152): Eigen-order qrot, qmat, qmul, qlength2, the rotation
//     vector `quat - quat` and the integrator `quat + float3`;
//   - std::min/std::max/std::clamp selections (libstdc++ definitions).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#define AVBD_HD __host__ __device__ __forceinline__

#ifdef AVBDG_FP64
// The FP64 build (-DAVBDG_FP64, libavbdg64.so): the same kernels with every floating-point value
// of the step in double precision, to state how far the float32 result is from it. A record of
// four doubles is 32 bytes, loaded and stored as two 16-byte halves.
struct __align__(32) avbdg_real4 {
    double x, y, z, w;
};
__device__ __forceinline__ avbdg_real4 __ldcg(const avbdg_real4 *p) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    return avbdg_real4{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ avbdg_real4 __ldg(const avbdg_real4 *p) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return avbdg_real4{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void __stcg(avbdg_real4 *p, avbdg_real4 v) {
    __stcg(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y));
    __stcg(reinterpret_cast<double2 *>(p) + 1, make_double2(v.z, v.w));
}
#endif

namespace avbdg {

// The step's scalar: float (the reference's precision, bit for bit) or, in the FP64 build, double.
// Constants keep their float values in both builds; the math wrappers call the float functions
// in the float build (sqrtf, fabsf, ...) and the double ones in the FP64 build.
#ifdef AVBDG_FP64
using real = double;
using real4 = avbdg_real4;
AVBD_HD real4 mk4(real x, real y, real z, real w) { return real4{x, y, z, w}; }
AVBD_HD real msqrt(real x) { return sqrt(x); }
AVBD_HD real mabs(real x) { return fabs(x); }
AVBD_HD real matan2(real y, real x) { return atan2(y, x); }
AVBD_HD real mmin2(real a, real b) { return fmin(a, b); }
AVBD_HD real mmax2(real a, real b) { return fmax(a, b); }
AVBD_HD real mcopysign(real a, real b) { return copysign(a, b); }
#else
using real = float;
using real4 = float4;
AVBD_HD real4 mk4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
AVBD_HD float msqrt(float x) { return sqrtf(x); }
AVBD_HD float mabs(float x) { return fabsf(x); }
AVBD_HD float matan2(float y, float x) { return atan2f(y, x); }
AVBD_HD float mmin2(float a, float b) { return fminf(a, b); }
AVBD_HD float mmax2(float a, float b) { return fmaxf(a, b); }
AVBD_HD float mcopysign(float a, float b) { return copysignf(a, b); }
#endif
// Ordered-integer reductions (scene bounds, the projection's early-exit depth, ray picks) run on
// the value rounded to float in both builds: they only choose discrete outcomes.
__device__ __forceinline__ int fbits(real x) { return __float_as_int(static_cast<float>(x)); }
__device__ __forceinline__ float bitsf(int i) { return __int_as_float(i); }

struct f3 {
    real x, y, z;
};
struct q4 {
    real x, y, z, w;
};
// Column-major 3x3: c0, c1, c2 are columns; m.c[col].row.
struct m3 {
    f3 c0, c1, c2;
};

AVBD_HD f3 mk3(real x, real y, real z) { return f3{x, y, z}; }
AVBD_HD real at(const f3 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
AVBD_HD void set(f3 &v, int i, real s) {
    if (i == 0)
        v.x = s;
    else if (i == 1)
        v.y = s;
    else
        v.z = s;
}
AVBD_HD f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
AVBD_HD f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
AVBD_HD f3 neg(f3 a) { return f3{-a.x, -a.y, -a.z}; }
AVBD_HD f3 scale(f3 a, real s) { return f3{a.x * s, a.y * s, a.z * s}; }
AVBD_HD f3 divs(f3 a, real s) { return f3{a.x / s, a.y / s, a.z / s}; }
AVBD_HD f3 cmul(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
AVBD_HD f3 vabs(f3 a) { return f3{mabs(a.x), mabs(a.y), mabs(a.z)}; }

// linalg dot: fold(+, 0, a*b).
AVBD_HD real dot(f3 a, f3 b) {
    const real px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    real s = 0.0f;
    s = s + px;
    s = s + py;
    s = s + pz;
    return s;
}
AVBD_HD real length2(f3 a) { return dot(a, a); }
AVBD_HD real length(f3 a) { return msqrt(length2(a)); }
AVBD_HD f3 normalize(f3 a) { return divs(a, length(a)); }
// linalg length of float2 {a, b}.
AVBD_HD real length2d(real a, real b) {
    const real pa = a * a, pb = b * b;
    real s = 0.0f;
    s = s + pa;
    s = s + pb;
    return msqrt(s);
}
AVBD_HD f3 cross(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Selections: linalg (l*) and std (s*).
AVBD_HD real lmin(real a, real b) { return a < b ? a : b; }
AVBD_HD real lclamp(real x, real l, real h) { return x < l ? l : (x < h ? x : h); }
AVBD_HD real smin(real a, real b) { return b < a ? b : a; }
AVBD_HD real smax(real a, real b) { return a < b ? b : a; }
AVBD_HD real sclamp(real v, real lo, real hi) { return v < lo ? lo : (hi < v ? hi : v); }
AVBD_HD f3 lminv(f3 a, f3 b) { return f3{lmin(a.x, b.x), lmin(a.y, b.y), lmin(a.z, b.z)}; }
AVBD_HD f3 lclampv(f3 x, real l, real h) { return f3{lclamp(x.x, l, h), lclamp(x.y, l, h), lclamp(x.z, l, h)}; }

// Matrices.
AVBD_HD m3 mcols(f3 a, f3 b, f3 c) { return m3{a, b, c}; }
AVBD_HD m3 mzero() { return m3{f3{0, 0, 0}, f3{0, 0, 0}, f3{0, 0, 0}}; }
AVBD_HD m3 mdiag(real a, real b, real c) { return m3{f3{a, 0, 0}, f3{0, b, 0}, f3{0, 0, c}}; }
AVBD_HD f3 col(const m3 &m, int c) { return c == 0 ? m.c0 : (c == 1 ? m.c1 : m.c2); }
AVBD_HD real mat(const m3 &m, int c, int r) { return at(col(m, c), r); }
AVBD_HD f3 mrow(const m3 &m, int r) { return f3{at(m.c0, r), at(m.c1, r), at(m.c2, r)}; }
AVBD_HD m3 transpose(const m3 &m) { return m3{mrow(m, 0), mrow(m, 1), mrow(m, 2)}; }
AVBD_HD f3 mul(const m3 &a, f3 b) { return add(add(scale(a.c0, b.x), scale(a.c1, b.y)), scale(a.c2, b.z)); }
AVBD_HD m3 mul(const m3 &a, const m3 &b) { return m3{mul(a, b.c0), mul(a, b.c1), mul(a, b.c2)}; }
AVBD_HD m3 madd(const m3 &a, const m3 &b) { return m3{add(a.c0, b.c0), add(a.c1, b.c1), add(a.c2, b.c2)}; }
AVBD_HD m3 mscale(const m3 &a, real s) { return m3{scale(a.c0, s), scale(a.c1, s), scale(a.c2, s)}; }
AVBD_HD m3 mdivs(const m3 &a, real s) { return m3{divs(a.c0, s), divs(a.c1, s), divs(a.c2, s)}; }
AVBD_HD m3 mneg(const m3 &a) { return m3{neg(a.c0), neg(a.c1), neg(a.c2)}; }

// Quaternions (maths.h:48-152).
AVBD_HD real qlength2(q4 q) { return (q.x * q.x + q.z * q.z) + (q.y * q.y + q.w * q.w); }
AVBD_HD q4 qnormalize(q4 q) {
    const real z = qlength2(q);
    if (z > 0.0f) {
        const real s = msqrt(z);
        return q4{q.x / s, q.y / s, q.z / s, q.w / s};
    }
    return q;
}
AVBD_HD q4 qconj(q4 q) { return q4{-q.x, -q.y, -q.z, q.w}; }
AVBD_HD q4 qmul(q4 a, q4 b) {
    return q4{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z,
              a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x,
              a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
AVBD_HD f3 qrot(q4 q, f3 v) {
    const f3 z{q.x, q.y, q.z};
    f3 uv = cross(z, v);
    uv = add(uv, uv);
    return add(add(v, scale(uv, q.w)), cross(z, uv));
}
AVBD_HD m3 qmat(q4 q) {
    const real tx = 2.0f * q.x, ty = 2.0f * q.y, tz = 2.0f * q.z;
    const real twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const real txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const real tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    return m3{f3{1.0f - (tyy + tzz), txy + twz, txz - twy},
              f3{txy - twz, 1.0f - (txx + tzz), tyz + twx},
              f3{txz + twy, tyz - twx, 1.0f - (txx + tyy)}};
}
// Rotation vector from b to a: 2 vec(a conj(b)).
AVBD_HD f3 qdiff(q4 a, q4 b) {
    const q4 d = qmul(a, qconj(b));
    return f3{d.x * 2.0f, d.y * 2.0f, d.z * 2.0f};
}
// First-order integration of a rotation vector, then renormalisation.
AVBD_HD q4 qintegrate(q4 a, f3 b) {
    const q4 omega{b.x, b.y, b.z, 0.0f};
    const q4 p = qmul(omega, a);
    return qnormalize(q4{a.x + p.x * 0.5f, a.y + p.y * 0.5f, a.z + p.z * 0.5f, a.w + p.w * 0.5f});
}
// Right-handed frame with `n` as its first row (maths.h:108-116).
AVBD_HD m3 orthonormal(f3 n) {
    f3 t1 = mabs(n.x) > mabs(n.z) ? f3{-n.y, n.x, 0.0f} : f3{0.0f, -n.z, n.y};
    t1 = normalize(t1);
    const f3 t2 = cross(n, t1);
    return transpose(m3{n, t1, t2});
}

// float4 packing helpers.
AVBD_HD f3 xyz(real4 v) { return f3{v.x, v.y, v.z}; }
AVBD_HD q4 asq(real4 v) { return q4{v.x, v.y, v.z, v.w}; }
AVBD_HD real4 f4(f3 v, real w) { return mk4(v.x, v.y, v.z, w); }
AVBD_HD real4 f4(q4 q) { return mk4(q.x, q.y, q.z, q.w); }

} // namespace avbdg
