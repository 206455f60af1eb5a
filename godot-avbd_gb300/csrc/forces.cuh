// Spring and GenericJoint on the device (godot-avbd src/avbd/spring.cpp, generic_joint.cpp).
//
// Both are non-manifold forces: they live in the force list with the ball joints and ignore
// pairs, are stamped into a body's block in adjacency order (force list order first) and take
// their dual step in the force dual pass. Expression order follows the reference: IEEE-exact
// except the twist angle, which calls atan2f where the reference calls the C library's atan2f,
// so scenes whose limited or sprung rotations read that angle match within a tolerance rather
// than bit for bit.
//
// Per-force record of a generic joint, fExt[f * kExtF4 + k]:
//   k = 0        rest orientation (B relative to A in A's frame, at creation)
//   k = 1 + i    axis i (0-2 linear x/y/z, 3-5 angular x/y/z): mode, lower, upper, spring stiffness
//   k = 7 + i    axis i: spring equilibrium, spring damping, lambda, penalty
//   k = 13, 14   the six step-start values (stabilisation of locked axes)
// A spring keeps its stiffness and rest length in fPar.xy.
#pragma once

#include "engine.cuh"

namespace avbdg {

constexpr int kForceBall = 0, kForceIgnore = 1, kForceSpring = 2, kForceGeneric = 3;
constexpr int kAxisFree = 0, kAxisLocked = 1, kAxisLimited = 2;

struct GAxis {
    int mode;
    real lower, upper, springK, springEq, springDamp, lambda, penalty, initial;
};

__device__ __forceinline__ GAxis loadAxis(const Dev &d, int f, int i) {
    const real4 *e = d.fExt + static_cast<size_t>(f) * kExtF4;
    const real4 a = e[1 + i], b = e[7 + i], c = e[13 + i / 4];
    const real init[4] = {c.x, c.y, c.z, c.w};
    return GAxis{static_cast<int>(a.x), a.y, a.z, a.w, b.x, b.y, b.z, b.w, init[i % 4]};
}

__device__ __forceinline__ f3 unitAxis(int i) { return i == 0 ? f3{1, 0, 0} : (i == 1 ? f3{0, 1, 0} : f3{0, 0, 1}); }
__device__ __forceinline__ real qcomp(q4 q, int i) { return i == 0 ? q.x : (i == 1 ? q.y : (i == 2 ? q.z : q.w)); }

__device__ __forceinline__ q4 frameOrientation(const Dev &d, int a) {
    return a >= 0 ? asq(d.q[a]) : q4{0.0f, 0.0f, 0.0f, 1.0f};
}

__device__ __forceinline__ m3 outerprod(f3 a, f3 b) { return mcols(scale(a, b.x), scale(a, b.y), scale(a, b.z)); }

// Linear measurement: qrot(conj(qA), anchorA - anchorB) (generic_joint.cpp:37-45, 100-104).
__device__ __forceinline__ f3 genericOffset(const Dev &d, int f) {
    const int2 ab = d.fAB[f];
    const f3 rA = xyz(d.fRA[f]);
    const f3 anchorA = ab.x >= 0 ? add(xyz(d.x[ab.x]), qrot(asq(d.q[ab.x]), rA)) : rA;
    const f3 anchorB = add(xyz(d.x[ab.y]), qrot(asq(d.q[ab.y]), xyz(d.fRB[f])));
    return qrot(qconj(frameOrientation(d, ab.x)), sub(anchorA, anchorB));
}

// Angular measurement, swing-twist split (generic_joint.cpp:49-98): each non-locked axis takes its
// twist 2 atan2(v.n, w) out of the deviation, the locked axes read the remaining swing.
__device__ __forceinline__ void genericAngles(const Dev &d, int f, real out[3]) {
    const int2 ab = d.fAB[f];
    const real4 *e = d.fExt + static_cast<size_t>(f) * kExtF4;
    const q4 qA = frameOrientation(d, ab.x);
    const q4 relativeNow = qmul(qconj(qA), qnormalize(asq(d.q[ab.y])));
    q4 dev = qmul(qnormalize(asq(e[0])), qconj(relativeNow));
    int locked[3];
    for (int i = 0; i < 3; i++)
        locked[i] = static_cast<int>(e[4 + i].x) == kAxisLocked;
    for (int i = 0; i < 3; i++) {
        if (locked[i])
            continue;
        const real proj = dot(f3{dev.x, dev.y, dev.z}, unitAxis(i));
        const q4 twist{dev.x * proj, dev.y * proj, dev.z * proj, dev.w};
        if (msqrt(qlength2(twist)) <= 1.0e-12f) {
            out[i] = 0.0f;
            continue;
        }
        out[i] = 2.0f * matan2(proj, dev.w);
        const real l = qlength2(twist); // qinv(twist) = conj(twist) / |twist|^2
        dev = qmul(qnormalize(dev), q4{-twist.x / l, -twist.y / l, -twist.z / l, twist.w / l});
    }
    for (int i = 0; i < 3; i++)
        if (locked[i])
            out[i] = qcomp(dev, i) * 2.0f;
}

// axisConstraint + axisForce (generic_joint.cpp:120-168).
__device__ __forceinline__ bool axisForce(const GAxis &ax, real value, real alpha, real &C, real &F) {
    if (ax.mode == kAxisLocked) {
        C = value;
    } else if (ax.mode == kAxisLimited) {
        if (value > ax.upper)
            C = value - ax.upper;
        else if (value < ax.lower)
            C = value - ax.lower;
        else
            return false;
    } else {
        return false;
    }
    if (ax.mode == kAxisLocked)
        C -= ax.initial * alpha;
    real force = ax.penalty * C + ax.lambda;
    if (ax.mode == kAxisLimited)
        force = C > 0.0f ? smax(force, 0.0f) : smin(force, 0.0f);
    F = force;
    return true;
}

// GenericJoint::stampAxis (generic_joint.cpp:170-196) into a block (lin, ang, cross, rhs).
template <typename Block>
__device__ __forceinline__ void stampAxis(Block &blk, const GAxis &ax, real value, real alpha, f3 jLin, f3 jAng,
                                          real rate) {
    real C, F;
    if (axisForce(ax, value, alpha, C, F)) {
        blk.lin = madd(blk.lin, mscale(outerprod(jLin, jLin), ax.penalty));
        blk.ang = madd(blk.ang, mscale(outerprod(jAng, jAng), ax.penalty));
        blk.crs = madd(blk.crs, mscale(outerprod(jAng, jLin), ax.penalty));
        blk.rl = add(blk.rl, scale(jLin, F));
        blk.ra = add(blk.ra, scale(jAng, F));
    }
    if (ax.springK > 0.0f) {
        const real Cs = value - ax.springEq;
        const real Fs = ax.springK * Cs - ax.springDamp * rate;
        blk.lin = madd(blk.lin, mscale(outerprod(jLin, jLin), ax.springK));
        blk.ang = madd(blk.ang, mscale(outerprod(jAng, jAng), ax.springK));
        blk.crs = madd(blk.crs, mscale(outerprod(jAng, jLin), ax.springK));
        blk.rl = add(blk.rl, scale(jLin, Fs));
        blk.ra = add(blk.ra, scale(jAng, Fs));
    }
}

// GenericJoint::updatePrimal (generic_joint.cpp:247-287).
template <typename Block>
__device__ __forceinline__ void genericStamp(const Dev &d, const StepParams &p, int f, int body, Block &blk) {
    const int2 ab = d.fAB[f];
    const q4 qA = frameOrientation(d, ab.x);
    const q4 qB = asq(d.q[ab.y]);
    const f3 rAWorld = qrot(qA, xyz(d.fRA[f]));
    const f3 rBWorld = qrot(qB, xyz(d.fRB[f]));
    const f3 offset = genericOffset(d, f);
    real ang[3];
    genericAngles(d, f, ang);
    const bool isA = body == ab.x;
    const real sign = isA ? 1.0f : -1.0f;
    const f3 arm = isA ? rAWorld : rBWorld;
    const f3 vA = ab.x >= 0 ? add(xyz(d.v[ab.x]), cross(xyz(d.w[ab.x]), rAWorld)) : f3{0, 0, 0};
    const f3 vB = add(xyz(d.v[ab.y]), cross(xyz(d.w[ab.y]), rBWorld));
    const f3 relV = sub(vA, vB);
    const f3 wA = ab.x >= 0 ? xyz(d.w[ab.x]) : f3{0, 0, 0};
    const f3 wB = xyz(d.w[ab.y]);
    for (int i = 0; i < 3; i++) {
        const f3 axis = qrot(qA, unitAxis(i));
        const f3 jLin = scale(axis, sign);
        const f3 jAng = cross(arm, jLin);
        stampAxis(blk, loadAxis(d, f, i), at(offset, i), p.alpha, jLin, jAng, dot(relV, axis));
        stampAxis(blk, loadAxis(d, f, 3 + i), ang[i], p.alpha, f3{0, 0, 0}, scale(axis, sign), dot(sub(wA, wB), axis));
    }
}

// Spring::updatePrimal (spring.cpp:31-70).
template <typename Block>
__device__ __forceinline__ void springStamp(const Dev &d, int f, int body, Block &blk) {
    const int2 ab = d.fAB[f];
    const real4 par = d.fPar[f];
    const q4 qa = asq(d.q[ab.x]), qb = asq(d.q[ab.y]);
    const f3 pA = add(xyz(d.x[ab.x]), qrot(qa, xyz(d.fRA[f])));
    const f3 pB = add(xyz(d.x[ab.y]), qrot(qb, xyz(d.fRB[f])));
    const f3 dv = sub(pA, pB);
    const real len = length(dv);
    if (len <= 1.0e-6f)
        return;
    const f3 n = divs(dv, len);
    const real C = len - par.y;
    const real force = par.x * C;
    f3 jLin, jAng;
    if (body == ab.x) {
        const f3 r = qrot(qa, xyz(d.fRA[f]));
        jLin = n;
        jAng = cross(r, n);
    } else {
        const f3 r = qrot(qb, xyz(d.fRB[f]));
        jLin = neg(n);
        jAng = neg(cross(r, n));
    }
    const f3 F = scale(jLin, force);
    const f3 tau = scale(jAng, force);
    const m3 kll = mscale(outerprod(jLin, jLin), par.x);
    const m3 kla = mscale(outerprod(jAng, jLin), par.x);
    const m3 kaa = mscale(outerprod(jAng, jAng), par.x);
    blk.lin = madd(blk.lin, kll);
    blk.ang = madd(blk.ang, kaa);
    blk.crs = madd(blk.crs, kla);
    blk.rl = add(blk.rl, F);
    blk.ra = add(blk.ra, tau);
}

// GenericJoint::penaltyLimit (generic_joint.cpp:198-222).
__device__ __forceinline__ real penaltyLimit(const Dev &d, const StepParams &p, int body, f3 axis, bool angular) {
    real effective;
    if (angular) {
        const f3 local = qrot(qconj(asq(d.q[body])), axis);
        const f3 mo = xyz(d.moment[body]);
        effective = local.x * local.x * mo.x + local.y * local.y * mo.y + local.z * local.z * mo.z;
    } else {
        effective = d.x[body].w;
    }
    if (effective <= 0.0f)
        return PENALTY_MAX;
    const real limit = effective * 0.25f * 0.25f / (p.dt * p.dt);
    return smin(limit, PENALTY_MAX);
}

// GenericJoint::initialize (generic_joint.cpp:224-245).
__device__ __forceinline__ void genericInit(const Dev &d, const StepParams &p, int f) {
    real ang[3];
    genericAngles(d, f, ang);
    const f3 offset = genericOffset(d, f);
    real4 *e = d.fExt + static_cast<size_t>(f) * kExtF4;
    real init[6];
    for (int i = 0; i < 3; i++) {
        init[i] = at(offset, i);
        init[3 + i] = ang[i];
    }
    for (int i = 0; i < 6; i++) {
        real4 s = e[7 + i];
        s.z = s.z * (p.alpha * p.gamma);
        s.w = sclamp(s.w * p.gamma, PENALTY_MIN, PENALTY_MAX);
        e[7 + i] = s;
    }
    e[13] = mk4(init[0], init[1], init[2], init[3]);
    e[14] = mk4(init[4], init[5], 0.0f, 0.0f);
}

// GenericJoint::updateDual (generic_joint.cpp:289-319).
__device__ __forceinline__ void genericDual(const Dev &d, const StepParams &p, int f) {
    real ang[3];
    genericAngles(d, f, ang);
    const f3 offset = genericOffset(d, f);
    const int2 ab = d.fAB[f];
    real4 *e = d.fExt + static_cast<size_t>(f) * kExtF4;
    for (int i = 0; i < 3; i++) {
        const real values[2] = {at(offset, i), ang[i]};
        const real betas[2] = {p.betaLin, p.betaAng};
        for (int k = 0; k < 2; k++) {
            const int idx = 3 * k + i;
            const GAxis ax = loadAxis(d, f, idx);
            real C, F;
            real4 s = e[7 + idx];
            if (!axisForce(ax, values[k], p.alpha, C, F)) {
                if (ax.mode == kAxisLimited) {
                    s.z = 0.0f;
                    e[7 + idx] = s;
                }
                continue;
            }
            s.z = F;
            const f3 dir = qrot(frameOrientation(d, ab.x), unitAxis(i));
            real cap = penaltyLimit(d, p, ab.y, dir, k == 1);
            if (ab.x >= 0)
                cap = smin(cap, penaltyLimit(d, p, ab.x, dir, k == 1));
            s.w = sclamp(ax.penalty + mabs(C) * betas[k], 0.0f, cap);
            e[7 + idx] = s;
        }
    }
}

} // namespace avbdg
