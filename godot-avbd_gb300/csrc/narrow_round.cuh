// Sphere and cylinder narrow phase (godot-avbd src/avbd/collide.cpp:493-999, dispatch
// :1001-1027): closest points for spheres (exact against boxes, spheres and cylinders), surface
// samples for cylinders against boxes and cylinders (cap centres and rims, interior rings, plus box
// corners inside the cylinder), candidates ranked by depth and emitted deepest first. Operation
// order follows the reference so the contact sets are bit-identical. One thread per manifold; the
// candidate arrays of the cylinder paths live in local memory.
#pragma once

#include <cfloat>

#include "narrow.cuh"

namespace avbdg {

namespace narrow {

constexpr int kRimSamples = 8, kAxialSamples = 3;
constexpr int kMaxCylSamples = 2 * (kRimSamples + 1) + kRimSamples * (kAxialSamples - 1);
constexpr int kMaxCandidates = 2 * kMaxCylSamples + 8;
constexpr unsigned kAxisCylSample = 3, kAxisCylCorner = 4;

// Rim directions: cos/sin of 2 pi * (5 i mod 8) / 8 (collide.cpp:731-753), computed on the host
// with the C library exactly as the reference does, then uploaded.
struct RimTable {
    real c[kRimSamples], s[kRimSamples];
};

struct RShape {
    int type; // 0 box, 1 sphere, 2 cylinder
    f3 center;
    q4 rot;
    f3 half;
    real radius, halfHeight;
    f3 axis;
};

__device__ __forceinline__ RShape makeShape(int type, f3 c, q4 q, f3 size) {
    return RShape{type, c, q, scale(size, 0.5f), size.x, size.z * 0.5f, qrot(q, f3{0, 0, 1})};
}

__device__ inline bool pointInBox(const RShape &box, f3 p, f3 &push, real &depth) {
    const f3 local = qrot(qconj(box.rot), sub(p, box.center));
    real best = FLT_MAX;
    int axis = 0;
    real sign = 1.0f;
    for (int i = 0; i < 3; ++i) {
        const real d = at(box.half, i) - mabs(at(local, i));
        if (d <= 0.0f)
            return false;
        if (d < best) {
            best = d;
            axis = i;
            sign = at(local, i) >= 0.0f ? 1.0f : -1.0f;
        }
    }
    f3 lp{0, 0, 0};
    set(lp, axis, sign);
    push = qrot(box.rot, lp);
    depth = best;
    return true;
}

__device__ inline bool pointNearBox(const RShape &box, f3 p, real margin, f3 &push, real &depth) {
    const f3 local = qrot(qconj(box.rot), sub(p, box.center));
    bool outside = false;
    for (int i = 0; i < 3; ++i)
        if (mabs(at(local, i)) >= at(box.half, i)) {
            outside = true;
            break;
        }
    if (!outside)
        return false;
    const f3 cl{sclamp(local.x, -box.half.x, box.half.x), sclamp(local.y, -box.half.y, box.half.y),
                sclamp(local.z, -box.half.z, box.half.z)};
    const f3 d = sub(local, cl);
    const real gap = length(d);
    if (gap > margin || gap <= 1.0e-9f)
        return false;
    push = qrot(box.rot, divs(d, gap));
    depth = -gap;
    return true;
}

__device__ inline f3 closestOnCylinder(const RShape &cyl, f3 p, f3 &outward, real &distance) {
    const f3 local = qrot(qconj(cyl.rot), sub(p, cyl.center));
    const real t = sclamp(local.z, -cyl.halfHeight, cyl.halfHeight);
    const real lenSq = (0.0f + local.x * local.x) + local.y * local.y; // linalg length2 of (x, y)
    f3 closest{0, 0, t};
    if (lenSq > cyl.radius * cyl.radius) {
        const real sc = cyl.radius / msqrt(lenSq);
        closest.x = local.x * sc;
        closest.y = local.y * sc;
    } else if (lenSq > 1.0e-12f) {
        closest.x = local.x;
        closest.y = local.y;
    } else {
        closest.x = cyl.radius;
    }
    const f3 on = add(qrot(cyl.rot, closest), cyl.center);
    const f3 d = sub(p, on);
    distance = length(d);
    outward = distance > 1.0e-9f ? divs(d, distance) : qrot(cyl.rot, f3{1, 0, 0});
    return on;
}

__device__ inline bool pointInCylinder(const RShape &cyl, f3 p, f3 &push, real &surface) {
    const f3 local = qrot(qconj(cyl.rot), sub(p, cyl.center));
    const real radialSq = local.x * local.x + local.y * local.y;
    if (radialSq >= cyl.radius * cyl.radius || mabs(local.z) >= cyl.halfHeight)
        return false;
    const real radialDepth = cyl.radius - msqrt(radialSq);
    const real capDepth = cyl.halfHeight - mabs(local.z);
    f3 pl{0, 0, 0};
    if (capDepth < radialDepth) {
        pl.z = local.z >= 0.0f ? 1.0f : -1.0f;
        surface = capDepth;
    } else {
        const real len = msqrt(radialSq);
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

__device__ inline bool pointNearCylinder(const RShape &cyl, f3 p, real margin, f3 &push, real &depth) {
    const f3 local = qrot(qconj(cyl.rot), sub(p, cyl.center));
    const real radialSq = local.x * local.x + local.y * local.y;
    if (radialSq < cyl.radius * cyl.radius && mabs(local.z) < cyl.halfHeight)
        return false;
    f3 outward;
    real distance;
    closestOnCylinder(cyl, p, outward, distance);
    if (distance > margin)
        return false;
    push = outward;
    depth = -distance;
    return true;
}

__device__ __forceinline__ bool sampleInBox(const RShape &box, f3 p, real margin, f3 &push, real &depth) {
    return pointInBox(box, p, push, depth) || (margin > 0.0f && pointNearBox(box, p, margin, push, depth));
}

__device__ __forceinline__ bool sampleInCylinder(const RShape &cyl, f3 p, real margin, f3 &push, real &depth) {
    return pointInCylinder(cyl, p, push, depth) || (margin > 0.0f && pointNearCylinder(cyl, p, margin, push, depth));
}

// Sample k of cylinderSamples (collide.cpp:755-783): cap centre then rim per end, then rings.
__device__ inline f3 cylinderSample(const RShape &cyl, const RimTable &rim, int k) {
    const f3 x = qrot(cyl.rot, f3{1, 0, 0});
    const f3 y = qrot(cyl.rot, f3{0, 1, 0});
    const int capCount = 2 * (kRimSamples + 1);
    if (k < capCount) {
        const int end = k < kRimSamples + 1 ? -1 : 1;
        const int j = k % (kRimSamples + 1);
        const f3 cap = add(cyl.center, scale(cyl.axis, cyl.halfHeight * static_cast<real>(end)));
        if (j == 0)
            return cap;
        return add(cap, scale(add(scale(x, rim.c[j - 1]), scale(y, rim.s[j - 1])), cyl.radius));
    }
    const int ring = 1 + (k - capCount) / kRimSamples, i = (k - capCount) % kRimSamples;
    const real t = -cyl.halfHeight + 2.0f * cyl.halfHeight * static_cast<real>(ring) / static_cast<real>(kAxialSamples);
    const f3 rc = add(cyl.center, scale(cyl.axis, t));
    return add(rc, scale(add(scale(x, rim.c[i]), scale(y, rim.s[i])), cyl.radius));
}

struct Candidate {
    f3 xA, xB, normal;
    real depth;
    unsigned feature;
};

// Deepest first, stable for equal depths; emission stops at the first contact the sink refuses
// (collide.cpp:699-729).
__device__ inline void emitRanked(const Candidate *cand, int n, Sink &sink) {
    unsigned char order[kMaxCandidates];
    for (int i = 0; i < n; ++i) {
        int j = i;
        while (j > 0 && cand[order[j - 1]].depth < cand[i].depth) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = static_cast<unsigned char>(i);
    }
    const int emit = n < 8 ? n : 8;
    for (int i = 0; i < emit; ++i)
        if (!sink.addc(cand[order[i]].xA, cand[order[i]].xB, static_cast<int>(cand[order[i]].feature)))
            break;
}

__device__ inline int sphereSphere(const RShape &a, const RShape &b, real margin, Sink &sink, m3 &basis) {
    const f3 d = sub(b.center, a.center);
    const real distSq = length2(d);
    const real sumPlus = a.radius + b.radius + margin;
    if (distSq >= sumPlus * sumPlus)
        return 0;
    const real dist = msqrt(distSq);
    const f3 n = dist > 1.0e-6f ? divs(d, dist) : f3{0, 0, 1};
    basis = orthonormal(neg(n));
    sink.addc(add(a.center, scale(n, a.radius)), sub(b.center, scale(n, b.radius)), 1);
    return sink.n;
}

__device__ inline int sphereBox(const RShape &a, const RShape &b, bool sphereIsA, real margin, Sink &sink,
                                m3 &basis) {
    const RShape &sphere = sphereIsA ? a : b;
    const RShape &box = sphereIsA ? b : a;
    const f3 local = qrot(qconj(box.rot), sub(sphere.center, box.center));
    const f3 cl{sclamp(local.x, -box.half.x, box.half.x), sclamp(local.y, -box.half.y, box.half.y),
                sclamp(local.z, -box.half.z, box.half.z)};
    const f3 closest = add(qrot(box.rot, cl), box.center);
    const f3 d = sub(sphere.center, closest);
    const real distSq = length2(d);
    const real radPlus = sphere.radius + margin;
    if (distSq >= radPlus * radPlus)
        return 0;
    const real dist = msqrt(distSq);
    f3 n;
    if (dist > 1.0e-6f) {
        n = divs(d, dist);
    } else {
        real depth;
        if (!pointInBox(box, sphere.center, n, depth))
            return 0;
    }
    basis = orthonormal(neg(sphereIsA ? neg(n) : n));
    const f3 onSphere = sub(sphere.center, scale(n, sphere.radius));
    sink.addc(sphereIsA ? onSphere : closest, sphereIsA ? closest : onSphere, 1);
    return sink.n;
}

__device__ inline int sphereCylinder(const RShape &a, const RShape &b, bool sphereIsA, real margin, Sink &sink,
                                     m3 &basis) {
    const RShape &sphere = sphereIsA ? a : b;
    const RShape &cyl = sphereIsA ? b : a;
    f3 outward;
    real distance;
    const f3 onCyl = closestOnCylinder(cyl, sphere.center, outward, distance);
    if (distance >= sphere.radius + margin)
        return 0;
    basis = orthonormal(neg(sphereIsA ? neg(outward) : outward));
    const f3 onSphere = sub(sphere.center, scale(outward, sphere.radius));
    sink.addc(sphereIsA ? onSphere : onCyl, sphereIsA ? onCyl : onSphere, 1);
    return sink.n;
}

__device__ inline int cylinderBox(const RShape &a, const RShape &b, bool cylIsA, const RimTable &rim, real margin,
                                  Sink &sink, m3 &basis) {
    const RShape &cyl = cylIsA ? a : b;
    const RShape &box = cylIsA ? b : a;
    Candidate cand[kMaxCylSamples + 8];
    int nc = 0;
    f3 normalAB{0, 0, 0};
    for (int i = 0; i < kMaxCylSamples; ++i) {
        const f3 s = cylinderSample(cyl, rim, i);
        f3 push;
        real depth;
        if (!sampleInBox(box, s, margin, push, depth))
            continue;
        Candidate &c = cand[nc++];
        c.xA = cylIsA ? s : add(s, scale(push, depth));
        c.xB = cylIsA ? add(s, scale(push, depth)) : s;
        c.normal = cylIsA ? neg(push) : push;
        c.depth = depth;
        c.feature = (kAxisCylSample << 24) | ((cylIsA ? 1u : 0u) << 20) | static_cast<unsigned>(i);
        normalAB = add(normalAB, c.normal);
    }
    for (int corner = 0; corner < 8; ++corner) {
        const f3 cl{(corner & 1) ? box.half.x : -box.half.x, (corner & 2) ? box.half.y : -box.half.y,
                    (corner & 4) ? box.half.z : -box.half.z};
        const f3 cw = add(qrot(box.rot, cl), box.center);
        f3 push;
        real surf;
        if (!sampleInCylinder(cyl, cw, margin, push, surf))
            continue;
        Candidate &c = cand[nc++];
        c.xA = cylIsA ? add(cw, scale(push, surf)) : cw;
        c.xB = cylIsA ? cw : add(cw, scale(push, surf));
        c.normal = cylIsA ? push : neg(push);
        c.depth = surf;
        c.feature = (kAxisCylCorner << 24) | ((cylIsA ? 0u : 1u) << 20) | static_cast<unsigned>(corner);
        normalAB = add(normalAB, c.normal);
    }
    if (!nc)
        return 0;
    basis = orthonormal(neg(length2(normalAB) > 1.0e-12f ? normalize(normalAB) : cyl.axis));
    emitRanked(cand, nc, sink);
    return sink.n;
}

__device__ inline int cylinderCylinder(const RShape &a, const RShape &b, const RimTable &rim, real margin, Sink &sink,
                                       m3 &basis) {
    Candidate cand[2 * kMaxCylSamples];
    int nc = 0;
    f3 normalAB{0, 0, 0};
    for (int pass = 0; pass < 2; ++pass) {
        const RShape &from = pass == 0 ? a : b;
        const RShape &into = pass == 0 ? b : a;
        const bool fromIsA = pass == 0;
        for (int i = 0; i < kMaxCylSamples; ++i) {
            const f3 s = cylinderSample(from, rim, i);
            f3 push;
            real surf;
            if (!sampleInCylinder(into, s, margin, push, surf))
                continue;
            Candidate &c = cand[nc++];
            c.xA = fromIsA ? s : add(s, scale(push, surf));
            c.xB = fromIsA ? add(s, scale(push, surf)) : s;
            c.normal = fromIsA ? neg(push) : push;
            c.depth = surf;
            c.feature = (kAxisCylSample << 24) | ((fromIsA ? 1u : 0u) << 20) | static_cast<unsigned>(i);
            normalAB = add(normalAB, c.normal);
        }
    }
    if (!nc)
        return 0;
    basis = orthonormal(neg(length2(normalAB) > 1.0e-12f ? normalize(normalAB) : a.axis));
    emitRanked(cand, nc, sink);
    return sink.n;
}

} // namespace narrow

// collideShapes for a pair with a sphere or a cylinder (collide.cpp:1007-1027).
__device__ inline int collideRound(int typeA, f3 ca, q4 qa, f3 sizeA, int typeB, f3 cb, q4 qb, f3 sizeB, real margin,
                                   const narrow::RimTable &rim, NContact *out, m3 &basis) {
    using namespace narrow;
    const RShape a = makeShape(typeA, ca, qa, sizeA), b = makeShape(typeB, cb, qb, sizeB);
    Sink sink{ca, cb, qa, qb, out, 0, {}};
    if (a.type == 1 && b.type == 1)
        return sphereSphere(a, b, margin, sink, basis);
    if (a.type == 1 || b.type == 1) {
        const bool sphereIsA = a.type == 1;
        if (a.type == 2 || b.type == 2)
            return sphereCylinder(a, b, sphereIsA, margin, sink, basis);
        return sphereBox(a, b, sphereIsA, margin, sink, basis);
    }
    if (a.type == 2 && b.type == 2)
        return cylinderCylinder(a, b, rim, margin, sink, basis);
    return cylinderBox(a, b, a.type == 2, rim, margin, sink, basis);
}

} // namespace avbdg
