// C API over the compiled reference solver (godot-avbd src/avbd/*.cpp), built by
// oracle/Makefile into oracle/_ref/libavbd_ref.so. Test infrastructure only: the parity tests
// and the CPU-baseline leg of bench.py drive it to pin the oracle port and to time the
// reference's own multithreaded CPU step. It exports the avbdg_* world API of include/avbdg.h
// under the prefix avbdr_, so one Python driver runs the GPU library, the oracle port and the
// reference side by side.
//
// Private solver state (LBVH codes and order, candidate pairs, manifold store, colouring) is
// read for the parity dumps; the standard headers are included first so that only the
// solver's own declarations see the access override below.

#include <algorithm>
#include <array>
#include <atomic>
#include <barrier>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iosfwd>
#include <latch>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <ranges>
#include <span>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#define private public
#include "avbd/solver.h"
#undef private

#include "avbdg.h"

using namespace avbd;

namespace {

thread_local std::string g_error;

int fail(int code, const char *msg) {
    g_error = msg;
    return code;
}

struct RefWorld {
    Solver solver;
    avbdg_params params{};
    std::vector<Rigid *> bodies; // creation order
    std::unordered_map<const Rigid *, int> bodyId;
    int steps = 0;
};

void applyParams(Solver &s, const avbdg_params &p) {
    s.dt = p.dt;
    s.gravity = p.gravity;
    s.iterations = p.iterations;
    s.alpha = p.alpha;
    s.betaLin = p.beta_lin;
    s.betaAng = p.beta_ang;
    s.gamma = p.gamma;
    s.newtonRatio = p.newton_ratio;
    s.stiffnessDecay = p.stiffness_decay;
    s.adaptiveBeta = p.adaptive_beta != 0;
    s.adaptiveBetaErrorFloor = p.adaptive_beta_error_floor;
    s.convergenceThreshold = p.convergence_threshold;
    s.jacobiRelaxation = p.jacobi_relaxation;
    s.contactOnlyOverflow = p.contact_only_overflow != 0;
    s.stickDriftHeal = p.stick_drift_heal;
    s.maxPenetration = p.max_penetration;
    s.jacobianRebuildDistance = p.jacobian_rebuild_distance;
    s.speculativeMargin = p.speculative_margin;
    s.positionProjection = p.position_projection != 0;
    s.projectionIterations = p.projection_iterations;
    s.projectionBeta = p.projection_beta;
    s.projectionSlop = p.projection_slop;
    s.projectionMaxCorrection = p.projection_max_correction;
    s.contactGraceTicks = p.contact_grace_ticks;
    s.sleepLinearThreshold = p.sleep_linear_threshold;
    s.sleepAngularThreshold = p.sleep_angular_threshold;
    s.sleepFrames = p.sleep_frames;
    s.threads = p.threads;
}

void readParams(const Solver &s, avbdg_params &p) {
    p.dt = s.dt;
    p.gravity = s.gravity;
    p.iterations = s.iterations;
    p.alpha = s.alpha;
    p.beta_lin = s.betaLin;
    p.beta_ang = s.betaAng;
    p.gamma = s.gamma;
    p.newton_ratio = s.newtonRatio;
    p.stiffness_decay = s.stiffnessDecay;
    p.adaptive_beta = s.adaptiveBeta ? 1 : 0;
    p.adaptive_beta_error_floor = s.adaptiveBetaErrorFloor;
    p.convergence_threshold = s.convergenceThreshold;
    p.jacobi_relaxation = s.jacobiRelaxation;
    p.contact_only_overflow = s.contactOnlyOverflow ? 1 : 0;
    p.stick_drift_heal = s.stickDriftHeal;
    p.max_penetration = s.maxPenetration;
    p.jacobian_rebuild_distance = s.jacobianRebuildDistance;
    p.speculative_margin = s.speculativeMargin;
    p.position_projection = s.positionProjection ? 1 : 0;
    p.projection_iterations = s.projectionIterations;
    p.projection_beta = s.projectionBeta;
    p.projection_slop = s.projectionSlop;
    p.projection_max_correction = s.projectionMaxCorrection;
    p.contact_grace_ticks = s.contactGraceTicks;
    p.sleep_linear_threshold = s.sleepLinearThreshold;
    p.sleep_angular_threshold = s.sleepAngularThreshold;
    p.sleep_frames = s.sleepFrames;
    p.threads = s.threads;
}

} // namespace

extern "C" {

const char *avbdr_last_error(void) { return g_error.c_str(); }

int avbdr_params_default(avbdg_params *out) {
    if (!out)
        return fail(AVBDG_ERR_INVALID, "null output");
    Solver s;
    readParams(s, *out);
    return AVBDG_OK;
}

int avbdr_world_create(const avbdg_params *params, int, int, RefWorld **out) {
    if (!out)
        return fail(AVBDG_ERR_INVALID, "null output");
    RefWorld *w = new RefWorld();
    if (params) {
        w->params = *params;
        applyParams(w->solver, *params);
    } else {
        readParams(w->solver, w->params);
    }
    *out = w;
    return AVBDG_OK;
}

int avbdr_world_destroy(RefWorld *w) {
    delete w;
    return AVBDG_OK;
}

int avbdr_world_clear(RefWorld *w) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->solver.clear();
    w->bodies.clear();
    w->bodyId.clear();
    return AVBDG_OK;
}

int avbdr_world_set_params(RefWorld *w, const avbdg_params *p) {
    if (!w || !p)
        return fail(AVBDG_ERR_INVALID, "null argument");
    w->params = *p;
    applyParams(w->solver, *p);
    return AVBDG_OK;
}

int avbdr_world_get_params(const RefWorld *w, avbdg_params *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    readParams(w->solver, *out);
    return AVBDG_OK;
}

int avbdr_world_add_bodies(RefWorld *w, int count, const avbdg_body_desc *d, int *ids) {
    if (!w || count < 0 || (count > 0 && !d))
        return fail(AVBDG_ERR_INVALID, "bad argument");
    for (int i = 0; i < count; i++) {
        const avbdg_body_desc &b = d[i];
        Rigid *r = new Rigid(&w->solver, float3{b.size[0], b.size[1], b.size[2]},
                static_cast<ShapeType>(b.shape), b.density, b.friction,
                float3{b.position[0], b.position[1], b.position[2]},
                float3{b.velocity[0], b.velocity[1], b.velocity[2]});
        r->positionAng = quat{b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]};
        r->velocityAng = float3{b.angular_velocity[0], b.angular_velocity[1], b.angular_velocity[2]};
        r->collisionLayer = b.collision_layer;
        r->collisionMask = b.collision_mask;
        r->axisLockLinear = static_cast<uint8_t>(b.axis_lock_linear);
        r->axisLockAngular = static_cast<uint8_t>(b.axis_lock_angular);
        r->sleep_mode = static_cast<int>(b.sleep_mode);
        const int id = static_cast<int>(w->bodies.size());
        w->bodies.push_back(r);
        w->bodyId[r] = id;
        if (ids)
            ids[i] = id;
    }
    return AVBDG_OK;
}

int avbdr_world_add_joint(RefWorld *w, int a, int b, const float *rA, const float *rB, float kLin,
        float kAng, float fracture, int *id) {
    if (!w || b < 0 || b >= (int)w->bodies.size() || a >= (int)w->bodies.size() || a < -1)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    Rigid *ba = a >= 0 ? w->bodies[a] : nullptr;
    Joint *j = new Joint(&w->solver, ba, w->bodies[b], float3{rA[0], rA[1], rA[2]},
            float3{rB[0], rB[1], rB[2]}, kLin, kAng, fracture);
    (void)j;
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdr_world_add_ignore_collision(RefWorld *w, int a, int b, int *id) {
    if (!w || a < 0 || b < 0 || a >= (int)w->bodies.size() || b >= (int)w->bodies.size())
        return fail(AVBDG_ERR_INVALID, "bad body index");
    new IgnoreCollision(&w->solver, w->bodies[a], w->bodies[b]);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdr_world_add_spring(RefWorld *w, int a, int b, const float *rA, const float *rB, float stiffness,
        float rest, int *id) {
    if (!w || a < 0 || b < 0 || a >= (int)w->bodies.size() || b >= (int)w->bodies.size())
        return fail(AVBDG_ERR_INVALID, "bad body index");
    new Spring(&w->solver, w->bodies[a], w->bodies[b], float3{rA[0], rA[1], rA[2]}, float3{rB[0], rB[1], rB[2]},
            stiffness, rest);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdr_world_add_generic_joint(RefWorld *w, int a, int b, const float *rA, const float *rB,
        const avbdg_joint_axis *axes, int *id) {
    if (!w || b < 0 || b >= (int)w->bodies.size() || a >= (int)w->bodies.size() || a < -1 || !axes)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    Rigid *ba = a >= 0 ? w->bodies[a] : nullptr;
    GenericJoint *j = new GenericJoint(&w->solver, ba, w->bodies[b], float3{rA[0], rA[1], rA[2]},
            float3{rB[0], rB[1], rB[2]});
    for (int i = 0; i < 6; i++) {
        JointAxis &ax = i < 3 ? j->linear[i] : j->angular[i - 3];
        ax.mode = static_cast<AxisMode>(axes[i].mode);
        ax.lower = axes[i].lower;
        ax.upper = axes[i].upper;
        ax.springStiffness = axes[i].spring_stiffness;
        ax.springEquilibrium = axes[i].spring_equilibrium;
        ax.springDamping = axes[i].spring_damping;
    }
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdr_world_step(RefWorld *w) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->solver.step();
    w->steps++;
    return AVBDG_OK;
}

int avbdr_world_step_interleaved(RefWorld *w, int substeps, int rounds) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->solver.stepInterleaved(substeps, rounds);
    w->steps++;
    return AVBDG_OK;
}

int avbdr_world_step_n(RefWorld *w, int count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    for (int i = 0; i < count; i++) {
        w->solver.step();
        w->steps++;
    }
    return AVBDG_OK;
}

int avbdr_world_sync(RefWorld *) { return AVBDG_OK; }

static int refIndex(RefWorld *w, Rigid *r) {
    for (int i = 0; i < (int)w->bodies.size(); i++)
        if (w->bodies[i] == r)
            return i;
    return -1;
}

int avbdr_world_pick(RefWorld *w, int count, const float *o, const float *d, uint32_t mask, int *outBody,
        float *outLocal) {
    if (!w || count < 0 || (count > 0 && (!o || !d || !outBody)))
        return fail(AVBDG_ERR_INVALID, "bad arguments");
    for (int i = 0; i < count; i++) {
        float3 local{0, 0, 0};
        Rigid *r = w->solver.pick(float3{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, float3{d[3 * i], d[3 * i + 1], d[3 * i + 2]},
                local, mask);
        outBody[i] = r ? refIndex(w, r) : -1;
        if (outLocal) {
            outLocal[3 * i] = r ? local.x : 0.0f;
            outLocal[3 * i + 1] = r ? local.y : 0.0f;
            outLocal[3 * i + 2] = r ? local.z : 0.0f;
        }
    }
    return AVBDG_OK;
}

int avbdr_world_collect_aabb(RefWorld *w, const float *lo, const float *hi, uint32_t mask, int capacity, int *out,
        int *outCount) {
    if (!w || !lo || !hi || capacity < 0 || (capacity > 0 && !out))
        return fail(AVBDG_ERR_INVALID, "bad arguments");
    std::vector<Rigid *> found;
    w->solver.collectAABB(float3{lo[0], lo[1], lo[2]}, float3{hi[0], hi[1], hi[2]}, mask, found);
    for (int i = 0; i < (int)found.size() && i < capacity; i++)
        out[i] = refIndex(w, found[i]);
    if (outCount)
        *outCount = static_cast<int>(found.size());
    return AVBDG_OK;
}

int avbdr_world_get_sleeping(RefWorld *w, int first, int count, uint8_t *out) {
    if (!w || first < 0 || count < 0 || first + count > (int)w->bodies.size() || (count > 0 && !out))
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++)
        out[i] = w->bodies[first + i]->sleeping ? 1 : 0;
    return AVBDG_OK;
}

int avbdr_world_get_body_state(RefWorld *w, int first, int count, float *p, float *q, float *v,
        float *av) {
    if (!w || first < 0 || count < 0 || first + count > (int)w->bodies.size())
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++) {
        const Rigid *r = w->bodies[first + i];
        if (p) {
            p[3 * i + 0] = r->positionLin.x;
            p[3 * i + 1] = r->positionLin.y;
            p[3 * i + 2] = r->positionLin.z;
        }
        if (q) {
            q[4 * i + 0] = r->positionAng.x;
            q[4 * i + 1] = r->positionAng.y;
            q[4 * i + 2] = r->positionAng.z;
            q[4 * i + 3] = r->positionAng.w;
        }
        if (v) {
            v[3 * i + 0] = r->velocityLin.x;
            v[3 * i + 1] = r->velocityLin.y;
            v[3 * i + 2] = r->velocityLin.z;
        }
        if (av) {
            av[3 * i + 0] = r->velocityAng.x;
            av[3 * i + 1] = r->velocityAng.y;
            av[3 * i + 2] = r->velocityAng.z;
        }
    }
    return AVBDG_OK;
}

int avbdr_world_set_body_state(RefWorld *w, int first, int count, const float *p, const float *q,
        const float *v, const float *av) {
    if (!w || first < 0 || count < 0 || first + count > (int)w->bodies.size())
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++) {
        Rigid *r = w->bodies[first + i];
        if (p)
            r->positionLin = float3{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
        if (q)
            r->positionAng = quat{q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]};
        if (v)
            r->velocityLin = float3{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        if (av)
            r->velocityAng = float3{av[3 * i], av[3 * i + 1], av[3 * i + 2]};
    }
    return AVBDG_OK;
}

int avbdr_world_get_stats(RefWorld *w, avbdg_stats *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof(*out));
    Solver &s = w->solver;
    for (const Rigid *b = s.bodies; b; b = b->next) {
        out->bodies++;
        if (b->mass > 0.0f)
            out->dynamic_bodies++;
    }
    for (const Force *f = s.forces; f; f = f->next)
        out->forces++;
    out->broad_pairs = s.broadPhasePairCount();
    out->manifolds = s.manifoldCount();
    out->contacts = s.manifoldContactPoints();
    out->colour_groups = s.colourGroups();
    out->overflow_bodies = s.overflowBodies();
    out->update_bodies = static_cast<int>(s.updateOrder.size());
    out->steps = w->steps;
    out->broad_ms = s.lastStepTimes.broadPhase;
    out->graph_ms = s.lastStepTimes.graph;
    out->solve_ms = s.lastStepTimes.solve;
    out->finish_ms = s.lastStepTimes.finish;
    out->total_ms = out->broad_ms + out->graph_ms + out->solve_ms + out->finish_ms;
    return AVBDG_OK;
}

int avbdr_world_digest(RefWorld *w, uint64_t *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; i++) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    for (Rigid *b = w->solver.bodies; b; b = b->next) {
        mix(&b->positionLin, sizeof(b->positionLin));
        mix(&b->positionAng, sizeof(b->positionAng));
        mix(&b->velocityLin, sizeof(b->velocityLin));
        mix(&b->velocityAng, sizeof(b->velocityAng));
    }
    *out = h;
    return AVBDG_OK;
}

int avbdr_world_dump_broadphase(RefWorld *w, uint64_t *codes, int32_t *order, int capN,
        uint64_t *pairs, int capP, int *nBodies, int *nPairs) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    Solver &s = w->solver;
    const int n = static_cast<int>(s.broadLbvh.codes.size());
    const int np = static_cast<int>(s.sweepPairs.size());
    if (nBodies)
        *nBodies = n;
    if (nPairs)
        *nPairs = np;
    for (int i = 0; i < n && i < capN; i++) {
        if (codes)
            codes[i] = s.broadLbvh.codes[i];
        if (order)
            order[i] = s.broadLbvh.order[i];
    }
    for (int i = 0; i < np && i < capP; i++)
        if (pairs)
            pairs[i] = s.sweepPairs[i];
    return AVBDG_OK;
}

int avbdr_world_dump_manifolds(RefWorld *w, int cap, int32_t *ba, int32_t *bb, int32_t *nc,
        int32_t *features, float *basis, float *c0, float *penalty, float *lambda, int *count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    ManifoldStore &m = w->solver.manifolds;
    const int n = m.count();
    if (count)
        *count = n;
    for (int i = 0; i < n && i < cap; i++) {
        const uint32_t slot = m.live[i];
        const int first = ManifoldStore::base(slot);
        if (ba)
            ba[i] = w->bodyId.at(m.bodyA[slot]);
        if (bb)
            bb[i] = w->bodyId.at(m.bodyB[slot]);
        const int k = m.numContacts[slot];
        if (nc)
            nc[i] = k;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                if (basis)
                    basis[9 * i + 3 * r + c] = m.basis[slot][c][r];
        for (int j = 0; j < 8; j++) {
            const bool on = j < k;
            if (features)
                features[8 * i + j] = on ? m.contacts[first + j].feature.key : 0;
            for (int e = 0; e < 3; e++) {
                if (c0)
                    c0[24 * i + 3 * j + e] = on ? m.contactC0[first + j][e] : 0.0f;
                if (penalty)
                    penalty[24 * i + 3 * j + e] = on ? m.contactPenalty[first + j][e] : 0.0f;
                if (lambda)
                    lambda[24 * i + 3 * j + e] = on ? m.contactLambda[first + j][e] : 0.0f;
            }
        }
    }
    return AVBDG_OK;
}

int avbdr_world_dump_colours(RefWorld *w, int cap, uint8_t *colour, int32_t *bodyIdOut, int *count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    Solver &s = w->solver;
    const int n = static_cast<int>(s.updateOrder.size());
    if (count)
        *count = n;
    for (int i = 0; i < n && i < cap; i++) {
        if (colour)
            colour[i] = i < (int)s.bodyColour.size() ? s.bodyColour[i] : 255;
        if (bodyIdOut)
            bodyIdOut[i] = w->bodyId.at(s.updateOrder[i]);
    }
    return AVBDG_OK;
}

} // extern "C"
