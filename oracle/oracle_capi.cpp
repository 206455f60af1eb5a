// C API of the oracle port (test infrastructure): the avbdg_* world API of include/avbdg.h
// under the prefix avbdo_, so the parity tests drive the GPU library, this port and the compiled
// reference (avbdr_*) through one Python driver.

#include <cmath>
#include <cstring>
#include <string>

#include "avbd_oracle.hpp"

using namespace oracle;

namespace {

thread_local std::string g_error;

int fail(int code, const char *msg) {
    g_error = msg;
    return code;
}

// The option set this restatement covers; anything else is reported, not approximated.
int checkParams(const avbdg_params &p) {
    if (p.iterations < 1 || !(p.dt > 0.0f))
        return fail(AVBDG_ERR_INVALID, "iterations must be >= 1 and dt > 0");
    return AVBDG_OK;
}

} // namespace

extern "C" {

const char *avbdo_last_error(void) { return g_error.c_str(); }

int avbdo_params_default(avbdg_params *p) {
    if (!p)
        return fail(AVBDG_ERR_INVALID, "null output");
    std::memset(p, 0, sizeof(*p));
    p->dt = 1.0f / 60.0f;
    p->gravity = -10.0f;
    p->iterations = 8;
    p->alpha = 0.99f;
    p->beta_lin = 10000.0f;
    p->beta_ang = 100.0f;
    p->gamma = 0.999f;
    p->newton_ratio = 1.0f;
    p->stiffness_decay = 1.0f;
    p->adaptive_beta = 0;
    p->adaptive_beta_error_floor = 1e-3f;
    p->convergence_threshold = 0.0f;
    p->jacobi_relaxation = 0.7f;
    p->contact_only_overflow = 1;
    p->stick_drift_heal = STICK_DRIFT_HEAL;
    p->max_penetration = CONTACT_MAX_PENETRATION;
    p->jacobian_rebuild_distance = 0.0f;
    p->speculative_margin = 0.01f;
    p->position_projection = 1;
    p->projection_iterations = 4;
    p->projection_beta = 1.0f;
    p->projection_slop = 0.008f;
    p->projection_max_correction = 0.0f;
    p->contact_grace_ticks = 0;
    p->sleep_linear_threshold = 0.1f;
    p->sleep_angular_threshold = 0.139626f;
    p->sleep_frames = 0;
    p->threads = 0;
    return AVBDG_OK;
}

int avbdo_world_create(const avbdg_params *params, int, int, World **out) {
    if (!out)
        return fail(AVBDG_ERR_INVALID, "null output");
    avbdg_params p;
    if (params)
        p = *params;
    else
        avbdo_params_default(&p);
    const int rc = checkParams(p);
    if (rc)
        return rc;
    *out = new World(p);
    return AVBDG_OK;
}

int avbdo_world_destroy(World *w) {
    delete w;
    return AVBDG_OK;
}

int avbdo_world_clear(World *w) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->bodies.clear();
    w->forces.clear();
    w->live.clear();
    w->invalidateTree();
    return AVBDG_OK;
}

int avbdo_world_set_params(World *w, const avbdg_params *p) {
    if (!w || !p)
        return fail(AVBDG_ERR_INVALID, "null argument");
    const int rc = checkParams(*p);
    if (rc)
        return rc;
    w->P = *p;
    return AVBDG_OK;
}

int avbdo_world_get_params(const World *w, avbdg_params *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    *out = w->P;
    return AVBDG_OK;
}

int avbdo_world_add_bodies(World *w, int count, const avbdg_body_desc *d, int *ids) {
    if (!w || count < 0 || (count > 0 && !d))
        return fail(AVBDG_ERR_INVALID, "bad argument");
    for (int i = 0; i < count; i++)
        if (d[i].shape < AVBDG_SHAPE_BOX || d[i].shape > AVBDG_SHAPE_CYLINDER)
            return fail(AVBDG_ERR_INVALID, "unknown shape");
    for (int i = 0; i < count; i++) {
        const int id = w->addBody(d[i]);
        if (ids)
            ids[i] = id;
    }
    return AVBDG_OK;
}

int avbdo_world_add_joint(World *w, int a, int b, const float *rA, const float *rB, float kLin, float kAng,
        float fracture, int *id) {
    if (!w || b < 0 || b >= w->count() || a < -1 || a >= w->count() || !rA || !rB)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    w->addJoint(a, b, V3{rA[0], rA[1], rA[2]}, V3{rB[0], rB[1], rB[2]}, kLin, kAng, fracture);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdo_world_add_ignore_collision(World *w, int a, int b, int *id) {
    if (!w || a < 0 || b < 0 || a >= w->count() || b >= w->count())
        return fail(AVBDG_ERR_INVALID, "bad body index");
    w->addIgnore(a, b);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdo_world_add_spring(World *w, int a, int b, const float *rA, const float *rB, float stiffness, float rest,
        int *id) {
    if (!w || a < 0 || b < 0 || a >= w->count() || b >= w->count() || !rA || !rB)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    w->addSpring(a, b, V3{rA[0], rA[1], rA[2]}, V3{rB[0], rB[1], rB[2]}, stiffness, rest);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdo_world_add_generic_joint(World *w, int a, int b, const float *rA, const float *rB,
        const avbdg_joint_axis *axes, int *id) {
    if (!w || b < 0 || b >= w->count() || a < -1 || a >= w->count() || !rA || !rB || !axes)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    Axis ax[6];
    for (int i = 0; i < 6; i++) {
        if (axes[i].mode < 0 || axes[i].mode > 2)
            return fail(AVBDG_ERR_INVALID, "bad axis mode");
        ax[i].mode = axes[i].mode;
        ax[i].lower = axes[i].lower;
        ax[i].upper = axes[i].upper;
        ax[i].springK = axes[i].spring_stiffness;
        ax[i].springEq = axes[i].spring_equilibrium;
        ax[i].springDamp = axes[i].spring_damping;
    }
    w->addGeneric(a, b, V3{rA[0], rA[1], rA[2]}, V3{rB[0], rB[1], rB[2]}, ax);
    if (id)
        *id = 0;
    return AVBDG_OK;
}

int avbdo_world_step(World *w) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->step();
    return AVBDG_OK;
}

int avbdo_world_step_interleaved(World *w, int substeps, int rounds) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    w->stepInterleaved(substeps, rounds);
    return AVBDG_OK;
}

int avbdo_world_step_n(World *w, int count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    for (int i = 0; i < count; i++)
        w->step();
    return AVBDG_OK;
}

int avbdo_world_sync(World *) { return AVBDG_OK; }

int avbdo_world_pick(World *w, int count, const float *o, const float *d, uint32_t mask, int *outBody,
        float *outLocal) {
    if (!w || count < 0 || (count > 0 && (!o || !d || !outBody)))
        return fail(AVBDG_ERR_INVALID, "bad arguments");
    for (int i = 0; i < count; i++) {
        V3 local{0, 0, 0};
        outBody[i] = w->pick(V3{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]}, mask,
                local);
        if (outLocal) {
            outLocal[3 * i] = local.x;
            outLocal[3 * i + 1] = local.y;
            outLocal[3 * i + 2] = local.z;
        }
    }
    return AVBDG_OK;
}

int avbdo_world_collect_aabb(World *w, const float *lo, const float *hi, uint32_t mask, int capacity, int *out,
        int *outCount) {
    if (!w || !lo || !hi || capacity < 0 || (capacity > 0 && !out))
        return fail(AVBDG_ERR_INVALID, "bad arguments");
    std::vector<int> ids;
    w->collectAABB(V3{lo[0], lo[1], lo[2]}, V3{hi[0], hi[1], hi[2]}, mask, ids);
    for (int i = 0; i < static_cast<int>(ids.size()) && i < capacity; i++)
        out[i] = ids[i];
    if (outCount)
        *outCount = static_cast<int>(ids.size());
    return AVBDG_OK;
}

int avbdo_world_get_sleeping(World *w, int first, int count, uint8_t *out) {
    if (!w || first < 0 || count < 0 || first + count > w->count() || (count > 0 && !out))
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++)
        out[i] = w->bodies[first + i].sleeping ? 1 : 0;
    return AVBDG_OK;
}

int avbdo_world_get_body_state(World *w, int first, int count, float *p, float *q, float *v, float *av) {
    if (!w || first < 0 || count < 0 || first + count > w->count())
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++) {
        const Body &b = w->bodies[first + i];
        if (p) {
            p[3 * i] = b.x.x;
            p[3 * i + 1] = b.x.y;
            p[3 * i + 2] = b.x.z;
        }
        if (q) {
            q[4 * i] = b.q.x;
            q[4 * i + 1] = b.q.y;
            q[4 * i + 2] = b.q.z;
            q[4 * i + 3] = b.q.w;
        }
        if (v) {
            v[3 * i] = b.v.x;
            v[3 * i + 1] = b.v.y;
            v[3 * i + 2] = b.v.z;
        }
        if (av) {
            av[3 * i] = b.w.x;
            av[3 * i + 1] = b.w.y;
            av[3 * i + 2] = b.w.z;
        }
    }
    return AVBDG_OK;
}

int avbdo_world_set_body_state(World *w, int first, int count, const float *p, const float *q, const float *v,
        const float *av) {
    if (!w || first < 0 || count < 0 || first + count > w->count())
        return fail(AVBDG_ERR_INVALID, "bad range");
    for (int i = 0; i < count; i++) {
        Body &b = w->bodies[first + i];
        if (p)
            b.x = V3{p[3 * i], p[3 * i + 1], p[3 * i + 2]};
        if (q)
            b.q = Q4{q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]};
        if (v)
            b.v = V3{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        if (av)
            b.w = V3{av[3 * i], av[3 * i + 1], av[3 * i + 2]};
    }
    return AVBDG_OK;
}

int avbdo_world_get_stats(World *w, avbdg_stats *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof(*out));
    out->bodies = w->count();
    for (const Body &b : w->bodies)
        if (b.mass > 0.0f)
            out->dynamic_bodies++;
    out->forces = static_cast<int>(w->forces.size());
    out->broad_pairs = static_cast<int>(w->pairs.size());
    out->manifolds = static_cast<int>(w->live.size());
    for (const Manifold &m : w->live)
        out->contacts += m.n;
    out->colour_groups = w->colourCount;
    out->overflow_bodies = w->overflowCount;
    out->update_bodies = static_cast<int>(w->updateOrder.size());
    out->steps = w->steps;
    return AVBDG_OK;
}

int avbdo_world_digest(World *w, uint64_t *out) {
    if (!w || !out)
        return fail(AVBDG_ERR_INVALID, "null argument");
    *out = w->digest();
    return AVBDG_OK;
}

int avbdo_world_dump_broadphase(World *w, uint64_t *codes, int32_t *order, int capN, uint64_t *pairs, int capP,
        int *nBodies, int *nPairs) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    const int n = static_cast<int>(w->codes.size());
    const int np = static_cast<int>(w->pairs.size());
    if (nBodies)
        *nBodies = n;
    if (nPairs)
        *nPairs = np;
    for (int i = 0; i < n && i < capN; i++) {
        if (codes)
            codes[i] = w->codes[i];
        if (order)
            order[i] = w->order[i];
    }
    for (int i = 0; i < np && i < capP; i++)
        if (pairs)
            pairs[i] = w->pairs[i];
    return AVBDG_OK;
}

int avbdo_world_dump_manifolds(World *w, int cap, int32_t *ba, int32_t *bb, int32_t *nc, int32_t *features,
        float *basis, float *c0, float *penalty, float *lambda, int *count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    const int n = static_cast<int>(w->live.size());
    if (count)
        *count = n;
    for (int i = 0; i < n && i < cap; i++) {
        const Manifold &m = w->live[i];
        if (ba)
            ba[i] = m.a;
        if (bb)
            bb[i] = m.b;
        if (nc)
            nc[i] = m.n;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                if (basis)
                    basis[9 * i + 3 * r + c] = m.basis.c[c][r];
        for (int j = 0; j < 8; j++) {
            const bool on = j < m.n;
            if (features)
                features[8 * i + j] = on ? m.c[j].key : 0;
            for (int e = 0; e < 3; e++) {
                if (c0)
                    c0[24 * i + 3 * j + e] = on ? m.c[j].C0[e] : 0.0f;
                if (penalty)
                    penalty[24 * i + 3 * j + e] = on ? m.c[j].k[e] : 0.0f;
                if (lambda)
                    lambda[24 * i + 3 * j + e] = on ? m.c[j].lam[e] : 0.0f;
            }
        }
    }
    return AVBDG_OK;
}

int avbdo_world_dump_colours(World *w, int cap, uint8_t *colour, int32_t *bodyId, int *count) {
    if (!w)
        return fail(AVBDG_ERR_INVALID, "null world");
    const int n = static_cast<int>(w->updateOrder.size());
    if (count)
        *count = n;
    for (int i = 0; i < n && i < cap; i++) {
        if (colour)
            colour[i] = i < (int)w->colour.size() ? w->colour[i] : 255;
        if (bodyId)
            bodyId[i] = w->updateOrder[i];
    }
    return AVBDG_OK;
}

} // extern "C"
