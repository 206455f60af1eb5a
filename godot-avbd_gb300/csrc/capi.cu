// C ABI (include/avbdg.h) over the host engine. Every entry point catches everything, records a
// message for avbdg_last_error and returns a status code; nothing throws across the boundary.

#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "avbdg.h"
#include "engine_host.hpp"
#include "server.hpp"

struct avbdg_world {
    avbdg::Engine engine;
    avbdg_world(const avbdg_params &p, int nb, int nf) : engine(p, nb, nf, 1) { engine.addWorld(); }
};

struct avbdg_batch {
    avbdg::Engine engine;
    avbdg_batch(const avbdg_params &p, int nw, int nb, int nf) : engine(p, nb, nf, nw) {}
};

struct avbdg_server {
    avbdg::Server server;
    avbdg_server(const avbdg_params &p, uint64_t budget, int maxResident) : server(p, budget, maxResident) {}
};

namespace {

thread_local std::string g_lastError;

int record(int rc, const avbdg::Engine *e) {
    if (rc != AVBDG_OK && e)
        g_lastError = e->error();
    return rc;
}

}

int failWith(int rc, const char *msg) {
    g_lastError = msg;
    return rc;
}

template <typename H, typename F>
int guarded(H *w, F &&fn) {
    if (!w)
        return failWith(AVBDG_ERR_INVALID, "null handle");
    try {
        return record(fn(w->engine), &w->engine);
    } catch (const std::bad_alloc &) {
        return failWith(AVBDG_ERR_CAPACITY, "host allocation failed");
    } catch (const std::exception &ex) {
        return failWith(AVBDG_ERR_INVALID, ex.what());
    } catch (...) {
        return failWith(AVBDG_ERR_INVALID, "unknown error");
    }
}

template <typename F>
int serverCall(avbdg_server *s, F &&fn) {
    if (!s)
        return failWith(AVBDG_ERR_INVALID, "null handle");
    try {
        const int rc = fn(s->server);
        if (rc != AVBDG_OK)
            g_lastError = s->server.error();
        return rc;
    } catch (const std::bad_alloc &) {
        return failWith(AVBDG_ERR_CAPACITY, "host allocation failed");
    } catch (const std::exception &ex) {
        return failWith(AVBDG_ERR_INVALID, ex.what());
    } catch (...) {
        return failWith(AVBDG_ERR_INVALID, "unknown error");
    }

} // namespace

namespace avbdg {
// Error channel shared with the entry points defined in other translation units.
void setLastError(const std::string &msg) { g_lastError = msg; }
} // namespace avbdg

extern "C" {

const char *avbdg_last_error(void) { return g_lastError.c_str(); }

int avbdg_params_default(avbdg_params *p) {
    if (!p)
        return failWith(AVBDG_ERR_INVALID, "null output");
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
    p->stick_drift_heal = 0.002f;
    p->max_penetration = 0.02f;
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

int avbdg_world_create(const avbdg_params *params, int max_bodies, int max_forces, avbdg_world **out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    *out = nullptr;
    avbdg_params p;
    if (params)
        p = *params;
    else
        avbdg_params_default(&p);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return failWith(AVBDG_ERR_CUDA, "no CUDA device: the GPU step has no CPU fallback");
    try {
        avbdg_world *w = new avbdg_world(p, max_bodies, max_forces);
        const int rc = w->engine.setParams(p);
        if (rc != AVBDG_OK) {
            g_lastError = w->engine.error();
            delete w;
            return rc;
        }
        *out = w;
        return AVBDG_OK;
    } catch (const std::bad_alloc &) {
        return failWith(AVBDG_ERR_CAPACITY, "host allocation failed");
    }
}

int avbdg_world_destroy(avbdg_world *w) {
    delete w;
    return AVBDG_OK;
}

int avbdg_world_clear(avbdg_world *w) {
    return guarded(w, [](avbdg::Engine &e) {
        e.clear();
        e.addWorld();
        return AVBDG_OK;
    });
}

int avbdg_world_set_params(avbdg_world *w, const avbdg_params *p) {
    if (!p)
        return failWith(AVBDG_ERR_INVALID, "null params");
    return guarded(w, [p](avbdg::Engine &e) { return e.setParams(*p); });
}

int avbdg_world_get_params(const avbdg_world *w, avbdg_params *out) {
    if (!w || !out)
        return failWith(AVBDG_ERR_INVALID, "null argument");
    *out = w->engine.params();
    return AVBDG_OK;
}

int avbdg_world_add_bodies(avbdg_world *w, int count, const avbdg_body_desc *descs, int *ids) {
    return guarded(w, [=](avbdg::Engine &e) { return e.addBodies(0, count, descs, ids); });
}

int avbdg_world_add_joint(avbdg_world *w, int a, int b, const float r_a[3], const float r_b[3], float kl, float ka,
                          float fr, int *id) {
    return guarded(w, [=](avbdg::Engine &e) {
        const int rc = e.addJoint(0, a, b, r_a, r_b, kl, ka, fr);
        if (rc == AVBDG_OK && id)
            *id = 0;
        return rc;
    });
}

int avbdg_world_add_ignore_collision(avbdg_world *w, int a, int b, int *id) {
    return guarded(w, [=](avbdg::Engine &e) {
        const int rc = e.addIgnore(0, a, b);
        if (rc == AVBDG_OK && id)
            *id = 0;
        return rc;
    });
}

int avbdg_world_add_spring(avbdg_world *w, int a, int b, const float r_a[3], const float r_b[3], float stiffness,
                           float rest, int *id) {
    if (!r_a || !r_b)
        return failWith(AVBDG_ERR_INVALID, "null anchor");
    avbdg_force_desc f{};
    f.kind = 2;
    f.body_a = a;
    f.body_b = b;
    std::memcpy(f.r_a, r_a, sizeof(f.r_a));
    std::memcpy(f.r_b, r_b, sizeof(f.r_b));
    f.stiffness_lin = stiffness;
    f.rest = rest;
    return guarded(w, [&](avbdg::Engine &e) {
        const int rc = e.addForces(0, 1, &f);
        if (rc == AVBDG_OK && id)
            *id = 0;
        return rc;
    });
}

int avbdg_world_add_generic_joint(avbdg_world *w, int a, int b, const float r_a[3], const float r_b[3],
                                  const avbdg_joint_axis axes[6], int *id) {
    if (!r_a || !r_b || !axes)
        return failWith(AVBDG_ERR_INVALID, "null anchor or axes");
    avbdg_force_desc f{};
    f.kind = 3;
    f.body_a = a;
    f.body_b = b;
    std::memcpy(f.r_a, r_a, sizeof(f.r_a));
    std::memcpy(f.r_b, r_b, sizeof(f.r_b));
    for (int i = 0; i < 6; i++)
        f.axes[i] = axes[i];
    return guarded(w, [&](avbdg::Engine &e) {
        const int rc = e.addForces(0, 1, &f);
        if (rc == AVBDG_OK && id)
            *id = 0;
        return rc;
    });
}

int avbdg_world_step(avbdg_world *w) {
    return guarded(w, [](avbdg::Engine &e) { return e.step(); });
}

int avbdg_world_step_interleaved(avbdg_world *w, int substeps, int rounds) {
    return guarded(w, [=](avbdg::Engine &e) { return e.stepInterleaved(substeps, rounds); });
}

int avbdg_world_step_n(avbdg_world *w, int count) {
    return guarded(w, [=](avbdg::Engine &e) { return e.stepMany(count, 1, 0); });
}

int avbdg_world_sync(avbdg_world *w) {
    return guarded(w, [](avbdg::Engine &e) { return e.sync(); });
}

int avbdg_world_get_sleeping(avbdg_world *w, int first, int count, uint8_t *out) {
    return guarded(w, [=](avbdg::Engine &e) { return e.getSleeping(0, first, count, out); });
}

int avbdg_world_pick(avbdg_world *w, int count, const float *origins, const float *dirs, uint32_t mask,
                     int *out_body, float *out_local) {
    return guarded(w, [=](avbdg::Engine &e) { return e.pick(0, count, origins, dirs, mask, out_body, out_local); });
}

int avbdg_world_collect_aabb(avbdg_world *w, const float lo[3], const float hi[3], uint32_t mask, int capacity,
                             int *out, int *out_count) {
    return guarded(w, [=](avbdg::Engine &e) { return e.collectAabb(0, lo, hi, mask, capacity, out, out_count); });
}

int avbdg_world_get_body_state(avbdg_world *w, int first, int count, float *p, float *q, float *v, float *av) {
    return guarded(w, [=](avbdg::Engine &e) { return e.getState(0, first, count, p, q, v, av); });
}

int avbdg_world_set_body_state(avbdg_world *w, int first, int count, const float *p, const float *q,
                               const float *v, const float *av) {
    return guarded(w, [=](avbdg::Engine &e) { return e.setState(0, first, count, p, q, v, av); });
}

int avbdg_world_get_stats(avbdg_world *w, avbdg_stats *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(w, [out](avbdg::Engine &e) { return e.stats(*out); });
}

int avbdg_world_digest(avbdg_world *w, uint64_t *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(w, [out](avbdg::Engine &e) { return e.digest(0, *out); });
}

int avbdg_batch_create(const avbdg_params *params, int max_worlds, int max_bodies, int max_forces,
                       avbdg_batch **out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    *out = nullptr;
    avbdg_params p;
    if (params)
        p = *params;
    else
        avbdg_params_default(&p);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return failWith(AVBDG_ERR_CUDA, "no CUDA device: the GPU step has no CPU fallback");
    try {
        avbdg_batch *b = new avbdg_batch(p, max_worlds, max_bodies, max_forces);
        const int rc = b->engine.setParams(p);
        if (rc != AVBDG_OK) {
            g_lastError = b->engine.error();
            delete b;
            return rc;
        }
        *out = b;
        return AVBDG_OK;
    } catch (const std::bad_alloc &) {
        return failWith(AVBDG_ERR_CAPACITY, "host allocation failed");
    }
}

int avbdg_batch_destroy(avbdg_batch *b) {
    delete b;
    return AVBDG_OK;
}

int avbdg_batch_add_world(avbdg_batch *b, int nb, const avbdg_body_desc *bodies, int nf, const avbdg_force_desc *forces,
                          int *outWorld) {
    if (nf < 0 || (nf > 0 && !forces))
        return failWith(AVBDG_ERR_INVALID, "bad force array");
    return guarded(b, [=](avbdg::Engine &e) {
        std::string why;
        int rc = avbdg::Engine::validateBodies(nb, bodies, why);
        if (rc == AVBDG_OK)
            rc = avbdg::Engine::validateForces(nb, nf, forces, why);
        if (rc != AVBDG_OK) {
            g_lastError = why;
            return rc;
        }
        const int w = e.addWorld();
        if (w < 0)
            return AVBDG_ERR_CAPACITY;
        rc = e.addBodies(w, nb, bodies, nullptr);
        if (rc == AVBDG_OK)
            rc = e.addForces(w, nf, forces);
        if (rc == AVBDG_OK && outWorld)
            *outWorld = w;
        return rc;
    });
}

int avbdg_batch_remove_worlds(avbdg_batch *b, int count, const int *worlds) {
    if (count < 0 || (count > 0 && !worlds))
        return failWith(AVBDG_ERR_INVALID, "bad world list");
    return guarded(b, [=](avbdg::Engine &e) { return e.removeWorlds(std::vector<int>(worlds, worlds + count)); });
}

int avbdg_batch_step(avbdg_batch *b, int count) {
    return guarded(b, [=](avbdg::Engine &e) { return e.stepMany(count, 1, 0); });
}

int avbdg_batch_sync(avbdg_batch *b) {
    return guarded(b, [](avbdg::Engine &e) { return e.sync(); });
}

int avbdg_batch_world_count(const avbdg_batch *b, int *out) {
    if (!b || !out)
        return failWith(AVBDG_ERR_INVALID, "null argument");
    *out = b->engine.worlds();
    return AVBDG_OK;
}

int avbdg_batch_get_body_state(avbdg_batch *b, int world, int first, int count, float *p, float *q, float *v,
                               float *av) {
    return guarded(b, [=](avbdg::Engine &e) { return e.getState(world, first, count, p, q, v, av); });
}

int avbdg_batch_set_body_state(avbdg_batch *b, int world, int first, int count, const float *p, const float *q,
                               const float *v, const float *av) {
    return guarded(b, [=](avbdg::Engine &e) { return e.setState(world, first, count, p, q, v, av); });
}

int avbdg_batch_digest(avbdg_batch *b, int world, uint64_t *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(b, [=](avbdg::Engine &e) { return e.digest(world, *out); });
}

int avbdg_batch_get_stats(avbdg_batch *b, avbdg_stats *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(b, [out](avbdg::Engine &e) { return e.stats(*out); });
}

int avbdg_batch_set_profiling(avbdg_batch *b, int enabled) {
    return guarded(b, [=](avbdg::Engine &e) {
        e.setProfiling(enabled != 0);
        return AVBDG_OK;
    });
}

int avbdg_batch_take_kernel_times(avbdg_batch *b, avbdg_kernel_times *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(b, [out](avbdg::Engine &e) {
        e.takeKernelTimes(*out);
        return AVBDG_OK;
    });
}

int avbdg_world_set_profiling(avbdg_world *w, int enabled) {
    return guarded(w, [=](avbdg::Engine &e) {
        e.setProfiling(enabled != 0);
        return AVBDG_OK;
    });
}

int avbdg_world_set_wait_limit(avbdg_world *w, long long spins) {
    return guarded(w, [=](avbdg::Engine &e) {
        e.setWaitLimit(spins);
        return AVBDG_OK;
    });
}

int avbdg_world_take_kernel_times(avbdg_world *w, avbdg_kernel_times *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return guarded(w, [out](avbdg::Engine &e) {
        e.takeKernelTimes(*out);
        return AVBDG_OK;
    });
}

int avbdg_world_dump_broadphase(avbdg_world *w, uint64_t *codes, int32_t *order, int capN, uint64_t *pairs,
                                int capP, int *nB, int *nP) {
    return guarded(w, [=](avbdg::Engine &e) { return e.dumpBroadphase(codes, order, capN, pairs, capP, nB, nP); });
}

int avbdg_world_dump_manifolds(avbdg_world *w, int cap, int32_t *ba, int32_t *bb, int32_t *nc, int32_t *features,
                               float *basis, float *c0, float *penalty, float *lambda, int *count) {
    return guarded(w, [=](avbdg::Engine &e) {
        return e.dumpManifolds(cap, ba, bb, nc, features, basis, c0, penalty, lambda, count);
    });
}

int avbdg_world_dump_colours(avbdg_world *w, int cap, uint8_t *colour, int32_t *ids, int *count) {
    return guarded(w, [=](avbdg::Engine &e) { return e.dumpColours(cap, colour, ids, count); });
}

int avbdg_server_create(const avbdg_params *params, uint64_t budget_bytes, int max_resident, avbdg_server **out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    *out = nullptr;
    if (budget_bytes == 0 || max_resident < 1)
        return failWith(AVBDG_ERR_INVALID, "the budget and the resident limit must be positive");
    avbdg_params p;
    if (params)
        p = *params;
    else
        avbdg_params_default(&p);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return failWith(AVBDG_ERR_CUDA, "no CUDA device: the GPU step has no CPU fallback");
    try {
        avbdg_server *s = new avbdg_server(p, budget_bytes, max_resident);
        const int rc = s->server.setParams(p);
        if (rc != AVBDG_OK) {
            g_lastError = s->server.error();
            delete s;
            return rc;
        }
        *out = s;
        return AVBDG_OK;
    } catch (const std::bad_alloc &) {
        return failWith(AVBDG_ERR_CAPACITY, "host allocation failed");
    }
}

int avbdg_server_destroy(avbdg_server *s) {
    if (!s)
        return failWith(AVBDG_ERR_INVALID, "null handle");
    delete s;
    return AVBDG_OK;
}

int avbdg_server_admit(avbdg_server *s, int nb, const avbdg_body_desc *bodies, int nf, const avbdg_force_desc *forces,
                       int steps, int64_t *out) {
    return serverCall(s, [=](avbdg::Server &srv) {
        int64_t id = -1;
        const int rc = srv.admit(nb, bodies, nf, forces, steps, id);
        if (out)
            *out = id;
        return rc;
    });
}

int avbdg_server_tick(avbdg_server *s, int *completed) {
    return serverCall(s, [=](avbdg::Server &srv) {
        int done = 0;
        const int rc = srv.tick(done);
        if (completed)
            *completed = done;
        return rc;
    });
}

int avbdg_server_poll(avbdg_server *s, int64_t *outRequest, int *outBodies) {
    if (!outRequest)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return serverCall(s, [=](avbdg::Server &srv) {
        int n = 0;
        srv.poll(*outRequest, n);
        if (outBodies)
            *outBodies = n;
        return AVBDG_OK;
    });
}

int avbdg_server_take_result(avbdg_server *s, int64_t request, int count, float *p, float *q, float *v, float *w) {
    return serverCall(s, [=](avbdg::Server &srv) { return srv.takeResult(request, count, p, q, v, w); });
}

int avbdg_server_evict(avbdg_server *s, int64_t request) {
    return serverCall(s, [=](avbdg::Server &srv) { return srv.evict(request); });
}

int avbdg_server_get_stats(avbdg_server *s, avbdg_server_stats *out) {
    if (!out)
        return failWith(AVBDG_ERR_INVALID, "null output");
    return serverCall(s, [=](avbdg::Server &srv) {
        srv.stats(*out);
        return AVBDG_OK;
    });
}

int avbdg_server_reset_stats(avbdg_server *s) {
    return serverCall(s, [](avbdg::Server &srv) {
        srv.resetStats();
        return AVBDG_OK;
    });
}

} // extern "C"
