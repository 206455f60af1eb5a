/*
 * avbdg.h - C ABI of the GB300 AVBD rigid-body time-step.
 *
 * This is the drop-in boundary for the CPU solver's step entry point. Every call maps onto
 * one piece of the reference solver's public surface (src/avbd/solver.h:50-374 of
 * godot-avbd); the citation next to each declaration names the reference interface it
 * replaces. Plain C: opaque handles, POD structs, plain pointers and sizes, no exceptions
 * across the boundary. Every call returns an int status (AVBDG_OK = 0, negative = error).
 *
 * Conventions (same as the reference core): metres, kilograms, seconds, +Z up, gravity along
 * -Z, boxes described by full widths, quaternions stored {x, y, z, w}.
 *
 * Body and force identity. A body id is its creation index within the world (0, 1, 2, ...).
 * The solver iterates bodies in *list order*, which is reverse creation order (the reference
 * prepends every new Rigid to an intrusive list, src/avbd/rigid.cpp:29-30); forces likewise
 * (src/avbd/force.cpp:19-21). State accessors take and return arrays in creation order.
 *
 * Threading. Calls on one world must be serialised by the caller (the reference Solver is
 * not thread-safe per instance either). Different worlds may be driven from different host
 * threads; each world owns its own CUDA stream.
 */
#ifndef AVBDG_H
#define AVBDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define AVBDG_OK 0
#define AVBDG_ERR_INVALID (-1)     /* bad handle, argument or index */
#define AVBDG_ERR_CAPACITY (-2)    /* a fixed-capacity device buffer would overflow */
#define AVBDG_ERR_NONFINITE (-3)   /* non-finite input state */
#define AVBDG_ERR_TIMEOUT (-4)     /* a bounded device wait gave up */
#define AVBDG_ERR_CUDA (-5)        /* CUDA runtime error (message via avbdg_last_error) */
#define AVBDG_ERR_UNSUPPORTED (-6) /* a reference feature this build does not implement */

/* Shapes (src/avbd/types.hpp:49-54). Only boxes are on the accelerated path. */
#define AVBDG_SHAPE_BOX 0
#define AVBDG_SHAPE_SPHERE 1
#define AVBDG_SHAPE_CYLINDER 2

/*
 * Solver parameters: the public fields of avbd::Solver (src/avbd/solver.h:54-144) that
 * shape a step. avbdg_params_default fills the reference defaults.
 */
typedef struct avbdg_params {
    float dt;                     /* time step (s) */
    float gravity;                /* signed magnitude along -Z; copied into each body at creation */
    int iterations;               /* solver rounds per step */
    float alpha;                  /* stabilisation, (0, 1] */
    float beta_lin;               /* penalty ramp, linear rows */
    float beta_ang;               /* penalty ramp, angular rows */
    float gamma;                  /* warm-start decay */
    float newton_ratio;           /* share of rounds running the primal */
    float stiffness_decay;        /* penalty decay of dual-only rounds */
    int adaptive_beta;            /* bool */
    float adaptive_beta_error_floor;
    float convergence_threshold;  /* 0 disables the early exit (solver_step.cpp:301-314) */
    float jacobi_relaxation;      /* overflow (block-Jacobi) combine factor */
    int contact_only_overflow;    /* bool */
    float stick_drift_heal;
    float max_penetration;
    float jacobian_rebuild_distance; /* > 0: drift-gated world-arm cache (manifold.cpp:600-668) */
    float speculative_margin;
    int position_projection;      /* bool */
    int projection_iterations;
    float projection_beta;
    float projection_slop;
    float projection_max_correction;
    int contact_grace_ticks;
    float sleep_linear_threshold;
    float sleep_angular_threshold;
    int sleep_frames;
    int threads;                  /* CPU worker count of the reference; ignored on the GPU */
} avbdg_params;

/* Creation record of one body: the arguments of Rigid::Rigid (src/avbd/types.hpp:114-117)
 * plus the public fields a host sets right after construction. */
typedef struct avbdg_body_desc {
    float size[3];                /* box: full extents */
    int shape;                    /* AVBDG_SHAPE_* */
    float density;                /* 0 = static body */
    float friction;
    float position[3];
    float orientation[4];         /* {x, y, z, w}; identity = {0, 0, 0, 1} */
    float velocity[3];
    float angular_velocity[3];
    uint32_t collision_layer;     /* Godot semantics; defaults 1/1 */
    uint32_t collision_mask;
    uint32_t axis_lock_linear;    /* bits 0..2 = x/y/z */
    uint32_t axis_lock_angular;
    uint32_t sleep_mode;          /* Rigid::sleep_mode: 0 never, 1 sleep when idle, 2 start asleep */
} avbdg_body_desc;

/* Per-step counters and phase timings (src/avbd/solver.h:160-275). */
typedef struct avbdg_stats {
    int bodies;
    int dynamic_bodies;           /* mass > 0 */
    int forces;                   /* non-manifold forces alive (joints, ignores) */
    int broad_pairs;              /* sorted unique candidate pairs (broadPhasePairCount) */
    int manifolds;                /* live manifolds (manifoldCount) */
    int contacts;                 /* contact points over live manifolds */
    int colour_groups;            /* colourGroups */
    int overflow_bodies;          /* overflowBodies */
    int update_bodies;            /* bodies in the update set */
    int steps;                    /* steps taken since creation */
    /* last step, milliseconds: broad, graph (warm start + colouring + brake), solve, finish */
    double broad_ms, graph_ms, solve_ms, finish_ms, total_ms;
    int manifold_sides;           /* (manifold, side) pairs whose body moves: stamps per round */
    int graph_step;               /* 1 if the last step ran as one CUDA graph launch */
    int kernel_launches;          /* kernels of this library in the last step */
    /* block sizes the autotuner picked (0 while it is still trying candidates): manifold dual,
     * overflow block solve, narrow phase, tree traversal */
    int block_dual, block_solve, block_narrow, block_traverse;
} avbdg_stats;

/* ------------------------------------------------------------------------------------ */
/* Library                                                                              */
/* ------------------------------------------------------------------------------------ */

/* Reference defaults of every Solver field (src/avbd/solver.h:54-144). */
int avbdg_params_default(avbdg_params *out);

/* Message of the last error on the calling thread ("" if none). Never NULL. */
const char *avbdg_last_error(void);

/* ------------------------------------------------------------------------------------ */
/* Worlds (one avbd::Solver each)                                                       */
/* ------------------------------------------------------------------------------------ */

typedef struct avbdg_world avbdg_world;

/* Solver::Solver (src/avbd/solver.cpp:21-23) with its fields assigned from `params`.
 * `max_bodies` / `max_forces` size the device store; 0 picks a default that grows on demand. */
int avbdg_world_create(const avbdg_params *params, int max_bodies, int max_forces,
                       avbdg_world **out);
/* Solver::~Solver (src/avbd/solver.cpp:25-28). */
int avbdg_world_destroy(avbdg_world *world);
/* Solver::clear (src/avbd/solver_step.cpp:29-40): removes every body, force and manifold. */
int avbdg_world_clear(avbdg_world *world);

/* Field assignment on a Solver (src/avbd/solver.h:54-144). Takes effect at the next step. */
int avbdg_world_set_params(avbdg_world *world, const avbdg_params *params);
int avbdg_world_get_params(const avbdg_world *world, avbdg_params *out);

/* `count` x new Rigid(...) (src/avbd/rigid.cpp:22-72) in array order; body gravity is the
 * world's current gravity. Writes the new ids to `out_ids` (may be NULL). */
int avbdg_world_add_bodies(avbdg_world *world, int count, const avbdg_body_desc *descs,
                           int *out_ids);

/* new Joint(solver, a, b, rA, rB, stiffnessLin, stiffnessAng, fracture)
 * (src/avbd/forces.hpp:58-87, src/avbd/joint.cpp:28-40). body_a = -1 anchors body_b to the
 * world point rA. */
int avbdg_world_add_joint(avbdg_world *world, int body_a, int body_b, const float r_a[3],
                          const float r_b[3], float stiffness_lin, float stiffness_ang,
                          float fracture, int *out_id);

/* new IgnoreCollision(solver, a, b) (src/avbd/forces.hpp:103-113). */
int avbdg_world_add_ignore_collision(avbdg_world *world, int body_a, int body_b, int *out_id);

/* new Spring(solver, a, b, rA, rB, stiffness, rest) (src/avbd/forces.hpp:89-101,
 * src/avbd/spring.cpp:16-27). Both bodies are required; rest < 0 takes the anchors' current
 * distance. */
int avbdg_world_add_spring(avbdg_world *world, int body_a, int body_b, const float r_a[3],
                           const float r_b[3], float stiffness, float rest, int *out_id);

/* One degree of freedom of a generic joint (JointAxis / AxisMode, src/avbd/forces.hpp:115-145). */
#define AVBDG_AXIS_FREE 0
#define AVBDG_AXIS_LOCKED 1
#define AVBDG_AXIS_LIMITED 2
typedef struct avbdg_joint_axis {
    int mode;                     /* AVBDG_AXIS_* */
    float lower, upper;           /* bounds of a limited axis */
    float spring_stiffness;       /* 0 = no spring */
    float spring_equilibrium;
    float spring_damping;
} avbdg_joint_axis;

/* new GenericJoint(solver, a, b, rA, rB) with its six axes set (src/avbd/forces.hpp:147-190,
 * src/avbd/generic_joint.cpp:24-30): axes[0..2] linear x/y/z, axes[3..5] angular x/y/z, in
 * A's frame (the world's for body_a = -1). The current arrangement is the joint's zero. */
int avbdg_world_add_generic_joint(avbdg_world *world, int body_a, int body_b, const float r_a[3],
                                  const float r_b[3], const avbdg_joint_axis axes[6], int *out_id);

/* Solver::step (src/avbd/solver_step.cpp:44-75). Enqueued on the world's stream; the state
 * accessors below synchronise. */
int avbdg_world_step(avbdg_world *world);

/* Solver::stepInterleaved (src/avbd/solver_step.cpp:109-160); `dt` must already be the
 * substep dt, as in the reference. */
int avbdg_world_step_interleaved(avbdg_world *world, int substeps, int rounds_per_substep);

/* Run `count` plain steps. While every buffer a step fills has at least 4x headroom, the next step
 * is queued before the previous one's counters are read back, so the device runs the steps back to
 * back; every step's counters (errors, forces, growth) are still checked in order. */
int avbdg_world_step_n(avbdg_world *world, int count);

/* Wait for every queued step of this world. */
int avbdg_world_sync(avbdg_world *world);

/* Read bodies [first, first+count) in creation order: the Rigid public fields
 * positionLin (3 floats), positionAng (4), velocityLin (3), velocityAng (3)
 * (src/avbd/types.hpp:79-88). Any pointer may be NULL. */
int avbdg_world_get_body_state(avbdg_world *world, int first, int count, float *position,
                               float *orientation, float *velocity, float *angular_velocity);
/* Rigid::sleeping of bodies [first, first+count) (creation order): 1 asleep, 0 awake. */
int avbdg_world_get_sleeping(avbdg_world *world, int first, int count, uint8_t *sleeping);

/* Solver::pick (src/avbd/solver_query.cpp:24-152) for `count` rays at once: ray i starts at
 * origins[3i..] along dirs[3i..] (not normalised; distances are in units of dir). out_body[i] is
 * the creation index of the nearest body hit whose layer meets `mask` (-1: none; the first in list
 * order wins a tie), out_local[3i..] the hit point in that body's frame. */
int avbdg_world_pick(avbdg_world *world, int count, const float *origins, const float *dirs, uint32_t mask,
                     int *out_body, float *out_local);
/* Solver::collectAABB (src/avbd/solver_query.cpp:154-170): bodies whose tight bounds overlap
 * [min, max] and whose layer meets `mask`, in list order (creation indices). Writes at most
 * `capacity` ids; *out_count is the number found. */
int avbdg_world_collect_aabb(avbdg_world *world, const float min[3], const float max[3], uint32_t mask,
                             int capacity, int *out_bodies, int *out_count);

/* Write the same fields (host edits between steps, e.g. integrated external forces,
 * src/server/avbd_physics_server3d.cpp:1503-1528). Any pointer may be NULL. A non-finite
 * position or velocity component returns AVBDG_ERR_NONFINITE and changes nothing. Returns when
 * the arrays may be reused. Transfers go straight from the caller's arrays where the device reads
 * host memory through the host's page tables, else through pinned staging (also forced by the
 * environment variable AVBDG_STAGED_IO=1 when the world is created). */
int avbdg_world_set_body_state(avbdg_world *world, int first, int count, const float *position,
                               const float *orientation, const float *velocity,
                               const float *angular_velocity);

/* Counters and phase times of the last step. */
int avbdg_world_get_stats(avbdg_world *world, avbdg_stats *out);

/* FNV-1a digest over positionLin, positionAng, velocityLin, velocityAng of every body in list
 * order: the reference test suite's state_digest (test/core_test.cpp:133-149). */
int avbdg_world_digest(avbdg_world *world, uint64_t *out);

/* Device time of the hot kernels, accumulated over steps while profiling is on (CUDA events on
 * the world's stream around each launch). Diagnostics beside the reference's PhaseTimes
 * (src/avbd/solver.h:251-275), which time the same phases on the CPU. */
typedef struct avbdg_kernel_times {
    double manifold_ms;   /* dual + stamp pass over manifolds (one launch per round) */
    int manifold_launches;
    double body_ms;       /* block-Jacobi body solve (one launch per Newton round) */
    int body_launches;
    double narrow_ms;     /* narrow phase + warm start (one launch per step) */
    int narrow_launches;
    int kernel_launches;  /* every kernel this library launched while profiling */
    int steps;
} avbdg_kernel_times;

int avbdg_world_set_profiling(avbdg_world *world, int enabled);
/* Read and reset the accumulated times. */
int avbdg_world_take_kernel_times(avbdg_world *world, avbdg_kernel_times *out);

/* Bound of the device's dataflow waits, in spins of ~64 ns. The greedy colouring and the
 * speculative brake sweep run as dataflows in which a body or brake candidate waits for its
 * predecessors (the reference runs both serially: solver_solve.cpp:365-424,
 * solver_projection.cpp:96-167); a wait that exceeds the bound stops its kernel, and the step
 * returns AVBDG_ERR_TIMEOUT with the world's state no longer trustworthy. The default
 * (4,000,000 spins, ~0.3 s per wait) is never reached by a real dependency chain; a small value
 * lets a test make a wait run out (0: give up at the first predecessor found unfinished).
 * spins < 0 restores the default. No reference counterpart. */
int avbdg_world_set_wait_limit(avbdg_world *world, long long spins);

/* ------------------------------------------------------------------------------------ */
/* Parity dumps (the integer stages, for bit-exact comparison with the reference)        */
/* ------------------------------------------------------------------------------------ */

/* Broad phase of the last step: Morton codes over swept-AABB centres per list index
 * (src/avbd/bvh_broadphase.cpp:19-36,70-85), the (code, index) sorted order (:87-96), and the
 * sorted, de-duplicated candidate pair keys (min << 32 | max over list indices,
 * src/avbd/solver_broadphase.cpp:124-137). Arrays may be NULL; counts are always written. */
int avbdg_world_dump_broadphase(avbdg_world *world, uint64_t *codes, int32_t *order, int cap_bodies,
                                uint64_t *pairs, int cap_pairs, int *n_bodies, int *n_pairs);

/* Live manifolds in live order (src/avbd/manifold.hpp:92): body ids of A and B, contact
 * count, eight feature keys per manifold (unused = 0), the 3x3 basis (row-major, normal first),
 * and per contact C0, penalty and lambda (8 x 3 floats each). Arrays may be NULL. */
int avbdg_world_dump_manifolds(avbdg_world *world, int cap, int32_t *body_a, int32_t *body_b,
                               int32_t *contact_count, int32_t *features, float *basis,
                               float *c0, float *penalty, float *lambda, int *count);

/* Colouring of the last step (src/avbd/solver_solve.cpp:365-424): per update-set index, the
 * colour (0..7, 8 = overflow) and the body id it refers to. */
int avbdg_world_dump_colours(avbdg_world *world, int cap, uint8_t *colour, int32_t *body_id,
                             int *count);

/* ------------------------------------------------------------------------------------ */
/* Batches: many independent worlds stepped together                                   */
/* ------------------------------------------------------------------------------------ */

/* A set of independent worlds (each one avbd::Solver, src/avbd/solver.h:50-374) that share one
 * device store and one CUDA stream: every kernel of a step covers all worlds in one launch. Each
 * world's result is bit-identical to stepping that world alone. All worlds share `params`
 * (gravity is copied into each body at creation, as Rigid::Rigid does). */
typedef struct avbdg_batch avbdg_batch;

/* One force of a world (forces.hpp:58-113): kind 0 = Joint, 1 = IgnoreCollision. Body indices
 * are creation indices within the world; body_a = -1 anchors a joint to the world point r_a. */
typedef struct avbdg_force_desc {
    int kind;                     /* 0 ball joint, 1 ignore pair, 2 spring, 3 generic joint */
    int body_a, body_b;
    float r_a[3], r_b[3];
    float stiffness_lin, stiffness_ang, fracture; /* ball joint; a spring's stiffness is stiffness_lin */
    float rest;                   /* spring rest length (< 0: the anchors' distance at creation) */
    avbdg_joint_axis axes[6];     /* generic joint */
} avbdg_force_desc;

int avbdg_batch_create(const avbdg_params *params, int max_worlds, int max_bodies, int max_forces,
                       avbdg_batch **out);
int avbdg_batch_destroy(avbdg_batch *batch);
/* Append a world with its bodies (creation order) and forces (creation order). */
int avbdg_batch_add_world(avbdg_batch *batch, int body_count, const avbdg_body_desc *bodies,
                          int force_count, const avbdg_force_desc *forces, int *out_world);
/* Remove `count` worlds (indices as returned by avbdg_batch_add_world). The other worlds keep
 * their order and are renumbered 0.. in it; their state and results are unaffected (Solver::clear
 * for the removed worlds, src/avbd/solver_step.cpp:29-40). */
int avbdg_batch_remove_worlds(avbdg_batch *batch, int count, const int *worlds);
/* `count` steps of every world (Solver::step each), queued back to back as avbdg_world_step_n. */
int avbdg_batch_step(avbdg_batch *batch, int count);
int avbdg_batch_sync(avbdg_batch *batch);
int avbdg_batch_world_count(const avbdg_batch *batch, int *out);
/* State of bodies [first, first+count) of `world` (creation order). world = -1 addresses all
 * bodies of all worlds, worlds in creation order, so the whole batch moves in one copy. */
int avbdg_batch_get_body_state(avbdg_batch *batch, int world, int first, int count, float *position,
                               float *orientation, float *velocity, float *angular_velocity);
int avbdg_batch_set_body_state(avbdg_batch *batch, int world, int first, int count,
                               const float *position, const float *orientation,
                               const float *velocity, const float *angular_velocity);
int avbdg_batch_digest(avbdg_batch *batch, int world, uint64_t *out);
/* Totals over all worlds; phase times of the last step. */
int avbdg_batch_get_stats(avbdg_batch *batch, avbdg_stats *out);
int avbdg_batch_set_profiling(avbdg_batch *batch, int enabled);
int avbdg_batch_take_kernel_times(avbdg_batch *batch, avbdg_kernel_times *out);

/* ------------------------------------------------------------------------------------ */
/* Served form: continuous batching of scenes on one device store                        */
/* ------------------------------------------------------------------------------------ */

/* Replaces the physics server's per-space stepping loop (AVBDPhysicsServer3D::_step,
 * src/server/avbd_physics_server3d.cpp:1396-1424, one Solver::step per active space in turn) for
 * many scenes at once: each request is one scene (one space, _space_create :318) asking for a
 * number of steps. Requests wait in arrival order until a slot and their device bytes fit the
 * budget, then stay resident on the device (bodies, manifolds with their duals, forces, tree)
 * until their steps are done; every tick advances every resident scene by one Solver::step in the
 * same launches, so requests that arrive while others run overlap with them on the device. A
 * scene's final state is identical to stepping it alone. Calls on one server are serialised by
 * the caller. */
typedef struct avbdg_server avbdg_server;

typedef struct avbdg_server_stats {
    int64_t submitted, admitted, completed, evicted; /* requests since creation */
    int64_t ticks;                /* ticks that stepped the device, since the last reset */
    int queued;                   /* waiting for a slot or for bytes */
    int resident;                 /* on the device */
    int resident_bodies;
    int resident_dynamic;
    uint64_t resident_bytes;      /* device bytes the resident requests are charged */
    uint64_t store_bytes;         /* device bytes the store holds now */
    uint64_t budget_bytes;
    double body_steps;            /* dynamic body-steps since the last reset */
    double busy_ms;               /* host wall time inside ticks since the last reset */
    double tick_p50_ms, tick_p99_ms, tick_max_ms; /* per-tick wall time (admit + step + retire) */
    double request_p50_ms, request_p99_ms;        /* admit call -> result ready */
    /* where tick time went since the last reset: admitting, stepping, retiring (ms), and how
     * many ticks stepped as one captured CUDA graph */
    double admit_ms, step_ms, retire_ms;
    int64_t graph_ticks;
} avbdg_server_stats;

/* `budget_bytes` bounds the device store (a request is charged what a store of its size needs);
 * `max_resident` bounds the scenes on the device at once. */
int avbdg_server_create(const avbdg_params *params, uint64_t budget_bytes, int max_resident,
                        avbdg_server **out);
int avbdg_server_destroy(avbdg_server *server);
/* Queue a scene: bodies and forces in creation order (as avbdg_batch_add_world) and the number of
 * steps it asks for (>= 1). Invalid scenes, and scenes larger than the whole budget, are refused
 * here (AVBDG_ERR_INVALID / UNSUPPORTED / NONFINITE / CAPACITY). */
int avbdg_server_admit(avbdg_server *server, int body_count, const avbdg_body_desc *bodies,
                       int force_count, const avbdg_force_desc *forces, int steps,
                       int64_t *out_request);
/* Admit what fits, step every resident scene once, retire finished scenes (results kept on the
 * host until taken). `completed` = requests finished by this tick. */
int avbdg_server_tick(avbdg_server *server, int *completed);
/* Oldest finished request whose result was not taken yet; *out_request = -1 if none. */
int avbdg_server_poll(avbdg_server *server, int64_t *out_request, int *out_body_count);
/* Final state of a finished request (count = its body count; NULL fields are skipped); the
 * result is released. Layout as avbdg_world_get_body_state. */
int avbdg_server_take_result(avbdg_server *server, int64_t request, int count, float *position,
                             float *orientation, float *velocity, float *angular_velocity);
/* Cancel a queued or resident request (no result), or release a finished one's result
 * (_free_rid :292 for a space). */
int avbdg_server_evict(avbdg_server *server, int64_t request);
int avbdg_server_get_stats(avbdg_server *server, avbdg_server_stats *out);
/* Restart the tick/latency/throughput window (counts of requests are kept). */
int avbdg_server_reset_stats(avbdg_server *server);

/* ------------------------------------------------------------------------------------ */
/* Standalone kernels                                                                   */
/* ------------------------------------------------------------------------------------ */

/* Sort `count` 64-bit keys held in device memory ascending and drop repeated keys, in place:
 * the reference's candidate-pair pass radix_std::sort_with_buffer + std::unique
 * (src/radixsort.hpp:24-83, src/avbd/solver_broadphase.cpp:136-137). Keys must be below
 * 2^key_bits (1..64). On return d_keys[0 .. *unique_count) holds the distinct keys in order.
 * Runs on `stream` (a cudaStream_t; NULL = the default stream) and waits for it. Scratch is
 * allocated with cudaMalloc for the duration of the call. */
int avbdg_sort_unique_keys(uint64_t *d_keys, int count, int key_bits, int *unique_count, void *stream);

/* The same sort + unique for callers that cannot allocate device memory: a host that gives its
 * physics code a fixed device budget and forbids new allocations, a plugin inside an engine whose
 * allocator owns the device, or code that runs while another component captures a stream (a
 * cudaMalloc there would break that capture). It allocates nothing: its scratch is a fixed
 * 4.5 MiB array compiled into this library, present on every GPU that loads the library until
 * the process exits. At most 262,144 keys per call; larger counts return AVBDG_ERR_CAPACITY.
 * The call itself is not capturable: it enqueues a memset, a copy of the count into host memory
 * and waits for `stream`. So `stream` must not be a stream under capture, and while another
 * stream is being captured it must be a non-blocking stream (not NULL, the legacy default
 * stream, whose implicit synchronisation would invalidate that capture), and that capture must
 * have been begun in cudaStreamCaptureModeRelaxed, or in cudaStreamCaptureModeThreadLocal by
 * another thread (a capture in cudaStreamCaptureModeGlobal forbids this call's copy and wait).
 * The first call on each device looks up the array's device address (with that device current);
 * make that first call before any stream capture begins. The address is kept for the life of the
 * device's context: do not call this again on a device after cudaDeviceReset. All calls share the
 * one array: calls whose GPU work overlaps (e.g. on two streams at once) race and corrupt each
 * other's results. No counterpart in the reference (it has no GPU and no allocation constraint). */
int avbdg_sort_unique_keys_static(uint64_t *d_keys, int count, int key_bits, int *unique_count, void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* AVBDG_H */
