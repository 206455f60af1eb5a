/* C++ facade with the public surface of the reference's core classes, over the C ABI.
 *
 * Mirrors avbd::Solver (src/avbd/solver.h:50-374), avbd::Rigid (src/avbd/types.hpp:75-139) and the
 * forces Joint, Spring, IgnoreCollision and GenericJoint (src/avbd/forces.hpp): the same class and
 * member names, constructor arguments, intrusive lists (a new body or force becomes the list head),
 * solver fields and step entry points, so host code written against the reference drives the GPU
 * step by changing its include and namespace. Vector types are plain {x, y, z(, w)} records; the
 * reference's linalg arithmetic on them is not provided.
 *
 * Semantics: step() first pushes new bodies and forces to the device world (creation order), then
 * the host-visible state of every body (position, orientation, velocities, so host edits between
 * steps take effect as in the reference), runs Solver::step on the GPU and reads the new state back
 * into the Rigid objects. Deleting a body or a force rebuilds the device world from the remaining
 * objects at the next step (warm-start state is lost, as when the Godot server rebuilds a space).
 * Broken joints are dropped on the device; their host objects remain until the host deletes them.
 * Errors of the C ABI raise avbdg::Error.
 */
#ifndef AVBDG_SOLVER_HPP
#define AVBDG_SOLVER_HPP

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "avbdg.h"

namespace avbdg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc) {
    if (rc != AVBDG_OK)
        throw Error(rc, avbdg_last_error());
}

struct float3 {
    float x = 0, y = 0, z = 0;
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct quat {
    float x = 0, y = 0, z = 0, w = 1;
};

constexpr quat quatIdentity{0, 0, 0, 1};

enum class ShapeType : int { Box = 0, Sphere = 1, Cylinder = 2 };
enum class AxisMode : int { Free = 0, Locked = 1, Limited = 2 };

struct JointAxis {
    AxisMode mode = AxisMode::Free;
    float lower = 0.0f, upper = 0.0f;
    float springStiffness = 0.0f, springEquilibrium = 0.0f, springDamping = 0.0f;
};

class Solver;

struct Rigid {
    Solver *solver;
    Rigid *next;
    float3 positionLin;
    quat positionAng;
    float3 velocityLin, velocityAng;
    float3 size;
    ShapeType shape;
    float density, friction;
    float mass = 0.0f, radius = 0.0f, gravity;
    float3 moment;
    uint32_t collisionLayer = 1, collisionMask = 1;
    uint8_t axisLockLinear = 0, axisLockAngular = 0;
    int sleep_mode = 0;   // 0 never, 1 sleep when idle, 2 start asleep
    bool sleeping = false; // read back after each step

    inline Rigid(Solver *p_solver, float3 p_size, ShapeType p_shape, float p_density, float p_friction,
                 float3 p_position, float3 p_velocity = {});
    inline ~Rigid();
    Rigid(const Rigid &) = delete;
    Rigid &operator=(const Rigid &) = delete;

    // Creation index in the device world (-1 until the next step uploads the body).
    int deviceIndex() const { return index; }

private:
    friend class Solver;
    int index = -1;
};

struct Force {
    Solver *solver;
    Rigid *bodyA, *bodyB;
    Force *next;
    void *owner = nullptr;

    inline Force(Solver *p_solver, Rigid *p_bodyA, Rigid *p_bodyB);
    inline virtual ~Force();
    Force(const Force &) = delete;
    Force &operator=(const Force &) = delete;

protected:
    friend class Solver;
    bool uploaded = false;
    virtual avbdg_force_desc describe() const = 0;
};

struct Joint : Force {
    float3 rA, rB;
    float stiffnessLin, stiffnessAng, fracture;
    Joint(Solver *s, Rigid *a, Rigid *b, float3 p_rA, float3 p_rB,
          float p_stiffnessLin = std::numeric_limits<float>::infinity(), float p_stiffnessAng = 0.0f,
          float p_fracture = std::numeric_limits<float>::infinity())
        : Force(s, a, b), rA(p_rA), rB(p_rB), stiffnessLin(p_stiffnessLin), stiffnessAng(p_stiffnessAng),
          fracture(p_fracture) {}

protected:
    inline avbdg_force_desc describe() const override;
};

struct Spring : Force {
    float3 rA, rB;
    float rest, stiffness;
    Spring(Solver *s, Rigid *a, Rigid *b, float3 p_rA, float3 p_rB, float p_stiffness, float p_rest = -1.0f)
        : Force(s, a, b), rA(p_rA), rB(p_rB), rest(p_rest), stiffness(p_stiffness) {}

protected:
    inline avbdg_force_desc describe() const override;
};

struct IgnoreCollision : Force {
    using Force::Force;

protected:
    inline avbdg_force_desc describe() const override;
};

struct GenericJoint : Force {
    float3 rA, rB;
    JointAxis linear[3];
    JointAxis angular[3];
    GenericJoint(Solver *s, Rigid *a, Rigid *b, float3 p_rA, float3 p_rB) : Force(s, a, b), rA(p_rA), rB(p_rB) {}

protected:
    inline avbdg_force_desc describe() const override;
};

class Solver {
public:
    // Solver fields (solver.h:54-144), reference defaults.
    float dt, gravity;
    int iterations;
    float alpha, betaLin, betaAng, gamma, newtonRatio, stiffnessDecay;
    bool adaptiveBeta;
    float adaptiveBetaErrorFloor, convergenceThreshold, jacobiRelaxation;
    bool contactOnlyOverflow;
    float stickDriftHeal, maxPenetration, jacobianRebuildDistance, speculativeMargin;
    bool positionProjection;
    int projectionIterations;
    float projectionBeta, projectionSlop, projectionMaxCorrection;
    int contactGraceTicks;
    float sleepLinearThreshold, sleepAngularThreshold;
    int sleepFrames, threads;

    Rigid *bodies = nullptr; // list order: newest first
    Force *forces = nullptr;

    Solver() {
        avbdg_params p;
        check(avbdg_params_default(&p));
        fromParams(p);
    }
    ~Solver() {
        clear();
        if (world)
            avbdg_world_destroy(world);
    }
    Solver(const Solver &) = delete;
    Solver &operator=(const Solver &) = delete;

    // Solver::clear (solver_step.cpp:29-40): deletes every body and force.
    void clear() {
        while (forces)
            delete forces;
        while (bodies)
            delete bodies;
        dirty = true;
    }

    void step() { run(1, 0); }
    void stepInterleaved(int substeps, int roundsPerSubstep = 0) { run(substeps, roundsPerSubstep); }

    int manifoldCount() const { return stats().manifolds; }
    int broadPhasePairCount() const { return stats().broad_pairs; }
    int colourGroups() const { return stats().colour_groups; }
    int overflowBodies() const { return stats().overflow_bodies; }

    Rigid *pick(float3 origin, float3 dir, float3 &local) { return pick(origin, dir, local, 0xFFFFFFFFu); }
    Rigid *pick(float3 origin, float3 dir, float3 &local, uint32_t mask) {
        if (!prepared())
            return nullptr;
        int id = -1;
        float l[3];
        const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
        check(avbdg_world_pick(world, 1, o, d, mask, &id, l));
        if (id < 0)
            return nullptr;
        local = float3{l[0], l[1], l[2]};
        return created[static_cast<size_t>(id)];
    }
    void collectAABB(float3 min, float3 max, uint32_t mask, std::vector<Rigid *> &out) {
        if (!prepared())
            return;
        const float lo[3] = {min.x, min.y, min.z}, hi[3] = {max.x, max.y, max.z};
        std::vector<int> ids(created.size());
        int found = 0;
        check(avbdg_world_collect_aabb(world, lo, hi, mask, static_cast<int>(ids.size()), ids.data(), &found));
        for (int i = 0; i < found && i < static_cast<int>(ids.size()); i++)
            out.push_back(created[static_cast<size_t>(ids[i])]);
    }

private:
    friend struct Rigid;
    friend struct Force;
    avbdg_world *world = nullptr;
    avbdg_params applied{};       // parameters the device world holds
    bool appliedValid = false;
    std::vector<Rigid *> created; // device creation order
    std::vector<Force *> forceOrder;
    bool dirty = true;            // a body or force was deleted: rebuild the device world

    void fromParams(const avbdg_params &p) {
        dt = p.dt;
        gravity = p.gravity;
        iterations = p.iterations;
        alpha = p.alpha;
        betaLin = p.beta_lin;
        betaAng = p.beta_ang;
        gamma = p.gamma;
        newtonRatio = p.newton_ratio;
        stiffnessDecay = p.stiffness_decay;
        adaptiveBeta = p.adaptive_beta != 0;
        adaptiveBetaErrorFloor = p.adaptive_beta_error_floor;
        convergenceThreshold = p.convergence_threshold;
        jacobiRelaxation = p.jacobi_relaxation;
        contactOnlyOverflow = p.contact_only_overflow != 0;
        stickDriftHeal = p.stick_drift_heal;
        maxPenetration = p.max_penetration;
        jacobianRebuildDistance = p.jacobian_rebuild_distance;
        speculativeMargin = p.speculative_margin;
        positionProjection = p.position_projection != 0;
        projectionIterations = p.projection_iterations;
        projectionBeta = p.projection_beta;
        projectionSlop = p.projection_slop;
        projectionMaxCorrection = p.projection_max_correction;
        contactGraceTicks = p.contact_grace_ticks;
        sleepLinearThreshold = p.sleep_linear_threshold;
        sleepAngularThreshold = p.sleep_angular_threshold;
        sleepFrames = p.sleep_frames;
        threads = p.threads;
    }

    avbdg_params toParams(float bodyGravity) const {
        avbdg_params p;
        p.dt = dt;
        p.gravity = bodyGravity;
        p.iterations = iterations;
        p.alpha = alpha;
        p.beta_lin = betaLin;
        p.beta_ang = betaAng;
        p.gamma = gamma;
        p.newton_ratio = newtonRatio;
        p.stiffness_decay = stiffnessDecay;
        p.adaptive_beta = adaptiveBeta ? 1 : 0;
        p.adaptive_beta_error_floor = adaptiveBetaErrorFloor;
        p.convergence_threshold = convergenceThreshold;
        p.jacobi_relaxation = jacobiRelaxation;
        p.contact_only_overflow = contactOnlyOverflow ? 1 : 0;
        p.stick_drift_heal = stickDriftHeal;
        p.max_penetration = maxPenetration;
        p.jacobian_rebuild_distance = jacobianRebuildDistance;
        p.speculative_margin = speculativeMargin;
        p.position_projection = positionProjection ? 1 : 0;
        p.projection_iterations = projectionIterations;
        p.projection_beta = projectionBeta;
        p.projection_slop = projectionSlop;
        p.projection_max_correction = projectionMaxCorrection;
        p.contact_grace_ticks = contactGraceTicks;
        p.sleep_linear_threshold = sleepLinearThreshold;
        p.sleep_angular_threshold = sleepAngularThreshold;
        p.sleep_frames = sleepFrames;
        p.threads = threads;
        return p;
    }

    // New parameters drop the world's captured step graphs, so only changes are sent.
    void apply(const avbdg_params &p) {
        if (appliedValid && std::memcmp(&p, &applied, sizeof(p)) == 0)
            return;
        check(avbdg_world_set_params(world, &p));
        applied = p;
        appliedValid = true;
    }

    avbdg_stats stats() const {
        avbdg_stats s{};
        if (world)
            check(avbdg_world_get_stats(world, &s));
        return s;
    }

    static avbdg_body_desc describe(const Rigid &b) {
        avbdg_body_desc d{};
        d.size[0] = b.size.x;
        d.size[1] = b.size.y;
        d.size[2] = b.size.z;
        d.shape = static_cast<int>(b.shape);
        d.density = b.density;
        d.friction = b.friction;
        d.position[0] = b.positionLin.x;
        d.position[1] = b.positionLin.y;
        d.position[2] = b.positionLin.z;
        d.orientation[0] = b.positionAng.x;
        d.orientation[1] = b.positionAng.y;
        d.orientation[2] = b.positionAng.z;
        d.orientation[3] = b.positionAng.w;
        d.velocity[0] = b.velocityLin.x;
        d.velocity[1] = b.velocityLin.y;
        d.velocity[2] = b.velocityLin.z;
        d.angular_velocity[0] = b.velocityAng.x;
        d.angular_velocity[1] = b.velocityAng.y;
        d.angular_velocity[2] = b.velocityAng.z;
        d.collision_layer = b.collisionLayer;
        d.collision_mask = b.collisionMask;
        d.axis_lock_linear = b.axisLockLinear;
        d.axis_lock_angular = b.axisLockAngular;
        d.sleep_mode = static_cast<uint32_t>(b.sleep_mode);
        return d;
    }

    // Bodies and forces in creation order (the lists run newest first).
    template <typename T>
    static std::vector<T *> creationOrder(T *head) {
        std::vector<T *> v;
        for (T *x = head; x; x = x->next)
            v.push_back(x);
        return std::vector<T *>(v.rbegin(), v.rend());
    }

    // Push new bodies (each group with the gravity it was created under) and forces.
    bool prepared() {
        if (dirty) {
            if (world)
                avbdg_world_destroy(world);
            world = nullptr;
            appliedValid = false;
            created.clear();
            forceOrder.clear();
            for (Force *f = forces; f; f = f->next)
                f->uploaded = false;
            for (Rigid *b = bodies; b; b = b->next)
                b->index = -1;
            dirty = false;
        }
        const std::vector<Rigid *> all = creationOrder(bodies);
        if (all.empty())
            return false;
        if (!world)
            check(avbdg_world_create(nullptr, static_cast<int>(all.size()), 0, &world));
        size_t i = 0;
        while (i < all.size()) {
            if (all[i]->index >= 0) {
                i++;
                continue;
            }
            // Rigid::Rigid copies the solver's gravity: a run of new bodies sharing one gravity
            // goes up under parameters carrying it.
            size_t j = i;
            std::vector<avbdg_body_desc> descs;
            while (j < all.size() && all[j]->index < 0 && all[j]->gravity == all[i]->gravity)
                descs.push_back(describe(*all[j++]));
            apply(toParams(all[i]->gravity));
            check(avbdg_world_add_bodies(world, static_cast<int>(descs.size()), descs.data(), nullptr));
            for (size_t k = i; k < j; k++) {
                all[k]->index = static_cast<int>(created.size());
                created.push_back(all[k]);
            }
            i = j;
        }
        for (Force *f : creationOrder(forces)) {
            if (f->uploaded)
                continue;
            const avbdg_force_desc d = f->describe();
            check(avbdg_world_add_generic_force(world, d));
            f->uploaded = true;
            forceOrder.push_back(f);
        }
        return true;
    }

    void run(int substeps, int rounds) {
        if (!prepared())
            return;
        apply(toParams(gravity));
        const int n = static_cast<int>(created.size());
        std::vector<float> pos(3 * n), rot(4 * n), vel(3 * n), ang(3 * n);
        for (int i = 0; i < n; i++) {
            const Rigid &b = *created[static_cast<size_t>(i)];
            pos[3 * i] = b.positionLin.x, pos[3 * i + 1] = b.positionLin.y, pos[3 * i + 2] = b.positionLin.z;
            rot[4 * i] = b.positionAng.x, rot[4 * i + 1] = b.positionAng.y;
            rot[4 * i + 2] = b.positionAng.z, rot[4 * i + 3] = b.positionAng.w;
            vel[3 * i] = b.velocityLin.x, vel[3 * i + 1] = b.velocityLin.y, vel[3 * i + 2] = b.velocityLin.z;
            ang[3 * i] = b.velocityAng.x, ang[3 * i + 1] = b.velocityAng.y, ang[3 * i + 2] = b.velocityAng.z;
        }
        check(avbdg_world_set_body_state(world, 0, n, pos.data(), rot.data(), vel.data(), ang.data()));
        if (substeps > 1)
            check(avbdg_world_step_interleaved(world, substeps, rounds));
        else
            check(avbdg_world_step(world));
        std::vector<uint8_t> sl(static_cast<size_t>(n));
        check(avbdg_world_get_body_state(world, 0, n, pos.data(), rot.data(), vel.data(), ang.data()));
        check(avbdg_world_get_sleeping(world, 0, n, sl.data()));
        for (int i = 0; i < n; i++) {
            Rigid &b = *created[static_cast<size_t>(i)];
            b.positionLin = float3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
            b.positionAng = quat{rot[4 * i], rot[4 * i + 1], rot[4 * i + 2], rot[4 * i + 3]};
            b.velocityLin = float3{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
            b.velocityAng = float3{ang[3 * i], ang[3 * i + 1], ang[3 * i + 2]};
            b.sleeping = sl[static_cast<size_t>(i)] != 0;
        }
    }

    // One force through the bulk form (kinds as avbdg_force_desc).
    static int avbdg_world_add_generic_force(avbdg_world *w, const avbdg_force_desc &d) {
        switch (d.kind) {
        case 0:
            return avbdg_world_add_joint(w, d.body_a, d.body_b, d.r_a, d.r_b, d.stiffness_lin, d.stiffness_ang,
                                         d.fracture, nullptr);
        case 1:
            return avbdg_world_add_ignore_collision(w, d.body_a, d.body_b, nullptr);
        case 2:
            return avbdg_world_add_spring(w, d.body_a, d.body_b, d.r_a, d.r_b, d.stiffness_lin, d.rest, nullptr);
        default:
            return avbdg_world_add_generic_joint(w, d.body_a, d.body_b, d.r_a, d.r_b, d.axes, nullptr);
        }
    }
};

// Rigid::Rigid (rigid.cpp:22-72): links itself as the list head; mass properties per shape.
inline Rigid::Rigid(Solver *p_solver, float3 p_size, ShapeType p_shape, float p_density, float p_friction,
                    float3 p_position, float3 p_velocity)
    : solver(p_solver), next(p_solver->bodies), positionLin(p_position), positionAng(quatIdentity),
      velocityLin(p_velocity), velocityAng{}, size(p_size), shape(p_shape), density(p_density),
      friction(p_friction), gravity(p_solver->gravity) {
    p_solver->bodies = this;
    const float pi = 3.14159265358979f;
    if (shape == ShapeType::Sphere) {
        const float r = size.x;
        mass = (4.0f / 3.0f) * pi * r * r * r * density;
        const float i = 0.4f * mass * r * r;
        moment = float3{i, i, i};
        radius = r;
    } else if (shape == ShapeType::Cylinder) {
        const float r = size.x, h = size.z;
        mass = pi * r * r * h * density;
        const float radial = mass * (3.0f * r * r + h * h) / 12.0f;
        moment = float3{radial, radial, 0.5f * mass * r * r};
        const float hh = h * 0.5f;
        radius = std::sqrt(((0.0f + r * r) + hh * hh) + r * r);
    } else {
        mass = size.x * size.y * size.z * density;
        moment = float3{(size.y * size.y + size.z * size.z) / 12.0f * mass,
                        (size.x * size.x + size.z * size.z) / 12.0f * mass,
                        (size.x * size.x + size.y * size.y) / 12.0f * mass};
        const float hx = size.x * 0.5f, hy = size.y * 0.5f, hz = size.z * 0.5f;
        radius = std::sqrt(((0.0f + hx * hx) + hy * hy) + hz * hz);
    }
}

inline Rigid::~Rigid() {
    Rigid **p = &solver->bodies;
    while (*p && *p != this)
        p = &(*p)->next;
    if (*p)
        *p = next;
    if (index >= 0)
        solver->dirty = true;
}

inline Force::Force(Solver *p_solver, Rigid *p_bodyA, Rigid *p_bodyB)
    : solver(p_solver), bodyA(p_bodyA), bodyB(p_bodyB), next(p_solver->forces) {
    p_solver->forces = this;
}

inline Force::~Force() {
    Force **p = &solver->forces;
    while (*p && *p != this)
        p = &(*p)->next;
    if (*p)
        *p = next;
    if (uploaded)
        solver->dirty = true;
}

namespace detail {
inline void anchors(avbdg_force_desc &d, const Force &f, float3 rA, float3 rB) {
    d.body_a = f.bodyA ? f.bodyA->deviceIndex() : -1;
    d.body_b = f.bodyB ? f.bodyB->deviceIndex() : -1;
    d.r_a[0] = rA.x, d.r_a[1] = rA.y, d.r_a[2] = rA.z;
    d.r_b[0] = rB.x, d.r_b[1] = rB.y, d.r_b[2] = rB.z;
}
} // namespace detail

inline avbdg_force_desc Joint::describe() const {
    avbdg_force_desc d{};
    d.kind = 0;
    detail::anchors(d, *this, rA, rB);
    d.stiffness_lin = stiffnessLin;
    d.stiffness_ang = stiffnessAng;
    d.fracture = fracture;
    return d;
}

inline avbdg_force_desc Spring::describe() const {
    avbdg_force_desc d{};
    d.kind = 2;
    detail::anchors(d, *this, rA, rB);
    d.stiffness_lin = stiffness;
    d.rest = rest;
    return d;
}

inline avbdg_force_desc IgnoreCollision::describe() const {
    avbdg_force_desc d{};
    d.kind = 1;
    detail::anchors(d, *this, float3{}, float3{});
    return d;
}

inline avbdg_force_desc GenericJoint::describe() const {
    avbdg_force_desc d{};
    d.kind = 3;
    detail::anchors(d, *this, rA, rB);
    for (int i = 0; i < 6; i++) {
        const JointAxis &a = i < 3 ? linear[i] : angular[i - 3];
        d.axes[i].mode = static_cast<int>(a.mode);
        d.axes[i].lower = a.lower;
        d.axes[i].upper = a.upper;
        d.axes[i].spring_stiffness = a.springStiffness;
        d.axes[i].spring_equilibrium = a.springEquilibrium;
        d.axes[i].spring_damping = a.springDamping;
    }
    return d;
}

} // namespace avbdg

#endif /* AVBDG_SOLVER_HPP */
