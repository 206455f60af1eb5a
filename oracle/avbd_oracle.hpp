// Oracle: serial CPU restatement of godot-avbd's AVBD time-step (avbd::Solver::step and
// stepInterleaved), used ONLY as the parity checker of the GPU library (tests, smoke check,
// CPU baseline of bench.py). It is not part of the product and nothing in the product links it.
//
// Pinning: the oracle reproduces the reference's pinned state digests
// (tools/baseline/digests.txt: stack_300, interleaved_300, mixed_240) and, where the reference
// compiles (oracle/_ref), its per-step body state bit for bit; see tests/test_oracle_pin.py.
//
// Data model (own design, not the reference's): bodies are held in creation order and walked in
// list order (reverse creation, src/avbd/rigid.cpp:29-30); forces are held in list order
// (src/avbd/force.cpp:19-21); manifolds are held densely in `live` order, which is the only
// order the reference's arithmetic depends on (its slot numbers never reach a float).
#pragma once

#include <cstdint>
#include <vector>

#include "omath.hpp"
#include "avbdg.h"

namespace oracle {

constexpr float PENALTY_MIN = 1.0f;                // src/avbd/types.hpp:24
constexpr float PENALTY_MAX = 10000000000.0f;      // :26
constexpr float ADAPTIVE_BETA_MAX = 64.0f;         // :28
constexpr float COLLISION_MARGIN = 0.001f;         // :31-33
constexpr float STICK_THRESH = 0.00001f;           // :35
constexpr float STICK_DRIFT_HEAL = 0.002f;         // :38
constexpr float CONTACT_RELEASE_GAP = 2.0e-3f;     // :41
constexpr float CONTACT_MAX_PENETRATION = 0.02f;   // :45
constexpr int kMaxContacts = 8;                    // src/avbd/manifold.hpp:25
constexpr int kMaxColours = 8;                     // src/avbd/solver.h:339
constexpr uint8_t kOverflowColour = 8;

struct Body {
    // Creation record (src/avbd/types.hpp:75-139).
    V3 size{};
    int shape = 0;
    float mass = 0, friction = 0, radius = 0, gravity = 0;
    V3 moment{};
    uint32_t layer = 1, mask = 1;
    uint8_t lockLin = 0, lockAng = 0;
    // Dynamic state.
    V3 x{}, x0{}, xi{};
    Q4 q{0, 0, 0, 1}, q0{0, 0, 0, 1}, qi{0, 0, 0, 1};
    V3 v{}, w{}, vprev{};
    bool sleeping = false;
    int stillFrames = 0;
    int sleepMode = 0; // 0 never, 1 sleep when idle, 2 start asleep (types.hpp:138)
    // Per-step bookkeeping.
    bool inUpdate = false;
    int updateIndex = -1;
    bool contactOnly = true;
};

enum ForceKind { kJoint = 0, kIgnore = 1, kSpring = 2, kGeneric = 3 };

// One degree of freedom of a generic joint (JointAxis, src/avbd/forces.hpp:130-145).
enum AxisMode { kFree = 0, kLocked = 1, kLimited = 2 };
struct Axis {
    int mode = kFree;
    float lower = 0, upper = 0;
    float springK = 0, springEq = 0, springDamp = 0;
    float lambda = 0, penalty = 0, initial = 0;
};

struct Force {
    ForceKind kind = kJoint;
    int a = -1, b = -1; // body ids; a = -1 means the world
    // Joint state (src/avbd/forces.hpp:58-87); rA/rB are also the Spring and GenericJoint anchors.
    V3 rA{}, rB{}, C0Lin{}, C0Ang{}, kLin{}, kAng{}, lamLin{}, lamAng{};
    float stiffLin = 0, stiffAng = 0, fracture = 0, torqueArm = 0;
    bool broken = false;
    // Spring (forces.hpp:89-101).
    float springK = 0, rest = 0;
    // GenericJoint (forces.hpp:147-190): B relative to A at creation, linear axes 0-2, angular 3-5.
    Q4 restQ{0, 0, 0, 1};
    Axis axis[6];
};

struct Contact {
    int32_t key = 0;
    V3 rA{}, rB{};                       // body-local anchors
    V3 C0{}, k{}, lam{};                 // step-start error, penalty, dual
    V3 F{}, rAW{}, rBW{};                // primal force cache and world arms
    uint8_t stick = 0;
    float betaScale = 1.0f;
    float S[6] = {0, 0, 0, 0, 0, 0};     // B^T K B
};

struct Manifold {
    int a = -1, b = -1; // body ids (a = smaller list index)
    M3 basis = mzero();
    float mu = 0;
    int n = 0;
    uint8_t flags = 0;
    // Arm cache (manifold.hpp:79-80): first columns of the body rotations when the world arms were
    // last captured by the dual.
    V3 rotACap{}, rotBCap{};
    // Contact grace (manifold.hpp:76-77): ticks parked without contacts, contacts kept for revival.
    int dormantTicks = 0, dormantSaved = 0;
    Contact c[kMaxContacts];
};

struct Ref {
    bool manifold;
    int index; // live index or force list index
};

class World {
public:
    explicit World(const avbdg_params &p) : P(p) {}

    avbdg_params P;
    std::vector<Body> bodies;  // creation order
    std::vector<Force> forces; // list order (front = newest)
    std::vector<Manifold> live;
    int steps = 0;

    // Diagnostics of the last step.
    std::vector<uint64_t> codes;   // per list index
    std::vector<int32_t> order;    // sorted list indices
    std::vector<uint64_t> pairs;   // sorted unique candidate keys
    std::vector<uint8_t> colour;   // per update index
    std::vector<int> updateOrder;  // body ids in list order
    int colourCount = 0, overflowCount = 0;

    int addBody(const avbdg_body_desc &d);
    void invalidateTree() { treeBodies = -1; }
    void addJoint(int a, int b, V3 rA, V3 rB, float kLin, float kAng, float fracture);
    void addIgnore(int a, int b);
    void addSpring(int a, int b, V3 rA, V3 rB, float stiffness, float rest);
    void addGeneric(int a, int b, V3 rA, V3 rB, const Axis axes[6]);
    void step();
    void stepInterleaved(int substeps, int rounds);
    // Solver::pick / collectAABB (src/avbd/solver_query.cpp): body ids, -1 = no hit.
    int pick(V3 origin, V3 dir, uint32_t mask, V3 &local) const;
    void collectAABB(V3 lo, V3 hi, uint32_t mask, std::vector<int> &out) const;
    uint64_t digest() const;

    // Independent per-body / per-manifold loops use all host threads unless `threads` is 1 (the
    // reference's Solver::threads convention); results do not depend on the thread count.
    bool parallel() const { return P.threads != 1; }

    int count() const { return static_cast<int>(bodies.size()); }
    int listIndex(int id) const { return count() - 1 - id; }
    int idAt(int listIdx) const { return count() - 1 - listIdx; }

private:
    float collisionDt = 0;
    // Adjacency per list index (src/avbd/manifold.hpp:157-176).
    std::vector<int> adjStart;
    std::vector<Ref> adjRefs;
    std::vector<int> overflowOrder, colourBegins, colourOrder;
    std::vector<V3> aabbCenter, aabbHalf;
    int treeBodies = -1, treeAge = 0; // code/order refresh schedule of the reference's LBVH

    void buildAdjacency();
    int otherBody(const Ref &r, int body) const;
    bool pairConstrained(int a, int b) const;
    void broadPhase();
    int warmstartForces();
    void selectUpdateBodies();
    void colourGraph();
    void runSubstep(int forceCount, int rounds, bool idleDetection);
    void iterate(int rounds, int forceCount);
    void warmstartBody(Body &b);
    void finishBody(Body &b, bool idleDetection);
    void islandSleep();
    void projectContacts(bool projectPositions, float window);
    void rebase(Manifold &m);

    // Manifold pieces (src/avbd/manifold.cpp).
    bool manifoldInitialize(Manifold &m);
    bool frozen(const Manifold &m) const;
    void preCompute(Manifold &m);
    void stampCached(const Manifold &m, int body, struct Block &block) const;
    void manifoldUpdatePrimal(Manifold &m, int body, struct Block &block);
    void manifoldUpdateDual(Manifold &m);
    void decayPenalty(Manifold &m, float decay);
    int collide(const Body &A, const Body &B, Contact *out, M3 &basis) const;

    // Joint pieces (src/avbd/joint.cpp).
    V3 jointLin(const Force &f) const;
    V3 jointAng(const Force &f) const;
    bool jointInitialize(Force &f);
    void jointUpdatePrimal(const Force &f, int body, struct Block &block) const;
    void jointUpdateDual(Force &f);
    // Spring and GenericJoint pieces (src/avbd/spring.cpp, generic_joint.cpp).
    void springUpdatePrimal(const Force &f, int body, struct Block &block) const;
    Q4 frameOrientation(const Force &f) const;
    V3 genericOffset(const Force &f) const;
    void genericAngles(const Force &f, float out[3]) const;
    float penaltyLimit(int body, V3 axis, bool angular) const;
    void genericInitialize(Force &f);
    void genericUpdatePrimal(const Force &f, int body, struct Block &block) const;
    void genericUpdateDual(Force &f);
    // Primal and dual of any non-manifold force.
    void forceUpdatePrimal(const Force &f, int body, struct Block &block) const;
    void forceUpdateDual(Force &f);
};

// Box-box narrow phase with a speculative margin (src/avbd/collide.cpp:1001-1098). Exposed for
// the collide parity test.
int collideBoxes(V3 ca, Q4 qa, V3 ha, V3 cb, Q4 qb, V3 hb, float margin, Contact *out, M3 &basis);

} // namespace oracle
