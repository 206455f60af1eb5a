// Device data layout and kernel entry points of the GB300 AVBD step.
//
// One Engine holds a SET of independent worlds (one for the plain avbdg_world API, thousands for
// the batched API). Each world owns a contiguous range of body slots; manifolds, forces, pairs
// and adjacency of all worlds live in shared arrays and never reference two worlds at once, so
// every kernel runs over the whole set in one launch.
//
// HBM layout (SoA, 16-byte records so each body or contact field is one 128-bit load):
//   bodies    x, q, x0, q0, xi, qi, v, w, vprev : float4   (x.w = mass, v.w = gravity)
//             size (xyz, w = bounding radius), moment (xyz, w = friction), meta (int4)
//   manifolds live order, dense: ab (int2), basis rows b0 (xyz, w = mu), b1, b2, count
//   contacts  stride 8 per manifold: key, rA (w = adaptive beta scale), rB, C0, k, lam (w = stick)
//   stamps    per (manifold, side) 7 float4: the Jacobi block contribution of that side
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dmath.cuh"

namespace avbdg {

constexpr int kMaxContacts = 8;
constexpr int kMaxColours = 8;
constexpr uint8_t kOverflowColour = 8;
constexpr uint8_t kUncoloured = 255;
constexpr int kStampF4 = 7; // float4 per (manifold, side) stamp
constexpr int kPairStash = 64; // partners kept per body by the counting walk
constexpr int kExtF4 = 16;  // float4 per force of the generic-joint record (forces.cuh)
// Spins (64 ns sleeps) a dataflow wait of the colouring or the brake sweep makes before it gives
// up and reports a timeout: ~0.3 s, far beyond any real dependency hop.
constexpr long long kDefaultWaitLimit = 4000000;

constexpr real PENALTY_MIN = 1.0f;
constexpr real PENALTY_MAX = 10000000000.0f;
constexpr real ADAPTIVE_BETA_MAX = 64.0f;
constexpr real COLLISION_MARGIN = 0.001f;
constexpr real STICK_THRESH = 0.00001f;
constexpr real CONTACT_RELEASE_GAP = 2.0e-3f;
constexpr real kReleaseAbove = COLLISION_MARGIN + CONTACT_RELEASE_GAP;

// Device counters (indices into Dev::ctr).
enum Counter {
    C_PAIRS = 0,      // candidate pairs this step
    C_LIVE,           // live manifolds
    C_CAND,           // live + newly acquired, before compaction
    C_FORCES,         // live forces
    C_ADJ,            // adjacency entries
    C_LONG,           // long segments (segmented sort scratch)
    C_SPECN,          // brake candidates in specList
    C_BODIES,         // body slots in use (all worlds)
    C_WORLDS,         // worlds
    C_ERRORS,         // capacity / timeout bits (kErr*)
    C_ONE,            // constant 1 (scan length helper)
    C_SOLVEFAIL,      // overflow bodies whose plain LDLT failed this round (solveFail)
    C_PAIRSPILL,      // bodies with more broad-phase partners than the stash holds (pairSpill)
    C_QSOLVE,         // round-loop queue: solve tiles a round (all worlds)
    C_QDUAL,          // round-loop queue: dual tiles a round (all worlds)
    C_TMP,
    C_COUNT
};

constexpr int kErrPairs = 1;
constexpr int kErrManifolds = 2;
constexpr int kErrAdjacency = 4;
constexpr int kErrBrakeTimeout = 8;
constexpr int kErrColourTimeout = 16;
constexpr int kErrBarrierTimeout = 32; // a grid barrier of a cooperative sweep gave up
constexpr int kErrQueueTimeout = 64;   // a tile of the round-loop queue waited too long for its world

// Solver fields a kernel reads (src/avbd/solver.h:54-144), with derived terms.
struct StepParams {
    real dt, dtSq, collisionDt;
    real alpha, oneMinusAlpha, betaLin, betaAng, gamma;
    real stiffnessDecay, jacobiRelax, stickDriftHeal, maxPen, specMargin;
    real projBeta, projSlop, projMaxCorr, adaptiveFloor;
    int adaptiveBeta, contactOnlyOverflow, projIters;
    int sleepFrames;              // 0 = sleeping off
    int graceTicks;               // Solver::contactGraceTicks (0 = off)
    real graceSeed;              // penalty of a fresh contact under grace: max(PENALTY_MIN, 0.05 betaLin)
    real sleepLin2, sleepAng2;   // squared velocity thresholds of idle detection
    int armCache;                 // Solver::jacobianRebuildDistance > 0
    real armRebuild2;            // its square
};

struct ManifoldBuf {
    int2 *ab;          // global body indices (a = smaller list index)
    real4 *b0, *b1, *b2;
    int *count;
    int2 *dormant;     // contact grace: x = ticks parked, y = contacts kept for revival
    int *key;          // contacts: slot-major, see cslot
    real4 *rA, *rB, *C0, *k, *lam;
    // Arm cache (Solver::jacobianRebuildDistance, manifold.cpp:600-668): world arms (slot-major like
    // the contacts), the first rotation columns captured with them and the kArmsCached flag.
    // Allocated only while the cache is on (Dev::ARM).
    real4 *armA, *armB;
    real4 *capA, *capB;
    uint8_t *armFlag;
};

struct Dev {
    int NB, MM, FF, PP, WW; // capacities
    int ARM;                // 1: the arm-cache arrays of ManifoldBuf are allocated
    long long waitLimit;    // spins a dataflow wait makes before it reports a timeout
    unsigned *gridBar;      // grid barrier of the cooperative sweeps: arrivals, generation
    // Round-loop tile queue (k_queue.cu): each world's live manifolds grouped together (wManStart,
    // wManList), the prefix sums of the worlds' solve and dual chunk counts (qPre: WW + 1 each), and
    // per world the phases completed (qStage) and the chunks of the current phase done (qDone).
    int *wManStart, *wManFill, *wManList;
    int *qPre, *qStage, *qDone;
    unsigned *qTicket;
    // worlds
    int *wBase, *wCount;    // body range
    int *wMaxDepth;         // projection: max depth bits per world (positive floats)
    int *wStop;             // projection: early-exit flag per world
    int *wBounds;           // Morton scene bounds per world: lo xyz, hi xyz (ordered ints)
    int *wActive;           // projection: movable manifolds per world (0 = skip the world)
    int *wColour;           // colouring: 1 if a force touches the world (its bodies need colours)
    int *wSleep;            // sleep: first compacted sleeper pair and their count, per world
    // bodies
    real4 *x, *q, *x0, *q0, *xi, *qi, *v, *w, *vprev;
    real4 *size, *moment;
    int4 *meta;             // x = world, y = layer, z = mask, w = lockLin | lockAng << 8 | sleepMode << 16
    int2 *sleep;            // x = sleeping, y = still frames (Rigid::sleeping, stillFrames)
    uint8_t *upd;           // this step's update set (Rigid::inUpdateSet)
    int *lpToBody;          // list position -> body
    uint8_t *contactOnly, *colour;
    real4 *aabbC, *aabbH;
    // LBVH
    uint64_t *codes;        // per body: the reference's Morton code of the last rebuild (dumps)
    uint64_t *treeCodes;    // per body: the code the tree is built from (true per-axis origin)
    uint64_t *sortK, *sortKAlt;
    uint32_t *sortV, *sortVAlt;
    int *leafBody;          // sorted position -> body
    int *nodeL, *nodeR, *nodeParent, *leafParent, *nodeFlag;
    int *nodeMaxLp;         // largest list position in the subtree (prunes the pair walk)
    real4 *nodeMin, *nodeMax;
    // What the pair walk reads at an internal node, written by the refit in one place: its
    // children's boxes (left min, left max, right min, right max) and (left, right, largest list
    // position under the left child, under the right child; a leaf's own position).
    real4 *nodeKids;
    int4 *nodeLink;
    // pairs
    int *pairStart;         // per list position (+1)
    uint64_t *pairs, *pairsTmp;
    int *pairValid;         // then exclusive rank
    // manifolds
    ManifoldBuf live, stage;
    int *mActive;           // then exclusive rank
    real4 *stamps;         // block stamps, one per adjacency entry (the entry of the stamped body)
    int2 *stampSlot;        // per live manifold: the adjacency entries of its side-A and side-B stamps
    uint8_t *mSpec, *mDone; // brake: candidate flag per manifold, done flag per candidate
    int *specList;
    int *solveFail;         // overflow bodies left to the pivoted fallback this round
    int *pairStash;         // broad phase: first kPairStash partners' list positions per body list position
    int *pairSpill;         // broad phase: bodies whose partners overflow the stash (walked again)
    int2 *specPred;         // brake: candidate index of the preceding candidate on each movable body (-1 = none)
    real4 *projLin, *projAng; // projection contributions, one per adjacency entry (w: side sign, 0 = none)
    real4 *dLin, *dAng;       // block-Jacobi deltas per body (when applied in a separate pass)
    // forces (creation order; list order is descending index)
    int2 *fAB;
    real4 *fRA, *fRB, *fC0L, *fC0A, *fKL, *fKA, *fLL, *fLA, *fPar; // fPar: stiffLin, stiffAng, fracture, torqueArm
    int *fKind, *fBroken, *fKeep;
    real4 *fExt;           // generic joints: kExtF4 float4 per force (forces.cuh)
    // adjacency (dynamic bodies only): sequence numbers, forces first (list order) then manifolds
    int *adjStart, *adjFill;
    uint32_t *adjSeq, *adjTmp;
    int *adjInfo;           // per adjacency entry: the other body (kNoBody: none) | side (0: body is a, 1: b) << 31
    // colouring
    int *colourList, *colourCount; // per colour c: bodies with colour c (c = 0..8)
    // scratch
    int *ctr;
    int *longList;
    void *scanScratch, *radixScratch;
    // sleep: compacted sleeper pairs (rank, list), union-find parent and island aggregates
    int *sleepRank, *sleepList;
    int *island, *islandAwake, *islandStill;
    // world removal: slot map (NB) + force ranks (FF), staging of max(NB, FF * kExtF4) records,
    // world remap
    int *relocInt;
    real4 *relocF4;
    int *relocRemap;        // 2 per world: new id (-1 = removed), new base slot
};

// ---- device helpers shared by the kernel files ----

__device__ __forceinline__ int bodyWorld(const Dev &d, int g) { return d.meta[g].x; }
// Contact slot c of manifold m. The contact arrays are slot-major (MM entries per slot), so a warp
// reading slot c of 32 consecutive manifolds reads 512 contiguous bytes.
AVBD_HD int cslot(const Dev &d, int m, int c) { return c * d.MM + m; }
// List position of body g: the world's bodies in list order (reverse creation) occupy
// [wBase, wBase + wCount).
__device__ __forceinline__ int listPos(const Dev &d, int g) {
    const int w = d.meta[g].x;
    return 2 * d.wBase[w] + d.wCount[w] - 1 - g;
}
__device__ __forceinline__ bool isDynamic(const Dev &d, int g) { return d.x[g].w > 0.0f; }
// Movable and not asleep (ManifoldStore::frozen's `awake`, manifold.cpp:168-172).
// Adjacency entry info: the other body of the entry's force or manifold and this body's side.
constexpr int kNoBody = 0x7fffffff;
__device__ __forceinline__ int adjInfoOther(int v) {
    const int o = v & 0x7fffffff;
    return o == kNoBody ? -1 : o;
}
__device__ __forceinline__ int adjInfoSide(int v) { return static_cast<int>(static_cast<unsigned>(v) >> 31); }
// In this step's update set (solved, braked, projected).
__device__ __forceinline__ bool inUpdate(const Dev &d, int g) { return d.upd[g] != 0; }
constexpr uint8_t kNotUpdated = 10; // colour of a movable body outside the update set

} // namespace avbdg
