// Host-side launchers of the step's kernels (one function per kernel or kernel group).
#pragma once

#include "engine.cuh"

namespace avbdg {

// Kernels with one thread per independent item take their block size from the autotuner (their
// results do not depend on it); the candidates are the sizes each kernel's registers allow.
constexpr int kTuneCandidates = 4;
struct TuneSpace {
    int sizes[kTuneCandidates];
    int count;
};
constexpr TuneSpace kTuneDual{{64, 128, 256, 512}, 4};     // dualKernel (one thread per manifold)
constexpr TuneSpace kTuneSolve{{32, 64, 128, 0}, 3};       // overflowSolveKernel (launch bound 128)
constexpr TuneSpace kTuneNarrow{{64, 128, 256, 512}, 4};   // manifoldInitKernel
constexpr TuneSpace kTuneTraverse{{64, 128, 256, 512}, 4}; // traverseKernel

// ---- broad phase (k_broad.cu) ----
// Body and world counts come from the device (C_BODIES, C_WORLDS); grids cover the capacities,
// so a captured step stays valid while worlds are added or removed.
void launchAabb(const Dev &d, const StepParams &p, cudaStream_t s);
// Morton codes per body, the stable (code, list position) sort, with `multiWorld` a second stable
// pass by world so each world's leaves are contiguous, then the Karras topology per world.
void launchRebuildTree(const Dev &d, bool multiWorld, cudaStream_t s);
void launchRefit(const Dev &d, cudaStream_t s);
// Candidate pairs: traversal count, scan, emit, per-segment sort. Leaves the count in C_PAIRS.
// `brute`: every world of the store is small, and each body tests its world's bodies directly
// (the same pair set; the tree's bounds are not needed).
void launchPairs(const Dev &d, int block, bool brute, cudaStream_t s);
// Exact filter and acquisition of new manifolds after the live ones (C_CAND = C_LIVE + new).
void launchFilterAcquire(const Dev &d, cudaStream_t s);

// ---- manifolds and adjacency (k_manifold.cu) ----
void launchAdjacency(const Dev &d, cudaStream_t s);
void launchManifoldInit(const Dev &d, const StepParams &p, bool round, int block, cudaStream_t s);
void launchManifoldCompact(const Dev &d, cudaStream_t s);
void launchRebase(const Dev &d, const StepParams &p, cudaStream_t s);
void launchForceInit(const Dev &d, const StepParams &p, bool forces, cudaStream_t s);

// ---- update set and colouring (k_solve.cu) ----
void launchContactOnly(const Dev &d, cudaStream_t s);
// Greedy colouring of dynamic bodies in list order (when `needGreedy`), colours in d.colour;
// unless `everyWorld`, only worlds a force touches are coloured (the rest go to overflow).
void launchColour(const Dev &d, bool needGreedy, bool everyWorld, cudaStream_t s);
// Contact-only bodies to the overflow colour, then per-colour body lists and counts.
void launchColourLists(const Dev &d, int contactOnlyOverflow, cudaStream_t s);

// ---- substep (k_solve.cu) ----
void launchWarmstartBodies(const Dev &d, const StepParams &p, cudaStream_t s);
// BDF1 velocities; with `idle` (the tick's last substep) also idle detection for sleeping.
void launchFinishBodies(const Dev &d, const StepParams &p, bool idle, cudaStream_t s);
// Stamps (precompute) of manifolds touching the overflow set; `mixedOnly` restricts to those that
// also touch a coloured body (recomputed after the colour passes).
void launchStamps(const Dev &d, const StepParams &p, bool mixedOnly, cudaStream_t s);
// `armsFromDual`: a dual pass ran since the manifolds were (re)initialised or rebased.
// The rounds of a substep for a store without forces or coloured bodies, as one persistent launch
// over a (round, phase, world, chunk) tile queue; per round: Newton (solve) or not, stamps written
// by its dual or not, and the stiffness decay of its dual.
constexpr int kMaxQueueRounds = 32;
struct QueueRounds {
    int rounds;
    unsigned newtonMask, stampMask;
    real decay[kMaxQueueRounds];
};
void launchRoundQueue(const Dev &d, const StepParams &p, const QueueRounds &qr, cudaStream_t s);

// One round's Gauss-Seidel colour passes, colours in order, in one cooperative launch.
void launchColourSweep(const Dev &d, const StepParams &p, bool armsFromDual, cudaStream_t s);
// Block-Jacobi solve of every dynamic body in the overflow colour (walked in slot order).
void launchOverflowSolve(const Dev &d, const StepParams &p, bool inPlace, bool forces, int block, cudaStream_t s);
void launchOverflowApply(const Dev &d, const StepParams &p, cudaStream_t s);
// Dual pass over live manifolds; with `stamps`, also the next round's stamps of manifolds whose
// bodies are all overflow or static. `decay` < 1 scales penalties first (dual-only rounds).
void launchDual(const Dev &d, const StepParams &p, bool stamps, real decay, int block, cudaStream_t s);
void launchForceDual(const Dev &d, const StepParams &p, bool forces, cudaStream_t s);

// ---- projection (k_proj.cu) ----
// projectionActive per world and the brake candidates (manifolds with an open gap).
void launchProjActive(const Dev &d, cudaStream_t s);
void launchBrake(const Dev &d, real window, cudaStream_t s);
void launchProjection(const Dev &d, const StepParams &p, cudaStream_t s);

int brakeGridBlocks();
int projectionGridBlocks();
// Constant tables of the narrow phase (cylinder rim directions); before any capture.
void prepareNarrowPhase();
int colourGridBlocks();
// Kernel attributes and cooperative grid sizes, set once before any stream capture.
void prepareKernels();
// Whether every instantiation of a tuned kernel can launch with `block` threads (the autotuner
// only tries sizes that fit; the FP64 build uses far more registers per thread).
bool dualBlockFits(int block);
bool solveBlockFits(int block);
bool narrowBlockFits(int block);
bool traverseBlockFits(int block);

// ---- host state exchange (k_io.cu) ----
// Layout of `buf`: [pos 3n | quat 4n | vel 3n | angvel 3n] for bodies [first, first + n).
void launchPackState(const Dev &d, int first, int count, float *buf, cudaStream_t s);
// `bad` (may be null): a device flag; when set, the unpack writes nothing.
void launchUnpackState(const Dev &d, int first, int count, const float *buf, int mask, const int *bad, cudaStream_t s);
void launchCheckState(int count, const float *buf, int mask, int *bad, cudaStream_t s);

// ---- sleeping (k_sleep.cu; only when Solver::sleepFrames > 0) ----
// Broad-phase wake-up over the valid pairs (after the filter), in pair order per world.
void launchSleepWakePairs(const Dev &d, cudaStream_t s);
// Wake pass over the adjacency, then island sleep (before the update set is chosen).
void launchSleepSelect(const Dev &d, const StepParams &p, cudaStream_t s);

// ---- queries (k_query.cu) ----
// Rays: 6 floats each (origin, dir). `best` holds one key per ray; results in world creation index.
void launchPick(const Dev &d, int base, int count, const float *rays, int nRays, unsigned mask,
                unsigned long long *best, int *outBody, float *outLocal, cudaStream_t s);
void launchCollectAabb(const Dev &d, int base, int count, f3 lo, f3 hi, unsigned mask, int *flags, int *rank,
                       int *total, void *scanScratch, int capacity, int *out, cudaStream_t s);

// ---- world removal (k_relocate.cu) ----
// Moves the surviving worlds' bodies down to their new bases (remap: per old world, new id or -1
// and new base), drops the removed worlds' manifolds and forces, keeping live and force order.
// The caller uploads the new world table afterwards and then rebuilds the list-position map.
void launchRelocateWorlds(const Dev &d, int nOld, int nNew, int nForces, const int *remap, cudaStream_t s);
void launchListPositions(const Dev &d, int nBodies, cudaStream_t s);

} // namespace avbdg
