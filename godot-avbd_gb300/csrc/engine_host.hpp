// Host orchestration of the GB300 AVBD step (C++ runtime under the C ABI).
//
// An Engine owns one CUDA stream and the device store of a set of worlds. `step()` enqueues the
// phases of avbd::Solver::step (src/avbd/solver_step.cpp:44-75) for every world at once; all
// counts stay on the device, so a step needs no host round trip except the capacity check at its
// end and, when joints exist, the colouring rounds.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "avbdg.h"
#include "engine.cuh"
#include "kernels.cuh"

namespace avbdg {

class Engine {
public:
    Engine(const avbdg_params &params, int maxBodies, int maxForces, int maxWorlds);
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Worlds. A new world's bodies occupy the next free slots; only the last world can grow.
    int addWorld();
    int addBodies(int world, int count, const avbdg_body_desc *descs, int *outIds);
    int addJoint(int world, int a, int b, const float rA[3], const float rB[3], float kLin, float kAng,
                 float fracture);
    int addIgnore(int world, int a, int b);
    // Forces of `world` in creation order (kind 0 ball joint, 1 ignore pair), one upload for all.
    int addForces(int world, int count, const avbdg_force_desc *descs);
    // Remove the listed worlds. The others keep their order and their results: they move down to
    // dense body slots and are renumbered 0.. in order; their manifolds and forces are carried.
    int removeWorlds(const std::vector<int> &ids);
    void clear();
    // A store with no worlds gives its device memory back down to the smallest capacities (64
    // bodies); the next worlds grow it again. No effect on a store that holds worlds.
    int shrinkEmpty();

    // Checks addBodies / addForces apply before touching the store (a world of `nb` bodies).
    static int validateBodies(int count, const avbdg_body_desc *descs, std::string &why);
    static int validateForces(int nb, int count, const avbdg_force_desc *descs, std::string &why);

    // Device bytes of a store with these capacities (bodies, manifolds, forces, pairs, worlds).
    static size_t storeBytes(int nb, int mm, int ff, int pp, int ww, bool arm = false);
    // Capacities for `nb` bodies the store grows to (manifolds and pairs follow the body count).
    static size_t storeBytesForBodies(int nb, int ff, int ww) { return storeBytes(nb, 8 * nb, ff, 16 * nb, ww); }
    size_t reservedBytes() const { return storeBytes(d.NB, d.MM, d.FF, d.PP, d.WW, d.ARM != 0); }
    // Upper bound on the store's device bytes (0 = none): growth headroom is cut to fit, and a
    // growth that cannot fit fails with AVBDG_ERR_CAPACITY.
    void setByteLimit(size_t bytes) { byteLimit = bytes; }

    int setParams(const avbdg_params &p);
    const avbdg_params &params() const { return P; }

    // Enqueue one step of every world (Solver::step / Solver::stepInterleaved).
    int step();
    // step() in two halves, for a caller that steps several stores at once on their own streams:
    // stepEnqueue hands the step to this store's stream, stepFinish waits for it and checks its
    // counters (growing the store as step() does). Nothing may change the store in between.
    int stepEnqueue();
    int stepFinish();
    int stepInterleaved(int substeps, int rounds);
    // `count` steps (substeps > 1: stepInterleaved(substeps, rounds)), queued back to back while the
    // store has room; each step's counters are still checked in order.
    int stepMany(int count, int substeps, int rounds);
    int sync();

    int getState(int world, int first, int count, float *pos, float *quat, float *vel, float *angVel);
    int getSleeping(int world, int first, int count, uint8_t *out);
    // Solver::pick / collectAABB of one world (body ids in creation order).
    int pick(int world, int count, const float *origins, const float *dirs, uint32_t mask, int *outBody,
             float *outLocal);
    int collectAabb(int world, const float lo[3], const float hi[3], uint32_t mask, int capacity, int *out,
                    int *outCount);
    int setState(int world, int first, int count, const float *pos, const float *quat, const float *vel,
                 const float *angVel);
    int stats(avbdg_stats &out);
    int digest(int world, uint64_t &out);
    int dumpBroadphase(uint64_t *codes, int32_t *order, int capN, uint64_t *pairs, int capP, int *nB, int *nP);
    int dumpManifolds(int cap, int32_t *ba, int32_t *bb, int32_t *nc, int32_t *features, float *basis, float *c0,
                      float *penalty, float *lambda, int *count);
    int dumpColours(int cap, uint8_t *colour, int32_t *bodyId, int *count);

    // Profiling times single launches, so it runs steps eagerly (outside the graph cache).
    void setProfiling(bool on) { profiling = on; }
    void setGraphs(bool on) {
        useGraphs = on;
        if (!on)
            dropGraphs();
    }
    bool graphsEnabled() const { return useGraphs; }
    // Bound of the dataflow waits (colouring, brake sweep) in spins; 0 gives up at the first
    // unfinished predecessor, a negative value restores the default.
    void setWaitLimit(long long spins) {
        waitLimit = spins < 0 ? kDefaultWaitLimit : spins;
        d.waitLimit = waitLimit;
        dropGraphs(); // the limit is part of every captured launch's arguments
    }
    void takeKernelTimes(avbdg_kernel_times &out);

    int worlds() const { return static_cast<int>(wBase.size()); }
    int worldBodies(int w) const { return wCount[w]; }
    int worldDynamic(int w) const { return wDyn[w]; }
    int bodies() const { return nBodies; }
    int dynamicBodies() const { return nDynamic; }
    int forces() const { return nForces; }
    cudaStream_t streamHandle() const { return stream; }
    // Kernel launches of the last step (this library's kernels only).
    int lastLaunches() const { return launches; }
    bool lastStepWasGraph() const { return lastGraph; }
    const std::string &error() const { return err; }

private:
    avbdg_params P;
    Dev d{};
    long long waitLimit = kDefaultWaitLimit;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    std::vector<int> wBase, wCount, wDyn, wRound;
    int nBodies = 0, nDynamic = 0, nForces = 0, nRound = 0; // nRound: spheres and cylinders
    int treeAge = 0;
    bool treeValid = false, adjValid = false;
    bool armStore = false; // the store carries the arm-cache arrays (set once the cache is first on)
    size_t byteLimit = 0;
    int steps = 0;
    int launches = 0;
    int hostCtr[C_COUNT] = {};
    // stepMany: counters of queued steps come back through a two-slot pinned ring, each slot with
    // the event that marks its copy; ctrFresh is true when hostCtr holds a step of the current
    // store (cleared whenever the store or its contents change).
    int *ctrRing = nullptr;
    cudaEvent_t ctrEvent[2] = {nullptr, nullptr};
    int ctrLaunches[2] = {0, 0};
    bool ctrFresh = false;
    int processCounters();
    int finishQueued(int slot);
    bool roomy() const;
    int colourSizes[kMaxColours + 1] = {};
    cudaEvent_t ev[5] = {};
    bool timed = false;
    std::string err;
    // Profiling: event pairs around the hot launches of the current step.
    bool profiling = false;
    enum KernelKind { kManifold = 0, kBody = 1, kNarrow = 2, kTraverse = 3, kKinds = 4 };
    struct Span {
        cudaEvent_t a, b;
        int kind;
    };
    std::vector<cudaEvent_t> evPool;
    std::vector<Span> spans;
    size_t evUsed = 0;
    avbdg_kernel_times acc{};
    int launchBase = 0;
    // Autotuned block sizes (candidates in kernels.cuh). After a store is created or regrown,
    // kTuneDelay steps run as usual, then kTuneTrials eager steps try the candidates in turn,
    // timed by events around each tuned launch; the fastest per kernel is kept.
    struct Tuned {
        int dual = 256, solve = 128, narrow = 256, traverse = 256;
    };
    Tuned tuned;
    Tuned tunedBase; // the default sizes, each replaced by the largest candidate that launches if it does not
    static constexpr int kTuneDelay = 4, kTuneTrials = 8;
    // Largest world whose candidate pairs come from the all-pairs test: each body of it walks up to
    // this many candidates, which costs less than refitting and walking the tree below this size.
    static constexpr int kBruteMaxBodies = 512;
    bool tuneEnabled = true, tuning = false;
    int tuneTrial = 0;
    double tuneMs[kKinds][kTuneCandidates] = {};
    int tuneN[kKinds][kTuneCandidates] = {};
    bool tuneFits[kKinds][kTuneCandidates] = {}; // the candidate can launch (occupancy >= 1 block)
    void armTuning();
    void configureTrial();
    void finishTrial();
    int beginSpan();
    void endSpan(int kind);
    void collectSpans();
    // Pinned host staging for state upload/download (13 floats per body).
    float *ioHost = nullptr;
    float *ioDev = nullptr;
    int *ioFlag = nullptr; // device: non-finite upload seen (after the 13 x ioCap floats of ioDev)
    int ioCap = 0;
    // Body state moves straight between the caller's (pageable) arrays and the device, where the
    // device reaches host memory through the host's page tables; else through pinned staging.
    bool roundQueue = false; // AVBDG_QUEUE=1: the round loop as one tile-queue launch where it applies
    bool bruteAllowed = true; // AVBDG_NO_BRUTE=1: candidate pairs always from the tree walk
    bool stepPending = false; // stepEnqueue ran, stepFinish has not
    int pendingLaunches = 0;  // kernels the pending step launched
    bool directIo = false;
    int ensureIo(int count);

    int fail(int code, const std::string &msg);
    int slotRange(int w, int first, int count, int &g0);
    int cudaCheck(const char *where);
    void allocate(int nb, int mm, int ff, int pp, int ww);
    void releaseAll();
    template <typename T>
    T *dalloc(size_t n);
    int ensureCapacity(int nb, int ff, int ww);
    void uploadCounts();
    bool fits(int nb, int mm, int ff, int pp, int ww) const {
        return byteLimit == 0 || storeBytes(nb, mm, ff, pp, ww, armStore) <= byteLimit;
    }
    StepParams stepParams(real collisionDt) const;
    // Host decisions of one step; the enqueued work depends on nothing else but device counts.
    struct StepPlan {
        int mode = 0; // 0 step, 1 interleaved
        int substeps = 1, rounds = 0;
        bool adjAtStart = false, anyTree = false, rebuild = false, forces = false, greedy = false;
        bool multiWorld = false, round = false;
        bool brute = false; // pairs by the all-pairs test within each world instead of the tree
        std::string key() const;
    };
    struct Graph {
        cudaGraphExec_t exec;
        int launches;
        std::vector<Span> spans; // profiling spans recorded by the graph's event nodes
    };
    const std::vector<Span> *graphSpans = nullptr; // spans of the graph the last step ran
    std::map<std::string, Graph> graphs;
    std::map<std::string, int> planSeen; // plans run since the cache was dropped (capture on reuse)
    bool useGraphs = true, capturing = false, lastGraph = false;
    std::string graphError;
    StepPlan planStep(int mode, int substeps, int rounds);
    bool enqueueStep(const StepPlan &plan); // false: a launch failed (the rest was not enqueued)
    int launchFailure();
    int enqueuePlan(const StepPlan &plan);
    int runPlan(const StepPlan &plan);
    void dropGraphs();
    void recordPhase(cudaEvent_t e);
    int broadPhase(const StepParams &sp, const StepPlan &plan);
    int warmstartAndSelect(const StepParams &sp);
    void projectContacts(const StepParams &sp, bool positions, real window);
    void runSubstep(const StepParams &sp, int rounds, bool idle);
    int finishStep();
    bool needGreedy() const;
};

} // namespace avbdg
