// Host orchestration of the GB300 AVBD step: device store, capacity management and the phase
// sequence of avbd::Solver::step / stepInterleaved (godot-avbd src/avbd/solver_step.cpp:44-160).

#include "engine_host.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <type_traits>
#include <unistd.h>
#include <vector>

#include "kernels.cuh"
#include "prims.cuh"

namespace avbdg {

namespace {

// Rigid::Rigid (src/avbd/rigid.cpp:22-72) per shape; host compiled with -ffp-contract=off.
void massProperties(const avbdg_body_desc &b, real &mass, real moment[3], real &radius) {
    if (b.shape == AVBDG_SHAPE_SPHERE) {
        const real r = b.size[0];
        mass = (4.0f / 3.0f) * 3.14159265358979f * r * r * r * b.density;
        const real i = 0.4f * mass * r * r;
        moment[0] = moment[1] = moment[2] = i;
        radius = r;
        return;
    }
    if (b.shape == AVBDG_SHAPE_CYLINDER) {
        const real r = b.size[0], h = b.size[2];
        mass = 3.14159265358979f * r * r * h * b.density;
        const real axial = 0.5f * mass * r * r;
        const real radialM = mass * (3.0f * r * r + h * h) / 12.0f;
        moment[0] = moment[1] = radialM;
        moment[2] = axial;
        const real hh = h * 0.5f;
        const real px = r * r, py = hh * hh, pz = r * r;
        real s = 0.0f;
        s = s + px;
        s = s + py;
        s = s + pz;
        radius = std::sqrt(s);
        return;
    }
    const real sx = b.size[0], sy = b.size[1], sz = b.size[2];
    mass = sx * sy * sz * b.density;
    moment[0] = (sy * sy + sz * sz) / 12.0f * mass;
    moment[1] = (sx * sx + sz * sz) / 12.0f * mass;
    moment[2] = (sx * sx + sy * sy) / 12.0f * mass;
    const real hx = sx * 0.5f, hy = sy * 0.5f, hz = sz * 0.5f;
    const real px = hx * hx, py = hy * hy, pz = hz * hz;
    real s = 0.0f;
    s = s + px;
    s = s + py;
    s = s + pz;
    radius = std::sqrt(s);
}

bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

constexpr int kRefitBudget = 16; // src/avbd/bvh_broadphase.hpp:40

// Every device buffer of a store, in one place: `take(ptr, count)` allocates (or counts) `count`
// elements of ptr's type.
template <typename Take>
void layoutStore(Dev &n, int nb, int mm, int ff, int pp, int ww, bool arm, Take &&take) {
    n.NB = nb;
    n.ARM = arm ? 1 : 0;
    n.MM = mm;
    n.FF = ff;
    n.PP = pp;
    n.WW = ww;
    take(n.wBase, ww);
    take(n.wCount, ww);
    take(n.wMaxDepth, ww);
    take(n.wStop, ww);
    take(n.wBounds, 6 * static_cast<size_t>(ww));
    take(n.wActive, ww);
    take(n.wColour, ww);
    take(n.wSleep, 2 * static_cast<size_t>(ww));
    take(n.gridBar, 2);
    take(n.wManStart, static_cast<size_t>(ww) + 1);
    take(n.wManFill, ww);
    take(n.qPre, 2 * (static_cast<size_t>(ww) + 1));
    take(n.qStage, ww);
    take(n.qDone, ww);
    take(n.qTicket, 1);
    take(n.x, nb);
    take(n.q, nb);
    take(n.x0, nb);
    take(n.q0, nb);
    take(n.xi, nb);
    take(n.qi, nb);
    take(n.v, nb);
    take(n.w, nb);
    take(n.vprev, nb);
    take(n.size, nb);
    take(n.moment, nb);
    take(n.meta, nb);
    take(n.sleep, nb);
    take(n.upd, nb);
    take(n.lpToBody, nb);
    take(n.contactOnly, nb);
    take(n.colour, nb);
    take(n.aabbC, nb);
    take(n.aabbH, nb);
    take(n.codes, nb);
    take(n.treeCodes, nb);
    take(n.sortK, nb);
    take(n.sortKAlt, nb);
    take(n.sortV, nb);
    take(n.sortVAlt, nb);
    take(n.leafBody, nb);
    take(n.nodeL, nb);
    take(n.nodeR, nb);
    take(n.nodeParent, nb);
    take(n.leafParent, nb);
    take(n.nodeFlag, nb);
    take(n.nodeMaxLp, nb);
    take(n.nodeMin, nb);
    take(n.nodeMax, nb);
    take(n.nodeKids, 4 * static_cast<size_t>(nb));
    take(n.nodeLink, nb);
    take(n.pairStart, static_cast<size_t>(nb) + 1);
    take(n.pairs, pp);
    take(n.pairsTmp, pp);
    const int flagsCap = std::max(pp, mm);
    take(n.pairValid, flagsCap);
    take(n.mActive, flagsCap);
    for (ManifoldBuf *b : {&n.live, &n.stage}) {
        take(b->ab, mm);
        take(b->b0, mm);
        take(b->b1, mm);
        take(b->b2, mm);
        take(b->count, mm);
        take(b->dormant, mm);
        const size_t mc = static_cast<size_t>(mm) * kMaxContacts;
        take(b->key, mc);
        take(b->rA, mc);
        take(b->rB, mc);
        take(b->C0, mc);
        take(b->k, mc);
        take(b->lam, mc);
        const size_t am = arm ? static_cast<size_t>(mm) : 0;
        take(b->armA, am * kMaxContacts);
        take(b->armB, am * kMaxContacts);
        take(b->capA, am);
        take(b->capB, am);
        take(b->armFlag, am);
    }
    take(n.stampSlot, mm);
    take(n.wManList, mm);
    take(n.mSpec, mm);
    take(n.mDone, mm);
    take(n.specList, mm);
    take(n.specPred, mm);
    take(n.solveFail, nb);
    take(n.pairStash, static_cast<size_t>(nb) * kPairStash);
    take(n.pairSpill, nb);
    take(n.dLin, nb);
    take(n.dAng, nb);
    take(n.fAB, ff);
    take(n.fRA, ff);
    take(n.fRB, ff);
    take(n.fC0L, ff);
    take(n.fC0A, ff);
    take(n.fKL, ff);
    take(n.fKA, ff);
    take(n.fLL, ff);
    take(n.fLA, ff);
    take(n.fPar, ff);
    take(n.fKind, ff);
    take(n.fBroken, ff);
    take(n.fKeep, ff);
    take(n.fExt, static_cast<size_t>(ff) * kExtF4);
    take(n.adjStart, static_cast<size_t>(nb) + 1);
    take(n.adjFill, nb);
    const size_t adjCap = 2 * (static_cast<size_t>(ff) + mm);
    take(n.adjSeq, adjCap);
    take(n.adjTmp, adjCap);
    take(n.adjInfo, adjCap);
    take(n.stamps, adjCap * kStampF4);
    take(n.projLin, adjCap);
    take(n.projAng, adjCap);
    take(n.colourList, static_cast<size_t>(nb) * (kMaxColours + 1));
    take(n.colourCount, kMaxColours + 1);
    take(n.ctr, C_COUNT);
    take(n.longList, static_cast<size_t>(std::max(nb, 1)) + 1);
    const int scanCap = std::max({pp, mm, nb + 1, 2 * (ff + mm)}) + 1;
    char *scan = nullptr, *radix = nullptr;
    take(scan, scanScratchBytes(scanCap));
    take(radix, radixScratchBytes(nb + 1));
    n.scanScratch = scan;
    n.radixScratch = radix;
    take(n.sleepRank, pp);
    take(n.sleepList, pp);
    take(n.island, nb);
    take(n.islandAwake, nb);
    take(n.islandStill, nb);
    take(n.relocInt, static_cast<size_t>(nb) + ff);
    take(n.relocF4, std::max(static_cast<size_t>(nb), static_cast<size_t>(ff) * kExtF4));
    take(n.relocRemap, 2 * static_cast<size_t>(ww));
}

} // namespace

Engine::Engine(const avbdg_params &params, int maxBodies, int maxForces, int maxWorlds) : P(params) {
    const char *noGraphs = std::getenv("AVBDG_NO_GRAPHS");
    useGraphs = !(noGraphs && noGraphs[0] == '1');
    d.waitLimit = waitLimit;
    const char *queue = std::getenv("AVBDG_QUEUE");
    roundQueue = queue && queue[0] == '1';
    const char *noBrute = std::getenv("AVBDG_NO_BRUTE");
    bruteAllowed = !(noBrute && noBrute[0] == '1');
    const char *noTune = std::getenv("AVBDG_NO_TUNE");
    tuneEnabled = !(noTune && noTune[0] == '1');
#ifdef AVBDG_FP64
    tuneEnabled = false; // the FP64 build states an error, not a speed: default block sizes
#endif
    int dev = 0, hostTables = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&hostTables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    const char *staged = std::getenv("AVBDG_STAGED_IO");
    directIo = hostTables == 1 && !(staged && staged[0] == '1');
    armTuning();
    prepareKernels(); // attributes and occupancy queries, never during a capture
    {
        const TuneSpace *spaces[kKinds] = {&kTuneDual, &kTuneSolve, &kTuneNarrow, &kTuneTraverse};
        bool (*fits[kKinds])(int) = {dualBlockFits, solveBlockFits, narrowBlockFits, traverseBlockFits};
        int *base[kKinds] = {&tunedBase.dual, &tunedBase.solve, &tunedBase.narrow, &tunedBase.traverse};
        for (int k = 0; k < kKinds; k++) {
            for (int c = 0; c < spaces[k]->count; c++)
                tuneFits[k][c] = fits[k](spaces[k]->sizes[c]);
            if (!fits[k](*base[k])) // a default above the kernel's launch bounds or registers
                for (int c = 0; c < spaces[k]->count; c++)
                    if (tuneFits[k][c])
                        *base[k] = spaces[k]->sizes[c];
        }
        tuned = tunedBase;
    }
    cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    for (auto &e : ev)
        cudaEventCreate(&e);
    armStore = P.jacobian_rebuild_distance > 0.0f;
    const int nb = std::max(maxBodies, 64);
    allocate(nb, std::max(1024, 8 * nb), std::max(maxForces, 16), std::max(4096, 16 * nb), std::max(maxWorlds, 1));
}

Engine::~Engine() {
    if (stream)
        cudaStreamSynchronize(stream);
    dropGraphs();
    releaseAll();
    if (ioHost)
        cudaFreeHost(ioHost);
    if (ctrRing)
        cudaFreeHost(ctrRing);
    for (cudaEvent_t e : ctrEvent)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : evPool)
        cudaEventDestroy(e);
    for (auto &e : ev)
        if (e)
            cudaEventDestroy(e);
    if (stream)
        cudaStreamDestroy(stream);
}

int Engine::fail(int code, const std::string &msg) {
    err = msg;
    return code;
}

int Engine::cudaCheck(const char *where) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(AVBDG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    return AVBDG_OK;
}

template <typename T>
T *Engine::dalloc(size_t n) {
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess)
        return nullptr;
    cudaMemsetAsync(p, 0, bytes, stream);
    allocs.push_back(p);
    return static_cast<T *>(p);
}

void Engine::releaseAll() {
    for (void *p : allocs)
        cudaFree(p);
    allocs.clear();
}

void Engine::allocate(int nb, int mm, int ff, int pp, int ww) {
    ctrFresh = false;
    dropGraphs(); // they hold the old buffers' addresses
    const Dev old = d;
    std::vector<void *> oldAllocs;
    oldAllocs.swap(allocs);
    Dev n{};
    layoutStore(n, nb, mm, ff, pp, ww, armStore, [this](auto *&ptr, size_t count) {
        using T = std::remove_reference_t<decltype(*ptr)>;
        ptr = dalloc<T>(count);
    });

    if (old.NB > 0) {
        // Carry the persistent state into the new store.
        const auto cp = [this](void *dst, const void *src, size_t bytes) {
            if (dst && src && bytes)
                cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream);
        };
        const size_t nbCopy = static_cast<size_t>(std::min(old.NB, nb));
        for (auto pr : {std::make_pair(n.x, old.x), std::make_pair(n.q, old.q), std::make_pair(n.x0, old.x0),
                        std::make_pair(n.q0, old.q0), std::make_pair(n.xi, old.xi), std::make_pair(n.qi, old.qi),
                        std::make_pair(n.v, old.v), std::make_pair(n.w, old.w), std::make_pair(n.vprev, old.vprev),
                        std::make_pair(n.size, old.size), std::make_pair(n.moment, old.moment)})
            cp(pr.first, pr.second, nbCopy * sizeof(real4));
        cp(n.meta, old.meta, nbCopy * sizeof(int4));
        cp(n.sleep, old.sleep, nbCopy * sizeof(int2));
        cp(n.lpToBody, old.lpToBody, nbCopy * sizeof(int));
        cp(n.codes, old.codes, nbCopy * sizeof(uint64_t));
        cp(n.ctr, old.ctr, C_COUNT * sizeof(int));
        cudaStreamSynchronize(stream);
        int liveCount = 0;
        cudaMemcpy(&liveCount, old.ctr + C_LIVE, sizeof(int), cudaMemcpyDeviceToHost);
        const size_t mCopy = static_cast<size_t>(std::min({liveCount, old.MM, mm}));
        const ManifoldBuf &s = old.live;
        const ManifoldBuf &t = n.live;
        cp(t.ab, s.ab, mCopy * sizeof(int2));
        cp(t.b0, s.b0, mCopy * sizeof(real4));
        cp(t.b1, s.b1, mCopy * sizeof(real4));
        cp(t.b2, s.b2, mCopy * sizeof(real4));
        cp(t.count, s.count, mCopy * sizeof(int));
        cp(t.dormant, s.dormant, mCopy * sizeof(int2));
        // Contact arrays are slot-major: slot c of the old store (old.MM entries apart) to slot c of
        // the new one (mm apart).
        const bool arms = old.ARM && n.ARM;
        for (int c = 0; c < kMaxContacts; c++) {
            const size_t so = static_cast<size_t>(c) * old.MM, sn = static_cast<size_t>(c) * mm;
            cp(t.key + sn, s.key + so, mCopy * sizeof(int));
            for (auto pr : {std::make_pair(t.rA, s.rA), std::make_pair(t.rB, s.rB), std::make_pair(t.C0, s.C0),
                            std::make_pair(t.k, s.k), std::make_pair(t.lam, s.lam)})
                cp(pr.first + sn, pr.second + so, mCopy * sizeof(real4));
            if (arms) {
                cp(t.armA + sn, s.armA + so, mCopy * sizeof(real4));
                cp(t.armB + sn, s.armB + so, mCopy * sizeof(real4));
            }
        }
        if (arms) {
            cp(t.capA, s.capA, mCopy * sizeof(real4));
            cp(t.capB, s.capB, mCopy * sizeof(real4));
            cp(t.armFlag, s.armFlag, mCopy * sizeof(uint8_t));
        }
        const size_t fCopy = static_cast<size_t>(std::min(old.FF, ff));
        cp(n.fAB, old.fAB, fCopy * sizeof(int2));
        for (auto pr : {std::make_pair(n.fRA, old.fRA), std::make_pair(n.fRB, old.fRB), std::make_pair(n.fC0L, old.fC0L),
                        std::make_pair(n.fC0A, old.fC0A), std::make_pair(n.fKL, old.fKL), std::make_pair(n.fKA, old.fKA),
                        std::make_pair(n.fLL, old.fLL), std::make_pair(n.fLA, old.fLA), std::make_pair(n.fPar, old.fPar)})
            cp(pr.first, pr.second, fCopy * sizeof(real4));
        cp(n.fKind, old.fKind, fCopy * sizeof(int));
        cp(n.fExt, old.fExt, fCopy * kExtF4 * sizeof(real4));
        cp(n.fBroken, old.fBroken, fCopy * sizeof(int));
        cudaStreamSynchronize(stream);
        for (void *p : oldAllocs)
            cudaFree(p);
        // The device staging buffer was one of the freed allocations.
        ioDev = nullptr;
        ioFlag = nullptr;
        ioCap = 0;
        treeValid = false;
        adjValid = false;
        armTuning(); // sizes changed: tune again
    }
    n.waitLimit = waitLimit;
    d = n;
    if (!wBase.empty()) {
        cudaMemcpyAsync(d.wBase, wBase.data(), wBase.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d.wCount, wCount.data(), wCount.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    }
    cudaStreamSynchronize(stream);
}

size_t Engine::storeBytes(int nb, int mm, int ff, int pp, int ww, bool arm) {
    size_t total = 0;
    Dev n{};
    layoutStore(n, nb, mm, ff, pp, ww, arm, [&total](auto *&ptr, size_t count) {
        using T = std::remove_reference_t<decltype(*ptr)>;
        total += (std::max<size_t>(count, 1) * sizeof(T) + 255) / 256 * 256; // cudaMalloc granularity
        ptr = nullptr;
    });
    return total;
}

int Engine::ensureCapacity(int nb, int ff, int ww) {
    if (nb <= d.NB && ff <= d.FF && ww <= d.WW)
        return AVBDG_OK;
    int nnb = nb <= d.NB ? d.NB : std::max(nb, 2 * d.NB);
    int nff = ff <= d.FF ? d.FF : std::max(ff, 2 * d.FF);
    int nww = ww <= d.WW ? d.WW : std::max(ww, 2 * d.WW);
    if (!fits(nnb, std::max(d.MM, 8 * nnb), nff, std::max(d.PP, 16 * nnb), nww)) {
        // No headroom under the byte limit: grow to exactly what is needed, or refuse.
        nnb = std::max(nb, d.NB);
        nff = std::max(ff, d.FF);
        nww = std::max(ww, d.WW);
        if (!fits(nnb, std::max(d.MM, 8 * nnb), nff, std::max(d.PP, 16 * nnb), nww))
            return fail(AVBDG_ERR_CAPACITY, "the store would exceed its device byte limit");
    }
    allocate(nnb, std::max(d.MM, 8 * nnb), nff, std::max(d.PP, 16 * nnb), nww);
    return cudaCheck("grow");
}

int Engine::validateBodies(int count, const avbdg_body_desc *descs, std::string &why) {
    for (int i = 0; i < count; i++) {
        const avbdg_body_desc &b = descs[i];
        if (b.shape < AVBDG_SHAPE_BOX || b.shape > AVBDG_SHAPE_CYLINDER) {
            why = "unknown shape";
            return AVBDG_ERR_INVALID;
        }
        if (b.sleep_mode > 2) {
            why = "sleep_mode must be 0, 1 or 2";
            return AVBDG_ERR_INVALID;
        }
        if (!finite3(b.size) || !finite3(b.position) || !finite3(b.velocity) || !finite3(b.angular_velocity) ||
            !std::isfinite(b.density) || !std::isfinite(b.friction) || !std::isfinite(b.orientation[0]) ||
            !std::isfinite(b.orientation[1]) || !std::isfinite(b.orientation[2]) || !std::isfinite(b.orientation[3])) {
            why = "non-finite body description";
            return AVBDG_ERR_NONFINITE;
        }
    }
    return AVBDG_OK;
}

int Engine::validateForces(int nb, int count, const avbdg_force_desc *descs, std::string &why) {
    for (int i = 0; i < count; i++) {
        const avbdg_force_desc &f = descs[i];
        if (f.kind < 0 || f.kind > 3) {
            why = "unknown force kind";
            return AVBDG_ERR_UNSUPPORTED;
        }
        // Ball and generic joints may anchor to the world (body_a = -1); springs and ignore pairs
        // join two bodies.
        const int aMin = (f.kind == 0 || f.kind == 3) ? -1 : 0;
        if (f.body_b < 0 || f.body_b >= nb || f.body_a < aMin || f.body_a >= nb) {
            why = "bad body index";
            return AVBDG_ERR_INVALID;
        }
        if (f.kind == 3)
            for (const avbdg_joint_axis &ax : f.axes)
                if (ax.mode < AVBDG_AXIS_FREE || ax.mode > AVBDG_AXIS_LIMITED) {
                    why = "bad generic joint axis mode";
                    return AVBDG_ERR_INVALID;
                }
    }
    return AVBDG_OK;
}

int Engine::addWorld() {
    ctrFresh = false;
    if (ensureCapacity(nBodies, nForces, worlds() + 1))
        return -1;
    wBase.push_back(nBodies);
    wCount.push_back(0);
    wDyn.push_back(0);
    wRound.push_back(0);
    const int w = worlds() - 1;
    cudaMemcpyAsync(d.wBase + w, &wBase[w], sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.wCount + w, &wCount[w], sizeof(int), cudaMemcpyHostToDevice, stream);
    uploadCounts();
    cudaStreamSynchronize(stream);
    return w;
}

int Engine::addBodies(int w, int count, const avbdg_body_desc *descs, int *outIds) {
    ctrFresh = false;
    if (w < 0 || w >= worlds() || count < 0 || (count > 0 && !descs))
        return fail(AVBDG_ERR_INVALID, "bad world or body array");
    if (w != worlds() - 1)
        return fail(AVBDG_ERR_INVALID, "only the most recently created world can receive bodies");
    std::string why;
    if (const int bad = validateBodies(count, descs, why))
        return fail(bad, why);
    if (count == 0)
        return AVBDG_OK;
    int rc = ensureCapacity(nBodies + count, nForces, worlds());
    if (rc)
        return rc;
    const int first = nBodies;
    std::vector<real4> x(count), q(count), v(count), wv(count), sz(count), mo(count), zero4(count);
    std::vector<int4> meta(count);
    for (int i = 0; i < count; i++) {
        const avbdg_body_desc &b = descs[i];
        real mass, moment[3], radius;
        massProperties(b, mass, moment, radius);
        x[i] = mk4(b.position[0], b.position[1], b.position[2], mass);
        q[i] = mk4(b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]);
        v[i] = mk4(b.velocity[0], b.velocity[1], b.velocity[2], P.gravity);
        wv[i] = mk4(b.angular_velocity[0], b.angular_velocity[1], b.angular_velocity[2], 0.0f);
        sz[i] = mk4(b.size[0], b.size[1], b.size[2], radius);
        mo[i] = mk4(moment[0], moment[1], moment[2], b.friction);
        meta[i] = make_int4(w, static_cast<int>(b.collision_layer), static_cast<int>(b.collision_mask),
                            static_cast<int>((b.axis_lock_linear & 0xff) | ((b.axis_lock_angular & 0xff) << 8) |
                                             ((b.sleep_mode & 0x3) << 16) | ((b.shape & 0x3) << 18)));
        zero4[i] = mk4(b.velocity[0], b.velocity[1], b.velocity[2], 0.0f);
        if (outIds)
            outIds[i] = first - wBase[w] + i;
        if (mass > 0.0f) {
            nDynamic++;
            wDyn[w]++;
        }
        if (b.shape != AVBDG_SHAPE_BOX) {
            nRound++;
            wRound[w]++;
        }
    }
    const size_t b4 = sizeof(real4) * static_cast<size_t>(count);
    cudaMemcpyAsync(d.x + first, x.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.q + first, q.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.v + first, v.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.vprev + first, zero4.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.w + first, wv.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.size + first, sz.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.moment + first, mo.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.meta + first, meta.data(), sizeof(int4) * static_cast<size_t>(count), cudaMemcpyHostToDevice,
                    stream);
    cudaMemsetAsync(d.sleep + first, 0, sizeof(int2) * static_cast<size_t>(count), stream);
    nBodies += count;
    wCount[w] += count;
    // The world's list order changed: rebuild its list-position map.
    std::vector<int> lp(wCount[w]);
    for (int i = 0; i < wCount[w]; i++)
        lp[i] = wBase[w] + wCount[w] - 1 - i; // list position wBase + i holds body (base + count - 1 - i)
    cudaMemcpyAsync(d.lpToBody + wBase[w], lp.data(), sizeof(int) * lp.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.wCount + w, &wCount[w], sizeof(int), cudaMemcpyHostToDevice, stream);
    uploadCounts();
    cudaStreamSynchronize(stream);
    treeValid = false;
    adjValid = false;
    return cudaCheck("addBodies");
}

int Engine::addJoint(int w, int a, int b, const float rA[3], const float rB[3], float kLin, float kAng,
                     float fracture) {
    ctrFresh = false;
    if (w < 0 || w >= worlds() || b < 0 || b >= wCount[w] || a < -1 || a >= wCount[w] || !rA || !rB)
        return fail(AVBDG_ERR_INVALID, "bad body index");
    int rc = ensureCapacity(nBodies, nForces + 1, worlds());
    if (rc)
        return rc;
    const int ga = a >= 0 ? wBase[w] + a : -1;
    const int gb = wBase[w] + b;
    // torqueArm = length2((A ? A.size : 0) + B.size) (joint.cpp:38-39), from host copies of sizes.
    real sa[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0};
    if (ga >= 0)
        cudaMemcpy(sa, d.size + ga, sizeof(real4), cudaMemcpyDeviceToHost);
    cudaMemcpy(sb, d.size + gb, sizeof(real4), cudaMemcpyDeviceToHost);
    const real tx = sa[0] + sb[0], ty = sa[1] + sb[1], tz = sa[2] + sb[2];
    const real px = tx * tx, py = ty * ty, pz = tz * tz;
    real arm = 0.0f;
    arm = arm + px;
    arm = arm + py;
    arm = arm + pz;
    const int f = nForces;
    const int2 ab = make_int2(ga, gb);
    const real4 ra = mk4(rA[0], rA[1], rA[2], 0.0f), rb = mk4(rB[0], rB[1], rB[2], 0.0f);
    const real4 zero = mk4(0, 0, 0, 0);
    const real4 par = mk4(kLin, kAng, fracture, arm);
    const int kind = 0, broken = 0;
    cudaMemcpyAsync(d.fAB + f, &ab, sizeof(int2), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fRA + f, &ra, sizeof(real4), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fRB + f, &rb, sizeof(real4), cudaMemcpyHostToDevice, stream);
    for (real4 *arr : {d.fC0L, d.fC0A, d.fKL, d.fKA, d.fLL, d.fLA})
        cudaMemcpyAsync(arr + f, &zero, sizeof(real4), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fPar + f, &par, sizeof(real4), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fKind + f, &kind, sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fBroken + f, &broken, sizeof(int), cudaMemcpyHostToDevice, stream);
    nForces++;
    cudaMemcpyAsync(d.ctr + C_FORCES, &nForces, sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaStreamSynchronize(stream);
    adjValid = false;
    return cudaCheck("addJoint");
}

int Engine::addIgnore(int w, int a, int b) {
    ctrFresh = false;
    if (w < 0 || w >= worlds() || a < 0 || b < 0 || a >= wCount[w] || b >= wCount[w])
        return fail(AVBDG_ERR_INVALID, "bad body index");
    int rc = ensureCapacity(nBodies, nForces + 1, worlds());
    if (rc)
        return rc;
    const int f = nForces;
    const int2 ab = make_int2(wBase[w] + a, wBase[w] + b);
    const int kind = 1, broken = 0;
    const real4 zero = mk4(0, 0, 0, 0);
    cudaMemcpyAsync(d.fAB + f, &ab, sizeof(int2), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fKind + f, &kind, sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fBroken + f, &broken, sizeof(int), cudaMemcpyHostToDevice, stream);
    for (real4 *arr : {d.fRA, d.fRB, d.fC0L, d.fC0A, d.fKL, d.fKA, d.fLL, d.fLA, d.fPar})
        cudaMemcpyAsync(arr + f, &zero, sizeof(real4), cudaMemcpyHostToDevice, stream);
    nForces++;
    cudaMemcpyAsync(d.ctr + C_FORCES, &nForces, sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaStreamSynchronize(stream);
    adjValid = false;
    return cudaCheck("addIgnore");
}

// Bulk form of addJoint/addIgnore: the same records, appended in the same order, with the joints'
// torque arms computed from one download of the world's body sizes.
int Engine::addForces(int w, int count, const avbdg_force_desc *descs) {
    ctrFresh = false;
    if (w < 0 || w >= worlds() || count < 0 || (count > 0 && !descs))
        return fail(AVBDG_ERR_INVALID, "bad world or force array");
    if (count == 0)
        return AVBDG_OK;
    const int n = wCount[w];
    std::string why;
    if (const int bad = validateForces(n, count, descs, why))
        return fail(bad, why);
    int rc = ensureCapacity(nBodies, nForces + count, worlds());
    if (rc)
        return rc;
    // Torque arms, spring rest lengths and generic-joint zeros read the bodies' current state.
    std::vector<real4> sizes(n), xs(n), qs(n);
    cudaMemcpy(sizes.data(), d.size + wBase[w], sizeof(real4) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(xs.data(), d.x + wBase[w], sizeof(real4) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(qs.data(), d.q + wBase[w], sizeof(real4) * n, cudaMemcpyDeviceToHost);
    std::vector<int2> ab(count);
    std::vector<real4> ra(count), rb(count), par(count), zero(count, mk4(0, 0, 0, 0));
    std::vector<real4> ext(static_cast<size_t>(count) * kExtF4, mk4(0, 0, 0, 0));
    std::vector<int> kind(count), broken(count, 0);
    for (int i = 0; i < count; i++) {
        const avbdg_force_desc &f = descs[i];
        kind[i] = f.kind;
        ab[i] = make_int2(f.body_a >= 0 ? wBase[w] + f.body_a : -1, wBase[w] + f.body_b);
        if (f.kind == 2) {
            // Spring::Spring (spring.cpp:16-27): rest < 0 -> the anchors' current distance.
            const f3 rA{f.r_a[0], f.r_a[1], f.r_a[2]}, rB{f.r_b[0], f.r_b[1], f.r_b[2]};
            real rest = f.rest;
            if (rest < 0.0f) {
                const f3 pA = add(xyz(xs[f.body_a]), qrot(asq(qs[f.body_a]), rA));
                const f3 pB = add(xyz(xs[f.body_b]), qrot(asq(qs[f.body_b]), rB));
                rest = length(sub(pA, pB));
            }
            ra[i] = mk4(rA.x, rA.y, rA.z, 0.0f);
            rb[i] = mk4(rB.x, rB.y, rB.z, 0.0f);
            par[i] = mk4(f.stiffness_lin, rest, 0.0f, 0.0f);
            continue;
        }
        if (f.kind == 3) {
            // GenericJoint::GenericJoint (generic_joint.cpp:24-30): zero = B relative to A now.
            const q4 qA = f.body_a >= 0 ? asq(qs[f.body_a]) : q4{0.0f, 0.0f, 0.0f, 1.0f};
            real4 *e = ext.data() + static_cast<size_t>(i) * kExtF4;
            e[0] = f4(qmul(qconj(qA), asq(qs[f.body_b])));
            for (int k = 0; k < 6; k++) {
                const avbdg_joint_axis &ax = f.axes[k];
                e[1 + k] = mk4(static_cast<real>(ax.mode), ax.lower, ax.upper, ax.spring_stiffness);
                e[7 + k] = mk4(ax.spring_equilibrium, ax.spring_damping, 0.0f, 0.0f);
            }
            ra[i] = mk4(f.r_a[0], f.r_a[1], f.r_a[2], 0.0f);
            rb[i] = mk4(f.r_b[0], f.r_b[1], f.r_b[2], 0.0f);
            par[i] = mk4(0, 0, 0, 0);
            continue;
        }
        if (f.kind == 0) {
            // torqueArm = length2((A ? A.size : 0) + B.size) (joint.cpp:38-39), as in addJoint.
            const real4 sa = f.body_a >= 0 ? sizes[f.body_a] : mk4(0, 0, 0, 0);
            const real4 sb = sizes[f.body_b];
            const real tx = sa.x + sb.x, ty = sa.y + sb.y, tz = sa.z + sb.z;
            const real px = tx * tx, py = ty * ty, pz = tz * tz;
            real arm = 0.0f;
            arm = arm + px;
            arm = arm + py;
            arm = arm + pz;
            ra[i] = mk4(f.r_a[0], f.r_a[1], f.r_a[2], 0.0f);
            rb[i] = mk4(f.r_b[0], f.r_b[1], f.r_b[2], 0.0f);
            par[i] = mk4(f.stiffness_lin, f.stiffness_ang, f.fracture, arm);
        } else {
            ra[i] = rb[i] = par[i] = mk4(0, 0, 0, 0);
        }
    }
    const int f0 = nForces;
    const size_t b4 = sizeof(real4) * static_cast<size_t>(count), bi = sizeof(int) * static_cast<size_t>(count);
    cudaMemcpyAsync(d.fAB + f0, ab.data(), sizeof(int2) * static_cast<size_t>(count), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fRA + f0, ra.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fRB + f0, rb.data(), b4, cudaMemcpyHostToDevice, stream);
    for (real4 *arr : {d.fC0L, d.fC0A, d.fKL, d.fKA, d.fLL, d.fLA})
        cudaMemcpyAsync(arr + f0, zero.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fPar + f0, par.data(), b4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fKind + f0, kind.data(), bi, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fBroken + f0, broken.data(), bi, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(d.fExt + static_cast<size_t>(f0) * kExtF4, ext.data(), sizeof(real4) * ext.size(),
                    cudaMemcpyHostToDevice, stream);
    nForces += count;
    cudaMemcpyAsync(d.ctr + C_FORCES, &nForces, sizeof(int), cudaMemcpyHostToDevice, stream);
    cudaStreamSynchronize(stream);
    adjValid = false;
    return cudaCheck("addForces");
}

// World removal between steps: one slot map, a device move of the survivors, a stable
// compaction of the manifold and force lists, then the new world table.
int Engine::removeWorlds(const std::vector<int> &ids) {
    ctrFresh = false;
    const int nw = worlds();
    std::vector<char> drop(nw, 0);
    for (int w : ids) {
        if (w < 0 || w >= nw)
            return fail(AVBDG_ERR_INVALID, "bad world");
        drop[w] = 1;
    }
    if (ids.empty())
        return AVBDG_OK;
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("removeWorlds");
    std::vector<int> remap(2 * static_cast<size_t>(nw)), base, count, dyn, round;
    int nb = 0, ndyn = 0, nround = 0;
    for (int w = 0; w < nw; w++) {
        if (drop[w]) {
            remap[2 * w] = -1;
            remap[2 * w + 1] = 0;
            continue;
        }
        remap[2 * w] = static_cast<int>(base.size());
        remap[2 * w + 1] = nb;
        base.push_back(nb);
        count.push_back(wCount[w]);
        dyn.push_back(wDyn[w]);
        round.push_back(wRound[w]);
        nb += wCount[w];
        ndyn += wDyn[w];
        nround += wRound[w];
    }
    cudaMemcpyAsync(d.relocRemap, remap.data(), sizeof(int) * remap.size(), cudaMemcpyHostToDevice, stream);
    launchRelocateWorlds(d, nBodies, nb, nForces, d.relocRemap, stream);
    wBase.swap(base);
    wCount.swap(count);
    wDyn.swap(dyn);
    wRound.swap(round);
    if (!wBase.empty()) {
        cudaMemcpyAsync(d.wBase, wBase.data(), wBase.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d.wCount, wCount.data(), wCount.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    }
    nBodies = nb;
    uploadCounts();
    launchListPositions(d, nb, stream);
    cudaMemcpyAsync(hostCtr, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("removeWorlds");
    nDynamic = ndyn;
    nRound = nround;
    nForces = hostCtr[C_FORCES];
    treeValid = false;
    adjValid = false;
    return cudaCheck("removeWorlds");
}

int Engine::shrinkEmpty() {
    if (!wBase.empty() || nBodies != 0)
        return AVBDG_OK;
    constexpr int nb = 64;
    if (d.NB <= nb)
        return AVBDG_OK;
    clear();
    allocate(nb, 8 * nb, std::min(d.FF, 64), 16 * nb, d.WW);
    return cudaCheck("shrink");
}

void Engine::clear() {
    ctrFresh = false;
    cudaStreamSynchronize(stream);
    dropGraphs();
    wBase.clear();
    wCount.clear();
    wDyn.clear();
    wRound.clear();
    nBodies = nDynamic = nForces = nRound = 0;
    cudaMemsetAsync(d.ctr, 0, sizeof(int) * C_COUNT, stream);
    cudaStreamSynchronize(stream);
    treeValid = adjValid = false;
    treeAge = 0;
    steps = 0;
}

// Body and world counts the step's kernels read from the device.
void Engine::uploadCounts() {
    const int counts[2] = {nBodies, worlds()};
    static_assert(C_WORLDS == C_BODIES + 1, "counts are uploaded together");
    cudaMemcpyAsync(d.ctr + C_BODIES, counts, sizeof(counts), cudaMemcpyHostToDevice, stream);
}

int Engine::setParams(const avbdg_params &p) {
    if (p.iterations < 1 || !(p.dt > 0.0f))
        return fail(AVBDG_ERR_INVALID, "iterations must be >= 1 and dt > 0");
    if (!(p.jacobian_rebuild_distance >= 0.0f))
        return fail(AVBDG_ERR_INVALID, "jacobian_rebuild_distance must be >= 0");
    if (p.contact_grace_ticks < 0)
        return fail(AVBDG_ERR_INVALID, "contact_grace_ticks must be >= 0");
    if (p.sleep_frames < 0)
        return fail(AVBDG_ERR_INVALID, "sleep_frames must be >= 0");
    P = p;
    dropGraphs(); // parameters are baked into captured launches
    if (p.jacobian_rebuild_distance > 0.0f && !armStore) {
        // The arm-cache arrays join the store (zeroed: no arms captured yet).
        armStore = true;
        if (d.NB > 0) {
            allocate(d.NB, d.MM, d.FF, d.PP, d.WW);
            return cudaCheck("arm cache");
        }
    }
    return AVBDG_OK;
}

StepParams Engine::stepParams(real collisionDt) const {
    StepParams s{};
    s.dt = P.dt;
    s.dtSq = P.dt * P.dt;
    s.collisionDt = collisionDt;
    s.alpha = P.alpha;
    s.oneMinusAlpha = 1 - P.alpha;
    s.betaLin = P.beta_lin;
    s.betaAng = P.beta_ang;
    s.gamma = P.gamma;
    s.stiffnessDecay = P.stiffness_decay;
    s.jacobiRelax = P.jacobi_relaxation;
    s.stickDriftHeal = P.stick_drift_heal;
    s.maxPen = P.max_penetration;
    s.specMargin = P.speculative_margin;
    s.projBeta = P.projection_beta;
    s.projSlop = P.projection_slop;
    s.projMaxCorr = P.projection_max_correction;
    s.adaptiveFloor = P.adaptive_beta_error_floor;
    s.adaptiveBeta = P.adaptive_beta;
    s.contactOnlyOverflow = P.contact_only_overflow;
    s.projIters = P.projection_iterations;
    s.sleepFrames = P.sleep_frames;
    s.graceTicks = P.contact_grace_ticks;
    s.graceSeed = std::max(PENALTY_MIN, static_cast<real>(0.05f) * P.beta_lin);
    s.sleepLin2 = P.sleep_linear_threshold * P.sleep_linear_threshold;
    s.sleepAng2 = P.sleep_angular_threshold * P.sleep_angular_threshold;
    s.armCache = P.jacobian_rebuild_distance > 0.0f && d.ARM ? 1 : 0;
    s.armRebuild2 = P.jacobian_rebuild_distance * P.jacobian_rebuild_distance;
    return s;
}

bool Engine::needGreedy() const { return nForces > 0 || !P.contact_only_overflow; }

// Solver::broadPhase (solver_broadphase.cpp:85-186).
// Host decisions of one step (everything the enqueued work depends on besides device counts).
Engine::StepPlan Engine::planStep(int mode, int substeps, int rounds) {
    StepPlan plan;
    plan.mode = mode;
    plan.substeps = substeps;
    plan.rounds = rounds;
    plan.adjAtStart = !adjValid;
    plan.anyTree = false;
    plan.brute = bruteAllowed;
    for (int c : wCount) {
        plan.anyTree = plan.anyTree || c >= 2;
        plan.brute = plan.brute && c <= kBruteMaxBodies;
    }
    // Rebuild from fresh Morton codes when the body set changed or after kRefitBudget refits
    // (bvh_broadphase.cpp:186-203), so the code/order dumps follow the reference's schedule.
    plan.rebuild = plan.anyTree && (!treeValid || treeAge >= kRefitBudget);
    if (plan.anyTree) {
        if (plan.rebuild) {
            treeValid = true;
            treeAge = 0;
        } else {
            treeAge++;
        }
    }
    adjValid = true; // the step rebuilds the adjacency after warm starting
    plan.forces = nForces > 0;
    plan.greedy = needGreedy();
    plan.multiWorld = worlds() > 1;
    plan.round = nRound > 0;
    return plan;
}

std::string Engine::StepPlan::key() const {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "%d/%d/%d/%d%d%d%d%d%d%d%d", mode, substeps, rounds, adjAtStart ? 1 : 0,
                  anyTree ? 1 : 0, rebuild ? 1 : 0, forces ? 1 : 0, greedy ? 1 : 0, multiWorld ? 1 : 0,
                  round ? 1 : 0, brute ? 1 : 0);
    return buf;
}

void Engine::recordPhase(cudaEvent_t e) {
    if (capturing)
        cudaEventRecordWithFlags(e, stream, cudaEventRecordExternal);
    else
        cudaEventRecord(e, stream);
}

int Engine::broadPhase(const StepParams &sp, const StepPlan &plan) {
    if (plan.adjAtStart)
        launchAdjacency(d, stream);
    launchAabb(d, sp, stream);
    if (!plan.anyTree) {
        cudaMemsetAsync(d.ctr + C_PAIRS, 0, sizeof(int), stream);
        cudaMemcpyAsync(d.ctr + C_CAND, d.ctr + C_LIVE, sizeof(int), cudaMemcpyDeviceToDevice, stream);
        return AVBDG_OK;
    }
    // The tree is rebuilt on the reference's schedule either way (its codes and order are dumped);
    // the all-pairs test needs no bounds, so only the tree walk refits it.
    if (plan.rebuild)
        launchRebuildTree(d, plan.multiWorld, stream);
    if (!plan.brute)
        launchRefit(d, stream);
    beginSpan();
    launchPairs(d, tuned.traverse, plan.brute, stream);
    endSpan(kTraverse);
    launchFilterAcquire(d, stream);
    if (sp.sleepFrames > 0)
        launchSleepWakePairs(d, stream);
    return AVBDG_OK;
}

// The whole step, enqueued on the stream without host round trips.
// A kernel whose launch fails (an invalid configuration) leaves its outputs unwritten, and the
// kernels after it would read them; so the step stops enqueuing at the first phase boundary that
// finds a launch error, and runPlan reports it instead of running what was enqueued as a step.
static bool launchesOk() { return cudaPeekAtLastError() == cudaSuccess; }

bool Engine::enqueueStep(const StepPlan &plan) {
    if (plan.mode == 0) {
        const StepParams sp = stepParams(P.dt);
        broadPhase(sp, plan);
        recordPhase(ev[1]);
        if (!launchesOk())
            return false;
        warmstartAndSelect(sp);
        projectContacts(sp, false, 0.0f);
        recordPhase(ev[2]);
        if (!launchesOk())
            return false;
        runSubstep(sp, P.iterations, true);
        recordPhase(ev[3]);
        if (!launchesOk())
            return false;
        projectContacts(sp, P.position_projection != 0, 0.0f);
        launchRebase(d, sp, stream);
        return launchesOk();
    }
    const int substeps = plan.substeps;
    const StepParams sp = stepParams(P.dt * static_cast<real>(substeps));
    broadPhase(sp, plan);
    recordPhase(ev[1]);
    if (!launchesOk())
        return false;
    warmstartAndSelect(sp);
    recordPhase(ev[2]);
    for (int sub = 0; sub < substeps; ++sub) {
        if (!launchesOk())
            return false;
        if (sub > 0)
            launchRebase(d, sp, stream);
        projectContacts(sp, false, P.dt * static_cast<real>(substeps - sub));
        runSubstep(sp, plan.rounds, sub + 1 == substeps);
    }
    recordPhase(ev[3]);
    if (!launchesOk())
        return false;
    projectContacts(sp, P.position_projection != 0, sp.collisionDt);
    launchRebase(d, sp, stream);
    return launchesOk();
}

int Engine::launchFailure() {
    const cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(stream);
    return fail(AVBDG_ERR_CUDA, std::string("step: a kernel launch failed (") + cudaGetErrorString(e) +
                                    "); the step was stopped and the world's state is not trustworthy");
}

void Engine::dropGraphs() {
    for (auto &kv : graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        for (const Span &s : kv.second.spans) {
            cudaEventDestroy(s.a);
            cudaEventDestroy(s.b);
        }
    }
    graphs.clear();
    planSeen.clear();
    graphSpans = nullptr;
}

// Enqueue the plan: from the graph cache (a plan is captured the second time it is seen; profiled
// plans, whose graphs carry the span events, are cached apart), or eagerly the first time, when
// graphs are disabled, during a tuning trial or when a capture failed.
int Engine::enqueuePlan(const StepPlan &plan) {
    launchBase = launchCount();
    graphSpans = nullptr;
    lastGraph = false;
    // The step's device time starts when its work is handed to the stream: after a capture and
    // instantiation (host work the device only waits for), before an eager enqueue or a launch.
    const auto startClock = [&] { cudaEventRecord(ev[0], stream); };
    const bool trial = tuning && tuneTrial >= 0;
    if (trial)
        configureTrial();
    if (useGraphs && !trial) {
        const std::string k = plan.key() + (profiling ? "/profiled" : "");
        auto it = graphs.find(k);
        // A plan runs eagerly the first time it is seen after the cache was dropped and is
        // captured when it comes back, so plans that never recur cost no capture. Body and world
        // counts are read on the device, so adding or removing worlds keeps the cache.
        const bool capture = it == graphs.end() && planSeen[k]++ > 0;
        if (it == graphs.end() && !capture) {
            startClock();
            if (!enqueueStep(plan))
                return launchFailure();
        } else if (it == graphs.end()) {
            const int before = launchCount();
            spans.clear();
            evUsed = 0;
            cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
            capturing = true;
            const bool launched = enqueueStep(plan);
            capturing = false;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(stream, &g);
            cudaGraphExec_t exec = nullptr;
            if (e == cudaSuccess && launched)
                e = cudaGraphInstantiate(&exec, g, 0);
            if (g)
                cudaGraphDestroy(g);
            if (!launched) { // a launch itself failed: running the step eagerly would fail the same way
                for (const Span &s : spans) {
                    cudaEventDestroy(s.a);
                    cudaEventDestroy(s.b);
                }
                spans.clear();
                return launchFailure();
            }
            if (e != cudaSuccess) {
                cudaGetLastError(); // capture refused: run eagerly from now on
                useGraphs = false;
                graphError = cudaGetErrorString(e);
                for (const Span &s : spans) {
                    cudaEventDestroy(s.a);
                    cudaEventDestroy(s.b);
                }
                spans.clear();
                startClock();
                if (!enqueueStep(plan))
                    return launchFailure();
            } else {
                Graph gr{exec, launchCount() - before, {}};
                gr.spans.swap(spans);
                it = graphs.emplace(k, std::move(gr)).first;
            }
        }
        if (it != graphs.end()) {
            startClock();
            cudaGraphLaunch(it->second.exec, stream);
            launchBase = launchCount() - it->second.launches; // kernels inside the graph
            graphSpans = &it->second.spans;
            lastGraph = true;
        }
    } else {
        startClock();
        if (!enqueueStep(plan))
            return launchFailure();
    }
    cudaEventRecord(ev[4], stream);
    timed = true;
    return AVBDG_OK;
}

int Engine::runPlan(const StepPlan &plan) {
    const int rc = enqueuePlan(plan);
    return rc ? rc : finishStep();
}

// warmstartForces + selectUpdateBodies (solver_solve.cpp:31-105, 263-424).
int Engine::warmstartAndSelect(const StepParams &sp) {
    launchForceInit(d, sp, nForces > 0, stream);
    beginSpan();
    launchManifoldInit(d, sp, nRound > 0, tuned.narrow, stream);
    endSpan(kNarrow);
    launchManifoldCompact(d, stream);
    launchAdjacency(d, stream);
    if (sp.sleepFrames > 0)
        launchSleepSelect(d, sp, stream);
    launchContactOnly(d, stream);
    launchColour(d, needGreedy(), !P.contact_only_overflow, stream);
    launchColourLists(d, P.contact_only_overflow, stream);
    return AVBDG_OK;
}

// Solver::projectContacts (solver_projection.cpp:67-281).
void Engine::projectContacts(const StepParams &sp, bool positions, real window) {
    launchProjActive(d, stream);
    if (sp.specMargin > 0.0f)
        launchBrake(d, window > 0.0f ? window : sp.collisionDt, stream);
    if (positions && sp.projIters > 0)
        launchProjection(d, sp, stream);
}

// Solver::runSubstep + iterateBody (solver_step.cpp:79-105, 195-316).
void Engine::runSubstep(const StepParams &sp, int rounds, bool idle) {
    launchWarmstartBodies(d, sp, stream);
    const int newtonRounds =
            std::clamp(static_cast<int>(std::ceil(P.newton_ratio * static_cast<float>(rounds))), 1, rounds);
    const bool colours = needGreedy();
    const bool inPlace = nForces == 0;
    // Convergence probe (solver_step.cpp:88, 301-314): after each round but the last, the mean
    // step-start penetration r (a mean of positive floats, so 0 <= r <= inf) is compared with the
    // previous probe's, starting from 0; the first probe's 0 - r < threshold holds for every
    // threshold > 0, so a positive threshold always stops the substep after its first round.
    const int run = (P.convergence_threshold > 0.0f && rounds > 1) ? 1 : rounds;
    launchStamps(d, sp, false, stream);
    if (roundQueue && !colours && nForces == 0 && run <= kMaxQueueRounds) {
        QueueRounds qr{};
        qr.rounds = run;
        for (int it = 0; it < run; it++) {
            const bool newton = it < newtonRounds;
            if (newton)
                qr.newtonMask |= 1u << it;
            if (it + 1 < newtonRounds)
                qr.stampMask |= 1u << it;
            qr.decay[it] = newton ? 1.0f : P.stiffness_decay;
        }
        launchRoundQueue(d, sp, qr, stream);
        launchFinishBodies(d, sp, idle, stream);
        return;
    }
    for (int it = 0; it < run; it++) {
        if (!launchesOk())
            return; // enqueueStep reports it
        const bool newton = it < newtonRounds;
        if (newton) {
            if (colours) {
                // The colours in one cooperative sweep (sizes read on the device, empty colours skipped).
                launchColourSweep(d, sp, it > 0, stream);
                launchStamps(d, sp, true, stream);
            }
            beginSpan();
            launchOverflowSolve(d, sp, inPlace, nForces > 0, tuned.solve, stream);
            endSpan(kBody);
            if (!inPlace)
                launchOverflowApply(d, sp, stream);
        }
        const bool nextNewton = it + 1 < newtonRounds;
        beginSpan();
        launchDual(d, sp, nextNewton, newton ? 1.0f : P.stiffness_decay, tuned.dual, stream);
        endSpan(kManifold);
        launchForceDual(d, sp, nForces > 0, stream);
    }
    launchFinishBodies(d, sp, idle, stream);
}

int Engine::finishStep() {
    cudaMemcpyAsync(hostCtr, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("step");
    int rc = cudaCheck("step");
    if (rc)
        return rc;
    launches = launchCount() - launchBase;
    return processCounters();
}

// The host's part of a finished step: its counters are in hostCtr.
int Engine::processCounters() {
    steps++;
    ctrFresh = true;
    if (profiling || tuning)
        collectSpans();
    if (profiling) {
        acc.kernel_launches += launches;
        acc.steps++;
    }
    if (tuning)
        finishTrial();
    nForces = hostCtr[C_FORCES];
    if (hostCtr[C_ERRORS]) {
        const int e = hostCtr[C_ERRORS];
        cudaMemsetAsync(d.ctr + C_ERRORS, 0, sizeof(int), stream);
        if (e & kErrBrakeTimeout)
            return fail(AVBDG_ERR_TIMEOUT, "brake sweep: a bounded wait for a preceding candidate gave up");
        if (e & kErrColourTimeout)
            return fail(AVBDG_ERR_TIMEOUT, "colouring: a bounded wait for an earlier neighbour gave up");
        if (e & kErrBarrierTimeout)
            return fail(AVBDG_ERR_TIMEOUT, "colour sweep: a bounded grid barrier gave up");
        if (e & kErrQueueTimeout)
            return fail(AVBDG_ERR_TIMEOUT, "round queue: a tile's bounded wait for its world gave up");
        return fail(AVBDG_ERR_CAPACITY, "a device buffer overflowed this step (state is not trustworthy)");
    }
    // Keep headroom for the next step's pairs and manifolds.
    if (hostCtr[C_PAIRS] * 2 > d.PP || hostCtr[C_CAND] * 2 > d.MM || hostCtr[C_ADJ] * 2 > 2 * (d.FF + d.MM)) {
        int mm = std::max(d.MM, 4 * hostCtr[C_CAND]), pp = std::max(d.PP, 4 * hostCtr[C_PAIRS]);
        if (!fits(d.NB, mm, d.FF, pp, d.WW)) {
            mm = std::max(d.MM, 2 * hostCtr[C_CAND]);
            pp = std::max(d.PP, 2 * hostCtr[C_PAIRS]);
        }
        // Under a byte limit that leaves no room, the store stays as it is; an overflow in a later
        // step is then reported as AVBDG_ERR_CAPACITY.
        if (fits(d.NB, mm, d.FF, pp, d.WW)) {
            allocate(d.NB, mm, d.FF, pp, d.WW);
            return cudaCheck("grow");
        }
    }
    return AVBDG_OK;
}

int Engine::step() {
    if (nBodies == 0)
        return AVBDG_OK;
    return runPlan(planStep(0, 1, P.iterations));
}

int Engine::stepEnqueue() {
    stepPending = false;
    if (nBodies == 0)
        return AVBDG_OK;
    const int rc = enqueuePlan(planStep(0, 1, P.iterations));
    pendingLaunches = launchCount() - launchBase;
    stepPending = rc == AVBDG_OK;
    return rc;
}

int Engine::stepFinish() {
    if (!stepPending)
        return AVBDG_OK;
    stepPending = false;
    launchBase = launchCount() - pendingLaunches; // launches of other stores in between are not this step's
    return finishStep();
}

// Every buffer a step fills has at least 4x headroom over the last checked step's counts, so the
// next step cannot overflow unless its counts more than quadruple.
bool Engine::roomy() const {
    return ctrFresh && hostCtr[C_PAIRS] * 4 <= d.PP && hostCtr[C_CAND] * 4 <= d.MM &&
           hostCtr[C_ADJ] * 4 <= 2 * (d.FF + d.MM);
}

// Waits for the queued step whose counters go to ring slot `slot` and checks them as finishStep does.
int Engine::finishQueued(int slot) {
    if (cudaEventSynchronize(ctrEvent[slot]) != cudaSuccess)
        return cudaCheck("step");
    const int rc = cudaCheck("step");
    if (rc)
        return rc;
    std::memcpy(hostCtr, ctrRing + slot * C_COUNT, sizeof(int) * C_COUNT);
    launches = ctrLaunches[slot];
    // An error or a growth replaces or resets buffers the step queued after this one still uses:
    // let that step finish first.
    const bool grow = hostCtr[C_PAIRS] * 2 > d.PP || hostCtr[C_CAND] * 2 > d.MM || hostCtr[C_ADJ] * 2 > 2 * (d.FF + d.MM);
    if (grow || hostCtr[C_ERRORS])
        cudaStreamSynchronize(stream);
    return processCounters();
}

// Steps `count` times. Without profiling or tuning, and while the last checked counters leave 4x
// headroom (roomy), step i is enqueued before step i-1's counters are read back: the host waits
// for the step before the one it just queued, so the device runs the steps back to back instead
// of idling while the host checks each one. Every step's counters are still checked in order;
// when a check finds an error the queued step is drained and the error returned (the state is
// then not trustworthy, as after a failed step), and when the headroom is short the next step
// waits for the check, which grows the store as step() does.
int Engine::stepMany(int count, int substeps, int rounds) {
    if (nBodies == 0 || count <= 0)
        return AVBDG_OK;
    const auto plan = [&] {
        if (substeps <= 1)
            return planStep(0, 1, P.iterations);
        const int r = rounds > 0 ? std::max(1, rounds) : std::max(2, (P.iterations + substeps - 1) / substeps);
        return planStep(1, substeps, r);
    };
    if (!ctrRing) {
        if (cudaMallocHost(&ctrRing, sizeof(int) * 2 * C_COUNT) != cudaSuccess)
            return fail(AVBDG_ERR_CAPACITY, "pinned counter allocation failed");
        for (cudaEvent_t &e : ctrEvent)
            cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    }
    int queued = -1; // ring slot of the step whose counters are not checked yet
    for (int i = 0; i < count; i++) {
        if (profiling || tuning) {
            if (queued >= 0) {
                const int rc = finishQueued(queued);
                queued = -1;
                if (rc)
                    return rc;
            }
            const int rc = runPlan(plan());
            if (rc)
                return rc;
            continue;
        }
        if (queued >= 0 && !roomy()) {
            const int rc = finishQueued(queued);
            queued = -1;
            if (rc)
                return rc;
        }
        const int slot = i & 1;
        int rc = enqueuePlan(plan());
        if (rc) {
            cudaStreamSynchronize(stream);
            return rc;
        }
        ctrLaunches[slot] = launchCount() - launchBase;
        cudaMemcpyAsync(ctrRing + slot * C_COUNT, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost, stream);
        cudaEventRecord(ctrEvent[slot], stream);
        if (queued >= 0) {
            rc = finishQueued(queued);
            if (rc) {
                cudaStreamSynchronize(stream);
                return rc;
            }
        }
        queued = slot;
    }
    return queued >= 0 ? finishQueued(queued) : AVBDG_OK;
}

int Engine::stepInterleaved(int substeps, int roundsPerSubstep) {
    if (substeps <= 1)
        return step();
    if (nBodies == 0)
        return AVBDG_OK;
    const int rounds = roundsPerSubstep > 0 ? std::max(1, roundsPerSubstep)
                                            : std::max(2, (P.iterations + substeps - 1) / substeps);
    return runPlan(planStep(1, substeps, rounds));
}

int Engine::sync() {
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("sync");
    return AVBDG_OK;
}

int Engine::ensureIo(int count) {
    if (count <= ioCap)
        return AVBDG_OK;
    const int cap = std::max(count, 2 * ioCap);
    if (ioHost)
        cudaFreeHost(ioHost);
    ioHost = nullptr;
    if (cudaMallocHost(&ioHost, sizeof(float) * 13 * static_cast<size_t>(cap)) != cudaSuccess)
        return fail(AVBDG_ERR_CAPACITY, "pinned staging allocation failed");
    ioDev = dalloc<float>(13 * static_cast<size_t>(cap) + 4);
    if (!ioDev)
        return fail(AVBDG_ERR_CAPACITY, "device staging allocation failed");
    ioFlag = reinterpret_cast<int *>(ioDev + 13 * static_cast<size_t>(cap));
    ioCap = cap;
    return AVBDG_OK;
}

// One device-side pack, one copy to pinned memory, one host copy per requested field.
// World -1 addresses every body slot of the set in world order (one copy for all worlds).
int Engine::slotRange(int w, int first, int count, int &g0) {
    const int limit = w == -1 ? nBodies : (w >= 0 && w < worlds() ? wCount[w] : -1);
    if (limit < 0 || first < 0 || count < 0 || first + count > limit)
        return fail(AVBDG_ERR_INVALID, "bad range");
    g0 = (w == -1 ? 0 : wBase[w]) + first;
    return AVBDG_OK;
}

int Engine::getSleeping(int w, int first, int count, uint8_t *out) {
    int g0 = 0;
    if (slotRange(w, first, count, g0))
        return AVBDG_ERR_INVALID;
    if (count == 0)
        return AVBDG_OK;
    if (!out)
        return fail(AVBDG_ERR_INVALID, "null output");
    std::vector<int2> s(static_cast<size_t>(count));
    sync();
    cudaMemcpy(s.data(), d.sleep + g0, sizeof(int2) * s.size(), cudaMemcpyDeviceToHost);
    for (int i = 0; i < count; i++)
        out[i] = s[i].x ? 1 : 0;
    return cudaCheck("getSleeping");
}

namespace {

// Device scratch of one query call, released on every path.
struct QueryScratch {
    std::vector<void *> ptrs;
    ~QueryScratch() {
        for (void *p : ptrs)
            cudaFree(p);
    }
    template <typename T>
    T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
            return nullptr;
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
};

} // namespace

int Engine::pick(int w, int count, const float *origins, const float *dirs, uint32_t mask, int *outBody,
                 float *outLocal) {
    if (w < 0 || w >= worlds() || count < 0 || (count > 0 && (!origins || !dirs || !outBody)))
        return fail(AVBDG_ERR_INVALID, "bad pick arguments");
    if (count == 0)
        return AVBDG_OK;
    std::vector<float> rays(6 * static_cast<size_t>(count));
    for (int i = 0; i < count; i++)
        for (int k = 0; k < 3; k++) {
            rays[6 * i + k] = origins[3 * i + k];
            rays[6 * i + 3 + k] = dirs[3 * i + k];
        }
    QueryScratch q;
    float *dRays = q.get<float>(rays.size());
    auto *dBest = q.get<unsigned long long>(count);
    int *dBody = q.get<int>(count);
    float *dLocal = q.get<float>(3 * static_cast<size_t>(count));
    if (!dRays || !dBest || !dBody || !dLocal)
        return fail(AVBDG_ERR_CAPACITY, "query scratch allocation failed");
    sync();
    cudaMemcpyAsync(dRays, rays.data(), sizeof(float) * rays.size(), cudaMemcpyHostToDevice, stream);
    launchPick(d, wBase[w], wCount[w], dRays, count, mask, dBest, dBody, dLocal, stream);
    std::vector<float> local(3 * static_cast<size_t>(count));
    cudaMemcpyAsync(outBody, dBody, sizeof(int) * static_cast<size_t>(count), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(local.data(), dLocal, sizeof(float) * local.size(), cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("pick");
    if (outLocal)
        std::memcpy(outLocal, local.data(), sizeof(float) * local.size());
    return cudaCheck("pick");
}

int Engine::collectAabb(int w, const float lo[3], const float hi[3], uint32_t mask, int capacity, int *out,
                        int *outCount) {
    if (w < 0 || w >= worlds() || !lo || !hi || capacity < 0 || (capacity > 0 && !out))
        return fail(AVBDG_ERR_INVALID, "bad collect arguments");
    const int n = wCount[w];
    QueryScratch q;
    int *flags = q.get<int>(n), *rank = q.get<int>(n), *total = q.get<int>(1), *ids = q.get<int>(n);
    if (!flags || !rank || !total || !ids)
        return fail(AVBDG_ERR_CAPACITY, "query scratch allocation failed");
    sync();
    launchCollectAabb(d, wBase[w], n, f3{lo[0], lo[1], lo[2]}, f3{hi[0], hi[1], hi[2]}, mask, flags, rank, total,
                      d.scanScratch, n, ids, stream);
    int found = 0;
    cudaMemcpyAsync(&found, total, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("collectAabb");
    const int k = std::min(found, capacity);
    if (k > 0)
        cudaMemcpy(out, ids, sizeof(int) * static_cast<size_t>(k), cudaMemcpyDeviceToHost);
    if (outCount)
        *outCount = found;
    return cudaCheck("collectAabb");
}

namespace {

// Host copies of body state between the caller's arrays and the pinned staging buffer, split over
// the host's cores for large transfers (one core's memcpy is far slower than the link). `check`
// also reports a non-finite value in the copied range.
struct HostCopy {
    float *dst;
    const float *src;
    size_t count;
    bool check;
};

// A process-wide pool of copy threads, started on first use and kept (never joined: it lives
// until the process ends), so a transfer pays no thread start-up. One caller at a time.
class CopyPool {
public:
    static CopyPool &get() {
        // A forked child has none of the parent's threads: it starts its own pool.
        static CopyPool *pool = nullptr;
        static pid_t owner = 0;
        static std::mutex made;
        std::lock_guard<std::mutex> l(made);
        if (!pool || owner != getpid()) {
            pool = new CopyPool(std::max(1u, std::min(16u, std::thread::hardware_concurrency())) - 1);
            owner = getpid();
        }
        return *pool;
    }
    unsigned threads() const { return static_cast<unsigned>(workers.size()) + 1; }
    // Runs f on every pool thread and on the caller; returns when all calls have returned.
    void run(const std::function<void()> &f) {
        std::lock_guard<std::mutex> one(callers);
        {
            std::lock_guard<std::mutex> l(mu);
            task = &f;
            pending = static_cast<int>(workers.size());
            ++generation;
        }
        wake.notify_all();
        f();
        std::unique_lock<std::mutex> l(mu);
        finished.wait(l, [&] { return pending == 0; });
        task = nullptr;
    }

private:
    explicit CopyPool(unsigned n) {
        for (unsigned i = 0; i < n; i++)
            workers.emplace_back([this] { loop(); });
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            const std::function<void()> *f = nullptr;
            {
                std::unique_lock<std::mutex> l(mu);
                wake.wait(l, [&] { return generation != seen; });
                seen = generation;
                f = task;
            }
            (*f)();
            std::lock_guard<std::mutex> l(mu);
            if (--pending == 0)
                finished.notify_all();
        }
    }
    std::vector<std::thread> workers;
    std::mutex mu, callers;
    std::condition_variable wake, finished;
    const std::function<void()> *task = nullptr;
    unsigned long long generation = 0;
    int pending = 0;
};

bool copyHostParallel(const std::vector<HostCopy> &jobs) {
    size_t total = 0;
    for (const HostCopy &j : jobs)
        total += j.count;
    const size_t chunk = size_t{1} << 16; // floats
    const bool parallel = total >= 4 * chunk;
    std::atomic<bool> finite{true};
    std::atomic<size_t> next{0};
    // Work items: (job, first float) pairs in order.
    std::vector<std::pair<size_t, size_t>> items;
    for (size_t j = 0; j < jobs.size(); j++)
        for (size_t f = 0; f < jobs[j].count; f += chunk)
            items.emplace_back(j, f);
    const auto run = [&]() {
        for (size_t i = next.fetch_add(1); i < items.size(); i = next.fetch_add(1)) {
            const HostCopy &job = jobs[items[i].first];
            const size_t f = items[i].second, n = std::min(chunk, job.count - f);
            const float *src = job.src + f;
            if (job.check) {
                bool ok = true;
                for (size_t k = 0; k < n; k++)
                    ok = ok && std::isfinite(src[k]);
                if (!ok)
                    finite.store(false);
            }
            std::memcpy(job.dst + f, src, sizeof(float) * n);
        }
    };
    if (parallel)
        CopyPool::get().run(run);
    else
        run();
    return finite.load();
}

} // namespace

int Engine::getState(int w, int first, int count, float *pos, float *quat, float *vel, float *angVel) {
    int g0 = 0;
    if (slotRange(w, first, count, g0))
        return AVBDG_ERR_INVALID;
    if (count == 0)
        return AVBDG_OK;
    int rc = ensureIo(count);
    if (rc)
        return rc;
    launchPackState(d, g0, count, ioDev, stream);
    const size_t n = static_cast<size_t>(count);
    if (directIo) {
        // One copy per requested field into the caller's arrays.
        if (pos)
            cudaMemcpyAsync(pos, ioDev, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, stream);
        if (quat)
            cudaMemcpyAsync(quat, ioDev + 3 * n, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, stream);
        if (vel)
            cudaMemcpyAsync(vel, ioDev + 7 * n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, stream);
        if (angVel)
            cudaMemcpyAsync(angVel, ioDev + 10 * n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        return cudaCheck("getState");
    }
    cudaMemcpyAsync(ioHost, ioDev, sizeof(float) * 13 * n, cudaMemcpyDeviceToHost, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        return cudaCheck("getState");
    std::vector<HostCopy> jobs;
    if (pos)
        jobs.push_back({pos, ioHost, 3 * n, false});
    if (quat)
        jobs.push_back({quat, ioHost + 3 * n, 4 * n, false});
    if (vel)
        jobs.push_back({vel, ioHost + 7 * n, 3 * n, false});
    if (angVel)
        jobs.push_back({angVel, ioHost + 10 * n, 3 * n, false});
    copyHostParallel(jobs);
    return cudaCheck("getState");
}

// Stage the given fields in pinned memory, one copy up, one device-side unpack (packed
// companions such as the mass in x.w are kept).
int Engine::setState(int w, int first, int count, const float *pos, const float *quat, const float *vel,
                     const float *angVel) {
    int g0 = 0;
    if (slotRange(w, first, count, g0))
        return AVBDG_ERR_INVALID;
    if (count == 0)
        return AVBDG_OK;
    int rc = ensureIo(count);
    if (rc)
        return rc;
    const size_t n = static_cast<size_t>(count);
    if (directIo) {
        // The fields go up as they are; the device checks them and unpacks only when all are
        // finite, so nothing changes on a rejected upload.
        const int mask = (pos ? 1 : 0) | (quat ? 2 : 0) | (vel ? 4 : 0) | (angVel ? 8 : 0);
        cudaMemsetAsync(ioFlag, 0, sizeof(int), stream);
        if (pos)
            cudaMemcpyAsync(ioDev, pos, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, stream);
        if (quat)
            cudaMemcpyAsync(ioDev + 3 * n, quat, sizeof(float) * 4 * n, cudaMemcpyHostToDevice, stream);
        if (vel)
            cudaMemcpyAsync(ioDev + 7 * n, vel, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, stream);
        if (angVel)
            cudaMemcpyAsync(ioDev + 10 * n, angVel, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, stream);
        launchCheckState(count, ioDev, mask, ioFlag, stream);
        launchUnpackState(d, g0, count, ioDev, mask, ioFlag, stream);
        int *flagHost = reinterpret_cast<int *>(ioHost);
        cudaMemcpyAsync(flagHost, ioFlag, sizeof(int), cudaMemcpyDeviceToHost, stream);
        if (cudaStreamSynchronize(stream) != cudaSuccess)
            return cudaCheck("setState");
        if (*flagHost)
            return fail(AVBDG_ERR_NONFINITE, "non-finite body state");
        return cudaCheck("setState");
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) // the staging buffer may still be in use
        return cudaCheck("setState");
    int mask = 0;
    std::vector<HostCopy> jobs;
    if (pos) {
        jobs.push_back({ioHost, pos, 3 * n, true});
        mask |= 1;
    }
    if (quat) {
        jobs.push_back({ioHost + 3 * n, quat, 4 * n, false});
        mask |= 2;
    }
    if (vel) {
        jobs.push_back({ioHost + 7 * n, vel, 3 * n, true});
        mask |= 4;
    }
    if (angVel) {
        jobs.push_back({ioHost + 10 * n, angVel, 3 * n, true});
        mask |= 8;
    }
    // Staged and checked in one pass; nothing reaches the device when a value is not finite.
    if (!copyHostParallel(jobs))
        return fail(AVBDG_ERR_NONFINITE, "non-finite body state");
    cudaMemcpyAsync(ioDev, ioHost, sizeof(float) * 13 * n, cudaMemcpyHostToDevice, stream);
    launchUnpackState(d, g0, count, ioDev, mask, nullptr, stream);
    return cudaCheck("setState");
}

// Spans of an eager step reuse pooled events; spans captured into a graph get events of their
// own, recorded by the graph's event nodes at every launch.
int Engine::beginSpan() {
    if (!profiling && !(tuning && tuneTrial >= 0))
        return -1;
    cudaEvent_t a, b;
    if (capturing) {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    } else {
        while (evPool.size() < evUsed + 2) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            evPool.push_back(e);
        }
        a = evPool[evUsed];
        b = evPool[evUsed + 1];
        evUsed += 2;
    }
    recordPhase(a);
    spans.push_back(Span{a, b, -1});
    return static_cast<int>(spans.size()) - 1;
}

void Engine::endSpan(int kind) {
    if ((!profiling && !(tuning && tuneTrial >= 0)) || spans.empty())
        return;
    spans.back().kind = kind;
    recordPhase(spans.back().b);
}

void Engine::collectSpans() {
    const std::vector<Span> &list = graphSpans ? *graphSpans : spans;
    const TuneSpace *spaces[kKinds] = {&kTuneDual, &kTuneSolve, &kTuneNarrow, &kTuneTraverse};
    for (const Span &s : list) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, s.a, s.b);
        if (tuning && tuneTrial >= 0 && s.kind >= 0 && s.kind < kKinds) {
            const int c = tuneTrial % spaces[s.kind]->count;
            tuneMs[s.kind][c] += ms;
            tuneN[s.kind][c]++;
        }
        if (!profiling)
            continue;
        if (s.kind == kManifold) {
            acc.manifold_ms += ms;
            acc.manifold_launches++;
        } else if (s.kind == kBody) {
            acc.body_ms += ms;
            acc.body_launches++;
        } else if (s.kind == kNarrow) {
            acc.narrow_ms += ms;
            acc.narrow_launches++;
        }
    }
    if (!graphSpans) {
        spans.clear();
        evUsed = 0;
    }
}

void Engine::armTuning() {
    tuning = tuneEnabled;
    tuneTrial = -kTuneDelay;
    std::memset(tuneMs, 0, sizeof(tuneMs));
    std::memset(tuneN, 0, sizeof(tuneN));
}

// Trial t runs candidate t mod (number of candidates) of every tuned kernel.
// A candidate that cannot launch (too many registers for its block size) is replaced by the
// default size for that trial and never chosen.
void Engine::configureTrial() {
    const TuneSpace *spaces[kKinds] = {&kTuneDual, &kTuneSolve, &kTuneNarrow, &kTuneTraverse};
    int *picks[kKinds] = {&tuned.dual, &tuned.solve, &tuned.narrow, &tuned.traverse};
    const int fallback[kKinds] = {tunedBase.dual, tunedBase.solve, tunedBase.narrow, tunedBase.traverse};
    for (int k = 0; k < kKinds; k++) {
        const int c = tuneTrial % spaces[k]->count;
        *picks[k] = tuneFits[k][c] ? spaces[k]->sizes[c] : fallback[k];
    }
}

void Engine::finishTrial() {
    if (++tuneTrial < kTuneTrials)
        return;
    const TuneSpace *spaces[kKinds] = {&kTuneDual, &kTuneSolve, &kTuneNarrow, &kTuneTraverse};
    int *picks[kKinds] = {&tuned.dual, &tuned.solve, &tuned.narrow, &tuned.traverse};
    const int fallback[kKinds] = {tunedBase.dual, tunedBase.solve, tunedBase.narrow, tunedBase.traverse};
    for (int k = 0; k < kKinds; k++) {
        int best = -1;
        double bestMs = 0.0;
        for (int c = 0; c < spaces[k]->count; c++) {
            if (tuneN[k][c] == 0 || !tuneFits[k][c])
                continue;
            const double avg = tuneMs[k][c] / tuneN[k][c];
            if (best < 0 || avg < bestMs) {
                best = c;
                bestMs = avg;
            }
        }
        *picks[k] = best >= 0 ? spaces[k]->sizes[best] : fallback[k];
    }
    tuning = false;
    dropGraphs(); // capture again with the chosen sizes
}

void Engine::takeKernelTimes(avbdg_kernel_times &out) {
    out = acc;
    acc = avbdg_kernel_times{};
}

int Engine::stats(avbdg_stats &out) {
    std::memset(&out, 0, sizeof(out));
    sync();
    cudaMemcpy(hostCtr, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost);
    out.bodies = nBodies;
    out.dynamic_bodies = nDynamic;
    out.forces = hostCtr[C_FORCES];
    out.broad_pairs = hostCtr[C_PAIRS];
    out.manifolds = hostCtr[C_LIVE];
    std::vector<int> counts(static_cast<size_t>(std::max(hostCtr[C_LIVE], 0)));
    if (!counts.empty())
        cudaMemcpy(counts.data(), d.live.count, sizeof(int) * counts.size(), cudaMemcpyDeviceToHost);
    for (int c : counts)
        out.contacts += c;
    if (!counts.empty() && nBodies > 0) {
        std::vector<int2> ab(counts.size());
        std::vector<real4> x(static_cast<size_t>(nBodies));
        cudaMemcpy(ab.data(), d.live.ab, sizeof(int2) * ab.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(x.data(), d.x, sizeof(real4) * x.size(), cudaMemcpyDeviceToHost);
        for (const int2 &m : ab)
            out.manifold_sides += (x[m.x].w > 0.0f ? 1 : 0) + (x[m.y].w > 0.0f ? 1 : 0);
    }
    int cc[kMaxColours + 1] = {};
    cudaMemcpy(cc, d.colourCount, sizeof(cc), cudaMemcpyDeviceToHost);
    for (int c = 0; c < kMaxColours; c++)
        if (cc[c] > 0)
            out.colour_groups = c + 1;
    out.overflow_bodies = cc[kMaxColours];
    out.update_bodies = nDynamic;
    out.steps = steps;
    out.graph_step = lastGraph ? 1 : 0;
    out.kernel_launches = launches;
    if (!tuning) {
        out.block_dual = tuned.dual;
        out.block_solve = tuned.solve;
        out.block_narrow = tuned.narrow;
        out.block_traverse = tuned.traverse;
    }
    if (timed) {
        float t[4] = {};
        for (int i = 0; i < 4; i++)
            cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]);
        out.broad_ms = t[0];
        out.graph_ms = t[1];
        out.solve_ms = t[2];
        out.finish_ms = t[3];
        out.total_ms = t[0] + t[1] + t[2] + t[3];
    }
    return cudaCheck("stats");
}

int Engine::digest(int w, uint64_t &out) {
    if (w < 0 || w >= worlds())
        return fail(AVBDG_ERR_INVALID, "bad world");
    const int n = wCount[w];
    std::vector<float> p(3 * n), q(4 * n), v(3 * n), av(3 * n);
    int rc = getState(w, 0, n, p.data(), q.data(), v.data(), av.data());
    if (rc)
        return rc;
    uint64_t h = 1469598103934665603ull;
    const auto mix = [&h](const void *ptr, size_t bytes) {
        const unsigned char *c = static_cast<const unsigned char *>(ptr);
        for (size_t i = 0; i < bytes; i++) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    for (int i = n - 1; i >= 0; i--) {
        mix(&p[3 * i], 12);
        mix(&q[4 * i], 16);
        mix(&v[3 * i], 12);
        mix(&av[3 * i], 12);
    }
    out = h;
    return AVBDG_OK;
}

int Engine::dumpBroadphase(uint64_t *codes, int32_t *order, int capN, uint64_t *pairs, int capP, int *nB, int *nP) {
    sync();
    cudaMemcpy(hostCtr, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost);
    const int n = nBodies;
    const int np = hostCtr[C_PAIRS];
    if (nB)
        *nB = n;
    if (nP)
        *nP = np;
    if ((codes || order) && n > 0) {
        std::vector<uint64_t> c(n);
        std::vector<int> l2b(n);
        cudaMemcpy(c.data(), d.codes, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(l2b.data(), d.lpToBody, sizeof(int) * n, cudaMemcpyDeviceToHost);
        // The reference's order: list positions of each world sorted by (code, list position)
        // (bvh_broadphase.cpp:87-96); the device tree is built from other codes.
        std::vector<int32_t> sv(n);
        for (int w = 0; w < worlds(); w++) {
            const int b = wBase[w], e = wBase[w] + wCount[w];
            for (int p = b; p < e; p++)
                sv[p] = p;
            std::stable_sort(sv.begin() + b, sv.begin() + e,
                             [&](int32_t x, int32_t y) { return c[l2b[x]] < c[l2b[y]]; });
        }
        for (int i = 0; i < n && i < capN; i++) {
            if (codes)
                codes[i] = c[l2b[i]];
            if (order)
                order[i] = sv[i];
        }
    }
    if (pairs && np > 0)
        cudaMemcpy(pairs, d.pairs, sizeof(uint64_t) * std::min(np, capP), cudaMemcpyDeviceToHost);
    return cudaCheck("dumpBroadphase");
}

int Engine::dumpManifolds(int cap, int32_t *ba, int32_t *bb, int32_t *nc, int32_t *features, float *basis,
                          float *c0, float *penalty, float *lambda, int *count) {
    sync();
    cudaMemcpy(hostCtr, d.ctr, sizeof(int) * C_COUNT, cudaMemcpyDeviceToHost);
    const int m = hostCtr[C_LIVE];
    if (count)
        *count = m;
    const int k = std::min(m, cap);
    if (k <= 0)
        return AVBDG_OK;
    std::vector<int2> ab(k);
    std::vector<int> cnt(k), keys(static_cast<size_t>(k) * kMaxContacts);
    std::vector<real4> b0(k), b1(k), b2(k);
    std::vector<real4> C(static_cast<size_t>(k) * kMaxContacts), K(C.size()), Lm(C.size());
    cudaMemcpy(ab.data(), d.live.ab, sizeof(int2) * k, cudaMemcpyDeviceToHost);
    cudaMemcpy(cnt.data(), d.live.count, sizeof(int) * k, cudaMemcpyDeviceToHost);
    cudaMemcpy(b0.data(), d.live.b0, sizeof(real4) * k, cudaMemcpyDeviceToHost);
    cudaMemcpy(b1.data(), d.live.b1, sizeof(real4) * k, cudaMemcpyDeviceToHost);
    cudaMemcpy(b2.data(), d.live.b2, sizeof(real4) * k, cudaMemcpyDeviceToHost);
    // Slot-major on the device; manifold-major (8 slots per manifold) here.
    const auto gather = [&](auto *dst, const auto *src) {
        using T = std::remove_const_t<std::remove_reference_t<decltype(*src)>>;
        std::vector<T> slot(static_cast<size_t>(k));
        for (int j = 0; j < kMaxContacts; j++) {
            cudaMemcpy(slot.data(), src + static_cast<size_t>(j) * d.MM, sizeof(T) * slot.size(), cudaMemcpyDeviceToHost);
            for (int i = 0; i < k; i++)
                dst[static_cast<size_t>(i) * kMaxContacts + j] = slot[static_cast<size_t>(i)];
        }
    };
    gather(keys.data(), d.live.key);
    gather(C.data(), d.live.C0);
    gather(K.data(), d.live.k);
    gather(Lm.data(), d.live.lam);
    const int base = wBase.empty() ? 0 : wBase[0];
    for (int i = 0; i < k; i++) {
        if (ba)
            ba[i] = ab[i].x - base;
        if (bb)
            bb[i] = ab[i].y - base;
        if (nc)
            nc[i] = cnt[i];
        const real4 rows[3] = {b0[i], b1[i], b2[i]};
        for (int r = 0; r < 3; r++)
            if (basis) {
                basis[9 * i + 3 * r + 0] = rows[r].x;
                basis[9 * i + 3 * r + 1] = rows[r].y;
                basis[9 * i + 3 * r + 2] = rows[r].z;
            }
        for (int j = 0; j < 8; j++) {
            const bool on = j < cnt[i];
            const size_t ci = static_cast<size_t>(i) * kMaxContacts + j;
            if (features)
                features[8 * i + j] = on ? keys[ci] : 0;
            const real *cv = &C[ci].x, *kv = &K[ci].x, *lv = &Lm[ci].x;
            for (int e = 0; e < 3; e++) {
                if (c0)
                    c0[24 * i + 3 * j + e] = on ? cv[e] : 0.0f;
                if (penalty)
                    penalty[24 * i + 3 * j + e] = on ? kv[e] : 0.0f;
                if (lambda)
                    lambda[24 * i + 3 * j + e] = on ? lv[e] : 0.0f;
            }
        }
    }
    return cudaCheck("dumpManifolds");
}

int Engine::dumpColours(int cap, uint8_t *colour, int32_t *bodyId, int *count) {
    sync();
    const int w = 0;
    if (worlds() == 0) {
        if (count)
            *count = 0;
        return AVBDG_OK;
    }
    const int n = wCount[w];
    std::vector<real4> x(n);
    std::vector<uint8_t> col(n), upd(n);
    cudaMemcpy(x.data(), d.x + wBase[w], sizeof(real4) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(col.data(), d.colour + wBase[w], n, cudaMemcpyDeviceToHost);
    cudaMemcpy(upd.data(), d.upd + wBase[w], n, cudaMemcpyDeviceToHost);
    int u = 0;
    for (int id = n - 1; id >= 0; id--) { // list order, update set only (sleepers are not in it)
        if (!(x[id].w > 0.0f) || !upd[id])
            continue;
        if (u < cap) {
            if (colour)
                colour[u] = col[id];
            if (bodyId)
                bodyId[u] = id;
        }
        u++;
    }
    if (count)
        *count = u;
    return cudaCheck("dumpColours");
}

} // namespace avbdg
