// Served form: continuous batching of independent scenes on one device store.
//
// The reference's physics server steps every active space with its own avbd::Solver, one after
// another (AVBDPhysicsServer3D::_step, src/server/avbd_physics_server3d.cpp:1396-1424; spaces are
// created and freed by _space_create :318 and _free_rid :292). Here every request is a scene (one
// space) that asks for a number of steps; the server
//   * queues requests as they arrive (admit) and moves them onto the device, in arrival order, as
//     soon as world slots and the device byte budget allow;
//   * keeps each admitted scene's bodies, manifolds (with their duals and penalties), forces and
//     tree resident between ticks;
//   * advances every resident scene by one Solver::step per tick, all of them in the same launches;
//   * downloads a scene's final state when its steps are done and removes it from the store.
// Scenes without forces and scenes with joints or springs are kept in two stores (lanes), each
// with its own CUDA stream: a store holding any force takes the coloured Gauss-Seidel passes, the
// deferred Jacobi update and the force duals for every body in it, and its dataflow sweeps wait
// along the longest chains, so the contact-only scenes step apart from them, and a tick hands both
// stores' steps to the device before it waits for either. A scene's results are the same as
// stepping it alone: worlds in one store share no state, and removal keeps every survivor's live
// and force order.
#pragma once

#include <chrono>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "avbdg.h"
#include "engine_host.hpp"

namespace avbdg {

class Server {
public:
    Server(const avbdg_params &params, uint64_t budgetBytes, int maxResident);
    // Solver parameters of every lane.
    int setParams(const avbdg_params &p);

    // Queue a scene (bodies and forces in creation order) for `steps` steps. Rejected at once when
    // it is invalid or could never fit the budget.
    int admit(int nb, const avbdg_body_desc *bodies, int nf, const avbdg_force_desc *forces, int steps,
              int64_t &id);
    // Admit what fits, step every resident scene once, retire the finished ones.
    int tick(int &completed);
    // Oldest finished request whose result has not been taken (id -1 if none).
    void poll(int64_t &id, int &bodies) const;
    int takeResult(int64_t id, int count, float *pos, float *quat, float *vel, float *angVel);
    // Cancel a queued or resident request, or drop a finished one's result.
    int evict(int64_t id);
    void stats(avbdg_server_stats &out) const;
    void resetStats();

    const std::string &error() const { return err; }

private:
    using Clock = std::chrono::steady_clock;
    struct Pending {
        int64_t id;
        std::vector<avbdg_body_desc> bodies;
        std::vector<avbdg_force_desc> forces;
        int steps;
        uint64_t bytes;
        Clock::time_point submitted;
    };
    struct Resident {
        int64_t id;
        int stepsLeft, bodies, dynamic;
        uint64_t bytes;
        Clock::time_point submitted;
    };
    struct Result {
        int bodies;
        std::vector<float> state; // [pos 3n | quat 4n | vel 3n | angvel 3n]
    };

    int fail(int code, const std::string &msg) {
        err = msg;
        return code;
    }
    int admitQueued();
    // An engine call failed: keep its message and pass its code on.
    int engineFail(const Engine &e, int code) {
        err = e.error();
        return code;
    }
    int residentCount() const;
    // A lane may grow up to the budget less what the other lane's store holds now.
    void limitLane(int lane);

    // Lane 0: scenes without forces; lane 1: scenes with forces.
    static constexpr int kLanes = 2;
    struct Lane {
        Engine eng;
        std::vector<Resident> resident; // in the store's world order
        Lane(const avbdg_params &params, int bodies, int forces, int worlds) : eng(params, bodies, forces, worlds) {}
    };
    std::unique_ptr<Lane> lanes[kLanes];
    uint64_t budget;
    int maxResident;
    std::deque<Pending> queue;
    std::map<int64_t, Result> results;
    std::deque<int64_t> ready;
    uint64_t residentBytes = 0;
    int64_t nextId = 1;
    int64_t submitted = 0, admitted = 0, completed = 0, evicted = 0, ticks = 0;
    double bodySteps = 0.0, busyMs = 0.0, admitMs = 0.0, stepMs = 0.0, retireMs = 0.0;
    int64_t graphTicks = 0;
    std::vector<float> tickMs, requestMs;
    std::string err;
};

} // namespace avbdg
