// Served form (host side): request queue, admission under a device byte budget, per-tick stepping
// of every resident scene in two stores (lanes), retirement. See server.hpp.

#include "server.hpp"

#include <algorithm>
#include <cmath>

namespace avbdg {

namespace {

double msSince(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

double percentile(std::vector<float> v, double p) {
    if (v.empty())
        return 0.0;
    const size_t k = std::min(v.size() - 1, static_cast<size_t>(std::ceil(p * static_cast<double>(v.size()))) - 1);
    std::nth_element(v.begin(), v.begin() + static_cast<long>(k), v.end());
    return v[k];
}

} // namespace

namespace {

// Initial body capacity of the store: 4096 bodies, or less when the budget is small.
int initialBodies(uint64_t budget, int worlds) {
    int nb = 4096;
    while (nb > 64 && Engine::storeBytesForBodies(nb, 64, worlds) > budget)
        nb /= 2;
    return nb;
}

} // namespace

Server::Server(const avbdg_params &params, uint64_t budgetBytes, int maxResidentScenes)
    : budget(budgetBytes), maxResident(std::max(1, maxResidentScenes)) {
    const int worlds = std::max(1, std::min(maxResidentScenes, 1024));
    // Each lane starts at no more than a sixteenth of the budget, so either one can grow to nearly
    // all of it when its scenes need it.
    const int nb = initialBodies(budgetBytes / 16, worlds);
    for (auto &lane : lanes)
        lane = std::make_unique<Lane>(params, nb, 64, worlds);
    for (int l = 0; l < kLanes; l++)
        limitLane(l);
}

int Server::setParams(const avbdg_params &p) {
    for (auto &lane : lanes) {
        const int rc = lane->eng.setParams(p);
        if (rc != AVBDG_OK)
            return engineFail(lane->eng, rc);
    }
    return AVBDG_OK;
}

int Server::residentCount() const {
    int n = 0;
    for (const auto &lane : lanes)
        n += static_cast<int>(lane->resident.size());
    return n;
}

void Server::limitLane(int lane) {
    uint64_t other = 0;
    for (int l = 0; l < kLanes; l++)
        if (l != lane)
            other += lanes[l]->eng.reservedBytes();
    // A limit of 0 would mean none: a lane left no room keeps a one-byte limit (no growth).
    lanes[lane]->eng.setByteLimit(budget > other + 1 ? budget - other : 1);
}

int Server::admit(int nb, const avbdg_body_desc *bodies, int nf, const avbdg_force_desc *forces, int steps,
                  int64_t &id) {
    id = -1;
    if (nb <= 0 || !bodies || nf < 0 || (nf > 0 && !forces) || steps < 1)
        return fail(AVBDG_ERR_INVALID, "a request needs bodies and at least one step");
    std::string why;
    int rc = Engine::validateBodies(nb, bodies, why);
    if (rc == AVBDG_OK)
        rc = Engine::validateForces(nb, nf, forces, why);
    if (rc != AVBDG_OK)
        return fail(rc, why);
    const uint64_t bytes = Engine::storeBytesForBodies(nb, nf, 1);
    if (bytes > budget)
        return fail(AVBDG_ERR_CAPACITY, "the scene alone exceeds the device byte budget");
    Pending p;
    p.id = nextId++;
    p.bodies.assign(bodies, bodies + nb);
    p.forces.assign(forces, forces + nf);
    p.steps = steps;
    p.bytes = bytes;
    p.submitted = Clock::now();
    id = p.id;
    queue.push_back(std::move(p));
    submitted++;
    return AVBDG_OK;
}

// Arrival order, no overtaking: the head waits until a slot and its bytes are free. A scene with
// forces goes to lane 1, any other to lane 0. When the head's lane cannot grow because the other
// lane's store holds the bytes and no scene, that store is shrunk and the head tried once more.
int Server::admitQueued() {
    bool shrunk = false;
    while (!queue.empty()) {
        Pending &p = queue.front();
        if (residentCount() >= maxResident || residentBytes + p.bytes > budget)
            break;
        const int l = p.forces.empty() ? 0 : 1;
        Lane &lane = *lanes[l];
        Lane &other = *lanes[1 - l];
        const auto retry = [&] {
            if (shrunk || !other.resident.empty())
                return false;
            shrunk = true;
            return other.eng.shrinkEmpty() == AVBDG_OK;
        };
        limitLane(l);
        const int w = lane.eng.addWorld();
        if (w < 0) { // the store cannot grow now
            if (retry())
                continue;
            break; // retry next tick
        }
        int rc = lane.eng.addBodies(w, static_cast<int>(p.bodies.size()), p.bodies.data(), nullptr);
        if (rc == AVBDG_OK)
            rc = lane.eng.addForces(w, static_cast<int>(p.forces.size()), p.forces.data());
        if (rc != AVBDG_OK) {
            const std::string why = lane.eng.error();
            lane.eng.removeWorlds({w});
            if (rc == AVBDG_ERR_CAPACITY) { // the byte limit bit before the budget estimate did
                if (retry())
                    continue;
                break; // retry next tick
            }
            return fail(rc, why);
        }
        lane.resident.push_back(Resident{p.id, p.steps, static_cast<int>(p.bodies.size()), lane.eng.worldDynamic(w),
                                         p.bytes, p.submitted});
        residentBytes += p.bytes;
        admitted++;
        queue.pop_front();
    }
    return AVBDG_OK;
}

int Server::tick(int &completedNow) {
    completedNow = 0;
    err.clear();
    const Clock::time_point t0 = Clock::now();
    int rc = admitQueued();
    if (rc != AVBDG_OK)
        return rc;
    if (residentCount() == 0)
        return AVBDG_OK; // nothing on the device: not a tick
    const Clock::time_point t1 = Clock::now();
    // Every lane's step goes to its stream before any is waited for; a lane's counters are then
    // checked (and its store grown) one lane after the other.
    bool stepped[kLanes] = {};
    int failed = AVBDG_OK;
    for (int l = 0; l < kLanes && failed == AVBDG_OK; l++) {
        if (lanes[l]->resident.empty())
            continue;
        rc = lanes[l]->eng.stepEnqueue();
        if (rc != AVBDG_OK)
            failed = engineFail(lanes[l]->eng, rc);
        else
            stepped[l] = true;
    }
    for (int l = 0; l < kLanes; l++) {
        if (!stepped[l])
            continue;
        limitLane(l);
        rc = lanes[l]->eng.stepFinish(); // a lane enqueued before a failure is still finished
        if (rc != AVBDG_OK && failed == AVBDG_OK)
            failed = engineFail(lanes[l]->eng, rc);
    }
    if (failed != AVBDG_OK)
        return failed;
    const Clock::time_point t2 = Clock::now();
    bool allGraphs = true;
    for (int l = 0; l < kLanes; l++)
        if (stepped[l])
            allGraphs = allGraphs && lanes[l]->eng.lastStepWasGraph();
    graphTicks += allGraphs ? 1 : 0;
    for (auto &lanePtr : lanes) {
        Lane &lane = *lanePtr;
        double dyn = 0.0;
        std::vector<int> done;
        for (size_t i = 0; i < lane.resident.size(); i++) {
            dyn += lane.resident[i].dynamic;
            if (--lane.resident[i].stepsLeft <= 0)
                done.push_back(static_cast<int>(i));
        }
        bodySteps += dyn;
        for (int w : done) {
            const Resident &r = lane.resident[w];
            Result res;
            res.bodies = r.bodies;
            const size_t n = static_cast<size_t>(r.bodies);
            res.state.resize(13 * n);
            float *s = res.state.data();
            rc = lane.eng.getState(w, 0, r.bodies, s, s + 3 * n, s + 7 * n, s + 10 * n);
            if (rc != AVBDG_OK)
                return engineFail(lane.eng, rc);
            results.emplace(r.id, std::move(res));
            ready.push_back(r.id);
            requestMs.push_back(static_cast<float>(msSince(r.submitted)));
            residentBytes -= r.bytes;
            completed++;
        }
        if (!done.empty()) {
            rc = lane.eng.removeWorlds(done);
            if (rc != AVBDG_OK)
                return engineFail(lane.eng, rc);
            for (auto it = done.rbegin(); it != done.rend(); ++it)
                lane.resident.erase(lane.resident.begin() + *it);
        }
        completedNow += static_cast<int>(done.size());
    }
    const double ms = msSince(t0);
    admitMs += std::chrono::duration<double, std::milli>(t1 - t0).count();
    stepMs += std::chrono::duration<double, std::milli>(t2 - t1).count();
    retireMs += msSince(t2);
    tickMs.push_back(static_cast<float>(ms));
    busyMs += ms;
    ticks++;
    return AVBDG_OK;
}

void Server::poll(int64_t &id, int &bodies) const {
    id = -1;
    bodies = 0;
    for (int64_t r : ready) {
        auto it = results.find(r);
        if (it != results.end()) {
            id = r;
            bodies = it->second.bodies;
            return;
        }
    }
}

int Server::takeResult(int64_t id, int count, float *pos, float *quat, float *vel, float *angVel) {
    auto it = results.find(id);
    if (it == results.end())
        return fail(AVBDG_ERR_INVALID, "no finished result for this request");
    const Result &r = it->second;
    if (count != r.bodies)
        return fail(AVBDG_ERR_INVALID, "count must equal the request's body count");
    const size_t n = static_cast<size_t>(r.bodies);
    const float *s = r.state.data();
    if (pos)
        std::copy(s, s + 3 * n, pos);
    if (quat)
        std::copy(s + 3 * n, s + 7 * n, quat);
    if (vel)
        std::copy(s + 7 * n, s + 10 * n, vel);
    if (angVel)
        std::copy(s + 10 * n, s + 13 * n, angVel);
    results.erase(it);
    ready.erase(std::remove(ready.begin(), ready.end(), id), ready.end());
    return AVBDG_OK;
}

int Server::evict(int64_t id) {
    for (auto it = queue.begin(); it != queue.end(); ++it)
        if (it->id == id) {
            queue.erase(it);
            evicted++;
            return AVBDG_OK;
        }
    for (auto &lanePtr : lanes) {
        Lane &lane = *lanePtr;
        for (size_t i = 0; i < lane.resident.size(); i++)
            if (lane.resident[i].id == id) {
                const int rc = lane.eng.removeWorlds({static_cast<int>(i)});
                if (rc != AVBDG_OK)
                    return engineFail(lane.eng, rc);
                residentBytes -= lane.resident[i].bytes;
                lane.resident.erase(lane.resident.begin() + static_cast<long>(i));
                evicted++;
                return AVBDG_OK;
            }
    }
    if (results.erase(id)) {
        ready.erase(std::remove(ready.begin(), ready.end(), id), ready.end());
        return AVBDG_OK;
    }
    return fail(AVBDG_ERR_INVALID, "unknown request");
}

void Server::stats(avbdg_server_stats &out) const {
    out = avbdg_server_stats{};
    out.submitted = submitted;
    out.admitted = admitted;
    out.completed = completed;
    out.evicted = evicted;
    out.ticks = ticks;
    out.queued = static_cast<int>(queue.size());
    out.resident = residentCount();
    for (const auto &lane : lanes) {
        for (const Resident &r : lane->resident) {
            out.resident_bodies += r.bodies;
            out.resident_dynamic += r.dynamic;
        }
        out.store_bytes += lane->eng.reservedBytes();
    }
    out.resident_bytes = residentBytes;
    out.budget_bytes = budget;
    out.body_steps = bodySteps;
    out.busy_ms = busyMs;
    out.tick_p50_ms = percentile(tickMs, 0.50);
    out.tick_p99_ms = percentile(tickMs, 0.99);
    out.tick_max_ms = tickMs.empty() ? 0.0 : *std::max_element(tickMs.begin(), tickMs.end());
    out.request_p50_ms = percentile(requestMs, 0.50);
    out.request_p99_ms = percentile(requestMs, 0.99);
    out.admit_ms = admitMs;
    out.step_ms = stepMs;
    out.retire_ms = retireMs;
    out.graph_ticks = graphTicks;
}

void Server::resetStats() {
    ticks = 0;
    bodySteps = busyMs = admitMs = stepMs = retireMs = 0.0;
    graphTicks = 0;
    tickMs.clear();
    requestMs.clear();
}

} // namespace avbdg
