// Served form (host side): request queue, admission under a device byte budget, per-tick stepping
// of every resident scene, retirement. See server.hpp.

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
    : eng(params, initialBodies(budgetBytes, std::max(1, std::min(maxResidentScenes, 1024))), 64,
          std::max(1, std::min(maxResidentScenes, 1024))),
      budget(budgetBytes), maxResident(std::max(1, maxResidentScenes)) {
    eng.setByteLimit(budget);
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

// Arrival order, no overtaking: the head waits until a slot and its bytes are free.
int Server::admitQueued() {
    while (!queue.empty()) {
        Pending &p = queue.front();
        if (static_cast<int>(resident.size()) >= maxResident || residentBytes + p.bytes > budget)
            break;
        const int w = eng.addWorld();
        if (w < 0)
            break; // the store cannot grow now; retry next tick
        int rc = eng.addBodies(w, static_cast<int>(p.bodies.size()), p.bodies.data(), nullptr);
        if (rc == AVBDG_OK)
            rc = eng.addForces(w, static_cast<int>(p.forces.size()), p.forces.data());
        if (rc != AVBDG_OK) {
            const std::string why = eng.error();
            eng.removeWorlds({w});
            if (rc == AVBDG_ERR_CAPACITY)
                break; // the byte limit bit before the budget estimate did; retry next tick
            return fail(rc, why);
        }
        resident.push_back(Resident{p.id, p.steps, static_cast<int>(p.bodies.size()), eng.worldDynamic(w), p.bytes,
                                    p.submitted});
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
    if (resident.empty())
        return AVBDG_OK; // nothing on the device: not a tick
    const Clock::time_point t1 = Clock::now();
    rc = eng.step();
    if (rc != AVBDG_OK)
        return rc;
    const Clock::time_point t2 = Clock::now();
    graphTicks += eng.lastStepWasGraph() ? 1 : 0;
    double dyn = 0.0;
    std::vector<int> done;
    for (size_t i = 0; i < resident.size(); i++) {
        dyn += resident[i].dynamic;
        if (--resident[i].stepsLeft <= 0)
            done.push_back(static_cast<int>(i));
    }
    bodySteps += dyn;
    for (int w : done) {
        const Resident &r = resident[w];
        Result res;
        res.bodies = r.bodies;
        const size_t n = static_cast<size_t>(r.bodies);
        res.state.resize(13 * n);
        float *s = res.state.data();
        rc = eng.getState(w, 0, r.bodies, s, s + 3 * n, s + 7 * n, s + 10 * n);
        if (rc != AVBDG_OK)
            return rc;
        results.emplace(r.id, std::move(res));
        ready.push_back(r.id);
        requestMs.push_back(static_cast<float>(msSince(r.submitted)));
        residentBytes -= r.bytes;
        completed++;
    }
    if (!done.empty()) {
        rc = eng.removeWorlds(done);
        if (rc != AVBDG_OK)
            return rc;
        for (auto it = done.rbegin(); it != done.rend(); ++it)
            resident.erase(resident.begin() + *it);
    }
    completedNow = static_cast<int>(done.size());
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
    for (size_t i = 0; i < resident.size(); i++)
        if (resident[i].id == id) {
            const int rc = eng.removeWorlds({static_cast<int>(i)});
            if (rc != AVBDG_OK)
                return rc;
            residentBytes -= resident[i].bytes;
            resident.erase(resident.begin() + static_cast<long>(i));
            evicted++;
            return AVBDG_OK;
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
    out.resident = static_cast<int>(resident.size());
    for (const Resident &r : resident) {
        out.resident_bodies += r.bodies;
        out.resident_dynamic += r.dynamic;
    }
    out.resident_bytes = residentBytes;
    out.store_bytes = eng.reservedBytes();
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
