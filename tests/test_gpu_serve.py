"""Served form and world removal on the GPU.

A scene's result must not depend on what else shares the device store: every request served in a
changing mix (admitted while others run, retired while others continue, evicted, held back by the
byte budget) must end bit-identical to the same scene stepped alone in a plain world, which the
parity tests tie to the reference solver.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(pkg, gpu, scene, steps):
    w = pkg.scenes.instantiate(gpu, scene)
    w.step(steps)
    out = w.state()
    w.close()
    return out


def _assert_same(a, b, what):
    for x, y, field in zip(a, b, ["position", "orientation", "velocity", "angular"]):
        assert np.array_equal(x, y), f"{what}: {field} differs (max {np.max(np.abs(x - y)):g})"


def _requests(pkg, sizes, steps, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for n, s in zip(sizes, steps):
        sc = pkg.scenes.request_world(rng, n)
        sc.params = dict(pkg.scenes.BENCH_PARAMS)
        sc.steps = s
        out.append(sc)
    return out


def test_gpu_batch_remove_worlds(pkg, gpu):
    """Worlds removed from a batch between steps leave the survivors' trajectories unchanged
    (bodies move to new slots, manifolds and joints are carried, order is kept)."""
    capi = pkg.capi
    scenes = _requests(pkg, [40, 90, 25, 150, 60, 33], [0] * 6, seed=9)
    p = gpu.default_params()
    pkg.scenes.apply_params(p, pkg.scenes.BENCH_PARAMS)
    b = capi.Batch(gpu.lib, p)
    for sc in scenes:
        b.add_scene(sc)
    b.step(12)
    b.remove_worlds([1, 4])
    b.step(10)
    b.remove_worlds([0])
    b.step(1)
    # Counts live on the device, so the captured steps survive removals (the rebuild plan of the
    # first step after a change was seen before and is now replayed as a graph).
    assert b.stats().graph_step == 1
    b.step(7)
    for world, idx in enumerate([2, 3, 5]):
        _assert_same(b.state(world), _alone(pkg, gpu, scenes[idx], 30), f"world {idx}")
    b.close()


def test_gpu_served_same_alone_and_in_mix(pkg, gpu):
    """Requests arriving while others run, with different lengths, all equal their solo runs."""
    capi = pkg.capi
    sizes = [30, 120, 18, 200, 64, 45, 90]
    steps = [25, 40, 10, 30, 35, 12, 20]
    arrive = [0, 0, 3, 5, 5, 11, 17]  # tick at which each request is submitted
    reqs = _requests(pkg, sizes, steps)
    # Jointed and contact-only scenes: both of the server's stores run.
    assert {bool(r.joints) for r in reqs} == {True, False}
    p = gpu.default_params()
    pkg.scenes.apply_params(p, pkg.scenes.BENCH_PARAMS)
    srv = capi.Server(gpu.lib, p, budget_bytes=8 * 10**9, max_resident=64)
    ids = {}
    results = {}
    tick = 0
    while len(results) < len(reqs):
        for i, t in enumerate(arrive):
            if t == tick:
                ids[srv.admit(reqs[i], reqs[i].steps)] = i
        srv.tick()
        results.update(srv.results())
        tick += 1
        assert tick < 200
    st = srv.stats()
    assert st.completed == len(reqs) and st.resident == 0 and st.queued == 0
    assert st.ticks == tick
    assert st.tick_p99_ms >= st.tick_p50_ms > 0
    for rid, state in results.items():
        i = ids[rid]
        _assert_same(state, _alone(pkg, gpu, reqs[i], reqs[i].steps), f"request {i}")
    srv.close()


def test_gpu_server_budget_and_eviction(pkg, gpu):
    """A budget that holds one scene at a time admits in arrival order as bytes free up; an
    evicted request leaves the others exact; a scene larger than the budget is refused."""
    capi = pkg.capi
    reqs = _requests(pkg, [1500, 1200, 1000, 900], [6, 5, 4, 8], seed=3)
    # The first scene has no joints and the next ones do: the jointed store can only grow once the
    # contact-only store, emptied, gives its bytes back.
    assert not reqs[0].joints and reqs[1].joints
    p = gpu.default_params()
    pkg.scenes.apply_params(p, pkg.scenes.BENCH_PARAMS)
    # The device bytes a request is charged, read from a server that admits the largest one.
    probe = capi.Server(gpu.lib, p, budget_bytes=8 * 10**9, max_resident=8)
    largest = max(range(len(reqs)), key=lambda i: reqs[i].n)
    probe.admit(reqs[largest], 2)
    probe.tick()  # admitted and stepped once; resident until the next tick
    charge = probe.stats().resident_bytes
    probe.close()
    assert charge > 0
    budget = int(charge * 1.1)  # one scene fits, no two of them do
    srv = capi.Server(gpu.lib, p, budget_bytes=budget, max_resident=8)
    big = pkg.scenes.request_world(np.random.default_rng(1), 4 * reqs[largest].n)
    with pytest.raises(capi.AvbdError) as e:
        srv.admit(big, 5)
    assert e.value.code == capi.ERR_CAPACITY
    ids = [srv.admit(r, r.steps) for r in reqs]
    srv.tick()
    st = srv.stats()
    assert st.resident == 1 and st.queued == 3, (st.resident, st.queued, st.resident_bytes, budget)
    assert st.store_bytes <= budget
    srv.evict(ids[2])  # cancel a queued request
    results = {}
    guard = 0
    while len(results) < 3:
        srv.tick()
        st = srv.stats()
        assert st.resident <= 1 and st.resident_bytes <= budget and st.store_bytes <= budget
        results.update(srv.results())
        guard += 1
        assert guard < 200
    assert st.evicted == 1 and set(results) == {ids[0], ids[1], ids[3]}
    for k in (0, 1, 3):
        _assert_same(results[ids[k]], _alone(pkg, gpu, reqs[k], reqs[k].steps), f"request {k}")
    srv.close()
    # Evict a resident request in the middle of its run; the other one is unaffected.
    srv2 = capi.Server(gpu.lib, p, budget_bytes=8 * 10**9, max_resident=8)
    a = srv2.admit(reqs[0], 20)
    b = srv2.admit(reqs[3], reqs[3].steps + 6)
    for _ in range(3):
        srv2.tick()
    srv2.evict(a)
    out = {}
    while b not in out:
        srv2.tick()
        out.update(srv2.results())
    assert a not in out
    _assert_same(out[b], _alone(pkg, gpu, reqs[3], reqs[3].steps + 6), "request after eviction")
    srv2.close()
