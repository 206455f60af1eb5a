"""The drift-gated arm cache (Solver::jacobianRebuildDistance, manifold.cpp:600-668) on the GPU:
batched worlds with removals, eager and captured steps, and the cache switched on mid-run (the
store gains its arm arrays), each bit for bit against the oracle."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["position", "orientation", "velocity", "angular"]


@pytest.mark.parametrize("graphs", [True, False])
def test_gpu_arm_cache_batch(pkg, gpu, oracle, monkeypatch, graphs):
    capi, scenes = pkg.capi, pkg.scenes
    monkeypatch.setenv("AVBDG_NO_GRAPHS", "0" if graphs else "1")
    sc = scenes.arm_cache_pile(steps=0)
    ref = scenes.instantiate(oracle, sc)
    ref.step(80)
    p = gpu.default_params()
    scenes.apply_params(p, sc.params)
    batch = capi.Batch(gpu.lib, p)
    batch.add_scene(scenes.arm_cache(steps=0))
    batch.add_scene(sc)
    batch.step(30)
    batch.remove_worlds([0])
    batch.step(50)
    for x, y, field in zip(batch.state(0), ref.state(), FIELDS):
        assert np.array_equal(x, y), f"graphs={graphs}: {field}"
    batch.close()


def test_gpu_arm_cache_switched_on(pkg, gpu, oracle):
    scenes = pkg.scenes
    on = scenes.arm_cache(steps=0)
    sc = scenes.arm_cache(steps=0)
    sc.params = dict(sc.params, jacobian_rebuild_distance=0.0)
    worlds = []
    for api in (gpu, oracle):
        w = scenes.instantiate(api, sc)
        w.step(40)
        p = w.params
        p.jacobian_rebuild_distance = on.params["jacobian_rebuild_distance"]
        w.params = p
        w.step(60)
        worlds.append(w)
    for x, y, field in zip(worlds[0].state(), worlds[1].state(), FIELDS):
        assert np.array_equal(x, y), field
