"""Idle sleep, islands and wake-ups on the GPU, bit for bit against the reference's recorded run
(per-step digests, poses and sleeping flags) and the oracle (interleaved substeps, where idle
detection runs on the tick's last substep only)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gpu_sleep_matches_reference(pkg, gpu, golden):
    scenes = pkg.scenes
    rec = golden["pose_runs"]["sleepers"]
    sc = scenes.sleepers()
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        w.step()
        assert f"{w.digest():016x}" == rec["digests"][s], f"step {s + 1}: digest differs"
        pose = rec["poses"].get(str(s + 1))
        if pose:
            assert np.array_equal(w.sleeping(), np.asarray(pose["sleeping"], np.uint8)), f"step {s + 1}: sleeping"
    assert w.sleeping().sum() > 0


def test_gpu_sleep_interleaved_matches_oracle(pkg, gpu, oracle):
    scenes = pkg.scenes
    sc = scenes.sleepers(steps=160)
    sc.substeps, sc.rounds = 2, 3
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    for s in range(sc.steps):
        a.step_interleaved(2, 3)
        b.step_interleaved(2, 3)
        for x, y, field in zip(a.state(), b.state(), ["position", "orientation", "velocity", "angular"]):
            assert np.array_equal(x, y), f"step {s + 1}: {field}"
        assert np.array_equal(a.sleeping(), b.sleeping()), f"step {s + 1}: sleeping"


def test_gpu_sleep_in_batch(pkg, gpu):
    """Sleeping worlds batched with others and with removals keep their solo trajectories."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.sleepers(steps=0)
    p = gpu.default_params()
    scenes.apply_params(p, sc.params)
    plain = scenes.instantiate(gpu, sc)
    plain.step(220)
    batch = capi.Batch(gpu.lib, p)
    filler = scenes.pyramid420()
    batch.add_scene(filler)
    batch.add_scene(sc)
    batch.add_scene(filler)
    batch.step(100)
    batch.remove_worlds([0])
    batch.step(120)
    for x, y, field in zip(batch.state(0), plain.state(), ["position", "orientation", "velocity", "angular"]):
        assert np.array_equal(x, y), f"batched sleepers: {field}"
    batch.close()


def test_gpu_contact_grace_matches_reference(pkg, gpu, golden):
    """Contact grace: parked manifolds keep their state for a few ticks and revive by feature key;
    every step's digest equals the reference's recorded run."""
    scenes = pkg.scenes
    rec = golden["pose_runs"]["pile_grace"]
    sc = scenes.pile_grace()
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        w.step()
        assert f"{w.digest():016x}" == rec["digests"][s], f"step {s + 1}: digest differs"


def test_gpu_contact_grace_batch_and_graphs(pkg, gpu, oracle, monkeypatch):
    """Grace with sleeping in one batch of worlds, eager and captured steps alike."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.pile_grace(count=120, chain_links=4)
    sc.params = dict(sc.params, sleep_frames=20)
    b = scenes.instantiate(oracle, sc)
    b.step(150)
    for graphs in ("1", "0"):
        monkeypatch.setenv("AVBDG_NO_GRAPHS", "0" if graphs == "1" else "1")
        p = gpu.default_params()
        scenes.apply_params(p, sc.params)
        batch = capi.Batch(gpu.lib, p)
        batch.add_scene(scenes.pyramid420())
        batch.add_scene(sc)
        batch.step(60)
        batch.remove_worlds([0])
        batch.step(90)
        for x, y, field in zip(batch.state(0), b.state(), ["position", "orientation", "velocity", "angular"]):
            assert np.array_equal(x, y), f"graphs={graphs}: {field}"
        batch.close()
