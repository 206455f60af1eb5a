"""The round loop as one persistent launch over a (round, phase, world, chunk) tile queue
(`roundQueueKernel`, AVBDG_QUEUE=1; stores without forces or coloured bodies): every world moves
through its rounds as soon as its own previous phase is done. The per-item arithmetic is the
separate kernels', so the results must be bit-identical: against the reference's recorded runs,
the full lattice, and a batch of uneven worlds stepped with the separate launches.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture
def queue(monkeypatch):
    monkeypatch.setenv("AVBDG_QUEUE", "1")


@pytest.mark.parametrize("run", ["stack", "interleaved", "pyramid420", "lattice", "shape_mix", "converge_interleaved"])
def test_queue_matches_reference_every_step(pkg, gpu, golden, queue, run):
    scenes = pkg.scenes
    rec = golden["runs"][run]
    sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"{run}: first differing step {s + 1}"


def test_queue_full_lattice(pkg, gpu, queue):
    with open(os.path.join(HERE, "golden", "full_runs.json")) as f:
        rec = json.load(f)["runs"]["lattice"]
    scenes = pkg.scenes
    sc = scenes.lattice()
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"lattice: first differing step {s + 1}"


@pytest.mark.parametrize("arm", [False, True])
def test_queue_batch_equals_separate_launches(pkg, gpu, monkeypatch, arm):
    """Uneven worlds (8-512 bodies), with and without the arm cache, stepped both ways."""
    capi, scenes = pkg.capi, pkg.scenes
    worlds = scenes.batch(worlds=256, seed=13)
    states = []
    for forced in ("0", "1"):
        monkeypatch.setenv("AVBDG_QUEUE", forced)
        p = gpu.default_params()
        scenes.apply_params(p, scenes.BENCH_PARAMS)
        if arm:
            p.jacobian_rebuild_distance = 0.02
        b = capi.Batch(gpu.lib, p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds))
        for w in worlds:
            b.add_scene(w)
        b.step(40)
        states.append(b.state_all())
        b.close()
    for x, y in zip(states[0], states[1]):
        assert np.array_equal(x, y)
