"""The multi-lane dual pass (dualLanesKernel: several lanes of a warp per manifold, the stamp terms
added in contact order) against the reference's recorded runs, forced for every store with
AVBDG_DUAL_LANES=1. The autotuner may pick either form, so both must be bit-identical to the
reference: every step's state digest is compared, with the arm cache on and off, coloured and
block-Jacobi bodies, one world and a batch.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture
def lanes(monkeypatch):
    monkeypatch.setenv("AVBDG_DUAL_LANES", "1")


@pytest.mark.parametrize("run", ["stack", "mixed", "pyramid420", "pile", "lattice", "shape_mix", "arm_cache",
                                 "arm_cache_pile", "arm_cache_sleep", "converge_interleaved"])
def test_lanes_match_reference_every_step(pkg, gpu, golden, lanes, run):
    scenes = pkg.scenes
    rec = golden["runs"][run]
    sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"{run}: first differing step {s + 1}"
    assert w.stats().block_dual == -128


def test_lanes_full_lattice(pkg, gpu, lanes):
    """The 65,536-box lattice for its 240 steps, the store the multi-lane form is for."""
    with open(os.path.join(HERE, "golden", "full_runs.json")) as f:
        rec = json.load(f)["runs"]["lattice"]
    scenes = pkg.scenes
    sc = scenes.lattice()
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"lattice: first differing step {s + 1}"


def test_lanes_batch_equals_single_thread_form(pkg, gpu, monkeypatch):
    """A batch of uneven worlds stepped with each form gives the same bits."""
    capi, scenes = pkg.capi, pkg.scenes
    worlds = scenes.batch(worlds=48, seed=5)
    states = []
    for forced in ("0", "1"):
        monkeypatch.setenv("AVBDG_DUAL_LANES", forced)
        monkeypatch.setenv("AVBDG_NO_TUNE", "1")
        p = gpu.default_params()
        scenes.apply_params(p, scenes.BENCH_PARAMS)
        b = capi.Batch(gpu.lib, p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds))
        for w in worlds:
            b.add_scene(w)
        b.step(30)
        states.append(b.state_all())
        b.close()
    for x, y in zip(states[0], states[1]):
        assert np.array_equal(x, y)
