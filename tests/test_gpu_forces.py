"""Springs and generic joints on the GPU (hinge, slider limit, limited and sprung rotations, world
anchor, spring chain, next to ball joints, ignore pairs and contacts).

Tolerance (the stated bar for floating point): body positions within 1e-4 m and rotations within
1e-4 rad of the reference over the first 30 steps. The only call whose rounding may differ is the
twist angle's atan2f (CUDA's against the C library's); it is read by the swing's limited and sprung
rotations alone, so every other body must stay bit-identical to the oracle.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-4  # m
ROT_TOL = 1e-4  # rad
SWING = 6       # joint_zoo body whose rotations read the twist angle


def rotation_error(q1, q2):
    """Angle between orientations (rad): 2 |q1 - q2| with the sign of q2 aligned, accurate for the
    small angles compared here (an arccos of the dot product is not, near identity)."""
    a = q1.astype(np.float64)
    b = q2.astype(np.float64)
    b = b * np.where(np.sum(a * b, axis=1) < 0.0, -1.0, 1.0)[:, None]
    return 2.0 * np.linalg.norm(a - b, axis=1)


def test_gpu_forces_match_reference_poses(pkg, gpu, golden):
    scenes = pkg.scenes
    rec = golden["pose_runs"]["joint_zoo"]
    sc = scenes.joint_zoo()
    w = scenes.instantiate(gpu, sc)
    for s in range(30):
        w.step()
        pose = rec["poses"].get(str(s + 1))
        if pose:
            p, q, _, _ = w.state()
            dp = np.max(np.abs(p - np.asarray(pose["position"], np.float32)))
            dq = np.max(rotation_error(q, np.asarray(pose["orientation"], np.float32)))
            assert dp <= POS_TOL and dq <= ROT_TOL, f"step {s + 1}: position {dp:g} m, rotation {dq:g} rad"


def test_gpu_forces_bit_exact_except_twist(pkg, gpu, oracle):
    scenes = pkg.scenes
    sc = scenes.joint_zoo()
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    others = np.ones(sc.n, bool)
    others[SWING] = False
    for s in range(120):
        a.step()
        b.step()
        for x, y, field in zip(a.state(), b.state(), ["position", "orientation", "velocity", "angular"]):
            assert np.array_equal(x[others], y[others]), f"step {s + 1}: {field} of a body without a twist angle"
    st = a.stats()
    assert st.forces == 10 and st.colour_groups > 0


def test_gpu_forces_in_batch_and_removal(pkg, gpu):
    """The same forces through the batched form (bulk force upload), with worlds removed around
    them (generic-joint records move with their forces)."""
    capi, scenes = pkg.capi, pkg.scenes
    zoo = scenes.joint_zoo()
    plain = scenes.instantiate(gpu, zoo)
    plain.step(40)
    want = plain.state()
    p = gpu.default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    batch = capi.Batch(gpu.lib, p)
    filler = scenes.mixed()
    filler.params = dict(scenes.BENCH_PARAMS)
    batch.add_scene(filler)
    batch.add_scene(zoo)
    batch.add_scene(filler)
    batch.step(15)
    batch.remove_worlds([0])
    batch.step(25)
    for x, y, field in zip(batch.state(0), want, ["position", "orientation", "velocity", "angular"]):
        assert np.array_equal(x, y), f"batched joint zoo: {field}"
    batch.close()


def test_gpu_shapes_in_batch(pkg, gpu):
    """Spheres and cylinders batched with boxes (the round-shape narrow phase runs beside box
    pairs in one launch) and with worlds removed: identical to the scene stepped alone."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.shape_mix()
    plain = scenes.instantiate(gpu, sc)
    plain.step(80)
    p = gpu.default_params()
    scenes.apply_params(p, sc.params)
    batch = capi.Batch(gpu.lib, p)
    batch.add_scene(scenes.pyramid420())
    batch.add_scene(sc)
    batch.step(30)
    batch.remove_worlds([0])
    batch.step(50)
    for x, y, field in zip(batch.state(0), plain.state(), ["position", "orientation", "velocity", "angular"]):
        assert np.array_equal(x, y), f"batched shape mix: {field}"
    batch.close()


def test_gpu_queries_match_oracle(pkg, gpu, oracle):
    """Ray picks (one launch for all rays) and box overlap collection on the device equal the
    oracle's serial scans (which match the reference's; see the oracle pin tests)."""
    scenes = pkg.scenes
    sc = scenes.shape_mix()
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    a.step(40)
    b.step(40)
    rng = np.random.default_rng(4)
    origins = rng.uniform([-15, -6, 1], [15, 6, 8], (256, 3)).astype(np.float32)
    dirs = (rng.uniform([-15, -3, -1], [15, 3, 2], (256, 3)) - origins).astype(np.float32)
    ga, la = a.pick(origins, dirs)
    gb, lb = b.pick(origins, dirs)
    assert np.array_equal(ga, gb) and np.array_equal(la, lb) and (ga >= 0).sum() > 40
    for lo, hi in [((-12, -2, 0), (-8, 2, 3)), ((-1, -1, 0), (1, 1, 5)), ((-30, -30, -2), (30, 30, 10))]:
        assert np.array_equal(a.collect_aabb(lo, hi), b.collect_aabb(lo, hi))
