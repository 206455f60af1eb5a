"""The FP64 build of the same kernels (libavbdg64.so: the same sources compiled with every
floating-point value of the step in double precision), and the float32 result's error against it.

The float32 library reproduces the reference's float32 solver bit for bit (the parity tests), so
the difference is also the reference's own float32 rounding error on these scenes, amplified by
the solver: 10 rounds leave contact-rich scenes far from converged, and a rounding difference that
flips a discrete choice (a contact kept or released, a stick flag, a clamp) grows from step to
step. On smooth dynamics (a hard jointed chain swinging, no contacts) the two builds agree to
rounding level, which shows that the FP64 build is the same algorithm. The FP64 state is read
back through the same float32 interface (resolution: half a float32 ulp of a coordinate).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu64(pkg):
    return pkg.gpu_api(fp64=True)


def run_pair(pkg, gpu, gpu64, scene, steps):
    from avbd_gb300 import stats

    scenes = pkg.scenes
    a = scenes.instantiate(gpu, scene)
    b = scenes.instantiate(gpu64, scene)
    scenes.advance(a, scene, steps)
    scenes.advance(b, scene, steps)
    pa, qa, _, _ = a.state()
    pb, qb, _, _ = b.state()
    return stats.pose_differences(pa, qa, pb, qb)


def test_fp64_build_is_double(pkg, gpu, gpu64):
    """The FP64 library really computes in double: a body in free fall from 10 m ends its 30th
    step at a different float32 position than the float32 library's, by less than float32's
    rounding can accumulate there (x rounds to ~5e-7 m a step, and v = (x - x0) / dt carries each
    rounding into every later step: at most ~n^2 * 5e-7 = 4.5e-4 m after n = 30 steps)."""
    capi = pkg.capi
    d = capi.make_body_descs([[1, 1, 1]], [1.0], [0.5], [[0.0, 0.0, 10.0]])
    z = []
    for api in (gpu, gpu64):
        w = capi.World(api)
        w.add_bodies(d)
        w.step(30)
        z.append(float(w.state()[0][0, 2]))
    assert z[0] != z[1]
    assert abs(z[0] - z[1]) < 1e-3


def test_fp64_agrees_on_smooth_dynamics(pkg, gpu, gpu64):
    """A 12-link hard ball-jointed chain hanging from a static anchor (no contacts): after 30
    steps the builds differ by rounding-level amounts only."""
    sc = pkg.scenes.hard_chain(links=12)
    dx, dq = run_pair(pkg, gpu, gpu64, sc, 30)
    print(f"hard chain: max |dx| {dx.max():.3e} m, max rotation {dq.max():.3e} rad after 30 steps")
    assert dx.max() < 1e-4 and dq.max() < 1e-4


@pytest.mark.parametrize("config", ["pyramid420", "pile", "lattice"])
def test_fp64_error_first_30_steps(pkg, gpu, gpu64, config):
    """After one step the builds agree to float32 resolution; after 30 the difference is the
    float32 rounding amplified by the unconverged contact solve (a 16-high lattice stack compresses
    by centimetres per interface at 10 rounds), reported, not bounded."""
    sc = getattr(pkg.scenes, config)()
    for steps in (1, 30):
        dx, dq = run_pair(pkg, gpu, gpu64, sc, steps)
        print(f"{config}: after {steps} steps max |dx| {dx.max():.3e} m (median {np.median(dx):.3e}), "
              f"max rotation {dq.max():.3e} rad (float32 vs FP64 build)")
        assert np.all(np.isfinite(dx)) and np.all(np.isfinite(dq))
        if steps == 1:
            assert dx.max() < 1e-5 and dq.max() < 1e-5
    assert dx.max() < 1.0 and dq.max() < 1.0
