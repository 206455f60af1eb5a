"""Error of the float32 step against an FP64 build of the same kernels (libavbdg64.so, compiled
from the same sources with every floating-point value of the step in double precision).

The float32 library reproduces the reference's float32 solver bit for bit (the parity tests), so
this is also the reference's own float32 rounding error on these scenes: for the three benchmark
configurations at full size, after their first 30 steps, the largest position difference (m) and
rotation difference (rad) of any body between the two builds. The FP64 state is read back
through the same float32 interface, so differences below half a float32 ulp of a coordinate
(~5e-7 m at 10 m) are not resolved. The figures are printed and must stay within a loose bound
(1e-2 m, 1e-2 rad); the stated numbers are the bench's `fp64_error` object.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu64(pkg):
    return pkg.gpu_api(fp64=True)


def fp64_error(pkg, gpu, gpu64, scene, steps=30):
    from avbd_gb300 import stats

    scenes = pkg.scenes
    a = scenes.instantiate(gpu, scene)
    b = scenes.instantiate(gpu64, scene)
    scenes.advance(a, scene, steps)
    scenes.advance(b, scene, steps)
    pa, qa, _, _ = a.state()
    pb, qb, _, _ = b.state()
    return stats.pose_difference(pa, qa, pb, qb)


def test_fp64_build_is_double(pkg, gpu, gpu64):
    """The FP64 library really computes in double: a body in free fall from 1 km ends its 120th
    step at a different float32 position than the float32 library's."""
    capi = pkg.capi
    d = capi.make_body_descs([[1, 1, 1]], [1.0], [0.5], [[0.0, 0.0, 1000.0]])
    z = []
    for api in (gpu, gpu64):
        w = capi.World(api)
        w.add_bodies(d)
        w.step(120)
        z.append(float(w.state()[0][0, 2]))
    assert z[0] != z[1]


@pytest.mark.parametrize("config", ["pyramid420", "pile", "lattice"])
def test_fp64_error_first_30_steps(pkg, gpu, gpu64, config):
    sc = getattr(pkg.scenes, config)()
    dx, dq = fp64_error(pkg, gpu, gpu64, sc)
    print(f"{config}: max |dx| {dx:.3e} m, max rotation {dq:.3e} rad after 30 steps (float32 vs FP64 build)")
    assert np.isfinite(dx) and np.isfinite(dq)
    assert dx < 1e-2 and dq < 1e-2
