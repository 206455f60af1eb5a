"""Body state exchange through the C ABI on both transfer paths: straight between the caller's
arrays and the device (hosts whose GPU reads host memory through the host's page tables) and
through pinned staging (`AVBDG_STAGED_IO=1`, every other host). Either way a state written back
is stepped exactly like the oracle's, and an upload holding a non-finite position or velocity is
refused with nothing changed (`Rigid` public fields, src/avbd/types.hpp:79-88)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["direct", "staged"])
def io_path(request, monkeypatch):
    if request.param == "staged":
        monkeypatch.setenv("AVBDG_STAGED_IO", "1")
    else:
        monkeypatch.delenv("AVBDG_STAGED_IO", raising=False)
    return request.param


def _equal(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_world_state_round_trip_and_refusal(pkg, gpu, oracle, io_path):
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.pyramid420(rows=8)
    w = scenes.instantiate(gpu, sc)
    ref = scenes.instantiate(oracle, sc)
    w.step(10)
    ref.step(10)
    assert _equal(w.state(), ref.state())
    # Written back unchanged, then edited the same way on both sides.
    p, q, v, av = w.state()
    w.set_state(position=p, orientation=q, velocity=v, angular_velocity=av)
    assert _equal(w.state(), (p, q, v, av))
    v2 = (v * 0.5).astype(np.float32)
    av2 = (av + np.float32(0.25)).astype(np.float32)
    w.set_state(velocity=v2, angular_velocity=av2)
    ref.set_state(velocity=v2, angular_velocity=av2)
    w.step(5)
    ref.step(5)
    assert _equal(w.state(), ref.state())
    # A non-finite value in any checked field is refused and changes nothing.
    before = w.state()
    into = tuple(np.empty_like(a) for a in before)
    assert w.state(out=into) is not None and _equal(into, before)
    for field, k in (("position", 0), ("velocity", 2), ("angular_velocity", 3)):
        bad = before[k].copy()
        bad[len(bad) // 2, 1] = np.inf if k else np.nan
        with pytest.raises(capi.AvbdError) as e:
            w.set_state(**{field: bad})
        assert e.value.code == capi.ERR_NONFINITE
        assert _equal(w.state(), before)
    w.step(3)
    ref.step(3)
    assert _equal(w.state(), ref.state())


def test_batch_state_all_round_trip(pkg, gpu, io_path):
    capi, scenes = pkg.capi, pkg.scenes
    worlds = scenes.batch(worlds=24, seed=5)
    p = gpu.default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    batch = capi.Batch(pkg.load_library(), p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds),
                       max_forces=max(1, sum(len(w.joints) for w in worlds)))
    for w in worlds:
        batch.add_scene(w)
    batch.step(4)
    state = batch.state_all()
    batch.set_state_all(*state)
    batch.step(4)
    after = batch.state_all()
    # The same worlds stepped 8 times without the round trip.
    for i in (0, 7, 23):
        sc = worlds[i]
        sc.params = dict(scenes.BENCH_PARAMS)
        alone = scenes.instantiate(gpu, sc)
        alone.step(8)
        start = sum(w.n for w in worlds[:i])
        for x, y in zip(after, alone.state()):
            assert np.array_equal(x[start:start + sc.n], y)
    bad = [a.copy() for a in after]
    bad[2][5, 0] = np.nan
    with pytest.raises(capi.AvbdError) as e:
        batch.set_state_all(*bad)
    assert e.value.code == capi.ERR_NONFINITE
    assert _equal(batch.state_all(), after)
    batch.close()
