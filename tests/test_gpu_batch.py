"""Batched form: independent worlds of uneven size stepped together in one device store. Every
world's state must equal that world stepped alone by the oracle, bit for bit."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch_scenes(scenes):
    worlds = scenes.batch(worlds=24, n_min=8, n_max=120, seed=11, steps=0)
    # Mix in joint scenes so coloured Gauss-Seidel, joints and overflow share one batch.
    worlds.insert(3, scenes.mixed(steps=0))
    worlds.insert(10, scenes.hard_chain(steps=0))
    chain = scenes.pile(count=60, chain_links=6, seed=5)
    worlds.append(chain)
    for w in worlds:
        w.params = dict(scenes.BENCH_PARAMS)
    return worlds


def test_batch_matches_worlds_stepped_alone(pkg, gpu, oracle):
    capi, scenes = pkg.capi, pkg.scenes
    worlds = _batch_scenes(scenes)
    p = gpu.default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    batch = capi.Batch(pkg.load_library(), p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds),
                       max_forces=sum(len(w.joints) for w in worlds))
    for w in worlds:
        batch.add_scene(w)
    refs = [scenes.instantiate(oracle, w) for w in worlds]
    for step in range(60):
        batch.step()
        for r in refs:
            r.step()
        if step % 10 == 9 or step < 3:
            for i, r in enumerate(refs):
                for a, b in zip(batch.state(i), r.state()):
                    assert np.array_equal(a, b), f"world {i} ({worlds[i].name}, {worlds[i].n} bodies) step {step + 1}"
    st = batch.stats()
    assert st.bodies == sum(w.n for w in worlds)
    assert st.manifolds > 0


def test_batch_digests_equal_single_world_gpu(pkg, gpu):
    capi, scenes = pkg.capi, pkg.scenes
    worlds = [scenes.stack(), scenes.mixed(), scenes.stack()]
    worlds[0].params = {}
    worlds[1].params = {}
    worlds[2].params = {}
    batch = capi.Batch(pkg.load_library(), gpu.default_params())
    for w in worlds:
        batch.add_scene(w)
    batch.step(240)
    single = scenes.instantiate(gpu, scenes.mixed())
    single.step(240)
    assert batch.digest(1) == single.digest() == scenes.PINNED_DIGESTS["mixed"]
    assert batch.digest(0) == batch.digest(2)


def test_full_size_batch_worlds_match_alone(pkg, gpu, oracle):
    """The bench's 4096-world batch (433k bodies) at full size: sampled worlds after 8 steps in the
    batch equal the same worlds stepped alone, on the GPU (the largest, the smallest and a spread
    between) and on the oracle (two of them), bit for bit; and again after 60 steps."""
    capi, scenes = pkg.capi, pkg.scenes
    worlds = scenes.batch(worlds=4096, seed=7)
    p = gpu.default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    batch = capi.Batch(pkg.load_library(), p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds),
                       max_forces=max(1, sum(len(w.joints) for w in worlds)))
    for w in worlds:
        batch.add_scene(w)
    batch.step(8)
    sizes = np.array([w.n for w in worlds])
    picks = sorted({int(sizes.argmax()), int(sizes.argmin()), 0, 1, 2047, 4095, 3000, 1234})
    for i in picks:
        sc = worlds[i]
        sc.params = dict(scenes.BENCH_PARAMS)
        alone = scenes.instantiate(gpu, sc)
        alone.step(8)
        assert batch.digest(i) == alone.digest(), f"world {i} ({sc.n} bodies)"
    for i in (int(sizes.argmin()), 1234):
        ref = scenes.instantiate(oracle, worlds[i])
        ref.step(8)
        for x, y in zip(batch.state(i), ref.state()):
            assert np.array_equal(x, y), f"world {i} vs the oracle"
    st = batch.stats()
    assert st.bodies == int(sizes.sum())
    # Longer: 60 steps in all (several Morton rebuilds, the piles settling into contact).
    batch.step(52)
    for i in (int(sizes.argmax()), 2047, 4095):
        sc = worlds[i]
        alone = scenes.instantiate(gpu, sc)
        alone.step(60)
        assert batch.digest(i) == alone.digest(), f"world {i} ({sc.n} bodies) after 60 steps"
    i = int(sizes.argmin())
    ref = scenes.instantiate(oracle, worlds[i])
    ref.step(60)
    for x, y in zip(batch.state(i), ref.state()):
        assert np.array_equal(x, y), f"world {i} vs the oracle after 60 steps"
    batch.close()
