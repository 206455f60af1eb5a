"""GPU parity: the sm_103a step against the reference (golden fixtures recorded from it) and the
oracle, through the C ABI.

Bar: bit-exact. Body state after every step must equal the reference's (FNV digests over
position, orientation and both velocities), and the integer stages (candidate pairs, Morton codes,
sorted order, manifold contact counts and feature keys, colouring) must be identical.
"""

import ctypes
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["stack", "interleaved", "mixed"])
def test_gpu_reproduces_pinned_digests(pkg, gpu, name):
    scenes = pkg.scenes
    sc = getattr(scenes, name)()
    w = scenes.instantiate(gpu, sc)
    scenes.advance(w, sc)
    assert w.digest() == scenes.PINNED_DIGESTS[name]


# Candidate pairs come from the all-pairs test within each world for stores of small worlds (every
# recorded run here) and from the tree walk otherwise; both paths are run against every recording.
@pytest.mark.parametrize("pair_path", ["direct", "tree"])
@pytest.mark.parametrize("run", ["stack", "interleaved", "mixed", "hard_chain", "pyramid420", "pile", "lattice",
                                 "shape_mix", "arm_cache", "arm_cache_pile", "arm_cache_sleep", "converge_pile",
                                 "converge_interleaved"])
def test_gpu_matches_reference_every_step(pkg, gpu, golden, monkeypatch, run, pair_path):
    monkeypatch.setenv("AVBDG_NO_BRUTE", "1" if pair_path == "tree" else "0")
    scenes = pkg.scenes
    rec = golden["runs"][run]
    sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
    w = scenes.instantiate(gpu, sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"{run}: first differing step {s + 1}"
        if s == 0:
            codes, order, pairs = w.broadphase()
            fs = rec["first_step"]
            assert pairs.size == fs["pairs"] and sha(pairs) == fs["pairs_sha"], "candidate pairs"
            assert sha(codes) == fs["codes_sha"], "Morton codes"
            assert sha(order) == fs["order_sha"], "sorted order"
            m = w.manifolds()
            assert sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + sha(m["features"]) == fs["manifolds_sha"]
    m = w.manifolds()
    col, ids = w.colours()
    ls = rec["last_step"]
    assert sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + sha(m["features"]) == ls["manifolds_sha"]
    assert sha(col) + sha(ids) == ls["colours_sha"]
    st = w.stats()
    assert st.colour_groups == ls["colour_groups"] and st.overflow_bodies == ls["overflow"]


def _compare_worlds(pkg, a, b, steps, check_every=1, rebuild_every=17):
    scenes = pkg.scenes
    for s in range(steps):
        a.step()
        b.step()
        if (s + 1) % check_every == 0 or s == steps - 1:
            for x, y, field in zip(a.state(), b.state(), ["position", "orientation", "velocity", "angular"]):
                assert np.array_equal(x, y), f"step {s + 1}: {field} differs (max {np.max(np.abs(x - y)):g})"
        if s % rebuild_every == 0:
            ca, oa, pa = a.broadphase()
            cb, ob, pb = b.broadphase()
            assert np.array_equal(pa, pb), f"step {s + 1}: pairs"
            assert np.array_equal(ca, cb) and np.array_equal(oa, ob), f"step {s + 1}: codes/order"
            ma, mb = a.manifolds(), b.manifolds()
            for key in ["body_a", "body_b", "count", "features"]:
                assert np.array_equal(ma[key], mb[key]), f"step {s + 1}: manifold {key}"
            for key in ["c0", "penalty", "lambda", "basis"]:
                assert np.array_equal(ma[key], mb[key]), f"step {s + 1}: manifold {key}"


@pytest.mark.parametrize("option", ["adaptive_beta", "stiffness_decay", "no_projection", "gs_contacts"])
def test_gpu_matches_oracle_with_options(pkg, gpu, oracle, option):
    scenes = pkg.scenes
    sc = scenes.pile(count=120, chain_links=6)

    def params(api):
        p = api.default_params()
        scenes.apply_params(p, sc.params)
        if option == "adaptive_beta":
            p.adaptive_beta = 1
        elif option == "stiffness_decay":
            p.newton_ratio = 0.5
            p.stiffness_decay = 0.9
        elif option == "no_projection":
            p.position_projection = 0
        elif option == "gs_contacts":
            p.contact_only_overflow = 0
        return p

    a = scenes.instantiate(gpu, sc, params=params(gpu))
    b = scenes.instantiate(oracle, sc, params=params(oracle))
    _compare_worlds(pkg, a, b, 60)


def test_gpu_matches_oracle_full_pile(pkg, gpu, oracle):
    """The 1653-box mass-ratio pile with its 32-link chain, first 30 steps, every field."""
    scenes = pkg.scenes
    sc = scenes.pile()
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    _compare_worlds(pkg, a, b, 30, check_every=1)


def test_gpu_matches_oracle_lattice_slice(pkg, gpu, oracle):
    """A 16 x 16 x 8 slice of the large lattice (2048 cubes), 40 steps."""
    scenes = pkg.scenes
    sc = scenes.lattice(nx=16, ny=16, nz=8)
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    _compare_worlds(pkg, a, b, 40, check_every=5)


def test_gpu_edge_cases(pkg, gpu, oracle):
    capi, scenes = pkg.capi, pkg.scenes
    # Empty world and a single body: stepping is a no-op / free fall, as in the reference.
    w = pkg.world()
    w.step()
    assert w.stats().manifolds == 0
    one = scenes.stack()
    one_g = capi.World(gpu)
    one_o = capi.World(oracle)
    d = capi.make_body_descs(one.size[1:2], one.density[1:2], one.friction[1:2], one.position[1:2])
    one_g.add_bodies(d)
    one_o.add_bodies(d)
    for _ in range(20):
        one_g.step()
        one_o.step()
    for x, y in zip(one_g.state(), one_o.state()):
        assert np.array_equal(x, y)
    # Non-finite input is rejected at the boundary.
    bad = capi.make_body_descs([[1, 1, 1]], [1.0], [0.5], [[0, 0, float("nan")]])
    with pytest.raises(capi.AvbdError) as e:
        pkg.world().add_bodies(bad)
    assert e.value.code == capi.ERR_NONFINITE
    # Unknown force kinds are reported, never approximated.
    batch = capi.Batch(gpu.lib)
    two = scenes.stack()
    two.joints = [(1, 2, (0, 0, 0.5), (0, 0, -0.5), 1000.0, 0.0, float("inf"))]
    descs = capi.scene_body_descs(two)
    forces = capi.make_force_descs(two.joints)
    forces[0].kind = 7
    out = ctypes.c_int()
    rc = batch.fn["batch_add_world"](batch.handle, two.n, descs, 1, forces, ctypes.byref(out))
    assert rc == capi.ERR_UNSUPPORTED
    batch.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_gpu_graph_and_eager_steps(pkg, gpu, golden, monkeypatch, graphs):
    """Steps run as one captured CUDA graph by default and eagerly when graphs are disabled; both
    must reproduce the reference's recorded runs (joints + colouring + overflow: `mixed`)."""
    scenes = pkg.scenes
    monkeypatch.setenv("AVBDG_NO_GRAPHS", "0" if graphs else "1")
    for run in ["mixed", "interleaved", "pyramid420"]:
        rec = golden["runs"][run]
        sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
        w = scenes.instantiate(gpu, sc)
        for s in range(min(rec["steps"], 60)):
            scenes.advance(w, sc, 1)
            assert f"{w.digest():016x}" == rec["digests"][s], f"{run} step {s + 1} graphs={graphs}"
        st = w.stats()
        assert st.graph_step == (1 if graphs else 0), f"graph capture state: {st.graph_step}"
        assert st.kernel_launches > 0


def test_gpu_store_growth(pkg, gpu, oracle):
    """A world created with the smallest store grows while bodies arrive in chunks and while its
    pairs and manifolds outgrow their buffers; results stay identical to the oracle."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.pyramid420()
    p = gpu.default_params()
    scenes.apply_params(p, sc.params)
    a = capi.World(gpu, p, max_bodies=1, max_forces=1)
    q = oracle.default_params()
    scenes.apply_params(q, sc.params)
    b = capi.World(oracle, q)
    for lo in range(0, sc.n, 50):
        hi = min(sc.n, lo + 50)
        d = capi.make_body_descs(sc.size[lo:hi], sc.density[lo:hi], sc.friction[lo:hi], sc.position[lo:hi],
                                 sc.orientation[lo:hi], sc.velocity[lo:hi])
        a.add_bodies(d)
        b.add_bodies(d)
        a.step()
        b.step()
        pa, qa, va, wa = a.state()
        a.set_state(velocity=va)
        for x, y in zip(a.state(), b.state()):
            assert np.array_equal(x, y)
    for _ in range(20):
        a.step()
        b.step()
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


def test_gpu_host_state_edits(pkg, gpu, oracle):
    """Velocity edits between steps (the server integrates host forces this way)."""
    scenes = pkg.scenes
    sc = scenes.pyramid420()
    a = scenes.instantiate(gpu, sc)
    b = scenes.instantiate(oracle, sc)
    for s in range(20):
        a.step()
        b.step()
        if s == 9:
            p, q, v, w = a.state()
            v[1:50, 0] += 0.5
            a.set_state(velocity=v)
            b.set_state(velocity=v)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


def test_gpu_queued_steps_with_growth(pkg, gpu, oracle, golden):
    """step(n) queues each step before the previous one's counters come back (they are checked one
    step behind, in order). A world created with the smallest store grows in its first steps and
    still equals the oracle, and a long run equals the reference's recorded digest."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.pile(count=300, chain_links=8)
    p = gpu.default_params()
    scenes.apply_params(p, sc.params)
    a = capi.World(gpu, p, max_bodies=1, max_forces=1)
    a.add_bodies(capi.scene_body_descs(sc))
    for force in sc.joints:
        a.add_force(force)
    b = scenes.instantiate(oracle, sc)
    a.step(60)
    b.step(60)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    rec = golden["runs"]["pile"]
    w = scenes.instantiate(gpu, scenes.pile(**rec["kwargs"]))
    w.step(rec["steps"])
    assert f"{w.digest():016x}" == rec["digests"][-1]
