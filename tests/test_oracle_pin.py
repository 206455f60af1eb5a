"""Pin the oracle (CPU restatement of the reference step) before trusting it as the checker.

1. The reference suite's pinned digests (tools/baseline/digests.txt:1-3) must come out exactly.
2. Per-step digests, candidate pairs, Morton codes, sorted order, manifold features and colouring
   must equal the golden fixtures recorded from the reference itself (tests/golden/).
3. Where the compiled reference is present, the oracle must match it step by step under
   non-default solver options too.
"""

import hashlib

import numpy as np
import pytest


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["stack", "interleaved", "mixed"])
def test_pinned_reference_digests(pkg, oracle, name):
    scenes = pkg.scenes
    sc = getattr(scenes, name)()
    w = scenes.instantiate(oracle, sc)
    scenes.advance(w, sc)
    assert w.digest() == scenes.PINNED_DIGESTS[name]


def test_golden_runs(pkg, oracle, golden):
    scenes = pkg.scenes
    for name, rec in golden["runs"].items():
        sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
        p = oracle.default_params()
        w = scenes.instantiate(oracle, sc, params=p)
        for s in range(rec["steps"]):
            scenes.advance(w, sc, 1)
            assert f"{w.digest():016x}" == rec["digests"][s], f"{name}: step {s + 1} digest differs"
            if s == 0:
                codes, order, pairs = w.broadphase()
                fs = rec["first_step"]
                assert pairs.size == fs["pairs"] and sha(pairs) == fs["pairs_sha"], name
                assert sha(codes) == fs["codes_sha"] and sha(order) == fs["order_sha"], name
                m = w.manifolds()
                assert sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + sha(m["features"]) == \
                    fs["manifolds_sha"], name
        m = w.manifolds()
        col, ids = w.colours()
        ls = rec["last_step"]
        assert sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + sha(m["features"]) == ls["manifolds_sha"]
        assert sha(col) + sha(ids) == ls["colours_sha"], name


def test_golden_pose_runs(pkg, oracle, golden):
    """Springs and generic joints (hinge, slider, limited and sprung rotations, world anchor), and
    idle sleep with islands and wake-ups: the oracle calls the same C library atan2 as the
    reference, so every step's digest, the stored poses and the sleeping flags are exact."""
    scenes = pkg.scenes
    for name, rec in golden["pose_runs"].items():
        sc = getattr(scenes, rec["scene"])(**rec["kwargs"])
        w = scenes.instantiate(oracle, sc)
        for s in range(rec["steps"]):
            scenes.advance(w, sc, 1)
            assert f"{w.digest():016x}" == rec["digests"][s], f"{name}: step {s + 1} digest differs"
            pose = rec["poses"].get(str(s + 1))
            if pose:
                p, q, _, _ = w.state()
                assert np.array_equal(p, np.asarray(pose["position"], np.float32))
                assert np.array_equal(q, np.asarray(pose["orientation"], np.float32))
                assert np.array_equal(w.sleeping(), np.asarray(pose["sleeping"], np.uint8))


@pytest.mark.parametrize("option", ["adaptive_beta", "stiffness_decay", "no_projection", "gs_contacts"])
def test_oracle_matches_reference_options(pkg, oracle, ref, option):
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
        p.threads = 1
        return p

    wo = scenes.instantiate(oracle, sc, params=params(oracle))
    wr = scenes.instantiate(ref, sc, params=params(ref))
    for s in range(90):
        wo.step()
        wr.step()
        assert wo.digest() == wr.digest(), f"{option}: step {s + 1}"


def test_oracle_matches_reference_interleaved_pile(pkg, oracle, ref):
    scenes = pkg.scenes
    sc = scenes.pile(count=150, chain_links=4)
    sc.params["dt"] = float(np.float32(1.0) / np.float32(240.0))
    wo = scenes.instantiate(oracle, sc)
    wr = scenes.instantiate(ref, sc)
    for s in range(60):
        wo.step_interleaved(4, 2)
        wr.step_interleaved(4, 2)
        assert wo.digest() == wr.digest(), f"step {s + 1}"


def test_oracle_convergence_probe_stops_after_one_round(pkg, oracle, ref):
    """The probe starts from a previous residual of 0 and the residual is a mean of positive
    penetrations, so any positive threshold stops each substep after its first round: a run at 10
    iterations with the probe on equals a run at 1 iteration, on the oracle and on the reference."""
    scenes = pkg.scenes
    sc = scenes.converge_pile(steps=0)
    one = scenes.converge_pile(steps=0)
    one.params = dict(one.params, convergence_threshold=0.0, iterations=1)
    for api in (oracle, ref):
        p = api.default_params()
        p.threads = 1  # two thread pools in one process would oversubscribe the host
        a = scenes.instantiate(api, sc, params=p)
        p = api.default_params()
        p.threads = 1
        b = scenes.instantiate(api, one, params=p)
        for s in range(40):
            a.step()
            b.step()
            assert a.digest() == b.digest(), f"step {s + 1}"


def _query_rays(n=64, seed=4):
    rng = np.random.default_rng(seed)
    origins = rng.uniform([-15, -6, 1], [15, 6, 8], (n, 3)).astype(np.float32)
    targets = rng.uniform([-15, -3, -1], [15, 3, 2], (n, 3)).astype(np.float32)
    return origins, targets - origins


def test_oracle_queries_match_reference(pkg, oracle, ref):
    """Solver::pick and collectAABB over boxes, spheres and cylinders, after 40 steps."""
    scenes = pkg.scenes
    sc = scenes.shape_mix()
    a = scenes.instantiate(oracle, sc)
    b = scenes.instantiate(ref, sc)
    a.step(40)
    b.step(40)
    origins, dirs = _query_rays()
    ba, la = a.pick(origins, dirs)
    bb, lb = b.pick(origins, dirs)
    assert np.array_equal(ba, bb) and np.array_equal(la, lb) and (ba >= 0).sum() > 10
    for lo, hi in [((-12, -2, 0), (-8, 2, 3)), ((-1, -1, 0), (1, 1, 5)), ((-30, -30, -2), (30, 30, 10))]:
        assert np.array_equal(a.collect_aabb(lo, hi), b.collect_aabb(lo, hi))
    box = ((-30, -30, -2), (30, 30, 10))
    assert np.array_equal(a.collect_aabb(*box, mask=2), b.collect_aabb(*box, mask=2))


@pytest.fixture(scope="module")
def full_golden():
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full_runs.json")) as f:
        return json.load(f)


def test_statistics_pinned_to_reference_diagnostic(full_golden):
    """The statistics code (godot-avbd_gb300/stats.py), run on the reference's own states by the
    golden maker, reproduces the RESULT line of the reference's `core_test --pyramid`."""
    rec = full_golden["runs"]["pyramid_dbl"]
    diag, pen = rec["reference_diagnostic"], rec["stats"]["penetration_m"]
    assert (round(pen["p50"], 4), round(pen["p95"], 4), round(pen["max"], 4)) == \
        (diag["p50"], diag["p95"], diag["max"])
    assert pen["samples"] == diag["samples"]
    assert sum(v > 0.05 for v in rec["overlap_samples"]) == diag["over5cm"]


@pytest.mark.parametrize("run", ["pyramid420", "pyramid_dbl"])
def test_oracle_full_config(pkg, oracle, full_golden, run):
    """The oracle over a full configuration: every step's digest and the long-run statistics equal
    the reference's recorded run."""
    from avbd_gb300 import stats

    scenes = pkg.scenes
    rec = full_golden["runs"][run]
    sc = getattr(scenes, run)()
    w = scenes.instantiate(oracle, sc)
    rs = stats.RunStats(sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"{run}: step {s + 1} digest differs"
        rs.sample(s + 1, w)
    assert rs.overlaps == rec["overlap_samples"]
    assert rs.summary()["penetration_m"] == rec["stats"]["penetration_m"]
