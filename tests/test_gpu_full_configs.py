"""The benchmark configurations at full size and full length, on the GPU, against the reference's
recorded runs (tests/golden/full_runs.json, made by `make_golden.py --full` from the compiled
reference):

  pyramid420   421 bodies, 300 steps       (two 20-row walls of unit cubes)
  pile         1687 bodies, 600 steps      (1653 mass-ratio boxes + a 32-link hard chain)
  lattice      65,537 bodies, 240 steps    (64 x 64 x 16 unit cubes)
  pyramid_dbl  421 bodies, 600 ticks       (the reference's `--pyramid` diagnostic scene:
                                            stepInterleaved(4, 2), arm cache, dropped wall)

Bar: the state digest of every step equals the reference's, and so do the long-run statistics
(penetration distribution by true SAT depth, joint error, rest energy), which then follow
exactly; for the diagnostic scene they also equal the RESULT line the reference's own
`core_test --pyramid` printed.
"""

import json
import os

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def full_golden():
    with open(os.path.join(HERE, "golden", "full_runs.json")) as f:
        return json.load(f)


def run_and_compare(pkg, api, rec):
    from avbd_gb300 import stats

    scenes = pkg.scenes
    sc = getattr(scenes, rec["scene"])()
    assert sc.n == rec["bodies"]
    w = scenes.instantiate(api, sc)
    rs = stats.RunStats(sc)
    for s in range(rec["steps"]):
        scenes.advance(w, sc, 1)
        assert f"{w.digest():016x}" == rec["digests"][s], f"{rec['scene']}: first differing step {s + 1}"
        rs.sample(s + 1, w)
    st = w.stats()
    last = rec["last_step"]
    assert (st.manifolds, st.contacts, st.broad_pairs) == (last["manifolds"], last["contacts"], last["pairs"])
    assert (st.colour_groups, st.overflow_bodies) == (last["colour_groups"], last["overflow"])
    got, want = rs.summary(), rec["stats"]
    assert rs.overlaps == rec["overlap_samples"]
    assert got["penetration_m"] == want["penetration_m"]
    assert got["max_joint_error_m"] == want["max_joint_error_m"]
    assert got["rest_kinetic_energy_j"] == pytest.approx(want["rest_kinetic_energy_j"], rel=1e-12, abs=1e-12)
    return got


@pytest.mark.parametrize("run", ["pyramid420", "pile", "lattice", "pyramid_dbl"])
def test_full_config_matches_reference(pkg, gpu, full_golden, run):
    rec = full_golden["runs"][run]
    got = run_and_compare(pkg, gpu, rec)
    if "reference_diagnostic" in rec:
        diag = rec["reference_diagnostic"]
        pen = got["penetration_m"]
        assert (round(pen["p50"], 4), round(pen["p95"], 4), round(pen["max"], 4)) == \
            (diag["p50"], diag["p95"], diag["max"])
        assert pen["samples"] == diag["samples"]
