"""Generate the golden fixtures of the parity tests from the reference solver itself.

Runs the reference core compiled from its own sources (oracle/_ref/libavbd_ref.so, built by
`make -C oracle ref` on a machine that has the reference tree) on the scenes of
godot-avbd_gb300/scenes.py and records, per scene:
  - the FNV-1a state digest after every step (test/core_test.cpp:133-149),
  - the sorted candidate pairs, Morton codes and (code, index) order after the first step,
  - the live manifolds' body ids, contact counts and feature keys after the first and last step,
  - the colouring of the last step.
Scenes whose arithmetic calls the C library's atan2 (generic joints with limited or sprung
rotations), and the sleeping scene, are recorded with per-step digests plus the full pose and
sleeping flag of every body at a few steps (pose tolerance where the GPU calls CUDA's atan2f).
Writes tests/golden/reference_runs.json. Usage: python tests/golden/make_golden.py

With `--full` it records instead the benchmark configurations at their full size and length
(the 420-box pyramid for 300 steps, the 1653-box pile with its 32-link chain for 600, the
65,536-box lattice for 240) and the reference's double-pyramid diagnostic scene for 600 ticks:
the digest of every step plus the long-run statistics of godot-avbd_gb300/stats.py (penetration
distribution by true SAT depth, joint error, rest energy). For the diagnostic scene it also runs
the reference's own `core_test --pyramid` (built by `make -C oracle reftest`) and stores its
RESULT line, which pins the statistics code. Writes tests/golden/full_runs.json.
"""

import ctypes
import hashlib
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

# (scene builder, keyword arguments, steps recorded)
RUNS = [
    ("stack", {}, 300),
    ("interleaved", {}, 300),
    ("mixed", {}, 240),
    ("hard_chain", {}, 120),
    ("pyramid420", {}, 120),
    ("pile", {"count": 300, "chain_links": 8}, 120),
    ("lattice", {"nx": 8, "ny": 8, "nz": 4}, 90),
    ("shape_mix", {}, 240),
    ("arm_cache", {}, 240),
    ("arm_cache_pile", {}, 120),
    ("arm_cache_sleep", {}, 300),
    ("converge_pile", {}, 120),
    ("converge_interleaved", {}, 300),
]


# (scene builder, keyword arguments, steps recorded, steps whose poses are stored)
POSE_RUNS = [
    ("joint_zoo", {}, 60, [1, 10, 20, 30, 60]),
    ("sleepers", {}, 300, [60, 150, 200, 300]),
    ("pile_grace", {}, 240, [120, 240]),
]


def sha(a):
    return hashlib.sha256(a.tobytes()).hexdigest()


def main():
    pkg = entry.load_package()
    capi, scenes = pkg.capi, pkg.scenes
    lib = os.path.join(ROOT, "oracle", "_ref", "libavbd_ref.so")
    ref = capi.Api(ctypes.CDLL(lib), "avbdr_")
    out = {"generator": "tests/golden/make_golden.py", "runs": {}}
    for name, kw, steps in RUNS:
        sc = getattr(scenes, name)(**kw)
        p = ref.default_params()
        p.threads = 1
        w = scenes.instantiate(ref, sc, params=p)
        digests = []
        rec = {"scene": name, "kwargs": kw, "steps": steps, "bodies": sc.n}
        for s in range(steps):
            scenes.advance(w, sc, 1)
            digests.append(f"{w.digest():016x}")
            if s == 0:
                codes, order, pairs = w.broadphase()
                rec["first_step"] = {
                    "pairs_sha": sha(pairs), "pairs": int(pairs.size),
                    "codes_sha": sha(codes), "order_sha": sha(order),
                }
                m = w.manifolds()
                rec["first_step"]["manifolds_sha"] = sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + \
                    sha(m["features"])
        m = w.manifolds()
        col, ids = w.colours()
        st = w.stats()
        rec["last_step"] = {
            "manifolds": int(m["count"].size), "contacts": int(m["count"].sum()),
            "manifolds_sha": sha(m["body_a"]) + sha(m["body_b"]) + sha(m["count"]) + sha(m["features"]),
            "colours_sha": sha(col) + sha(ids), "colour_groups": st.colour_groups,
            "overflow": st.overflow_bodies,
        }
        rec["digests"] = digests
        out["runs"][name] = rec
        print(name, sc.n, "bodies", steps, "steps, last digest", digests[-1], flush=True)
    out["pose_runs"] = {}
    for name, kw, steps, keep in POSE_RUNS:
        sc = getattr(scenes, name)(**kw)
        p = ref.default_params()
        p.threads = 1
        w = scenes.instantiate(ref, sc, params=p)
        rec = {"scene": name, "kwargs": kw, "steps": steps, "bodies": sc.n, "digests": [], "poses": {}}
        for s in range(steps):
            scenes.advance(w, sc, 1)
            rec["digests"].append(f"{w.digest():016x}")
            if s + 1 in keep:
                pos, quat, _, _ = w.state()
                rec["poses"][str(s + 1)] = {"position": [[float(v) for v in r] for r in pos],
                                            "orientation": [[float(v) for v in r] for r in quat],
                                            "sleeping": [int(v) for v in w.sleeping()]}
        out["pose_runs"][name] = rec
        print(name, sc.n, "bodies", steps, "steps (poses kept)", flush=True)
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(out, f, indent=1)


# (scene builder, steps): the benchmark configurations at full size and length.
FULL_RUNS = [("pyramid420", 300), ("pile", 600), ("lattice", 240), ("pyramid_dbl", 600)]


def reference_pyramid_diagnostic(steps):
    """The RESULT line of the reference's `core_test --pyramid --steps N`, parsed."""
    exe = os.path.join(ROOT, "oracle", "_ref", "core_test")
    out = subprocess.run([exe, "--pyramid", "--steps", str(steps)], capture_output=True, text=True,
                         check=True).stdout
    line = [ln for ln in out.splitlines() if ln.startswith("RESULT")][-1]
    rec = {"line": line}
    for key in ("p50", "p95", "max", "lowest"):
        rec[key] = float(re.search(rf"\b{key}=(-?[0-9.]+)", line).group(1))
    over, n = re.search(r"over5cm=(\d+)/(\d+)", line).groups()
    rec["over5cm"], rec["samples"] = int(over), int(n)
    return rec


def main_full():
    pkg = entry.load_package()
    capi, scenes = pkg.capi, pkg.scenes
    from avbd_gb300 import stats

    ref = capi.Api(ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libavbd_ref.so")), "avbdr_")
    out = {"generator": "tests/golden/make_golden.py --full", "runs": {}}
    for name, steps in FULL_RUNS:
        sc = getattr(scenes, name)()
        p = ref.default_params()
        p.threads = 1
        w = scenes.instantiate(ref, sc, params=p)
        rs = stats.RunStats(sc)
        digests = []
        for s in range(steps):
            scenes.advance(w, sc, 1)
            digests.append(f"{w.digest():016x}")
            rs.sample(s + 1, w)
        st = w.stats()
        rec = {"scene": name, "steps": steps, "bodies": sc.n, "dynamic": sc.dynamic, "digests": digests,
               "stats": rs.summary(), "overlap_samples": [float(v) for v in rs.overlaps],
               "last_step": {"manifolds": st.manifolds, "contacts": st.contacts, "pairs": st.broad_pairs,
                             "colour_groups": st.colour_groups, "overflow": st.overflow_bodies}}
        if name == "pyramid_dbl":
            rec["reference_diagnostic"] = reference_pyramid_diagnostic(steps)
        out["runs"][name] = rec
        print(name, sc.n, "bodies", steps, "steps, last digest", digests[-1], rec["stats"], flush=True)
    with open(os.path.join(HERE, "full_runs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main_full() if "--full" in sys.argv else main()
