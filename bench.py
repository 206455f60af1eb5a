"""Benchmark of the GB300 AVBD time-step: dynamic body-steps per second at 10 solver iterations.

One JSON line on rank 0. Workloads (seeded synthetic scenes, identical inputs on every arm):
  pile       1653 boxes, edges log-uniform 0.25-2 m, densities log-uniform 100-1e4 kg/m^3, random
             orientations, dropped on a 200 x 1 x 200 m ground, plus a 32-link hard ball-joint
             chain (0.2 x 0.2 x 1 m links) hung from a static anchor. dt 1/60 s, 10 iterations.
  pyramid420 two 20-row walls of unit cubes (420 boxes). dt 1/60 s, 10 iterations.
  lattice    64 x 64 x 16 unit cubes, 5 cm gaps, 2 cm jitter, 500 m ground. dt 1/60 s, 10 iterations.
  batch      (default) 4096 independent worlds of 8-512 boxes in one store, beside the plain per-scene
             step on a sample of them; the line also carries the served sweep (below, unless
             --no-serve), the lattice as a `lattice` sub-object (unless --no-lattice) and the
             float32 result's error against the FP64 build of the same kernels for the pyramid,
             pile and lattice (`fp64_error`, unless --no-fp64).
  serve      a stream of requests (16-16,384-box scenes, 60-600 steps each) arriving as Poisson
             processes at each rate of --rates, served by continuous batching under a 120 GB budget:
             throughput, p50/p99 tick and request latency, beside the plain per-scene step.

--impl gpu (default): the sm_103a library. `value` times each step on the library's stream with
CUDA events (the device is idle between steps while the host reads the step's counters), with L2
flushed by a 512 MB write before every timed step and no per-kernel profiling events inside the
step; the rooflines' per-launch kernel times come from a profiled pass of as many further steps
(CUDA events around each timed kernel). `e2e` runs the same workload through the C ABI
with host buffers: every step uploads the bodies' positions, orientations and velocities from
host memory and reads them back.
pile / pyramid420 / lattice also run the configuration over its full length and report the
long-run statistics (penetration distribution by true SAT depth, joint error, rest energy) beside
the reference's recorded ones, every step's digest checked against the reference (--no-stats to
skip; --oracle-stats adds the CPU step's own run).
CPU baselines (batch): the reference's CPU step with one world per host thread (`cpu_baseline`,
the fastest CPU arrangement for these worlds), worlds one after another on all threads, and one
thread.
--impl reference: the reference's CPU step on this machine's host cores (the reference compiled
from its own sources when present here, otherwise the oracle restatement of it, which runs at
0.99x its speed), all threads; for the batch one world per host thread.
Multi-GPU: one independent replica per rank (the path does not shard a single scene).
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

METRIC = "body-steps/s @10 iters"
UNIT = "body-steps/s"


def max_over_ranks(x, world_size):
    """The largest value of x over all ranks: the job takes as long as its slowest rank. The tensor
    lives where the process group's backend wants it (GPU for NCCL, host for gloo)."""
    if world_size <= 1:
        return x
    import torch

    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())
L2_FLUSH_BYTES = 512 << 20


def workload(name):
    scenes = entry.load_package().scenes
    if name == "pile":
        sc = scenes.pile()
        desc = ("mass-ratio pile: 1653 boxes (edges log-uniform 0.25-2 m, densities 100-1e4 kg/m^3, random "
                "orientations) + 32-link hard ball-joint chain, dt 1/60, 10 iterations")
    elif name == "pyramid420":
        sc = scenes.pyramid420()
        desc = "two 20-row walls of 1 m cubes (420 boxes) on a static ground, dt 1/60, 10 iterations"
    elif name == "lattice":
        sc = scenes.lattice()
        desc = "65,536 unit cubes on a 64x64x16 lattice (5 cm gaps, 2 cm jitter) dropped on a 500 m ground, " \
               "dt 1/60, 10 iterations"
    else:
        raise SystemExit(f"unknown workload {name}")
    return sc, desc


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        mhz, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": max(maxes), "reasons": sorted(reasons),
                "samples": len(mhz)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def manifold_pass_bytes(world, dynamic_mask, iterations):
    """Algorithmic bytes of one dual+stamp pass over the live manifolds (the dominant kernel).

    Per non-frozen manifold: body indices, basis and friction, contact count (60 B); position,
    orientation and start-of-step pose of both bodies (128 B). Per contact: anchors, step-start
    error, penalty and dual read (80 B), penalty and dual written (32 B). Per overflow side the
    pass writes a 112 B block stamp on all but the last round of a step.
    """
    m = world.manifolds()
    dyn_a = dynamic_mask[m["body_a"]]
    dyn_b = dynamic_mask[m["body_b"]]
    active = dyn_a | dyn_b
    n_m = int(active.sum())
    n_c = int(m["count"][active].sum())
    sides = int(dyn_a.sum() + dyn_b.sum())
    base = 188 * n_m + 112 * n_c
    avg = base + 112 * sides * (iterations - 1) / iterations
    return avg, {"manifolds": n_m, "contacts": n_c, "stamp_sides": sides}


PROJECTION_PASSES = 4


def traffic_per_launch(workload, algorithmic_bytes):
    """DRAM bytes of one dualKernel launch: the DRAM-to-algorithmic ratio an ncu capture of this
    workload measured (profiles/traffic_<workload>.json) times this run's algorithmic bytes of a
    launch, so the figure describes the same steps as `achieved`. None without a capture."""
    path = os.path.join(ROOT, "profiles", f"traffic_{workload}.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        ratio = json.load(f).get("dram_over_algorithmic")
    return None if ratio is None else ratio * algorithmic_bytes


def profiled_pass(w, flush, steps):
    """Per-launch kernel times for the rooflines: `steps` more steps of `w` (a world or a batch) with
    the library's profiling spans on (CUDA events around each timed kernel, on the library's stream),
    L2 flushed before each, after two steps that capture the profiled step graphs. Returns the kernel
    times and the last step's counters."""
    import torch

    w.set_profiling(True)
    w.step(2)
    torch.cuda.synchronize()
    w.take_kernel_times()
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        w.step()
    torch.cuda.synchronize()
    kt = w.take_kernel_times()
    st = w.stats()
    w.set_profiling(False)
    return kt, st


def body_solve_roofline(st, kt, peak, peak_kind):
    """The block-Jacobi body solve (`overflowSolveKernel`): per overflow body its pose, inertial
    pose, mass and inertia read and its pose written (96 B), plus one 112 B stamp record per
    stamped side; counts from the last timed step, time the mean launch of the timed steps."""
    launch_ms = kt.body_ms / max(kt.body_launches, 1)
    nbytes = 96 * st.overflow_bodies + 112 * st.manifold_sides
    achieved = nbytes / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else 0.0
    return {"bound": "hbm", "kernel": "overflowSolveKernel", "achieved": achieved, "peak": peak,
            "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "algorithmic_bytes_per_launch": nbytes, "launch_ms": launch_ms}


def step_bytes(st, iterations=10, projection_passes=PROJECTION_PASSES):
    """Algorithmic bytes of one whole step from that step's counters (float32 SoA, counted once).

    Per round: 100 B per updated body (pose, inertial pose, mass and inertia read; pose written),
    144 B per contact (primal and dual reads of anchors, step-start error, penalty and dual; dual
    writes) and 304 B per manifold (basis, friction and both bodies' poses, for the primal and the
    dual). Once a step: 56 B per body (bounds, Morton code, warm start, finish), 16 B per candidate
    pair (keys sorted), 200 B per manifold (narrow phase), and per projection pass 152 B per
    manifold plus 60 B per contact (passes counted at their cap; early exit can run fewer).
    """
    per_round = 100 * st.update_bodies + 144 * st.contacts + 304 * st.manifolds
    once = (56 * st.bodies + 16 * st.broad_pairs + 200 * st.manifolds
            + projection_passes * (152 * st.manifolds + 60 * st.contacts))
    return iterations * per_round + once


def step_roofline(total_bytes, total_ms, steps, peak, peak_kind):
    achieved = total_bytes / (total_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
            "frac": achieved / peak, "algorithmic_bytes_per_step": total_bytes / max(steps, 1),
            "note": "whole step: algorithmic bytes of every timed step (its own counters) over the timed "
                    "device time; rounds after the first read L2-resident state, so this is a lower bound "
                    f"on DRAM-side efficiency; projection passes counted at {PROJECTION_PASSES}"}


# Single-thread speed of the oracle port over the compiled reference on the same batch worlds,
# both built at -O3 (the reference's shipped level), measured where the reference tree exists
# (x86-64; 48 random worlds of the batch, steps 6-25): the port stands in for the reference on
# machines without its sources.
PORT_OVER_REFERENCE = 0.99


def cpu_reference_api():
    """The reference CPU step: the reference compiled from its own sources if present here, else
    the oracle port of it. Returns (api, kind)."""
    pkg = entry.load_package()
    capi = pkg.capi
    ref_lib = os.path.join(ROOT, "oracle", "_ref", "libavbd_ref.so")
    if os.path.exists(ref_lib):
        return capi.Api(ctypes.CDLL(ref_lib), "avbdr_"), "reference"
    lib = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return capi.Api(ctypes.CDLL(lib), "avbdo_"), "port"


def run_cpu_reference(sc, steps, warmup, threads, time_budget_s=None):
    """Time the reference CPU step (compiled reference if present here, else the oracle port)."""
    pkg = entry.load_package()
    scenes = pkg.scenes
    api, kind = cpu_reference_api()
    p = api.default_params()
    scenes.apply_params(p, sc.params)
    p.threads = threads
    w = scenes.instantiate(api, sc, params=p)
    w.step(warmup) if warmup > 0 else None
    done, t0 = 0, time.perf_counter()
    per_step = []
    for _ in range(steps):
        t = time.perf_counter()
        w.step()
        per_step.append(time.perf_counter() - t)
        done += 1
        if time_budget_s and time.perf_counter() - t0 > time_budget_s:
            break
    elapsed = sum(per_step)
    return sc.dynamic * done / elapsed, kind, done, elapsed


def run_gpu(args, rank, world_size):
    import numpy as np
    import torch

    pkg = entry.load_package()
    capi, scenes = pkg.capi, pkg.scenes
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    sc, desc = workload(args.workload)
    gpu = pkg.gpu_api()
    w = scenes.instantiate(gpu, sc)
    dyn_mask = sc.density > 0
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        w.step()
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    # The timed steps run without per-kernel profiling spans: their events would split the step's
    # chain of dependent launches. Each step's device time comes from the events the library records
    # at the step's phase boundaries on its own stream.
    step_ms = []
    sum_bytes = 0
    launches = 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            w.step()
            st_i = w.stats()
            step_ms.append(st_i.total_ms)
            sum_bytes += step_bytes(st_i)
            launches += st_i.kernel_launches
        torch.cuda.synchronize()
    kt, st_r = profiled_pass(w, flush, args.steps)
    total_ms = float(sum(step_ms))
    total_ms = max_over_ranks(total_ms, world_size)
    body_steps = sc.dynamic * args.steps * world_size
    value = body_steps / (total_ms / 1e3)

    # End to end through the C ABI with host buffers, on a fresh world after the same warm-up, so it
    # covers the same steps as the device-timed value.
    w.close()
    w = scenes.instantiate(gpu, sc)
    for _ in range(args.warmup):
        w.step()
    p, q, v, av = w.state()
    h2d = d2h = 13 * 4 * sc.n
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w.set_state(position=p, orientation=q, velocity=v, angular_velocity=av)
        w.step()
        p, q, v, av = w.state(out=(p, q, v, av))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world_size)
    e2e = {"value": body_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "steps": [args.warmup + 1, args.warmup + args.steps]}

    peak, peak_kind = measured_peak_hbm()
    bytes_per_launch, counts = manifold_pass_bytes(w, dyn_mask, 10)
    launch_ms = kt.manifold_ms / max(kt.manifold_launches, 1)
    achieved = bytes_per_launch / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else 0.0
    traffic = traffic_per_launch(args.workload, bytes_per_launch)
    roofline = {"bound": "hbm", "kernel": "dualKernel (manifold dual + block stamps)", "achieved": achieved,
                "peak": peak, "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "algorithmic_bytes_per_launch": bytes_per_launch,
                "launch_ms": launch_ms, "counts": counts,
                "note": "working set fits in L2 (126 MB); L2 flushed before each step, not between launches; "
                        "launch times from a profiled pass of as many further steps (kernel spans on)"}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
           "config": {"workload": desc, "bodies": sc.n, "dynamic_bodies": sc.dynamic, "joints": len(sc.joints),
                      "iterations": 10, "dt": "1/60", "form": "plain per-scene step",
                      "timed_steps": [args.warmup + 1, args.warmup + args.steps],
                      "l2": "flushed (512 MB write) before every timed step", "parallelism": f"replicas x{world_size}"},
           "roofline": roofline, "step_roofline": step_roofline(sum_bytes, total_ms, args.steps, peak, peak_kind),
           "e2e": e2e, "gpu_launches": launches,
           "clocks": clocks.summary(),
           "phase_ms_last_step": {k: getattr(w.stats(), k) for k in ["broad_ms", "graph_ms", "solve_ms", "finish_ms"]},
           "kernel_ms": {"manifold_pass_per_launch": launch_ms, "body_solve_per_launch":
                         kt.body_ms / max(kt.body_launches, 1), "narrow_per_step": kt.narrow_ms / max(kt.narrow_launches, 1)},
           "roofline_body_solve": body_solve_roofline(st_r, kt, peak, peak_kind)}
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline:
        cpu_threads = os.cpu_count() or 1
        v_cpu, kind, done, elapsed = run_cpu_reference(sc, args.steps, args.warmup, 0, time_budget_s=20.0)
        out["cpu_baseline"] = {"value": v_cpu, "unit": UNIT, "cores": cpu_threads, "kind": kind,
                               "sample": f"steps {args.warmup + 1}-{args.warmup + done} of the same scene "
                                         f"({elapsed:.1f} s of CPU step time, all {cpu_threads} threads)"}
    return out


def fp64_error_report(checkpoints=(1, 10, 30)):
    """Error of the float32 step, which is bit-identical to the reference's float32 solver, against
    the FP64 build of the same kernels (libavbdg64.so): per benchmark configuration at full size,
    after each checkpoint step, the largest and the median position difference (m) and the largest
    rotation difference (rad) of any body. The FP64 state is read through the same float32
    interface (resolution: half a float32 ulp of a coordinate)."""
    import numpy as np

    pkg = entry.load_package()
    scenes = pkg.scenes
    from avbd_gb300 import stats

    gpu, gpu64 = pkg.gpu_api(), pkg.gpu_api(fp64=True)
    out = {"against": "FP64 build of the same GPU kernels (libavbdg64.so)", "steps": list(checkpoints)}
    for name in ("pyramid420", "pile", "lattice"):
        sc = getattr(scenes, name)()
        a = scenes.instantiate(gpu, sc)
        b = scenes.instantiate(gpu64, sc)
        rec, done = {"bodies": sc.n}, 0
        for k in checkpoints:
            scenes.advance(a, sc, k - done)
            scenes.advance(b, sc, k - done)
            done = k
            pa, qa, _, _ = a.state()
            pb, qb, _, _ = b.state()
            dx, dq = stats.pose_differences(pa, qa, pb, qb)
            rec[f"step_{k}"] = {"max_position_m": float(dx.max()), "median_position_m": float(np.median(dx)),
                                "max_rotation_rad": float(dq.max())}
        out[name] = rec
        a.close()
        b.close()
    return out


def full_run_golden(name):
    path = os.path.join(ROOT, "tests", "golden", "full_runs.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)["runs"].get(name)


def long_run_stats(name, with_oracle):
    """The configuration over its full length on the GPU, every step's state digest checked against
    the reference's recorded run, with the long-run statistics (penetration distribution by true
    SAT depth, joint error, rest energy) beside the reference's recorded ones and, when asked, the
    oracle's (the CPU restatement, run here)."""
    pkg = entry.load_package()
    scenes = pkg.scenes
    from avbd_gb300 import stats

    rec = full_run_golden(name)

    def run(api, check):
        sc = getattr(scenes, name)()
        w = scenes.instantiate(api, sc)
        rs = stats.RunStats(sc)
        mismatch = 0
        for s in range(sc.steps):
            scenes.advance(w, sc, 1)
            if check and rec and f"{w.digest():016x}" != rec["digests"][s]:
                mismatch += 1
            rs.sample(s + 1, w)
        w.close()
        return rs.summary(), mismatch, sc.steps

    gpu_stats, mismatch, steps = run(pkg.gpu_api(), True)
    out = {"steps": steps, "gpu": gpu_stats}
    if rec:
        out["reference_recorded"] = rec["stats"]
        out["steps_whose_digest_differs_from_reference"] = mismatch
        out["penetration_identical_to_reference"] = gpu_stats["penetration_m"] == rec["stats"]["penetration_m"]
    if with_oracle:
        api, kind = cpu_reference_api()
        out["cpu_" + kind] = run(api, False)[0]
    return out


BATCH_DESC = ("4096 independent worlds, dynamic body counts log-uniform in 8-512 (each a 3-20 row pyramid wall "
              "or a random box pile with log-uniform sizes/densities, own static ground), dt 1/60, 10 iterations")


def run_batch(args, rank, world_size):
    """Batched form: all worlds in one device store, one launch per kernel per step; compared
    with the plain per-scene step (one world object per scene, stepped one after another) on a
    bounded sample of the same worlds."""
    import numpy as np
    import torch

    pkg = entry.load_package()
    capi, scenes = pkg.capi, pkg.scenes
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    worlds = scenes.batch(worlds=args.worlds, seed=7 + rank)
    p = pkg.gpu_api().default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    def make_batch():
        b = capi.Batch(pkg.load_library(), p, max_worlds=len(worlds), max_bodies=sum(w.n for w in worlds),
                       max_forces=max(1, sum(len(w.joints) for w in worlds)))
        for w in worlds:
            b.add_scene(w)
        return b

    batch = make_batch()
    dynamic = sum(w.dynamic for w in worlds)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    batch.step(args.warmup)
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    # Timed without per-kernel profiling spans (see run_gpu); the step's phase events give its time.
    step_ms = []
    sum_bytes = 0
    launches = 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            batch.step()
            st_i = batch.stats()
            step_ms.append(st_i.total_ms)
            sum_bytes += step_bytes(st_i)
            launches += st_i.kernel_launches
        torch.cuda.synchronize()
    kt, st = profiled_pass(batch, flush, args.steps)
    total_ms = float(sum(step_ms))
    total_ms = max_over_ranks(total_ms, world_size)
    value = dynamic * args.steps * world_size / (total_ms / 1e3)

    # Roofline of the manifold dual + stamp pass (the per-round kernel carrying the contact state).
    peak, peak_kind = measured_peak_hbm()
    iters = 10
    bytes_per_launch = 188 * st.manifolds + 112 * st.contacts + 112 * st.manifold_sides * (iters - 1) / iters
    launch_ms = kt.manifold_ms / max(kt.manifold_launches, 1)
    achieved = bytes_per_launch / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else 0.0
    traffic = traffic_per_launch("batch", bytes_per_launch)
    roofline = {"bound": "hbm", "kernel": "dualKernel (manifold dual + block stamps)", "achieved": achieved,
                "peak": peak, "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": bytes_per_launch, "launch_ms": launch_ms,
                "counts": {"manifolds": st.manifolds, "contacts": st.contacts, "stamp_sides": st.manifold_sides},
                "note": "L2 flushed before each step, not between the rounds of a step; launch times from a "
                        "profiled pass of as many further steps (kernel spans on)"}

    # End to end: every step uploads all bodies' state from host memory and reads it back, one copy
    # each way for the whole batch, through the C ABI; on a fresh batch of the same worlds after the
    # same warm-up, so it covers the same steps as the device-timed value.
    batch.close()
    batch = make_batch()
    batch.step(args.warmup)
    state = batch.state_all()
    torch.cuda.synchronize()
    e2e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.set_state_all(*state)
        batch.step()
        state = batch.state_all(state)
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world_size)
    nbytes = 13 * 4 * sum(w.n for w in worlds)
    e2e = {"value": dynamic * e2e_steps * world_size / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes}
    # Where an end-to-end step goes, from a few more steps after the timed ones (each part timed
    # alone on the host clock, the step's device time from its own events).
    split = {"upload_ms": 0.0, "step_wall_ms": 0.0, "step_device_ms": 0.0, "download_ms": 0.0}
    split_steps = 5
    for _ in range(split_steps):
        t = time.perf_counter()
        batch.set_state_all(*state)
        t1 = time.perf_counter()
        batch.step()
        t2 = time.perf_counter()
        state = batch.state_all(state)
        t3 = time.perf_counter()
        split["upload_ms"] += (t1 - t) * 1e3 / split_steps
        split["step_wall_ms"] += (t2 - t1) * 1e3 / split_steps
        split["download_ms"] += (t3 - t2) * 1e3 / split_steps
        split["step_device_ms"] += batch.stats().total_ms / split_steps
    e2e["ms_per_step"] = e2e_s * 1e3 / e2e_steps
    e2e["steps"] = [args.warmup + 1, args.warmup + e2e_steps]
    e2e["split_after_timed_steps"] = split

    # Plain per-scene GPU step on a sample of the worlds, each its own avbdg_world.
    rng = np.random.default_rng(1)
    sample = [worlds[i] for i in rng.choice(len(worlds), size=min(args.plain_sample, len(worlds)), replace=False)]
    gpu = pkg.gpu_api()
    plain_body_steps, plain_s = 0, 0.0
    for sc in sample:
        w = scenes.instantiate(gpu, sc)
        w.step(args.warmup)
        torch.cuda.synchronize()
        t = time.perf_counter()
        w.step(args.plain_steps)
        w.sync()
        plain_s += time.perf_counter() - t
        plain_body_steps += sc.dynamic * args.plain_steps
        w.close()
    plain_value = plain_body_steps / plain_s
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
           "config": {"workload": BATCH_DESC, "worlds": len(worlds), "bodies": sum(w.n for w in worlds),
                      "dynamic_bodies": dynamic, "iterations": 10, "dt": "1/60", "form": "batched",
                      "l2": "flushed (512 MB write) before every timed step", "parallelism": f"replicas x{world_size}"},
           "plain_per_scene": {"value": plain_value, "unit": UNIT, "sample_worlds": len(sample),
                               "steps_per_world": args.plain_steps, "batched_over_plain": value / plain_value},
           "roofline": roofline, "step_roofline": step_roofline(sum_bytes, total_ms, args.steps, peak, peak_kind),
           "e2e": e2e, "gpu_launches": launches, "clocks": clocks.summary(),
           "counts": {"manifolds": st.manifolds, "contacts": st.contacts, "pairs": st.broad_pairs},
           "autotuned_block_sizes": {"dualKernel": st.block_dual, "overflowSolveKernel": st.block_solve,
                                     "manifoldInitKernel": st.block_narrow, "traverseKernel": st.block_traverse},
           "phase_ms_last_step": {k: getattr(st, k) for k in ["broad_ms", "graph_ms", "solve_ms", "finish_ms"]},
           "kernel_ms": {"manifold_pass_per_launch": launch_ms,
                         "body_solve_per_launch": kt.body_ms / max(kt.body_launches, 1),
                         "narrow_per_step": kt.narrow_ms / max(kt.narrow_launches, 1)},
           "roofline_body_solve": body_solve_roofline(st, kt, peak, peak_kind)}
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline:
        v_cpu, kind, done, elapsed, cores = run_cpu_parallel_worlds(worlds, args.warmup, args.steps, budget_s=20.0)
        out["cpu_baseline"] = {"value": v_cpu, "unit": UNIT, "cores": cores, "kind": kind,
                               "port_over_reference": PORT_OVER_REFERENCE if kind == "port" else None,
                               "sample": f"{done} world-steps (one world per host thread, each solver "
                                         f"single-threaded, steps {args.warmup + 1}-{args.warmup + args.steps}), "
                                         f"{elapsed:.1f} s of step time per thread on {cores} threads"}
        out["e2e_over_cpu_baseline"] = out["e2e"]["value"] / v_cpu
        v_seq, kind_s, done_s, elapsed_s, _ = run_cpu_batch_sample(worlds, args.warmup, args.steps, budget_s=10.0)
        out["cpu_baseline_one_world_at_a_time"] = {
            "value": v_seq, "unit": UNIT, "cores": cores, "kind": kind_s,
            "sample": f"{done_s} world-steps (worlds stepped one after another, each on all {cores} threads), "
                      f"{elapsed_s:.1f} s"}
        v1, kind1, done1, elapsed1, _ = run_cpu_batch_sample(worlds, args.warmup, args.steps, budget_s=10.0,
                                                            threads=1)
        out["cpu_baseline_1thread"] = {"value": v1, "unit": UNIT, "cores": 1, "kind": kind1,
                                       "sample": f"{done1} world-steps, same sampling, {elapsed1:.1f} s, one thread"}
    return out


SERVE_DESC = ("served request stream: Poisson arrivals, each request a seeded scene of 16-16,384 boxes "
              "(log-uniform; parallel pyramid walls of 3-20 rows, or a mass-ratio pile with an 8-link ball-joint "
              "chain) asking for 60-600 steps, dt 1/60, 10 iterations, admitted under a 120 GB device budget")


def serve_stream(capi, lib, params, reqs, packed, rate, seed, budget):
    """Run one Poisson stream through a server: requests are submitted when their arrival time has
    passed, every tick steps whatever is resident. Returns throughput and latency figures."""
    import numpy as np

    srv = capi.Server(lib, params, budget_bytes=budget, max_resident=4096)
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    arrivals -= arrivals[0]
    n, nxt, finished, peak_resident = len(reqs), 0, 0, 0
    arriving = None  # (seconds, body-steps) when the last request arrived
    trace = []  # after each tick: (seconds, body-steps so far, requests in flight)
    t0 = time.perf_counter()
    while finished < n:
        now = time.perf_counter() - t0
        while nxt < n and arrivals[nxt] <= now:
            descs, forces = packed[nxt]
            srv.admit(reqs[nxt], reqs[nxt].steps, descs, forces)
            nxt += 1
            if nxt == n:
                arriving = (time.perf_counter() - t0, srv.stats().body_steps)
        if nxt - finished == 0:
            time.sleep(max(0.0, arrivals[nxt] - now))
            continue
        finished += srv.tick()
        srv.results()
        peak_resident = max(peak_resident, nxt - finished)
        trace.append((time.perf_counter() - t0, srv.stats().body_steps, nxt - finished))
    wall = time.perf_counter() - t0
    st = srv.stats()
    # Steady state: the ticks during which at least 80 % of the peak number of requests were in
    # flight (the ramp while requests arrive and the drain at the end are left out).
    steady_steps = steady_s = 0.0
    prev_t, prev_b = 0.0, 0.0
    for t, b, flight in trace:
        if flight >= 0.8 * peak_resident:
            steady_steps += b - prev_b
            steady_s += t - prev_t
        prev_t, prev_b = t, b
    out = {"rate_per_s": rate, "requests": n, "body_steps_per_s": st.body_steps / wall, "wall_s": wall,
           "body_steps_per_s_while_arriving": arriving[1] / arriving[0] if arriving and arriving[0] > 0 else None,
           "body_steps_per_s_steady": steady_steps / steady_s if steady_s > 0 else None,
           "steady_share_of_wall": steady_s / wall if wall > 0 else None,
           "ticks": st.ticks, "tick_p50_ms": st.tick_p50_ms, "tick_p99_ms": st.tick_p99_ms,
           "tick_max_ms": st.tick_max_ms, "request_p50_ms": st.request_p50_ms, "request_p99_ms": st.request_p99_ms,
           "peak_in_flight": peak_resident, "busy_s": st.busy_ms / 1e3,
           "tick_split_s": {"admit": st.admit_ms / 1e3, "step": st.step_ms / 1e3, "retire": st.retire_ms / 1e3},
           "graph_ticks": st.graph_ticks}
    srv.close()
    return out


def plain_stream_sample(pkg, reqs, sample, warmup, steps):
    """The plain per-scene GPU step on the same request stream: requests one at a time, each its
    own world; per-request step time measured on a sample, applied to each request's step count."""
    import numpy as np

    gpu = pkg.gpu_api()
    rng = np.random.default_rng(3)
    idx = rng.choice(len(reqs), size=min(sample, len(reqs)), replace=False)
    work, secs = 0.0, 0.0
    for i in idx:
        sc = reqs[i]
        w = pkg.scenes.instantiate(gpu, sc)
        w.step(warmup)
        w.sync()
        t = time.perf_counter()
        w.step(steps)
        w.sync()
        per_step = (time.perf_counter() - t) / steps
        w.close()
        work += sc.dynamic * sc.steps
        secs += per_step * sc.steps
    return {"value": work / secs, "unit": UNIT, "sample_requests": len(idx), "steps_timed_per_request": steps}


def run_serve(args, rank, world_size, standalone=True):
    """Served form (continuous batching) over a rate sweep, beside the plain per-scene step."""
    pkg = entry.load_package()
    capi, scenes = pkg.capi, pkg.scenes
    reqs = scenes.request_stream(requests=args.requests, seed=11 + rank)
    p = pkg.gpu_api().default_params()
    scenes.apply_params(p, scenes.BENCH_PARAMS)
    lib = pkg.load_library()
    packed = [(capi.make_body_descs(r.size, r.density, r.friction, r.position, r.orientation, r.velocity),
               capi.make_force_descs(r.joints)) for r in reqs]
    budget = 120 * 10**9
    # Warm-up stream (first-use costs: allocations, module load), not reported.
    serve_stream(capi, lib, p, reqs[:8], packed[:8], 1000.0, 99, budget)
    sweep = [serve_stream(capi, lib, p, reqs, packed, rate, 100 + k, budget)
             for k, rate in enumerate(args.rates)]
    best = max(sweep, key=lambda r: r["body_steps_per_s"])
    plain = plain_stream_sample(pkg, reqs, args.plain_sample, 3, args.plain_steps)
    total_work = sum(r.dynamic * r.steps for r in reqs)
    served = {"value": best["body_steps_per_s"], "unit": UNIT, "rate_per_s": best["rate_per_s"],
              "steady_value": best["body_steps_per_s_steady"], "steady_share_of_wall": best["steady_share_of_wall"],
              "tick_p50_ms": best["tick_p50_ms"], "tick_p99_ms": best["tick_p99_ms"],
              "request_p50_ms": best["request_p50_ms"], "request_p99_ms": best["request_p99_ms"],
              "served_over_plain": best["body_steps_per_s"] / plain["value"], "plain_per_scene": plain,
              "sweep": sweep, "requests": len(reqs), "body_steps_per_stream": total_work,
              "workload": SERVE_DESC}
    if not standalone:
        return served
    out = {"metric": METRIC, "value": served["value"], "unit": UNIT, "n_gpus": world_size,
           "steps": sum(r.steps for r in reqs), "warmup": 8, "ms_per_step": best["tick_p50_ms"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scene generator)",
           "config": {"workload": SERVE_DESC, "requests": len(reqs), "rates_per_s": args.rates,
                      "form": "served (continuous batching)", "iterations": 10, "dt": "1/60",
                      "l2": "inputs (all resident scenes) larger than L2 at load; not flushed between ticks",
                      "parallelism": f"replicas x{world_size}"},
           "served": served,
           "e2e": {"value": served["value"], "unit": UNIT,
                   "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                   "note": "serving is end to end by construction: scenes uploaded at admission, results read "
                           "back at retirement, inside the timed stream"}}
    return out


def run_cpu_parallel_worlds(worlds, warmup, steps, budget_s, threads=0):
    """The reference's CPU step over the batch's worlds with one world per host thread (each solver
    on one thread, every core busy): how a CPU server steps many independent spaces, and the
    fastest CPU arrangement for worlds of ~100 bodies (one world over all threads pays a barrier
    per phase; the reference runs concurrent solvers on separate threads, test/core_test.cpp:637-658).
    Threads take worlds in a random order from a shared queue until the wall-clock budget is
    spent; each times its own steps, and the aggregate is the sum of the threads' rates."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor

    scenes = entry.load_package().scenes
    api, kind = cpu_reference_api()
    threads = threads if threads > 0 else (os.cpu_count() or 1)
    queue = list(np.random.default_rng(2).permutation(len(worlds)))
    lock = threading.Lock()
    deadline = time.perf_counter() + budget_s

    def worker(_):
        body_steps, elapsed, done = 0, 0.0, 0
        while time.perf_counter() < deadline:
            with lock:
                if not queue:
                    break
                sc = worlds[queue.pop()]
            p = api.default_params()
            scenes.apply_params(p, sc.params)
            p.threads = 1
            w = scenes.instantiate(api, sc, params=p)
            if warmup > 0:
                w.step(warmup)
            t = time.perf_counter()
            w.step(steps)  # one C call: the GIL is released while it runs
            elapsed += time.perf_counter() - t
            body_steps += sc.dynamic * steps
            done += steps
            w.close()
        return body_steps, elapsed, done

    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(worker, range(threads)))
    rate = sum(b / e for b, e, _ in res if e > 0)
    return rate, kind, sum(r[2] for r in res), max(r[1] for r in res), threads


def run_cpu_batch_sample(worlds, warmup, steps, budget_s, threads=0):
    """The reference's CPU step over the batch's worlds, one world at a time with all host threads
    (threads=0, how the reference would serve them) or the given count, on a bounded sample of
    worlds."""
    import numpy as np

    rng = np.random.default_rng(2)
    order = rng.permutation(len(worlds))
    body_steps, elapsed, done, kind = 0, 0.0, 0, "port"
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    for i in order:
        sc = worlds[i]
        v, kind, n_done, t = run_cpu_reference(sc, steps, warmup, threads)
        body_steps += sc.dynamic * n_done
        elapsed += t
        done += n_done
        if elapsed > budget_s:
            break
    return body_steps / elapsed, kind, done, elapsed, cores


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "serve", "pile", "pyramid420", "lattice"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--requests", type=int, default=200, help="served stream length")
    ap.add_argument("--rates", type=float, nargs="+", default=[25.0, 50.0, 100.0, 400.0],
                    help="served stream arrival rates (requests/s)")
    ap.add_argument("--no-serve", action="store_true", help="batch workload without the served sweep")
    ap.add_argument("--no-lattice", action="store_true", help="batch workload without the lattice sub-line")
    ap.add_argument("--no-fp64", action="store_true", help="batch workload without the FP64 error figures")
    ap.add_argument("--no-stats", action="store_true",
                    help="pile/pyramid420/lattice without the full-length run and its long-run statistics")
    ap.add_argument("--oracle-stats", action="store_true",
                    help="also run the CPU reference step over the full length for its statistics")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference" and args.workload == "batch":
        if rank != 0:
            return
        worlds = entry.load_package().scenes.batch(worlds=args.worlds, seed=7)
        v, kind, done, elapsed, cores = run_cpu_parallel_worlds(worlds, args.warmup, args.steps, budget_s=60.0)
        out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)", "impl": "reference",
               "config": {"workload": BATCH_DESC, "worlds": len(worlds), "iterations": 10, "dt": "1/60",
                          "form": "CPU solver step, one world per host thread (each solver single-threaded)"},
               "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                                "port_over_reference": PORT_OVER_REFERENCE if kind == "port" else None,
                                "sample": f"{done} world-steps of randomly chosen worlds (steps {args.warmup + 1}-"
                                          f"{args.warmup + args.steps}), one world per thread on {cores} threads, "
                                          f"{elapsed:.1f} s of step time per thread"},
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        sc, desc = workload(args.workload)
        threads = os.cpu_count() or 1
        v, kind, done, elapsed = run_cpu_reference(sc, args.steps, args.warmup, 0)
        out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world_size, "steps": done,
               "warmup": args.warmup, "ms_per_step": elapsed / max(done, 1) * 1e3, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
               "impl": "reference",
               "config": {"workload": desc, "bodies": sc.n, "dynamic_bodies": sc.dynamic, "iterations": 10,
                          "dt": "1/60", "form": "CPU solver step"},
               "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                                "sample": f"steps {args.warmup + 1}-{args.warmup + done}, all {threads} threads"},
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return

    if world_size > 1:
        import torch

        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.workload == "batch":
        out = run_batch(args, rank, world_size)
        if not args.no_serve:
            out["served"] = run_serve(args, rank, world_size, standalone=False)
        if not args.no_lattice:
            # The 65,536-box lattice as a plain per-scene step: its own warm-up (the cubes land in
            # the first steps) and the same number of timed steps.
            lat = run_gpu(argparse.Namespace(**dict(vars(args), workload="lattice", warmup=max(args.warmup, 20),
                                                    no_cpu_baseline=True)), rank, world_size)
            out["lattice"] = {k: lat[k] for k in ["value", "unit", "ms_per_step", "steps", "warmup", "config",
                                                  "roofline", "roofline_body_solve", "step_roofline", "e2e",
                                                  "gpu_launches", "kernel_ms", "clocks"]}
        if not args.no_fp64 and rank == 0:
            out["fp64_error"] = fp64_error_report()
    elif args.workload == "serve":
        out = run_serve(args, rank, world_size)
    else:
        out = run_gpu(args, rank, world_size)
        if rank == 0 and not args.no_stats:
            out["long_run_stats"] = long_run_stats(args.workload, with_oracle=args.oracle_stats)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world_size > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
