"""Long-run statistics of a stepped scene: penetration distribution, constraint violation and
kinetic energy, computed on the host from any world's body state (GPU, oracle or reference).

The penetration figure is the reference's own diagnostic (test/core_test.cpp:485-529,
`satBoxDepth`, sampled as `--pyramid` does at :2064-2243): every fifth tick, the worst true
separating-axis overlap of any two dynamic boxes at the current pose; the distribution of those
per-sample maxima gives p50 / p95 / p99 / max with the reference's index convention
(samples[n/2], samples[int(n*0.95)], ...). The reference scans all box pairs within 1.2 m in x
and z; here the pairs are those whose bounding spheres touch (a k-d tree over the centres), a
superset of every overlapping pair, so the worst overlap is the same.

Pairs joined by a force or an IgnoreCollision are left out, since the solver never collides them
(solver_internal.hpp:70-86). Max constraint violation is the largest distance between the two world anchors of any ball
joint (the constraint `Joint` drives to zero, joint.cpp:80-160). Rest energy is the kinetic
energy 1/2 m|v|^2 + 1/2 w.(R I R^T) w summed over dynamic bodies (double precision), with box
masses and moments as Rigid::Rigid computes them (rigid.cpp:34-72).
"""

import numpy as np

F32 = np.float32


def qrot(q, v):
    """maths.h:48-58 qrot, vectorised over rows, float32: t = 2 (z x v); v + w t + z x t."""
    q = np.asarray(q, F32)
    v = np.asarray(v, F32)
    z = q[:, :3]
    w = q[:, 3:4]
    t = F32(2.0) * np.cross(z, v).astype(F32)
    return (v + w * t + np.cross(z, t).astype(F32)).astype(F32)


def _dot(a, b):
    """linalg dot: a left fold from 0 of the products."""
    s = np.zeros(a.shape[0], F32)
    s = s + a[:, 0] * b[:, 0]
    s = s + a[:, 1] * b[:, 1]
    s = s + a[:, 2] * b[:, 2]
    return s


def sat_box_depth(pa, qa, sa, pb, qb, sb):
    """Minimum separating-axis overlap of box pairs (test/core_test.cpp:485-529), float32.

    Each argument holds one row per pair. Returns the overlap depth of every pair, 0 where an axis
    separates the boxes."""
    n = pa.shape[0]
    ha = np.asarray(sa, F32) * F32(0.5)
    hb = np.asarray(sb, F32) * F32(0.5)
    eye = np.eye(3, dtype=F32)
    ea = [qrot(qa, np.broadcast_to(eye[i], (n, 3))) for i in range(3)]
    eb = [qrot(qb, np.broadcast_to(eye[i], (n, 3))) for i in range(3)]
    d = (np.asarray(pb, F32) - np.asarray(pa, F32)).astype(F32)
    best = np.full(n, F32(1.0e9), F32)
    apart = np.zeros(n, bool)

    def axis(nv, ra, rb, valid=None):
        nonlocal best, apart
        sep = np.abs(_dot(nv, d)) - (ra + rb)
        use = ~apart if valid is None else (~apart & valid)
        apart = apart | (use & (sep > 0))
        take = use & ~(sep > 0)
        best = np.where(take, np.minimum(best, -sep), best)

    for i in range(3):
        ra = ha[:, i]
        rb = np.zeros(n, F32)
        for j in range(3):
            rb = rb + hb[:, j] * np.abs(_dot(ea[i], eb[j]))
        axis(ea[i], ra, rb)
        rb2 = hb[:, i]
        ra2 = np.zeros(n, F32)
        for j in range(3):
            ra2 = ra2 + ha[:, j] * np.abs(_dot(ea[j], eb[i]))
        axis(eb[i], ra2, rb2)
    for i in range(3):
        for j in range(3):
            e = np.cross(ea[i], eb[j]).astype(F32)
            len2 = _dot(e, e)
            valid = ~(len2 < F32(1.0e-8))
            e = (e / np.sqrt(np.where(valid, len2, F32(1.0)))[:, None]).astype(F32)
            r1 = np.zeros(n, F32)
            r2 = np.zeros(n, F32)
            for k in range(3):
                r1 = r1 + ha[:, k] * np.abs(_dot(ea[k], e))
                r2 = r2 + hb[:, k] * np.abs(_dot(eb[k], e))
            axis(e, r1, r2, valid)
    return np.where(apart, F32(0.0), best).astype(F32)


def near_pairs(position, radius, candidates):
    """Index pairs (i < j) among `candidates` whose bounding spheres touch."""
    from scipy.spatial import cKDTree

    idx = np.asarray(candidates, np.int64)
    if idx.size < 2:
        return np.zeros((0, 2), np.int64)
    pos = np.asarray(position, np.float64)[idx]
    rad = np.asarray(radius, np.float64)[idx]
    pairs = cKDTree(pos).query_pairs(2.0 * float(rad.max()), output_type="ndarray")
    if pairs.size == 0:
        return np.zeros((0, 2), np.int64)
    dist = np.linalg.norm(pos[pairs[:, 0]] - pos[pairs[:, 1]], axis=1)
    keep = dist <= rad[pairs[:, 0]] + rad[pairs[:, 1]]
    return idx[pairs[keep]]


def dynamic_boxes(scene):
    """Creation indices of the scene's dynamic boxes (the bodies the reference's scan covers)."""
    box = np.ones(scene.n, bool) if scene.shape is None else np.asarray(scene.shape) == 0
    return np.nonzero(box & (np.asarray(scene.density) > 0))[0]


def exempt_pairs(scene):
    """Creation-index pairs the solver never collides (joined by a force or an IgnoreCollision;
    solver_internal.hpp:70-86), as a set of (min, max) tuples."""
    out = set()
    for j in scene.joints:
        a, b = (j[1], j[2]) if isinstance(j[0], str) else (j[0], j[1])
        if a >= 0 and b >= 0:
            out.add((min(a, b), max(a, b)))
    return out


def worst_overlap(scene, position, orientation, boxes=None, exempt=None):
    """The deepest true overlap of any two dynamic boxes at this pose (metres), leaving out the
    pairs the solver never collides."""
    boxes = dynamic_boxes(scene) if boxes is None else boxes
    exempt = exempt_pairs(scene) if exempt is None else exempt
    size = np.asarray(scene.size, F32)
    radius = 0.5 * np.linalg.norm(size.astype(np.float64), axis=1)
    pairs = near_pairs(position, radius, boxes)
    if exempt and pairs.shape[0]:
        lo, hi = np.minimum(pairs[:, 0], pairs[:, 1]), np.maximum(pairs[:, 0], pairs[:, 1])
        pairs = pairs[np.array([(int(x), int(y)) not in exempt for x, y in zip(lo, hi)], bool)]
    if pairs.shape[0] == 0:
        return 0.0
    # Pairs whose world AABBs are apart by more than a millimetre cannot overlap (a world axis
    # separates them, and the 15 box axes always find a separating axis then): skip them.
    rot = np.abs(np.stack([qrot(orientation, np.broadcast_to(np.eye(3, dtype=F32)[i], (len(orientation), 3)))
                           for i in range(3)], axis=2).astype(np.float64))
    half = np.einsum("nij,nj->ni", rot, 0.5 * size.astype(np.float64))
    a, b = pairs[:, 0], pairs[:, 1]
    gap = np.abs(position[a].astype(np.float64) - position[b]) - (half[a] + half[b])
    touch = np.all(gap < 1e-3, axis=1)
    if not np.any(touch):
        return 0.0
    a, b = a[touch], b[touch]
    depth = sat_box_depth(position[a], orientation[a], size[a], position[b], orientation[b], size[b])
    return float(depth.max())


def joint_error(scene, position, orientation):
    """Largest world-anchor separation of the scene's ball joints (metres); 0 without joints."""
    worst = 0.0
    for j in scene.joints:
        if not isinstance(j[0], (int, np.integer)):
            continue
        a, b, ra, rb = j[0], j[1], j[2], j[3]
        wa = (np.asarray(ra, F32) if a < 0 else
              position[a] + qrot(orientation[a:a + 1], np.asarray([ra], F32))[0])
        wb = (np.asarray(rb, F32) if b < 0 else
              position[b] + qrot(orientation[b:b + 1], np.asarray([rb], F32))[0])
        worst = max(worst, float(np.linalg.norm(wa.astype(np.float64) - wb.astype(np.float64))))
    return worst


def kinetic_energy(scene, orientation, velocity, angular):
    """Sum over dynamic bodies of 1/2 m |v|^2 + 1/2 w.(R I R^T) w, in joules (double precision).
    Boxes only: mass = density * volume, moments m (y^2 + z^2) / 12 etc. (rigid.cpp:34-47)."""
    size = np.asarray(scene.size, np.float64)
    dens = np.asarray(scene.density, np.float64)
    dyn = dens > 0
    if scene.shape is not None:
        dyn &= np.asarray(scene.shape) == 0
    m = dens * size[:, 0] * size[:, 1] * size[:, 2]
    sq = size ** 2
    inertia = np.stack([sq[:, 1] + sq[:, 2], sq[:, 0] + sq[:, 2], sq[:, 0] + sq[:, 1]], axis=1) * (m / 12.0)[:, None]
    q = np.asarray(orientation, np.float64)
    w = np.asarray(angular, np.float64)
    # Body-frame angular velocity: R^T w = conj(q) w q.
    z, s = -q[:, :3], q[:, 3:4]
    t = 2.0 * np.cross(z, w)
    wb = w + s * t + np.cross(z, t)
    v = np.asarray(velocity, np.float64)
    e = 0.5 * m * np.sum(v * v, axis=1) + 0.5 * np.sum(inertia * wb * wb, axis=1)
    return float(np.sum(e[dyn]))


def percentiles(samples):
    """p50 / p95 / p99 / max of per-sample maxima with the reference's indexing (sorted[n/2],
    sorted[int(n*0.95)], sorted[int(n*0.99)], sorted[n-1])."""
    s = np.sort(np.asarray(samples, np.float64))
    n = s.size
    if n == 0:
        return {"p50": 0.0, "p95": 0.0, "p99": 0.0, "max": 0.0, "samples": 0}
    return {"p50": float(s[n // 2]), "p95": float(s[int(n * 0.95)]), "p99": float(s[int(n * 0.99)]),
            "max": float(s[-1]), "samples": int(n)}


class RunStats:
    """Accumulates the statistics over a run: call `sample(step, world)` after each step."""

    def __init__(self, scene, every=5):
        self.scene = scene
        self.every = every
        self.boxes = dynamic_boxes(scene)
        self.exempt = exempt_pairs(scene)
        self.overlaps = []
        self.joint_max = 0.0
        self.final = None

    def sample(self, step, world):
        """`step` counts from 1. Samples every `every`-th step (tick % 5 == 4 in the reference)."""
        if step % self.every != 0:
            return
        pos, quat, vel, ang = world.state()
        self.overlaps.append(worst_overlap(self.scene, pos, quat, self.boxes, self.exempt))
        self.joint_max = max(self.joint_max, joint_error(self.scene, pos, quat))
        self.final = (step, kinetic_energy(self.scene, quat, vel, ang),
                      float(np.max(np.linalg.norm(vel.astype(np.float64), axis=1))) if len(vel) else 0.0)

    def summary(self):
        out = {"penetration_m": percentiles(self.overlaps), "max_joint_error_m": self.joint_max}
        if self.final is not None:
            out["rest_step"], out["rest_kinetic_energy_j"], out["rest_max_speed_mps"] = self.final
        return out


def pose_differences(pos_a, quat_a, pos_b, quat_b):
    """Per-body position distance (m) and rotation angle (rad) between two states of the same
    bodies, in double precision."""
    pa = np.asarray(pos_a, np.float64)
    pb = np.asarray(pos_b, np.float64)
    qa = np.asarray(quat_a, np.float64)
    qb = np.asarray(quat_b, np.float64)
    qa = qa / np.linalg.norm(qa, axis=1, keepdims=True)
    qb = qb / np.linalg.norm(qb, axis=1, keepdims=True)
    c = np.clip(np.abs(np.sum(qa * qb, axis=1)), 0.0, 1.0)
    return np.linalg.norm(pa - pb, axis=1), 2.0 * np.arccos(c)


def pose_difference(pos_a, quat_a, pos_b, quat_b):
    """Largest position distance (m) and rotation angle (rad) between two states of the same
    bodies, in double precision."""
    dx, dq = pose_differences(pos_a, quat_a, pos_b, quat_b)
    return (float(dx.max()) if dx.size else 0.0), (float(dq.max()) if dq.size else 0.0)
