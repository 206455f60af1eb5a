"""ctypes binding of the C ABI declared in include/avbdg.h.

The binding is generic over the symbol prefix: the GPU library exports ``avbdg_*``; test
infrastructure builds other libraries that export the same world API under other prefixes and
drives them through this same class.
"""

import ctypes as C

import numpy as np

OK = 0
ERR_INVALID = -1
ERR_CAPACITY = -2
ERR_NONFINITE = -3
ERR_TIMEOUT = -4
ERR_CUDA = -5
ERR_UNSUPPORTED = -6

SHAPE_BOX = 0
SHAPE_SPHERE = 1
SHAPE_CYLINDER = 2


class Params(C.Structure):
    """avbdg_params: the public fields of avbd::Solver (src/avbd/solver.h:54-144)."""

    _fields_ = [
        ("dt", C.c_float),
        ("gravity", C.c_float),
        ("iterations", C.c_int),
        ("alpha", C.c_float),
        ("beta_lin", C.c_float),
        ("beta_ang", C.c_float),
        ("gamma", C.c_float),
        ("newton_ratio", C.c_float),
        ("stiffness_decay", C.c_float),
        ("adaptive_beta", C.c_int),
        ("adaptive_beta_error_floor", C.c_float),
        ("convergence_threshold", C.c_float),
        ("jacobi_relaxation", C.c_float),
        ("contact_only_overflow", C.c_int),
        ("stick_drift_heal", C.c_float),
        ("max_penetration", C.c_float),
        ("jacobian_rebuild_distance", C.c_float),
        ("speculative_margin", C.c_float),
        ("position_projection", C.c_int),
        ("projection_iterations", C.c_int),
        ("projection_beta", C.c_float),
        ("projection_slop", C.c_float),
        ("projection_max_correction", C.c_float),
        ("contact_grace_ticks", C.c_int),
        ("sleep_linear_threshold", C.c_float),
        ("sleep_angular_threshold", C.c_float),
        ("sleep_frames", C.c_int),
        ("threads", C.c_int),
    ]


class BodyDesc(C.Structure):
    """avbdg_body_desc: arguments of Rigid::Rigid plus post-construction fields."""

    _fields_ = [
        ("size", C.c_float * 3),
        ("shape", C.c_int),
        ("density", C.c_float),
        ("friction", C.c_float),
        ("position", C.c_float * 3),
        ("orientation", C.c_float * 4),
        ("velocity", C.c_float * 3),
        ("angular_velocity", C.c_float * 3),
        ("collision_layer", C.c_uint32),
        ("collision_mask", C.c_uint32),
        ("axis_lock_linear", C.c_uint32),
        ("axis_lock_angular", C.c_uint32),
        ("sleep_mode", C.c_uint32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("bodies", C.c_int),
        ("dynamic_bodies", C.c_int),
        ("forces", C.c_int),
        ("broad_pairs", C.c_int),
        ("manifolds", C.c_int),
        ("contacts", C.c_int),
        ("colour_groups", C.c_int),
        ("overflow_bodies", C.c_int),
        ("update_bodies", C.c_int),
        ("steps", C.c_int),
        ("broad_ms", C.c_double),
        ("graph_ms", C.c_double),
        ("solve_ms", C.c_double),
        ("finish_ms", C.c_double),
        ("total_ms", C.c_double),
        ("manifold_sides", C.c_int),
        ("graph_step", C.c_int),
        ("kernel_launches", C.c_int),
        ("block_dual", C.c_int), ("block_solve", C.c_int), ("block_narrow", C.c_int), ("block_traverse", C.c_int),
    ]


class KernelTimes(C.Structure):
    _fields_ = [
        ("manifold_ms", C.c_double),
        ("manifold_launches", C.c_int),
        ("body_ms", C.c_double),
        ("body_launches", C.c_int),
        ("narrow_ms", C.c_double),
        ("narrow_launches", C.c_int),
        ("kernel_launches", C.c_int),
        ("steps", C.c_int),
    ]


AXIS_FREE, AXIS_LOCKED, AXIS_LIMITED = 0, 1, 2


class JointAxis(C.Structure):
    """avbdg_joint_axis: one degree of freedom of a generic joint."""

    _fields_ = [
        ("mode", C.c_int),
        ("lower", C.c_float),
        ("upper", C.c_float),
        ("spring_stiffness", C.c_float),
        ("spring_equilibrium", C.c_float),
        ("spring_damping", C.c_float),
    ]


def make_axes(axes):
    """Six (mode, lower, upper, spring_stiffness, spring_equilibrium, spring_damping) tuples ->
    avbdg_joint_axis[6] (linear x, y, z, then angular x, y, z)."""
    out = (JointAxis * 6)()
    for i, ax in enumerate(axes):
        out[i].mode = int(ax[0])
        out[i].lower, out[i].upper = float(ax[1]), float(ax[2])
        out[i].spring_stiffness, out[i].spring_equilibrium, out[i].spring_damping = (float(ax[3]), float(ax[4]),
                                                                                     float(ax[5]))
    return out


class ForceDesc(C.Structure):
    """avbdg_force_desc: kind 0 = Joint, 1 = IgnoreCollision, 2 = Spring, 3 = GenericJoint."""

    _fields_ = [
        ("kind", C.c_int),
        ("body_a", C.c_int),
        ("body_b", C.c_int),
        ("r_a", C.c_float * 3),
        ("r_b", C.c_float * 3),
        ("stiffness_lin", C.c_float),
        ("stiffness_ang", C.c_float),
        ("fracture", C.c_float),
        ("rest", C.c_float),
        ("axes", JointAxis * 6),
    ]


class AvbdError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"AVBD call failed ({code}): {message}")
        self.code = code


_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint64)
_bp = C.POINTER(C.c_uint8)

# name -> argtypes (after the handle where one is taken); all return int.
_WORLD_FUNCS = {
    "params_default": [C.POINTER(Params)],
    "world_create": [C.POINTER(Params), C.c_int, C.c_int, C.POINTER(C.c_void_p)],
    "world_destroy": [C.c_void_p],
    "world_clear": [C.c_void_p],
    "world_set_params": [C.c_void_p, C.POINTER(Params)],
    "world_get_params": [C.c_void_p, C.POINTER(Params)],
    "world_add_bodies": [C.c_void_p, C.c_int, C.POINTER(BodyDesc), C.POINTER(C.c_int)],
    "world_add_joint": [C.c_void_p, C.c_int, C.c_int, _fp, _fp, C.c_float, C.c_float, C.c_float,
                        C.POINTER(C.c_int)],
    "world_add_ignore_collision": [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)],
    "world_add_spring": [C.c_void_p, C.c_int, C.c_int, _fp, _fp, C.c_float, C.c_float, C.POINTER(C.c_int)],
    "world_add_generic_joint": [C.c_void_p, C.c_int, C.c_int, _fp, _fp, C.POINTER(JointAxis), C.POINTER(C.c_int)],
    "world_step": [C.c_void_p],
    "world_step_interleaved": [C.c_void_p, C.c_int, C.c_int],
    "world_step_n": [C.c_void_p, C.c_int],
    "world_sync": [C.c_void_p],
    "world_get_body_state": [C.c_void_p, C.c_int, C.c_int, _fp, _fp, _fp, _fp],
    "world_get_sleeping": [C.c_void_p, C.c_int, C.c_int, _bp],
    "world_pick": [C.c_void_p, C.c_int, _fp, _fp, C.c_uint32, _ip, _fp],
    "world_collect_aabb": [C.c_void_p, _fp, _fp, C.c_uint32, C.c_int, _ip, C.POINTER(C.c_int)],
    "world_set_body_state": [C.c_void_p, C.c_int, C.c_int, _fp, _fp, _fp, _fp],
    "world_get_stats": [C.c_void_p, C.POINTER(Stats)],
    "world_digest": [C.c_void_p, _up],
    "world_dump_broadphase": [C.c_void_p, _up, _ip, C.c_int, _up, C.c_int, C.POINTER(C.c_int),
                              C.POINTER(C.c_int)],
    "world_dump_manifolds": [C.c_void_p, C.c_int, _ip, _ip, _ip, _ip, _fp, _fp, _fp, _fp,
                             C.POINTER(C.c_int)],
    "world_dump_colours": [C.c_void_p, C.c_int, _bp, _ip, C.POINTER(C.c_int)],
}


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


class Api:
    """The world API of one shared library, bound under `prefix` (e.g. "avbdg_")."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.prefix = prefix
        for name, argtypes in _WORLD_FUNCS.items():
            fn = getattr(lib, prefix + name)
            fn.argtypes = argtypes
            fn.restype = C.c_int
            setattr(self, name, fn)
        err = getattr(lib, prefix + "last_error")
        err.argtypes = []
        err.restype = C.c_char_p
        self._last_error = err

    def check(self, rc):
        if rc != OK:
            raise AvbdError(rc, self._last_error().decode(errors="replace"))
        return rc

    def default_params(self):
        p = Params()
        self.check(self.params_default(C.byref(p)))
        return p


def make_body_descs(size, density, friction, position, orientation=None, velocity=None,
                    angular_velocity=None, sleep_mode=None, shape=None):
    """Pack per-body arrays (n x 3 / n x 4 / n) into an avbdg_body_desc array."""
    size = np.asarray(size, np.float32).reshape(-1, 3)
    n = size.shape[0]
    density = np.broadcast_to(np.asarray(density, np.float32), (n,))
    friction = np.broadcast_to(np.asarray(friction, np.float32), (n,))
    position = np.asarray(position, np.float32).reshape(n, 3)
    if orientation is None:
        orientation = np.tile(np.array([0, 0, 0, 1], np.float32), (n, 1))
    orientation = np.asarray(orientation, np.float32).reshape(n, 4)
    velocity = np.zeros((n, 3), np.float32) if velocity is None else np.asarray(velocity, np.float32).reshape(n, 3)
    if angular_velocity is None:
        angular_velocity = np.zeros((n, 3), np.float32)
    angular_velocity = np.asarray(angular_velocity, np.float32).reshape(n, 3)
    sleep_mode = np.broadcast_to(np.asarray(0 if sleep_mode is None else sleep_mode, np.int64), (n,))
    shape = np.broadcast_to(np.asarray(SHAPE_BOX if shape is None else shape, np.int64), (n,))
    descs = (BodyDesc * n)()
    for i in range(n):
        d = descs[i]
        d.size[:] = size[i].tolist()
        d.shape = int(shape[i])
        d.density = float(density[i])
        d.friction = float(friction[i])
        d.position[:] = position[i].tolist()
        d.orientation[:] = orientation[i].tolist()
        d.velocity[:] = velocity[i].tolist()
        d.angular_velocity[:] = angular_velocity[i].tolist()
        d.collision_layer = 1
        d.collision_mask = 1
        d.axis_lock_linear = 0
        d.axis_lock_angular = 0
        d.sleep_mode = int(sleep_mode[i])
    return descs


def scene_body_descs(scene):
    """avbdg_body_desc array of a scenes.Scene, creation order."""
    return make_body_descs(scene.size, scene.density, scene.friction, scene.position, scene.orientation,
                           scene.velocity, sleep_mode=getattr(scene, "sleep_mode", None),
                           shape=getattr(scene, "shape", None))


class World:
    """One avbd::Solver behind the C ABI (any implementation bound by `Api`)."""

    def __init__(self, api, params=None, max_bodies=0, max_forces=0):
        self.api = api
        p = api.default_params() if params is None else params
        h = C.c_void_p()
        api.check(api.world_create(C.byref(p), int(max_bodies), int(max_forces), C.byref(h)))
        self.handle = h
        self.n_bodies = 0

    def close(self):
        if self.handle:
            self.api.world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        p = Params()
        self.api.check(self.api.world_get_params(self.handle, C.byref(p)))
        return p

    @params.setter
    def params(self, p):
        self.api.check(self.api.world_set_params(self.handle, C.byref(p)))

    def add_bodies(self, descs):
        n = len(descs)
        ids = (C.c_int * n)()
        self.api.check(self.api.world_add_bodies(self.handle, n, descs, ids))
        self.n_bodies += n
        return list(ids)

    def add_joint(self, a, b, r_a, r_b, stiffness_lin=float("inf"), stiffness_ang=0.0,
                  fracture=float("inf")):
        ra = (C.c_float * 3)(*r_a)
        rb = (C.c_float * 3)(*r_b)
        out = C.c_int()
        self.api.check(self.api.world_add_joint(self.handle, int(a), int(b), ra, rb,
                                                float(stiffness_lin), float(stiffness_ang),
                                                float(fracture), C.byref(out)))
        return out.value

    def add_ignore_collision(self, a, b):
        out = C.c_int()
        self.api.check(self.api.world_add_ignore_collision(self.handle, int(a), int(b), C.byref(out)))
        return out.value

    def add_spring(self, a, b, r_a, r_b, stiffness, rest=-1.0):
        ra = (C.c_float * 3)(*r_a)
        rb = (C.c_float * 3)(*r_b)
        out = C.c_int()
        self.api.check(self.api.world_add_spring(self.handle, int(a), int(b), ra, rb, float(stiffness), float(rest),
                                                 C.byref(out)))
        return out.value

    def add_generic_joint(self, a, b, r_a, r_b, axes):
        ra = (C.c_float * 3)(*r_a)
        rb = (C.c_float * 3)(*r_b)
        out = C.c_int()
        self.api.check(self.api.world_add_generic_joint(self.handle, int(a), int(b), ra, rb, make_axes(axes),
                                                        C.byref(out)))
        return out.value

    def add_force(self, force):
        """One scene force record (see scenes.Scene.joints) in creation order."""
        if force[0] == "spring":
            _, a, b, ra, rb, k, rest = force
            return self.add_spring(a, b, ra, rb, k, rest)
        if force[0] == "generic":
            _, a, b, ra, rb, axes = force
            return self.add_generic_joint(a, b, ra, rb, axes)
        if force[0] == "ignore":
            return self.add_ignore_collision(force[1], force[2])
        a, b, ra, rb, kl, ka, fr = force
        return self.add_joint(a, b, ra, rb, kl, ka, fr)

    def step(self, n=1):
        if n == 1:
            self.api.check(self.api.world_step(self.handle))
        else:
            self.api.check(self.api.world_step_n(self.handle, int(n)))

    def step_interleaved(self, substeps, rounds):
        self.api.check(self.api.world_step_interleaved(self.handle, int(substeps), int(rounds)))

    def sync(self):
        self.api.check(self.api.world_sync(self.handle))

    def state(self, out=None):
        """(position n x 3, orientation n x 4, velocity n x 3, angular velocity n x 3), creation order;
        into `out` (four float32 C-contiguous arrays of those shapes) when given."""
        n = self.n_bodies
        if out is not None:
            p, q, v, w = out
            for a, k in zip(out, (3, 4, 3, 3)):
                if a.dtype != np.float32 or a.shape != (n, k) or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError("state(out=...) wants float32 C-contiguous arrays of n x 3, 4, 3, 3")
        else:
            p = np.zeros((n, 3), np.float32)
            q = np.zeros((n, 4), np.float32)
            v = np.zeros((n, 3), np.float32)
            w = np.zeros((n, 3), np.float32)
        self.api.check(self.api.world_get_body_state(self.handle, 0, n, _ptr(p, C.c_float), _ptr(q, C.c_float),
                                                     _ptr(v, C.c_float), _ptr(w, C.c_float)))
        return p, q, v, w

    def set_state(self, position=None, orientation=None, velocity=None, angular_velocity=None):
        n = self.n_bodies

        def arr(a, k):
            return None if a is None else np.ascontiguousarray(np.asarray(a, np.float32).reshape(n, k))

        p, q, v, w = arr(position, 3), arr(orientation, 4), arr(velocity, 3), arr(angular_velocity, 3)
        self.api.check(self.api.world_set_body_state(self.handle, 0, n, _ptr(p, C.c_float), _ptr(q, C.c_float),
                                                     _ptr(v, C.c_float), _ptr(w, C.c_float)))

    def pick(self, origins, dirs, mask=0xFFFFFFFF):
        """Solver::pick for each ray: (body creation indices, -1 = no hit; hit points in body frames)."""
        o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        dvec = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = o.shape[0]
        body = np.zeros(n, np.int32)
        local = np.zeros((n, 3), np.float32)
        self.api.check(self.api.world_pick(self.handle, n, _ptr(o, C.c_float), _ptr(dvec, C.c_float), int(mask),
                                           _ptr(body, C.c_int32), _ptr(local, C.c_float)))
        return body, local

    def collect_aabb(self, lo, hi, mask=0xFFFFFFFF):
        """Solver::collectAABB: creation indices of bodies overlapping [lo, hi], in list order."""
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        out = np.zeros(max(self.n_bodies, 1), np.int32)
        cnt = C.c_int()
        self.api.check(self.api.world_collect_aabb(self.handle, _ptr(lo, C.c_float), _ptr(hi, C.c_float), int(mask),
                                                   len(out), _ptr(out, C.c_int32), C.byref(cnt)))
        return out[:min(cnt.value, len(out))].copy()

    def sleeping(self):
        out = np.zeros(self.n_bodies, np.uint8)
        self.api.check(self.api.world_get_sleeping(self.handle, 0, self.n_bodies, _ptr(out, C.c_uint8)))
        return out

    def stats(self):
        s = Stats()
        self.api.check(self.api.world_get_stats(self.handle, C.byref(s)))
        return s

    def set_profiling(self, on=True):
        fn = getattr(self.api.lib, self.api.prefix + "world_set_profiling")
        fn.argtypes = [C.c_void_p, C.c_int]
        self.api.check(fn(self.handle, 1 if on else 0))

    def set_wait_limit(self, spins):
        """Bound of the device's dataflow waits (GPU library only): 0 gives up at the first
        unfinished predecessor, a negative value restores the default."""
        fn = getattr(self.api.lib, self.api.prefix + "world_set_wait_limit")
        fn.argtypes = [C.c_void_p, C.c_longlong]
        self.api.check(fn(self.handle, int(spins)))

    def take_kernel_times(self):
        fn = getattr(self.api.lib, self.api.prefix + "world_take_kernel_times")
        fn.argtypes = [C.c_void_p, C.POINTER(KernelTimes)]
        t = KernelTimes()
        self.api.check(fn(self.handle, C.byref(t)))
        return t

    def digest(self):
        out = C.c_uint64()
        self.api.check(self.api.world_digest(self.handle, C.byref(out)))
        return out.value

    def broadphase(self):
        nb, np_ = C.c_int(), C.c_int()
        self.api.check(self.api.world_dump_broadphase(self.handle, None, None, 0, None, 0, C.byref(nb),
                                                      C.byref(np_)))
        codes = np.zeros(nb.value, np.uint64)
        order = np.zeros(nb.value, np.int32)
        pairs = np.zeros(np_.value, np.uint64)
        self.api.check(self.api.world_dump_broadphase(self.handle, _ptr(codes, C.c_uint64), _ptr(order, C.c_int32),
                                                      nb.value, _ptr(pairs, C.c_uint64), np_.value,
                                                      C.byref(nb), C.byref(np_)))
        return codes, order, pairs

    def manifolds(self):
        cnt = C.c_int()
        self.api.check(self.api.world_dump_manifolds(self.handle, 0, None, None, None, None, None, None, None,
                                                     None, C.byref(cnt)))
        m = cnt.value
        out = {
            "body_a": np.zeros(m, np.int32),
            "body_b": np.zeros(m, np.int32),
            "count": np.zeros(m, np.int32),
            "features": np.zeros((m, 8), np.int32),
            "basis": np.zeros((m, 3, 3), np.float32),
            "c0": np.zeros((m, 8, 3), np.float32),
            "penalty": np.zeros((m, 8, 3), np.float32),
            "lambda": np.zeros((m, 8, 3), np.float32),
        }
        self.api.check(self.api.world_dump_manifolds(
            self.handle, m, _ptr(out["body_a"], C.c_int32), _ptr(out["body_b"], C.c_int32),
            _ptr(out["count"], C.c_int32), _ptr(out["features"], C.c_int32), _ptr(out["basis"], C.c_float),
            _ptr(out["c0"], C.c_float), _ptr(out["penalty"], C.c_float), _ptr(out["lambda"], C.c_float),
            C.byref(cnt)))
        return out

    def colours(self):
        cnt = C.c_int()
        self.api.check(self.api.world_dump_colours(self.handle, 0, None, None, C.byref(cnt)))
        col = np.zeros(cnt.value, np.uint8)
        ids = np.zeros(cnt.value, np.int32)
        self.api.check(self.api.world_dump_colours(self.handle, cnt.value, _ptr(col, C.c_uint8),
                                                   _ptr(ids, C.c_int32), C.byref(cnt)))
        return col, ids


def make_force_descs(joints):
    """Pack scene force records (ball-joint tuples (a, b, rA, rB, kLin, kAng, fracture), or
    ("spring", a, b, rA, rB, k, rest), ("generic", a, b, rA, rB, axes), ("ignore", a, b)) into an
    avbdg_force_desc array, creation order kept."""
    descs = (ForceDesc * max(len(joints), 1))()
    for i, force in enumerate(joints):
        d = descs[i]
        if force[0] == "spring":
            _, a, b, ra, rb, k, rest = force
            d.kind, d.stiffness_lin, d.rest = 2, float(k), float(rest)
        elif force[0] == "generic":
            _, a, b, ra, rb, axes = force
            d.kind = 3
            d.axes[:] = list(make_axes(axes))
        elif force[0] == "ignore":
            _, a, b = force
            ra = rb = (0.0, 0.0, 0.0)
            d.kind = 1
        else:
            a, b, ra, rb, kl, ka, fr = force
            d.kind = 0
            d.stiffness_lin, d.stiffness_ang, d.fracture = float(kl), float(ka), float(fr)
        d.body_a, d.body_b = int(a), int(b)
        d.r_a[:] = list(ra)
        d.r_b[:] = list(rb)
    return descs


class Batch:
    """Many independent worlds stepped together (avbdg_batch_*, GPU library only)."""

    def __init__(self, lib, params=None, max_worlds=0, max_bodies=0, max_forces=0):
        self.lib = lib
        self._api = Api(lib, "avbdg_")
        p = self._api.default_params() if params is None else params
        sig = {
            "batch_create": ([C.POINTER(Params), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
            "batch_destroy": ([C.c_void_p]),
            "batch_add_world": ([C.c_void_p, C.c_int, C.POINTER(BodyDesc), C.c_int, C.POINTER(ForceDesc),
                                 C.POINTER(C.c_int)]),
            "batch_remove_worlds": ([C.c_void_p, C.c_int, _ip]),
            "batch_step": ([C.c_void_p, C.c_int]),
            "batch_sync": ([C.c_void_p]),
            "batch_get_body_state": ([C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _fp]),
            "batch_set_body_state": ([C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp, _fp, _fp]),
            "batch_digest": ([C.c_void_p, C.c_int, _up]),
            "batch_get_stats": ([C.c_void_p, C.POINTER(Stats)]),
        }
        self.fn = {}
        for name, argtypes in sig.items():
            f = getattr(lib, "avbdg_" + name)
            f.argtypes = argtypes
            f.restype = C.c_int
            self.fn[name] = f
        h = C.c_void_p()
        self._api.check(self.fn["batch_create"](C.byref(p), int(max_worlds), int(max_bodies), int(max_forces),
                                                C.byref(h)))
        self.handle = h
        self.sizes = []

    def close(self):
        if self.handle:
            self.fn["batch_destroy"](self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene):
        descs = scene_body_descs(scene)
        forces = make_force_descs(scene.joints)
        out = C.c_int()
        self._api.check(self.fn["batch_add_world"](self.handle, scene.n, descs, len(scene.joints), forces,
                                                   C.byref(out)))
        self.sizes.append(scene.n)
        return out.value

    def remove_worlds(self, worlds):
        ids = np.asarray(sorted(set(int(w) for w in worlds)), np.int32)
        self._api.check(self.fn["batch_remove_worlds"](self.handle, len(ids), _ptr(ids, C.c_int32)))
        drop = set(ids.tolist())
        self.sizes = [n for i, n in enumerate(self.sizes) if i not in drop]

    def step(self, n=1):
        self._api.check(self.fn["batch_step"](self.handle, int(n)))

    def sync(self):
        self._api.check(self.fn["batch_sync"](self.handle))

    def state(self, world):
        n = self.sizes[world]
        p = np.zeros((n, 3), np.float32)
        q = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 3), np.float32)
        w = np.zeros((n, 3), np.float32)
        self._api.check(self.fn["batch_get_body_state"](self.handle, world, 0, n, _ptr(p, C.c_float),
                                                        _ptr(q, C.c_float), _ptr(v, C.c_float),
                                                        _ptr(w, C.c_float)))
        return p, q, v, w

    def digest(self, world):
        out = C.c_uint64()
        self._api.check(self.fn["batch_digest"](self.handle, world, C.byref(out)))
        return out.value

    def state_all(self, out=None):
        """All bodies of all worlds in world order, one device-to-host copy."""
        n = sum(self.sizes)
        p, q, v, w = out if out is not None else (np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32),
                                                  np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32))
        self._api.check(self.fn["batch_get_body_state"](self.handle, -1, 0, n, _ptr(p, C.c_float),
                                                        _ptr(q, C.c_float), _ptr(v, C.c_float),
                                                        _ptr(w, C.c_float)))
        return p, q, v, w

    def set_state_all(self, position=None, orientation=None, velocity=None, angular_velocity=None):
        n = sum(self.sizes)
        self._api.check(self.fn["batch_set_body_state"](self.handle, -1, 0, n, _ptr(position, C.c_float),
                                                        _ptr(orientation, C.c_float), _ptr(velocity, C.c_float),
                                                        _ptr(angular_velocity, C.c_float)))

    def set_profiling(self, on=True):
        fn = self.lib.avbdg_batch_set_profiling
        fn.argtypes = [C.c_void_p, C.c_int]
        self._api.check(fn(self.handle, 1 if on else 0))

    def take_kernel_times(self):
        fn = self.lib.avbdg_batch_take_kernel_times
        fn.argtypes = [C.c_void_p, C.POINTER(KernelTimes)]
        t = KernelTimes()
        self._api.check(fn(self.handle, C.byref(t)))
        return t

    def stats(self):
        s = Stats()
        self._api.check(self.fn["batch_get_stats"](self.handle, C.byref(s)))
        return s


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64), ("evicted", C.c_int64),
        ("ticks", C.c_int64),
        ("queued", C.c_int), ("resident", C.c_int), ("resident_bodies", C.c_int), ("resident_dynamic", C.c_int),
        ("resident_bytes", C.c_uint64), ("store_bytes", C.c_uint64), ("budget_bytes", C.c_uint64),
        ("body_steps", C.c_double), ("busy_ms", C.c_double),
        ("tick_p50_ms", C.c_double), ("tick_p99_ms", C.c_double), ("tick_max_ms", C.c_double),
        ("request_p50_ms", C.c_double), ("request_p99_ms", C.c_double),
        ("admit_ms", C.c_double), ("step_ms", C.c_double), ("retire_ms", C.c_double), ("graph_ticks", C.c_int64),
    ]


class Server:
    """Served form (avbdg_server_*): scenes queued as requests, admitted under a device byte budget,
    resident between ticks, all stepped together once per tick, retired when their steps are done."""

    def __init__(self, lib, params=None, budget_bytes=120 * 10**9, max_resident=4096):
        self.lib = lib
        self._api = Api(lib, "avbdg_")
        p = self._api.default_params() if params is None else params
        sig = {
            "server_create": [C.POINTER(Params), C.c_uint64, C.c_int, C.POINTER(C.c_void_p)],
            "server_destroy": [C.c_void_p],
            "server_admit": [C.c_void_p, C.c_int, C.POINTER(BodyDesc), C.c_int, C.POINTER(ForceDesc), C.c_int,
                             C.POINTER(C.c_int64)],
            "server_tick": [C.c_void_p, C.POINTER(C.c_int)],
            "server_poll": [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int)],
            "server_take_result": [C.c_void_p, C.c_int64, C.c_int, _fp, _fp, _fp, _fp],
            "server_evict": [C.c_void_p, C.c_int64],
            "server_get_stats": [C.c_void_p, C.POINTER(ServerStats)],
            "server_reset_stats": [C.c_void_p],
        }
        self.fn = {}
        for name, argtypes in sig.items():
            f = getattr(lib, "avbdg_" + name)
            f.argtypes = argtypes
            f.restype = C.c_int
            self.fn[name] = f
        h = C.c_void_p()
        self._api.check(self.fn["server_create"](C.byref(p), int(budget_bytes), int(max_resident), C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.fn["server_destroy"](self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, scene, steps, descs=None, forces=None):
        """Queue `scene` for `steps` steps; returns the request id. Pre-packed descriptor arrays
        (make_body_descs / make_force_descs) may be passed to keep packing out of a timed loop."""
        if descs is None:
            descs = scene_body_descs(scene)
        if forces is None:
            forces = make_force_descs(scene.joints)
        out = C.c_int64()
        self._api.check(self.fn["server_admit"](self.handle, scene.n, descs, len(scene.joints), forces, int(steps),
                                                C.byref(out)))
        return out.value

    def tick(self):
        done = C.c_int()
        self._api.check(self.fn["server_tick"](self.handle, C.byref(done)))
        return done.value

    def poll(self):
        rid, n = C.c_int64(), C.c_int()
        self._api.check(self.fn["server_poll"](self.handle, C.byref(rid), C.byref(n)))
        return rid.value, n.value

    def take_result(self, request, n):
        p = np.zeros((n, 3), np.float32)
        q = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 3), np.float32)
        w = np.zeros((n, 3), np.float32)
        self._api.check(self.fn["server_take_result"](self.handle, int(request), n, _ptr(p, C.c_float),
                                                      _ptr(q, C.c_float), _ptr(v, C.c_float), _ptr(w, C.c_float)))
        return p, q, v, w

    def results(self):
        """Take every finished result: {request id: (position, orientation, velocity, angular)}."""
        out = {}
        while True:
            rid, n = self.poll()
            if rid < 0:
                return out
            out[rid] = self.take_result(rid, n)

    def evict(self, request):
        self._api.check(self.fn["server_evict"](self.handle, int(request)))

    def stats(self):
        s = ServerStats()
        self._api.check(self.fn["server_get_stats"](self.handle, C.byref(s)))
        return s

    def reset_stats(self):
        self._api.check(self.fn["server_reset_stats"](self.handle))
