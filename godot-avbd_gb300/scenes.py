"""Scene builders: the reference test suite's pinned scenes and the seeded synthetic workloads.

A scene is a plain description (creation-ordered body arrays, joints, solver overrides) that any
implementation of the world API can instantiate, so the GPU library and its checkers receive
bit-identical float32 inputs. Body creation order matters: the solver walks bodies in reverse
creation order, and that order reaches the arithmetic.

Pinned scenes restate the reference's test fixtures:
  stack        test/core_test.cpp:391-399   (10-box stack, defaults, digest stack_300)
  interleaved  test/core_test.cpp:404-414   (same stack, dt 1/120, stepInterleaved(2, 3))
  mixed        test/core_test.cpp:612-631   (30-link soft-jointed chain + 40 boxes, mixed_240)
Synthetic workloads (seeded, numpy PCG64) follow the benchmark configurations:
  pyramid420   two 20-row walls of unit cubes on a 100 x 1 x 100 ground
  pile         log-uniform box sizes and densities + a 32-link ball-jointed chain
  lattice      64 x 64 x 16 unit cubes with 5 cm gaps and 2 cm jitter on a 500 m ground
  batch        many independent small worlds (pyramids or piles), log-uniform sizes
"""

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32
INF = float("inf")


@dataclass
class Scene:
    name: str
    size: np.ndarray          # n x 3 full extents
    density: np.ndarray       # n
    friction: np.ndarray      # n
    position: np.ndarray      # n x 3
    orientation: np.ndarray   # n x 4 {x, y, z, w}
    velocity: np.ndarray      # n x 3
    # Forces in creation order: ball joints (a, b, rA, rB, kLin, kAng, fracture),
    # ("spring", a, b, rA, rB, k, rest), ("generic", a, b, rA, rB, six axis tuples)
    joints: list = field(default_factory=list)
    params: dict = field(default_factory=dict)   # solver field overrides
    steps: int = 0
    substeps: int = 0          # > 1: stepInterleaved(substeps, rounds)
    rounds: int = 0
    sleep_mode: np.ndarray = None  # n: Rigid::sleep_mode (None = 0, never sleep)
    shape: np.ndarray = None       # n: 0 box, 1 sphere (size.x = radius), 2 cylinder (size.x radius, .z height)

    @property
    def n(self):
        return int(self.size.shape[0])

    @property
    def dynamic(self):
        return int(np.count_nonzero(self.density > 0))


class _Builder:
    def __init__(self):
        self.size, self.density, self.friction, self.position, self.orientation = [], [], [], [], []
        self.velocity = []
        self.shapes = []
        self.joints = []

    def box(self, size, density, friction, position, orientation=(0, 0, 0, 1), velocity=(0, 0, 0), shape=0):
        self.shapes.append(int(shape))
        self.size.append(np.asarray(size, F32))
        self.density.append(F32(density))
        self.friction.append(F32(friction))
        self.position.append(np.asarray(position, F32))
        self.orientation.append(np.asarray(orientation, F32))
        self.velocity.append(np.asarray(velocity, F32))
        return len(self.size) - 1

    def joint(self, a, b, ra, rb, k_lin=INF, k_ang=0.0, fracture=INF):
        self.joints.append((a, b, tuple(float(x) for x in ra), tuple(float(x) for x in rb),
                            float(k_lin), float(k_ang), float(fracture)))

    def spring(self, a, b, ra, rb, stiffness, rest=-1.0):
        self.joints.append(("spring", a, b, tuple(float(x) for x in ra), tuple(float(x) for x in rb),
                            float(stiffness), float(rest)))

    def generic(self, a, b, ra, rb, axes):
        self.joints.append(("generic", a, b, tuple(float(x) for x in ra), tuple(float(x) for x in rb),
                            tuple(tuple(float(v) for v in ax) for ax in axes)))

    def sphere(self, radius, density, friction, position, velocity=(0, 0, 0)):
        return self.box((radius, radius, radius), density, friction, position, velocity=velocity, shape=1)

    def cylinder(self, radius, height, density, friction, position, orientation=(0, 0, 0, 1)):
        return self.box((radius, radius, height), density, friction, position, orientation, shape=2)

    def scene(self, name, **kw):
        n = len(self.size)
        if any(self.shapes):
            kw.setdefault("shape", np.asarray(self.shapes, np.int64))
        return Scene(
            name=name,
            size=np.array(self.size, F32).reshape(n, 3),
            density=np.array(self.density, F32).reshape(n),
            friction=np.array(self.friction, F32).reshape(n),
            position=np.array(self.position, F32).reshape(n, 3),
            orientation=np.array(self.orientation, F32).reshape(n, 4),
            velocity=np.array(self.velocity, F32).reshape(n, 3),
            joints=list(self.joints),
            **kw,
        )


def _f(x):
    return F32(x)


# ----------------------------------------------------------------------------------------------
# Pinned scenes of the reference test suite
# ----------------------------------------------------------------------------------------------

def stack(steps=300):
    """test/core_test.cpp:391-399: ground + 10 unit boxes at z = i * 1.5 + 1 (defaults)."""
    b = _Builder()
    b.box((100, 100, 1), 0.0, 0.5, (0, 0, 0))
    for i in range(10):
        b.box((1, 1, 1), 1.0, 0.5, (0, 0, _f(i) * _f(1.5) + _f(1.0)))
    return b.scene("stack", steps=steps)


def interleaved(steps=300):
    """test/core_test.cpp:404-414: the stack at dt = 1/120 with stepInterleaved(2, 3)."""
    s = stack(steps)
    s.name = "interleaved"
    s.params = {"dt": float(_f(1.0) / _f(120.0))}
    s.substeps, s.rounds = 2, 3
    return s


def mixed(steps=240):
    """test/core_test.cpp:612-631: 30-link chain (Joint 1000 / 250) + 40 free boxes."""
    b = _Builder()
    b.box((100, 100, 1), 0.0, 0.5, (0, 0, 0))
    prev = None
    for i in range(30):
        link = b.box((1, 1, 1), 1.0, 0.5, (0, 0, _f(20.0) - _f(i) * _f(1.5)))
        if prev is not None:
            b.joint(prev, link, (0, 0, -0.5), (0, 0, 0.5), 1000.0, 250.0)
        prev = link
    for i in range(40):
        b.box((1, 1, 1), 1.0, 0.5, (_f(5.0) + _f(i) * _f(1.2), 0, _f(3.0) + _f(i % 5)))
    return b.scene("mixed", steps=steps)


# Digests the reference suite pins for these scenes (tools/baseline/digests.txt:1-3).
PINNED_DIGESTS = {
    "stack": 0xFBAC4F08CB1C977C,
    "interleaved": 0xB03ADEB37742850A,
    "mixed": 0xFB3CA7A3162035C2,
}


def hard_chain(links=4, steps=300):
    """test/core_test.cpp:271-300: static anchor + hard ball-jointed chain."""
    b = _Builder()
    prev = b.box((1, 1, 1), 0.0, 0.5, (0, 0, 10))
    for i in range(links):
        link = b.box((1, 1, 1), 1.0, 0.5, (0, 0, _f(9.0) - _f(i)))
        b.joint(prev, link, (0, 0, -0.5), (0, 0, 0.5), INF, 0.0)
        prev = link
    return b.scene("hard_chain", steps=steps)


# Axis presets of a generic joint: (mode, lower, upper, spring stiffness, equilibrium, damping).
FREE = (0, 0.0, 0.0, 0.0, 0.0, 0.0)
LOCK = (1, 0.0, 0.0, 0.0, 0.0, 0.0)


def limited(lower, upper):
    return (2, lower, upper, 0.0, 0.0, 0.0)


def sprung(stiffness, equilibrium=0.0, damping=0.0):
    return (0, 0.0, 0.0, stiffness, equilibrium, damping)


def joint_zoo(steps=240):
    """Every force kind the step supports, each in its own corner of one ground: a hinged
    pendulum (GenericJoint, one free rotation), a vertical slider that falls to its limit, a
    sprung-and-damped swing, a bungee (sprung linear axis) under a world anchor, a hanging chain
    of Springs, a ball-jointed pair, an ignore pair resting inside each other, and free boxes
    dropped onto the pendulum and the slider."""
    b = _Builder()
    b.box((60, 60, 1), 0.0, 0.5, (0, 0, -0.5))
    # Hinge about x: a post, a 2 m arm pivoting at the post's top, released horizontally.
    post = b.box((0.4, 0.4, 6), 0.0, 0.5, (-10, 0, 3))
    arm = b.box((0.3, 2.0, 0.3), 2.0, 0.5, (-10, 1.2, 6.2))
    b.generic(post, arm, (0, 0.2, 3.2), (0, -1.0, 0), (LOCK, LOCK, LOCK, FREE, LOCK, LOCK))
    # Slider along z, limited to [-1.5, 0] below its start, everything else locked.
    rail = b.box((0.5, 0.5, 0.5), 0.0, 0.5, (-4, 0, 8))
    car = b.box((1, 1, 1), 1.0, 0.5, (-4, 0, 6))
    b.generic(rail, car, (0, 0, -2), (0, 0, 0), (LOCK, LOCK, limited(-1.5, 0.0), LOCK, LOCK, LOCK))
    # Swing with a sprung, damped rotation about y (equilibrium tilted) and a limited x rotation.
    pivot = b.box((0.4, 0.4, 0.4), 0.0, 0.5, (2, 0, 7))
    swing = b.box((0.5, 0.5, 2.0), 1.5, 0.5, (2, 0, 5.6))
    b.generic(pivot, swing, (0, 0, -0.2), (0, 0, 1.2),
              (LOCK, LOCK, LOCK, limited(-0.3, 0.3), sprung(40.0, 0.4, 3.0), LOCK))
    # Bungee: world-anchored, linear z sprung, x/y locked, rotations free.
    bob = b.box((0.6, 0.6, 0.6), 1.0, 0.5, (8, 0, 6))
    b.generic(-1, bob, (8, 0, 9), (0, 0, 0.3), (LOCK, LOCK, sprung(60.0, 2.7, 1.5), FREE, FREE, FREE))
    # Chain of Springs from a static hook, rest lengths from the creation pose, one explicit.
    hook = b.box((0.3, 0.3, 0.3), 0.0, 0.5, (14, 0, 10))
    prev = hook
    for i in range(4):
        link = b.box((0.4, 0.4, 0.4), 1.0, 0.5, (14, 0, _f(9.0) - _f(i) * _f(1.2)))
        b.spring(prev, link, (0, 0, -0.15), (0, 0, 0.2), 300.0, -1.0 if i else 0.9)
        prev = link
    # Ball-jointed pair and an ignore pair.
    a1 = b.box((1, 1, 1), 1.0, 0.5, (-16, 0, 3))
    a2 = b.box((1, 1, 1), 1.0, 0.5, (-16, 0, 4.2))
    b.joint(a1, a2, (0, 0, 0.6), (0, 0, -0.6), INF, 0.0)
    g1 = b.box((1, 1, 1), 1.0, 0.5, (16, -8, 0.5))
    g2 = b.box((0.6, 0.6, 0.6), 1.0, 0.5, (16, -8, 0.7))
    b.joints.append(("ignore", g1, g2))
    # Free boxes falling onto the pendulum arm and the slider car.
    for i in range(4):
        b.box((0.5, 0.5, 0.5), 1.0, 0.5, (_f(-10.0), _f(1.6), _f(8.0) + _f(i) * _f(0.8)))
    for i in range(3):
        b.box((0.6, 0.6, 0.6), 1.0, 0.5, (_f(-4.0), _f(0.0), _f(9.0) + _f(i) * _f(1.0)))
    return b.scene("joint_zoo", params=dict(BENCH_PARAMS), steps=steps)


def sleepers(steps=300, sleep_frames=30):
    """Idle sleep, islands and wake-ups: a pyramid wall and a hanging ball-jointed chain settle and
    fall asleep (sleep mode 1), a box released high above them wakes the wall on impact, a box
    that starts asleep (mode 2) floats until a falling box reaches it, and a never-sleeping
    stack (mode 0) keeps running beside them."""
    b = _Builder()
    modes = []

    def box(*args, mode=1, **kw):
        modes.append(mode)
        return b.box(*args, **kw)

    box((60, 60, 1), 0.0, 0.5, (0, 0, -0.5), mode=0)
    rows = 8
    for r in range(rows):
        cnt = rows - r
        for k in range(cnt):
            box((1, 1, 1), 1.0, 0.5, ((_f(k) - _f(cnt - 1) * _f(0.5)) * _f(1.01), 0.0, _f(0.5) + _f(r)))
    anchor = box((0.3, 0.3, 0.3), 0.0, 0.5, (8, 0, 8), mode=0)
    prev = anchor
    for i in range(5):
        link = box((0.3, 0.3, 1.0), 1.0, 0.5, (_f(8.0), 0.0, _f(7.35) - _f(i) * _f(1.0)))
        b.joint(prev, link, (0, 0, -0.15), (0, 0, 0.5), INF, 0.0)
        prev = link
    box((1.5, 1.5, 1.5), 2.0, 0.5, (0.3, 0.0, 40.0))               # falls onto the wall
    box((1, 1, 1), 1.0, 0.5, (-8, 0, 3.0), mode=2)                # starts asleep in the air
    box((0.8, 0.8, 0.8), 1.0, 0.5, (-8, 0.1, 12.0))              # lands on it later
    for i in range(3):                                            # never sleeps
        box((1, 1, 1), 1.0, 0.5, (-16, 0, _f(0.5) + _f(i)), mode=0)
    sc = b.scene("sleepers", params=dict(BENCH_PARAMS, sleep_frames=sleep_frames), steps=steps)
    sc.sleep_mode = np.asarray(modes, np.int64)
    return sc


def pile_grace(steps=240, count=250, chain_links=6, grace=4):
    """A smaller mass-ratio pile with contact grace: manifolds whose contacts vanish for up to
    `grace` ticks are parked with their state and revived by feature key when they touch again."""
    sc = pile(steps=steps, count=count, chain_links=chain_links)
    sc.name = "pile_grace"
    sc.params = dict(sc.params, contact_grace_ticks=grace)
    return sc


def arm_cache(steps=240, rebuild=0.05):
    """The mixed scene (a jointed chain on coloured Gauss-Seidel, free boxes on block Jacobi) with
    the drift-gated arm cache on (Solver::jacobianRebuildDistance, manifold.cpp:600-668)."""
    sc = mixed(steps=steps)
    sc.name = "arm_cache"
    sc.params = dict(BENCH_PARAMS, jacobian_rebuild_distance=rebuild)
    return sc


def arm_cache_pile(steps=120, rebuild=0.02):
    """A 300-box pile with jointed chains (colours and overflow in one world), arm cache on."""
    sc = pile(steps=steps, count=300, chain_links=8)
    sc.name = "arm_cache_pile"
    sc.params = dict(sc.params, jacobian_rebuild_distance=rebuild)
    return sc


def arm_cache_sleep(steps=300, rebuild=0.05):
    """The sleepers scene stepped with stepInterleaved(2, 5) and the arm cache on: frozen manifolds
    keep their captured arms while parked, and the per-substep rebase keeps the cache."""
    sc = sleepers(steps=steps)
    sc.name = "arm_cache_sleep"
    sc.params = dict(sc.params, jacobian_rebuild_distance=rebuild, dt=float(_f(1.0) / _f(120.0)))
    sc.substeps, sc.rounds = 2, 5
    return sc


def converge_pile(steps=120, threshold=1e-3):
    """The 300-box jointed pile with the convergence probe on (Solver::convergenceThreshold,
    solver_step.cpp:301-314)."""
    sc = pile(steps=steps, count=300, chain_links=8)
    sc.name = "converge_pile"
    sc.params = dict(sc.params, convergence_threshold=threshold)
    return sc


def converge_interleaved(steps=300, threshold=1e-4):
    """The interleaved stack (stepInterleaved(2, 3)) with the convergence probe on."""
    sc = interleaved(steps=steps)
    sc.name = "converge_interleaved"
    sc.params = dict(sc.params, convergence_threshold=threshold)
    return sc


def shape_mix(steps=240):
    """Spheres and cylinders with boxes: a sphere pile, standing and lying cylinders, a cylinder
    stack, spheres rolling on a tilted box ramp and against cylinders, and boxes on cylinders."""
    b = _Builder()
    b.box((60, 60, 1), 0.0, 0.5, (0, 0, -0.5))
    ramp = (F32(0.0), F32(0.130526), F32(0.0), F32(0.991445))  # 15 degrees about y
    b.box((8, 3, 0.5), 0.0, 0.5, (-10, 0, 2.0), ramp)
    for i in range(4):
        b.sphere(0.4, 1.0, 0.5, (_f(-12.5) + _f(i) * _f(0.9), 0.0, _f(4.0) + _f(i) * _f(0.3)))
    for i in range(3):  # cylinder stack
        b.cylinder(0.6, 0.8, 1.0, 0.5, (0.0, 0.0, _f(0.4) + _f(i) * _f(0.85)))
    lying = (F32(0.707107), F32(0.0), F32(0.0), F32(0.707107))  # axis along y
    for i in range(3):  # lying cylinders
        b.cylinder(0.5, 2.0, 1.0, 0.5, (_f(4.0) + _f(i) * _f(1.2), 0.0, 0.5), lying)
    b.box((2.5, 1.0, 0.3), 1.0, 0.5, (5.2, 0.0, 1.3))  # a plank across them
    for i in range(9):  # sphere pile
        x, y = i % 3, i // 3
        b.sphere(0.35, 2.0, 0.5, (_f(10.0) + _f(x) * _f(0.75), _f(y) * _f(0.75), _f(0.4) + _f(i % 2) * _f(0.8)))
    for i in range(3):  # spheres and a box dropped on the stack
        b.sphere(0.3, 1.0, 0.5, (_f(0.1) * _f(i), 0.0, _f(4.0) + _f(i) * _f(0.8)))
    b.box((0.7, 0.7, 0.7), 1.0, 0.5, (0.2, 0.1, 6.5))
    b.cylinder(0.3, 1.0, 1.0, 0.5, (-3.0, 0.0, 3.0), (F32(0.258819), F32(0.0), F32(0.0), F32(0.965926)))
    return b.scene("shape_mix", params=dict(BENCH_PARAMS), steps=steps)


# ----------------------------------------------------------------------------------------------
# Synthetic workloads
# ----------------------------------------------------------------------------------------------

BENCH_PARAMS = {"gravity": -9.81, "iterations": 10, "dt": float(_f(1.0) / _f(60.0))}


def pyramid420(steps=300, rows=20, spacing=1.01):
    """Two parallel walls (y = -1.5 and +1.5) of `rows` rows (rows, rows-1, ..., 1 unit cubes,
    1 kg, friction 0.5) on a static 100 x 1 x 100 ground whose top face is z = 0."""
    b = _Builder()
    b.box((100, 100, 1), 0.0, 0.5, (0, 0, -0.5))
    for y in (-1.5, 1.5):
        for r in range(rows):
            count = rows - r
            for k in range(count):
                x = (_f(k) - _f(count - 1) * _f(0.5)) * _f(spacing)
                b.box((1, 1, 1), 1.0, 0.5, (x, y, _f(0.5) + _f(r)))
    return b.scene("pyramid420", params=dict(BENCH_PARAMS), steps=steps)


def pyramid_dbl(steps=600):
    """test/core_test.cpp:1915-1925 and :1948-1962 (`--pyramid`): a 20-row wall of 1 x 1 x 0.5 m
    boxes (density 2) on an 80 x 20 x 1 ground, and an identical wall 11.813 m above it that drops
    onto it; the solver settings of that diagnostic (dt 1/240 stepped as stepInterleaved(4, 2) per
    tick, 12 iterations, beta_lin 1e5, margin 0.02, arm cache 0.02, projection cap 0.1)."""
    b = _Builder()
    b.box((80, 20, 1), 0.0, 0.5, (0, 0, -0.5))
    for tier in range(2):
        for row in range(20):
            n = 20 - row
            z = _f(0.25) + _f(row) * _f(0.52) + _f(tier) * _f(11.813)
            for i in range(n):
                x = (_f(i) - _f(n - 1) * _f(0.5)) * _f(1.01)
                b.box((1, 1, 0.5), 2.0, 0.5, (x, 0.0, z))
    sc = b.scene("pyramid_dbl", steps=steps,
                 params={"gravity": -9.8, "dt": float(_f(1.0) / _f(240.0)), "iterations": 12,
                         "beta_lin": 100000.0, "speculative_margin": 0.02, "jacobian_rebuild_distance": 0.02,
                         "position_projection": 1, "projection_max_correction": 0.1, "contact_only_overflow": 1,
                         "sleep_frames": 30})
    sc.substeps, sc.rounds = 4, 2
    return sc


def _random_quats(rng, n):
    """Uniform random unit quaternions (Shoemake's method)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, c = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  c * np.sin(2 * np.pi * u3), c * np.cos(2 * np.pi * u3)], axis=1)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(F32)


def _place_pile(rng, b, count, lo, hi, edge_range=(0.25, 2.0), density_range=(100.0, 1e4), friction=0.5):
    """Boxes with log-uniform edges and densities, random orientations, placed without overlap by
    rejection against bounding spheres inside the box [lo, hi]."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    sizes = np.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1]), (count, 3)))
    dens = np.exp(rng.uniform(math.log(density_range[0]), math.log(density_range[1]), count))
    quats = _random_quats(rng, count)
    radii = 0.5 * np.linalg.norm(sizes, axis=1)
    # Uniform grid hash on the largest diameter for the overlap rejection.
    cell = 2.0 * radii.max()
    grid = {}
    centres = np.zeros((count, 3))
    for i in range(count):
        r = radii[i]
        for _ in range(10000):
            c = rng.uniform(lo + r, hi - r)
            key = tuple((c // cell).astype(int))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                            if np.sum((centres[j] - c) ** 2) < (radii[j] + r) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        else:
            raise RuntimeError("pile placement failed: volume too small")
        centres[i] = c
        grid.setdefault(key, []).append(i)
        b.box(sizes[i].astype(F32), dens[i], friction, centres[i].astype(F32), quats[i])


def pile(steps=600, count=1653, chain_links=32, seed=1):
    """Mass-ratio pile: `count` boxes (edges log-uniform 0.25-2 m per axis, densities log-uniform
    100-10^4 kg/m^3, uniform random orientations) placed without overlap in a 40 x 40 x 60 m volume
    above a static 200 x 1 x 200 ground (top face z = 0), plus a `chain_links`-link chain of
    0.2 x 0.2 x 1 m boxes hung by hard ball joints from a static anchor."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    b.box((200, 200, 1), 0.0, 0.5, (0, 0, -0.5))
    _place_pile(rng, b, count, (-20.0, -20.0, 1.0), (20.0, 20.0, 61.0))
    if chain_links > 0:
        prev = b.box((0.2, 0.2, 1.0), 0.0, 0.5, (26.0, 0.0, 45.0))
        for i in range(chain_links):
            link = b.box((0.2, 0.2, 1.0), 1000.0, 0.5, (26.0, 0.0, _f(44.0) - _f(i)))
            b.joint(prev, link, (0, 0, -0.5), (0, 0, 0.5), INF, 0.0)
            prev = link
    return b.scene("pile", params=dict(BENCH_PARAMS), steps=steps)


def lattice(steps=240, nx=64, ny=64, nz=16, pitch=1.05, jitter=0.02, seed=3):
    """Unit cubes (1 kg, friction 0.6) on an nx x ny x nz lattice with `pitch` spacing and uniform
    +/- `jitter` per coordinate, above a static 500 x 1 x 500 ground (top face z = 0)."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    b.box((500, 500, 1), 0.0, 0.6, (0, 0, -0.5))
    n = nx * ny * nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pos = np.stack([(ix.ravel() - (nx - 1) * 0.5) * pitch,
                    (iy.ravel() - (ny - 1) * 0.5) * pitch,
                    0.5 + (pitch - 1.0) + iz.ravel() * pitch], axis=1)
    pos += rng.uniform(-jitter, jitter, pos.shape)
    pos = pos.astype(F32)
    for i in range(n):
        b.box((1, 1, 1), 1.0, 0.6, pos[i])
    return b.scene("lattice", params=dict(BENCH_PARAMS), steps=steps)


def small_world(rng, n_target):
    """One world of the batched workload: a pyramid wall (rows 3-20) or a small pile, each with its
    own static ground, about `n_target` dynamic bodies."""
    b = _Builder()
    b.box((60, 60, 1), 0.0, 0.5, (0, 0, -0.5))
    if rng.random() < 0.5:
        # One pyramid wall of 3-20 rows, the row count closest to the drawn size.
        rows = int(min(20, max(3, round((math.sqrt(8 * n_target + 1) - 1) / 2))))
        for r in range(rows):
            cnt = rows - r
            for k in range(cnt):
                x = (_f(k) - _f(cnt - 1) * _f(0.5)) * _f(1.01)
                b.box((1, 1, 1), 1.0, 0.5, (x, 0.0, _f(0.5) + _f(r)))
    else:
        side = max(8.0, (n_target * 20.0) ** (1.0 / 3.0) * 1.5)
        _place_pile(rng, b, n_target, (-side / 2, -side / 2, 1.0), (side / 2, side / 2, 1.0 + side))
    return b.scene("world")


def batch(worlds=4096, n_min=8, n_max=512, seed=7, steps=120):
    """Independent worlds whose dynamic body counts are log-uniform in [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(worlds):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        w = small_world(rng, n)
        w.params = dict(BENCH_PARAMS)
        w.steps = steps
        out.append(w)
    return out


def _grid_pile(rng, b, count, z0=1.0, edge_range=(0.25, 2.0), density_range=(100.0, 1e4), friction=0.5):
    """A pile for large requests without the per-body rejection loop: the same size, density and
    orientation distributions as `_place_pile`, each box centred at a random point of its own cell
    of a cubic grid (cell = the largest bounding diameter), cells filled bottom-up, so no two
    bounding spheres overlap."""
    sizes = np.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1]), (count, 3)))
    dens = np.exp(rng.uniform(math.log(density_range[0]), math.log(density_range[1]), count))
    quats = _random_quats(rng, count)
    radii = 0.5 * np.linalg.norm(sizes, axis=1)
    cell = 2.0 * float(radii.max()) + 0.05
    side = max(2, int(math.ceil((count / 2.0) ** (1.0 / 3.0))))  # footprint side x side, ~2x as tall
    idx = np.arange(count)
    ij = np.stack([idx % side, (idx // side) % side, idx // (side * side)], axis=1).astype(np.float64)
    slack = (cell / 2.0 - radii)[:, None]
    centres = (ij + 0.5) * cell + rng.uniform(-1.0, 1.0, (count, 3)) * slack
    centres[:, 0] -= side * cell / 2.0
    centres[:, 1] -= side * cell / 2.0
    centres[:, 2] += z0
    for i in range(count):
        b.box(sizes[i].astype(F32), dens[i], friction, centres[i].astype(F32), quats[i])
    return side * cell


def request_world(rng, n_target, chain_links=8):
    """One request of the served stream, about `n_target` dynamic boxes: pyramid walls (3-20 rows,
    as many parallel walls as the size asks for) or a pile (sizes, densities and orientations as
    the mass-ratio pile) with a short ball-jointed chain, each on its own static ground."""
    b = _Builder()
    if rng.random() < 0.5:
        rows = int(rng.integers(3, 21))
        per_wall = rows * (rows + 1) // 2
        walls = max(1, int(round(n_target / per_wall)))
        extent = max(60.0, 1.6 * walls + 2.0 * rows)
        b.box((extent, extent, 1), 0.0, 0.5, (0, 0, -0.5))
        for wall in range(walls):
            y = (_f(wall) - _f(walls - 1) * _f(0.5)) * _f(1.6)
            for r in range(rows):
                cnt = rows - r
                for k in range(cnt):
                    x = (_f(k) - _f(cnt - 1) * _f(0.5)) * _f(1.01)
                    b.box((1, 1, 1), 1.0, 0.5, (x, y, _f(0.5) + _f(r)))
    else:
        count = max(1, n_target - chain_links)
        b.box((400, 400, 1), 0.0, 0.5, (0, 0, -0.5))
        width = _grid_pile(rng, b, count)
        if chain_links > 0:
            x0 = width / 2.0 + 4.0
            prev = b.box((0.2, 0.2, 1.0), 0.0, 0.5, (x0, 0.0, chain_links + 4.0))
            for i in range(chain_links):
                link = b.box((0.2, 0.2, 1.0), 1000.0, 0.5, (x0, 0.0, _f(chain_links + 3.0) - _f(i)))
                b.joint(prev, link, (0, 0, -0.5), (0, 0, 0.5), INF, 0.0)
                prev = link
    return b.scene("request")


def request_stream(requests=200, n_min=16, n_max=16384, steps_min=60, steps_max=600, seed=11):
    """Requests of the served workload: body counts log-uniform in [n_min, n_max], steps uniform in
    [steps_min, steps_max]; each scene carries its step count in `steps`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(requests):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        w = request_world(rng, n)
        w.params = dict(BENCH_PARAMS)
        w.steps = int(rng.integers(steps_min, steps_max + 1))
        out.append(w)
    return out


# ----------------------------------------------------------------------------------------------
# Instantiation
# ----------------------------------------------------------------------------------------------

def apply_params(p, overrides):
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def instantiate(api, scene, world_cls=None, params=None):
    """Create a world on `api` holding `scene` (solver overrides applied before any body, since
    bodies copy the solver's gravity at construction)."""
    from . import capi

    world_cls = world_cls or capi.World
    p = api.default_params() if params is None else params
    apply_params(p, scene.params)
    w = world_cls(api, p, max_bodies=scene.n, max_forces=len(scene.joints))
    descs = capi.scene_body_descs(scene)
    w.add_bodies(descs)
    for force in scene.joints:
        w.add_force(force)
    return w


def advance(world, scene, steps=None):
    """Advance `world` by `steps` ticks of the scene's stepping mode."""
    steps = scene.steps if steps is None else steps
    if scene.substeps > 1:
        for _ in range(steps):
            world.step_interleaved(scene.substeps, scene.rounds)
    elif steps > 0:
        world.step(steps)
