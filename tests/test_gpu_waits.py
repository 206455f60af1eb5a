"""Bounded device waits: the greedy colouring and the speculative brake sweep run as dataflows in
which a body (or brake candidate) waits for its predecessors. Each wait is bounded; one that runs
out stops its kernel and the step returns AVBDG_ERR_TIMEOUT. These tests lower the bound so that
the waits run out (no GPU fault is involved: the waiting threads give up and return), then check
that the status reaches the caller, that nothing is left running on the device, and that the
context still steps a fresh world bit for bit as the reference does.

The reference runs both sweeps serially (solver_solve.cpp:365-424, solver_projection.cpp:96-167),
so it has no wait to bound.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def approaching_column(pkg, boxes=16):
    """A column of unit cubes 2 cm apart, each falling 3 m/s faster than the one below it: every
    neighbouring pair is an approaching speculative contact, so each brake candidate waits on the
    one below it (a dependency chain through every body of the column)."""
    capi = pkg.capi
    size = [[40, 40, 1]] + [[1, 1, 1]] * boxes
    density = [0.0] + [1.0] * boxes
    friction = [0.5] * (boxes + 1)
    position = [[0, 0, -0.5]] + [[0, 0, 0.52 + 1.02 * i] for i in range(boxes)]
    velocity = [[0, 0, 0]] + [[0, 0, -3.0 * i] for i in range(boxes)]
    return capi.make_body_descs(size, density, friction, position, velocity=velocity)


def check_context_usable(pkg, gpu):
    """A fresh world on the same device reproduces the reference's pinned digest."""
    scenes = pkg.scenes
    sc = scenes.mixed()
    w = scenes.instantiate(gpu, sc)
    scenes.advance(w, sc)
    assert w.digest() == scenes.PINNED_DIGESTS["mixed"]


def step_until_timeout(w, steps=5):
    """Steps until one fails; returns the exception (None if every step succeeded)."""
    for _ in range(steps):
        try:
            w.step()
        except RuntimeError as e:  # capi.AvbdError
            return e
    return None


def test_colouring_wait_runs_out(pkg, gpu):
    """A hard ball-jointed chain: its links are coloured greedily, each waiting for the colour of
    the link before it. With a bound of zero spins the first such wait gives up."""
    capi, scenes = pkg.capi, pkg.scenes
    sc = scenes.hard_chain(links=12)
    w = scenes.instantiate(gpu, sc)
    w.set_wait_limit(0)
    err = step_until_timeout(w)
    assert isinstance(err, capi.AvbdError), "no colouring wait ran out"
    assert err.code == capi.ERR_TIMEOUT and "colouring" in str(err)
    w.sync()  # nothing of the failed step is still running
    w.set_wait_limit(-1)  # the default bound: the world steps again
    w.step()
    pos, quat, vel, ang = w.state()
    assert np.all(np.isfinite(pos)) and np.all(np.isfinite(quat))
    check_context_usable(pkg, gpu)


def test_brake_wait_runs_out(pkg, gpu):
    """The approaching column: each brake candidate waits for the candidate below it."""
    capi = pkg.capi
    w = capi.World(gpu)
    w.add_bodies(approaching_column(pkg))
    w.set_wait_limit(0)
    err = step_until_timeout(w)
    assert isinstance(err, capi.AvbdError), "no brake wait ran out"
    assert err.code == capi.ERR_TIMEOUT and "brake" in str(err)
    w.sync()
    w.set_wait_limit(-1)
    w.step()
    check_context_usable(pkg, gpu)


def test_default_bound_never_reached(pkg, gpu, oracle):
    """With the default bound the same two scenes step without a timeout and equal the oracle."""
    capi, scenes = pkg.capi, pkg.scenes
    a = capi.World(gpu)
    b = capi.World(oracle)
    d = approaching_column(pkg)
    a.add_bodies(d)
    b.add_bodies(d)
    sc = scenes.hard_chain(links=12)
    c = scenes.instantiate(gpu, sc)
    e = scenes.instantiate(oracle, sc)
    for _ in range(30):
        a.step()
        b.step()
        c.step()
        e.step()
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    for x, y in zip(c.state(), e.state()):
        assert np.array_equal(x, y)
