"""The dual-number build of the oracle (the same C source compiled as C++
with `real` = (value, tangent)): its values equal the FP64 build's bit for
bit, and its tangents are the directional derivatives of the FP64 replay
(central differences agree, and tangents are linear in the seed).  These
tangents are the exact reference the GPU adjoint is checked against."""
import numpy as np
import pytest

from helpers import params_nolib
from oracle import Oracle, OracleDual
from particlesolver_gb300 import FLAG_DELTA_OVER_RHO0
from particlesolver_gb300 import workloads as W


def cloth():
    return W.cloth_ropes_grains(cloth=8, ropes=2, rope_particles=8, grains=12, drop=0.8, seed=5, stiffness_seed=9)


def fluid():
    sc = W.dam_break(8, 8, 6, xsph=0.01)
    sc.params["flags"] = sc.params["flags"] | FLAG_DELTA_OVER_RHO0
    return sc


def boxes():
    sc = W.rigid_boxes(count=3, stiffness=0.6)
    rng = np.random.default_rng(5)
    vel = np.zeros((sc.n, 4), np.float32)
    for f, cnt, _ in sc.bodies:
        w = rng.standard_normal(3) * 2.0
        r = sc.pos_w[f:f + cnt, :3] - sc.pos_w[f:f + cnt, :3].mean(0)
        vel[f:f + cnt, :3] = rng.standard_normal(3) + np.cross(w, r)
    sc.vel = vel
    return sc


SCENES = {"cloth_ropes_grains": (cloth, 8), "pbf_block": (fluid, 2), "rigid_boxes": (boxes, 3)}


def make(cls, sc, stiffness, x0, v0):
    o = cls(params_nolib(sc.params), sc.n)
    W.apply_to(W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, rest_density=sc.rest_density, pairs=sc.pairs,
                       rest=sc.rest, stiffness=stiffness, pins=sc.pins, pin_points=sc.pin_points,
                       bodies=sc.bodies), o)
    pos = sc.pos_w.astype(np.float64).copy()
    pos[:, :3] = x0
    vel = np.zeros((sc.n, 4))
    vel[:, :3] = v0
    o.set_positions(pos)
    o.set_velocities(vel)
    return o


def state(sc):
    s0 = None if sc.pairs is None else (sc.stiffness if sc.stiffness is not None
                                        else np.ones(len(sc.pairs))).astype(np.float64)
    v0 = np.zeros((sc.n, 3)) if sc.vel is None else sc.vel[:, :3].astype(np.float64)
    return s0, sc.pos_w[:, :3].astype(np.float64), v0


def direction(sc, s0, seed):
    rng = np.random.default_rng(seed)
    ds = None if s0 is None else rng.uniform(-1, 1, len(s0))
    return ds, rng.standard_normal((sc.n, 3)) * 0.1, rng.standard_normal((sc.n, 3))


def tangent(sc, s0, x0, v0, d, steps):
    o = make(OracleDual, sc, s0, x0, v0)
    o.seed_tangents(d[1], d[2], d[0])
    for _ in range(steps):
        o.update(sc.dt)
    return o, o.tangents()


@pytest.mark.parametrize("name", list(SCENES))
def test_dual_values_equal_fp64_build(name):
    build, steps = SCENES[name]
    sc = build()
    s0, x0, v0 = state(sc)
    o = make(Oracle, sc, s0, x0, v0)
    od, _ = tangent(sc, s0, x0, v0, direction(sc, s0, 1), steps)
    for _ in range(steps):
        o.update(sc.dt)
    np.testing.assert_array_equal(od.positions(), o.positions())
    np.testing.assert_array_equal(od.velocities(), o.velocities())


@pytest.mark.parametrize("name", list(SCENES))
def test_dual_tangent_matches_central_difference(name):
    build, steps = SCENES[name]
    sc = build()
    s0, x0, v0 = state(sc)
    d = direction(sc, s0, 2)
    _, (tx, tv) = tangent(sc, s0, x0, v0, d, steps)
    eps = 1e-7
    shift = lambda sgn: make(Oracle, sc, None if s0 is None else s0 + sgn * eps * d[0],  # noqa: E731
                             x0 + sgn * eps * d[1], v0 + sgn * eps * d[2])
    a, b = shift(1), shift(-1)
    for _ in range(steps):
        a.update(sc.dt)
        b.update(sc.dt)
    fx = (a.positions()[:, :3] - b.positions()[:, :3]) / (2 * eps)
    fv = (a.velocities()[:, :3] - b.velocities()[:, :3]) / (2 * eps)
    np.testing.assert_allclose(tx[:, :3], fx, atol=1e-5 * np.abs(fx).max())
    np.testing.assert_allclose(tv[:, :3], fv, atol=1e-5 * np.abs(fv).max())


def test_dual_tangent_is_linear_in_the_seed():
    sc = cloth()
    s0, x0, v0 = state(sc)
    d1, d2 = direction(sc, s0, 3), direction(sc, s0, 4)
    comb = tuple(2.0 * a - 0.5 * b for a, b in zip(d1, d2))
    t1 = tangent(sc, s0, x0, v0, d1, 6)[1][0]
    t2 = tangent(sc, s0, x0, v0, d2, 6)[1][0]
    t12 = tangent(sc, s0, x0, v0, comb, 6)[1][0]
    np.testing.assert_allclose(t12, 2.0 * t1 - 0.5 * t2, atol=1e-9 * np.abs(t12).max())
