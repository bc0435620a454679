"""Parity at the benchmark configurations' full sizes, through the C ABI.

The other parity files check every stage on scenes the oracle replays in
well under a second.  Here the same checks run on the configurations the
benchmark measures, so the grid shape, the neighbour counts and the
wrapping of those configurations are covered too:

* the 1,048,576-particle dam break (128 x 128 x 64 lattice, grid
  256 x 64 x 32 cells of h): one iteration from the start and one from a
  state 40 steps into the flow -- grid, sorted indices and cell ranges
  bit-exact, lambda within 1e-5 (normalised max error) and the delta pass's
  correction within 1e-5 of the largest correction plus one FP32 ulp;
* the 833,536-particle mixed scene (256^2 cloth, 2,000 ropes, 10,000
  shape-matched boxes), 45 steps into the fall with its layers squeezed
  to 0.6 of their height (so that every projector moves particles far more
  than FP32 rounding of the coordinates): every projector of one
  iteration within the same 1e-5 bound;
* the 512-scene batch (7.9M particles): one batched step, 16 seeded scenes
  compared with their solo runs (2 FP32 ulp) and with the oracle.

The oracle runs on every host thread.
"""
import numpy as np
import pytest

from helpers import assert_projection, check_granular, check_trajectory, norm_err
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_STAGE = 1e-5


def make_pair(scene):
    p = default_params(**scene.params)
    g = ParticleSystem(p, scene.n)
    W.apply_to(scene, g)
    o = Oracle(p, scene.n)
    W.apply_to(scene, o)
    return g, o


def fluid_iteration(g, o):
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)
    before = g.positions()
    g.solve_fluids()
    o.solve_fluids()
    err = norm_err(g.lambdas(), o.lambdas())
    assert err < TOL_STAGE, err
    return assert_projection(g.positions(), o.positions(), before, TOL_STAGE)


@pytest.fixture(scope="module")
def dam_break_1m():
    return W.dam_break()


def test_dam_break_1m_first_iteration(dam_break_1m):
    sc = dam_break_1m
    assert sc.n == 1 << 20
    g, o = make_pair(sc)
    assert list(g.get_params().grid_size) == [256, 64, 32]
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    o.set_positions(g.positions().astype(np.float64))
    fluid_iteration(g, o)


def test_dam_break_1m_iteration_inside_the_flow(dam_break_1m):
    """40 full steps on the GPU, then the oracle takes the GPU's FP32
    positions and both run one more iteration's grid and PBF passes."""
    sc = dam_break_1m
    g, o = make_pair(sc)
    for _ in range(40):
        g.update(sc.dt)
    pos = g.positions()
    o.set_positions(pos.astype(np.float64))
    fluid_iteration(g, o)


def test_mixed_scene_full_size_stages():
    sc = W.mixed_scene()
    assert sc.n == 833536
    adv = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, adv)
    for _ in range(45):
        adv.update(sc.dt)
    pos = adv.positions()
    adv.close()
    # squeeze the layers together (as the small instance does) so that every
    # projector has corrections far above FP32 rounding of the coordinates
    pos[:, 1] = 10.0 + (pos[:, 1] - 10.0) * 0.6
    g, o = make_pair(sc)
    g.set_positions(pos)
    o.set_positions(pos.astype(np.float64))
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)
    moved = {}
    for stage in ("collide", "collide_world", "solve_distance_constraints", "solve_point_constraints",
                  "solve_shapes"):
        before = g.positions()
        getattr(g, stage)()
        getattr(o, stage)()
        moved[stage] = float(np.max(np.abs(o.positions()[:, :3] - before[:, :3])))
        try:
            assert_projection(g.positions(), o.positions(), before, TOL_STAGE)
        except AssertionError as e:
            raise AssertionError(f"{stage}: {e} (max corrections so far {moved})") from None
        o.set_positions(g.positions().astype(np.float64))
    # the state is one with contacts, stretched constraints and rotated bodies
    assert moved["collide"] > 1e-3 and moved["solve_distance_constraints"] > 1e-4 and moved["solve_shapes"] > 1e-4


def test_batch_512_scenes_one_step_sampled():
    scenes = W.batched_scenes(512)
    total = sum(sc.n for sc in scenes)
    batch = ParticleSystem(default_params(**scenes[0].params), total)
    firsts = []
    for k, sc in enumerate(scenes):
        if k:
            batch.begin_scene(default_params(**sc.params))
        firsts.append(batch.num_particles)
        W.apply_to(sc, batch)
    dt = 1.0 / 60.0
    batch.update(dt)
    pos, vel = batch.positions(), batch.velocities()
    batch.close()
    sample = np.random.default_rng(512).choice(len(scenes), 16, replace=False)
    for k in sorted(sample):
        sc = scenes[k]
        sl = slice(firsts[k], firsts[k] + sc.n)
        alone = ParticleSystem(default_params(**sc.params), sc.n)
        W.apply_to(sc, alone)
        alone.update(dt)
        for a, b, what in ((pos[sl], alone.positions(), "positions"), (vel[sl], alone.velocities(), "velocities")):
            a = np.asarray(a, np.float64)[:, :3]
            b = np.asarray(b, np.float64)[:, :3]
            ulp = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32)).astype(np.float64)
            assert np.max(np.abs(a - b) / ulp) <= 2.0, f"scene {k} ({sc.name}) {what}"
        alone.close()
        o = Oracle(default_params(**sc.params), sc.n)
        W.apply_to(sc, o)
        o.update(dt)
        if sc.name == "granular_column":
            check_granular(pos[sl], o.positions(), 1e-3)
        else:
            check_trajectory(pos[sl], o.positions(), sc.pos_w)
