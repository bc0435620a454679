"""Batched scenes: many independent scenes in one system, every stage one
launch over all of them.  Each scene of a batch must give the result it
gives alone (same kernels, its own parameters, iteration count and dt
clamp), and the batch must keep scenes apart (no cross-scene neighbours,
constraints or bodies)."""
import numpy as np
import pytest

from helpers import check_granular, check_trajectory
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def mixed_batch():
    """Scenes of every kind with different sizes, iteration counts (3, 4,
    5), dt clamps, grids and 2-D / 3-D flags."""
    return [
        W.pbf_block(1500, seed=1),
        W.granular_column(900, seed=2),
        W.rope_and_cloth(),
        W.pbf_block(3100, seed=3, iterations=3, xsph=0.0),
        W.rigid_boxes(count=5),
        W.granular_column(400, width=10, seed=4, iterations=4),
        W.pbf_block(700, seed=5, cell_div=2),
        W.mixed_scene(cloth=12, ropes=4, rope_particles=8, bodies=6, rope_lift=0.6, body_lift=1.6),
    ]


def load_batch(scenes):
    total = sum(sc.n for sc in scenes)
    sys = ParticleSystem(default_params(**scenes[0].params), total)
    firsts = []
    for k, sc in enumerate(scenes):
        if k:
            assert sys.begin_scene(default_params(**sc.params)) == k
        first = sys.num_particles
        firsts.append(first)
        shifted = W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, vel=sc.vel, rest_density=sc.rest_density,
                          pairs=None if sc.pairs is None else sc.pairs + first, rest=sc.rest,
                          stiffness=sc.stiffness, pins=None if sc.pins is None else sc.pins + first,
                          pin_points=sc.pin_points, bodies=[(f + first, c, s) for f, c, s in sc.bodies],
                          open_gas=[(f + first, c) for f, c in sc.open_gas], sdf=sc.sdf)
        W.apply_to(shifted, sys)
    return sys, firsts


def load_alone(sc):
    sys = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, sys)
    return sys


def assert_same_state(a, b, what):
    """Equal up to 2 FP32 ulps of the coordinate (the batched and the
    single-scene instantiations of a kernel may contract differently)."""
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    ulp = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32)).astype(np.float64)
    err = np.abs(a - b) / ulp
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err[worst] <= 2.0, f"{what}: {err[worst]:.1f} ulp at {worst} ({a[worst]} vs {b[worst]})"


def test_scene_table_bookkeeping():
    scenes = mixed_batch()
    sys, firsts = load_batch(scenes)
    assert sys.num_scenes == len(scenes)
    for k, sc in enumerate(scenes):
        first, count, p = sys.scene(k)
        assert (first, count) == (firsts[k], sc.n)
        assert p.iterations == sc.params["iterations"]
    cells = sum(int(np.prod(sc.params["grid_size"])) for sc in scenes)
    assert sys.num_cells == cells


def test_batch_rejects_cross_scene_links():
    a, b = W.granular_column(100, seed=7), W.granular_column(100, seed=8)
    sys, firsts = load_batch([a, b])
    with pytest.raises(PbdError):
        sys.add_distance_constraints([[firsts[0], firsts[1]]], [0.5])
    with pytest.raises(PbdError):
        sys.add_rigid_body(firsts[1] - 4, 8)
    sys.add_distance_constraints([[firsts[1], firsts[1] + 1]], [0.5])  # inside one scene: fine


def test_batch_one_step_equals_each_scene_alone():
    scenes = mixed_batch()
    batch, firsts = load_batch(scenes)
    batch.update(1.0 / 60.0)
    pos, vel = batch.positions(), batch.velocities()
    for k, sc in enumerate(scenes):
        alone = load_alone(sc)
        alone.update(1.0 / 60.0)
        sl = slice(firsts[k], firsts[k] + sc.n)
        assert_same_state(pos[sl], alone.positions(), f"scene {k} ({sc.name}) positions")
        assert_same_state(vel[sl], alone.velocities(), f"scene {k} ({sc.name}) velocities")


def test_batch_with_long_neighbour_rows():
    """A batch with a PBF block squeezed to 0.6 of its lattice spacing (rows
    of more than 32 candidates, more row chunks than the 12 a walk keeps in
    shared memory), a plain block and a granular column: each scene equals
    its solo run, and the batch's list path equals the batch's exact walk
    (no lists) bit for bit."""
    dense = W.pbf_block(3000, seed=21)
    dense.pos_w[:, :3] *= 0.6
    scenes = [dense, W.pbf_block(1500, seed=22), W.granular_column(400, seed=23)]
    a, firsts = load_batch(scenes)
    b, _ = load_batch(scenes)
    b.set_tuning(threads_per_particle=1, neighbor_list_capacity=0)
    for _ in range(2):
        a.update(1.0 / 60.0)
        b.update(1.0 / 60.0)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())
    pos = a.positions()
    for k, sc in enumerate(scenes):
        alone = load_alone(sc)
        for _ in range(2):
            alone.update(1.0 / 60.0)
        assert_same_state(pos[firsts[k]:firsts[k] + sc.n], alone.positions(), f"scene {k} ({sc.name}) positions")


def test_batch_trajectories_match_oracle():
    """Several steps: every scene of the batch against the FP64 oracle run
    on that scene alone, by invariants."""
    scenes = mixed_batch()
    batch, firsts = load_batch(scenes)
    for _ in range(5):
        batch.update(1.0 / 60.0)
    pos = batch.positions()
    for k, sc in enumerate(scenes):
        o = Oracle(default_params(**sc.params), sc.n)
        W.apply_to(sc, o)
        for _ in range(5):
            o.update(1.0 / 60.0)
        mine = pos[firsts[k]:firsts[k] + sc.n]
        if sc.name == "granular_column":  # contact-threshold chaos: invariants only
            check_granular(mine, o.positions(), 1e-3)
        else:
            check_trajectory(mine, o.positions(), sc.pos_w)


def test_batch_graph_replay_matches_eager_bitwise():
    scenes = mixed_batch()
    a, _ = load_batch(scenes)
    b, _ = load_batch(scenes)
    for _ in range(4):
        a.update(1.0 / 60.0)
    b.update_graph(1.0 / 60.0, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


def test_batch_scene_params_can_change():
    scenes = [W.granular_column(300, seed=11), W.pbf_block(800, seed=12)]
    batch, firsts = load_batch(scenes)
    p = default_params(**scenes[1].params)
    p.iterations = 2
    batch.set_scene_params(1, p)
    batch.update(1.0 / 60.0)
    sc = W.pbf_block(800, seed=12)
    sc.params["iterations"] = 2
    alone = load_alone(sc)
    alone.update(1.0 / 60.0)
    assert_same_state(batch.positions()[firsts[1]:], alone.positions(), "pbf block with 2 iterations")


def test_batch_with_skin_lists_matches_oracle():
    scenes = mixed_batch()
    batch, firsts = load_batch(scenes)
    batch.set_tuning(neighbor_skin=0.2, neighbor_list_capacity=128)
    for _ in range(5):
        batch.update(1.0 / 60.0)
    pos = batch.positions()
    for k, sc in enumerate(scenes):
        o = Oracle(default_params(**sc.params), sc.n)
        W.apply_to(sc, o)
        for _ in range(5):
            o.update(1.0 / 60.0)
        mine = pos[firsts[k]:firsts[k] + sc.n]
        if sc.name == "granular_column":
            check_granular(mine, o.positions(), 1e-3)
        else:
            check_trajectory(mine, o.positions(), sc.pos_w)
