"""Parity of the CUDA path (through the C ABI) with the oracle and with the
golden fixtures made from the reference's own kernels.

Tolerances (written per test): grids, sorted indices and cell ranges are
bit-exact; one projection of one iteration agrees with the FP64 oracle to
1e-5 as max_i |d_gpu - d_64| / max_i |d_64| over the displacement the stage
produces; several full steps are compared by invariants (90th percentile of
the per-particle error and the centre-of-mass motion).
"""
import numpy as np
import pytest

from helpers import (assert_projection, check_against_golden, check_trajectory, density_error, displacement,
                     golden_scene, norm_err, run_stages)
from conftest import GOLDEN
from oracle import Oracle
from particlesolver_gb300 import (FLAG_DELTA_OVER_RHO0, FLAG_DENSITY_NEIGHBOR_MASS, FLAG_DISTANCE_MASS_WEIGHTED,
                                  ParticleSystem, default_params)
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_STAGE = 1e-5


def make_pair(scene, **overrides):
    d = dict(scene.params)
    d.update(overrides)
    p = default_params(**d)
    g = ParticleSystem(p, scene.n)
    W.apply_to(scene, g)
    o = Oracle(p, scene.n)
    W.apply_to(scene, o)
    return g, o


def sync_positions(g, o):
    """Give the oracle the GPU's FP32 positions (so both sides start from
    identical inputs and the FP32 grid / neighbour decisions coincide)."""
    o.set_positions(g.positions().astype(np.float64))


# ---------------------------------------------------------------- grid

@pytest.mark.parametrize("builder", [W.reference_fluid, W.reference_granular, W.rope_and_cloth,
                                     lambda: W.dam_break(24, 20, 12)])
def test_grid_bit_exact(builder):
    sc = builder()
    g, o = make_pair(sc)
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)


def test_grid_wraps_and_aliases_like_reference():
    # particles far outside a tiny power-of-two grid alias into its cells
    sc = W.reference_fluid(ll=(-4, 0, -4), ur=(4, 4, 4), grid=(4, 8, 2))
    pos = sc.pos_w.copy()
    pos[::5, 0] += 37.0
    pos[::7, 2] -= 23.0
    sc.pos_w = pos
    g, o = make_pair(sc)
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE


def test_empty_and_single_particle():
    p = default_params()
    g = ParticleSystem(p, 4)
    g.update(1 / 60)  # no particles: a no-op
    g.add_particles(np.array([[1.0, 5.0, 2.0, 1.0]], np.float32), phase=[3])
    g.update(1 / 60)
    x = g.positions()
    assert np.isclose(x[0, 1], 5.0 - 9.8 / 60 / 60, atol=1e-5)


# ----------------------------------------------------------------- PBF

@pytest.mark.parametrize("flags", [0, FLAG_DENSITY_NEIGHBOR_MASS, FLAG_DELTA_OVER_RHO0,
                                   FLAG_DENSITY_NEIGHBOR_MASS | FLAG_DELTA_OVER_RHO0])
def test_pbf_lambda_and_delta_reference_constants(flags):
    a = W.reference_fluid(ll=(-4, 0, -3), ur=(4, 3, 3), density=2.0, mass=1.0, seed=1)
    b = W.reference_fluid(ll=(-4, 3, -3), ur=(4, 6, 3), density=3.0, mass=0.5, seed=2)
    sc = W.Scene("two", a.params, np.concatenate([a.pos_w, b.pos_w]), np.concatenate([a.phase, b.phase]),
                 rest_density=np.concatenate([a.rest_density, b.rest_density]))
    g, o = make_pair(sc, flags=flags)
    g.build_grid()
    o.build_grid()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)


def fluid_around_solid():
    """A fluid block with a solid column through it and solid grains
    below: fluid particles with solid neighbours."""
    a = W.reference_fluid(ll=(-4, 0, -3), ur=(4, 4, 3), density=2.0, mass=1.0, seed=3)
    inside = (np.abs(a.pos_w[:, 0]) < 1.0) & (np.abs(a.pos_w[:, 2]) < 1.0)
    phase = a.phase.copy()
    phase[inside] = W.PHASE_SOLID
    return W.Scene("fluid_solid", a.params, a.pos_w, phase, rest_density=a.rest_density)


@pytest.mark.parametrize("weight", [0.0, 0.5, 1.0])
def test_fluid_solid_coupling_weight(weight):
    """pbd_params.solid_density_weight: solid-like neighbours in a fluid
    particle's density and own gradient (0 = the CPU reference's S_SOLID,
    1 = the GPU reference)."""
    sc = fluid_around_solid()
    g, o = make_pair(sc, solid_density_weight=weight)
    g.build_grid()
    o.build_grid()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)


def test_fluid_solid_weight_changes_lambda():
    sc = fluid_around_solid()
    out = []
    for weight in (0.0, 1.0):
        g, _ = make_pair(sc, solid_density_weight=weight)
        g.build_grid()
        g.solve_fluids()
        out.append(g.lambdas())
    fluid = sc.phase == W.PHASE_FLUID
    assert np.max(np.abs(out[0][fluid] - out[1][fluid])) > 1e-3


@pytest.mark.parametrize("dims,cell_div", [((16, 16, 8), 1), ((40, 24, 20), 1), ((24, 20, 12), 2),
                                           ((20, 16, 12), 3)])
def test_pbf_dam_break_block_one_iteration(dims, cell_div):
    sc = W.dam_break(*dims, cell_div=cell_div)
    g, o = make_pair(sc)
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    sync_positions(g, o)
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)
    before = g.positions()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
    assert_projection(g.positions(), o.positions(), before, TOL_STAGE)


# ------------------------------------------------------------ contacts

def test_contacts_with_friction_and_mass_scaling():
    sc = W.reference_granular()
    vel = np.zeros((sc.n, 4), np.float32)
    vel[:, 0] = 0.3
    sc.vel = vel
    g, o = make_pair(sc)
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    sync_positions(g, o)
    g.build_grid()
    o.build_grid()
    before = g.positions()
    g.collide()
    o.collide()
    assert np.max(np.abs(displacement(o.positions(), before))) > 1e-4
    assert_projection(g.positions(), o.positions(), before, TOL_STAGE)


def test_contacts_between_objects_skip_same_object():
    sc = W.rope_and_cloth()
    g, o = make_pair(sc)
    g.build_grid()
    o.build_grid()
    g.collide()
    o.collide()
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)


# --------------------------------------------------------------- walls

@pytest.mark.parametrize("twod", [False, True])
def test_world_walls_with_jitter(twod):
    from particlesolver_gb300 import FLAG_TWOD

    sc = W.reference_granular(ll=(-3, 0, -3), ur=(3, 2, 3))
    g, o = make_pair(sc, flags=FLAG_TWOD if twod else 0, twod_z=0.5)
    jitter = [0.3, 0.7, 0.2, 0.9, 0.5, 0.1]
    g.set_wall_jitter(jitter)
    o.set_wall_jitter(jitter)
    pos = sc.pos_w.copy()
    pos[:, 0] += 0.01
    pos[:, 1] -= 0.4
    pos[::7, 0] = -50.3
    pos[::11, 2] = 50.6
    g.set_positions(pos)
    o.set_positions(pos.astype(np.float64))
    g.build_grid()
    o.build_grid()
    g.collide_world()
    o.collide_world()
    # clamps and wall friction: within one FP32 ulp of the stored coordinate
    xo = o.positions()[:, :3]
    ulp = np.spacing(np.abs(xo).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(g.positions()[:, :3] - xo) <= ulp)


# ---------------------------------------------------- distance / pins

@pytest.mark.parametrize("flags", [0, FLAG_DISTANCE_MASS_WEIGHTED])
def test_distance_constraints_and_pins(flags):
    sc = W.rope_and_cloth()
    sc.stiffness = W.uniform(99, (len(sc.rest),), 0.2, 1.0).astype(np.float32)
    g, o = make_pair(sc, flags=flags)
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    sync_positions(g, o)
    before = g.positions()
    g.solve_distance_constraints()
    o.solve_distance_constraints()
    assert np.max(np.abs(displacement(o.positions(), before))) > 1e-3
    assert_projection(g.positions(), o.positions(), before, TOL_STAGE)
    g.solve_point_constraints()
    o.solve_point_constraints()
    np.testing.assert_array_equal(g.positions()[sc.pins, :3], o.positions()[sc.pins, :3].astype(np.float32))


def test_distance_constraints_any_particle_order():
    """Constrained particles after unconstrained ones (the case the
    reference's segment indexing got wrong, solver.cu:227-230)."""
    fl = W.reference_fluid(ll=(-2, 0, -2), ur=(2, 2, 2))
    rc = W.rope_and_cloth(ropes=2, cloth=(5, 4))
    off = fl.n
    sc = W.Scene("mix", fl.params, np.concatenate([fl.pos_w, rc.pos_w]), np.concatenate([fl.phase, rc.phase]),
                 rest_density=np.concatenate([fl.rest_density, np.ones(rc.n, np.float32)]),
                 pairs=rc.pairs + off, rest=rc.rest, pins=rc.pins + off, pin_points=rc.pin_points)
    g, o = make_pair(sc)
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    sync_positions(g, o)
    before = g.positions()
    g.solve_distance_constraints()
    o.solve_distance_constraints()
    assert_projection(g.positions(), o.positions(), before, TOL_STAGE)


# -------------------------------------------------------- shape matching

def test_shape_matching_recovers_rotation():
    sc = W.rigid_boxes(count=6)
    g, o = make_pair(sc)
    noise = W.uniform(77, (sc.n, 3), -0.05, 0.05).astype(np.float32)
    pos = sc.pos_w.copy()
    pos[:, :3] += noise
    g.set_positions(pos)
    o.set_positions(pos.astype(np.float64))
    g.solve_shapes()
    o.solve_shapes()
    assert_projection(g.positions(), o.positions(), pos, TOL_STAGE)
    # a rigid motion of the rest shape (random rotations about each centre)
    # is a fixed point: the rotation extraction must find it from identity
    g2, _ = make_pair(sc)
    rot = sc.pos_w.astype(np.float64).copy()
    qs = W.random_quaternions(1234, len(sc.bodies))
    for b, (f, c, _) in enumerate(sc.bodies):
        com = rot[f:f + c, :3].mean(0)
        rot[f:f + c, :3] = W.quat_rotate(np.broadcast_to(qs[b], (c, 4)), rot[f:f + c, :3] - com) + com
    rot = rot.astype(np.float32)
    g2.set_positions(rot)
    g2.solve_shapes()
    assert np.max(np.abs(g2.positions()[:, :3] - rot[:, :3])) < 2e-5


# ----------------------------------------------------- velocity / XSPH

def test_velocity_and_xsph():
    sc = W.dam_break(16, 16, 8)
    g, o = make_pair(sc)
    g.update(sc.dt)
    o.set_positions(g.positions().astype(np.float64))
    o.set_velocities(g.velocities().astype(np.float64))
    # velocity from positions, then XSPH, from identical inputs
    g.build_grid()
    o.build_grid()
    g.apply_xsph()
    o.apply_xsph()
    assert norm_err(g.velocities()[:, :3], o.velocities()[:, :3]) < TOL_STAGE


# ---------------------------------------------------------- full steps

@pytest.mark.parametrize("builder,steps", [(W.reference_fluid, 4), (W.reference_granular, 4),
                                           (W.rope_and_cloth, 4), (lambda: W.rigid_boxes(count=8), 4),
                                           (lambda: W.dam_break(16, 16, 8), 6),
                                           (lambda: W.pbf_block(2000), 4)])
def test_full_update_trajectory(builder, steps):
    sc = builder()
    g, o = make_pair(sc)
    for _ in range(steps):
        g.update(sc.dt)
        o.update(sc.dt)
    check_trajectory(g.positions(), o.positions(), sc.pos_w)


def test_granular_column_collapse():
    """The 2-D granular column (1,600 particles, 40 x 40, spacing 2r, mu_s
    0.5, mu_k 0.3, 3 iterations, dt 1/60).  Its lattice sits at the contact
    threshold, so trajectories are chaotic: each step is checked from a
    common state (the oracle restarted from the GPU's positions and
    velocities), and 60 free-running steps by pile invariants."""
    from helpers import check_granular

    sc = W.granular_column()
    g, o = make_pair(sc)
    for step in range(12):
        o.set_positions(g.positions().astype(np.float64))
        o.set_velocities(g.velocities().astype(np.float64))
        start = g.positions()
        g.update(sc.dt)
        o.update(sc.dt)
        d_g, d_o = displacement(g.positions(), start), displacement(o.positions(), start)
        # per particle: 1e-4 of the step's largest move plus 4 FP32 ulps of
        # the coordinate; a minority may switch contacts at the threshold
        ulp = np.spacing(np.abs(o.positions()[:, :3]).astype(np.float32)).astype(np.float64).max(1)
        excess = np.linalg.norm(d_g - d_o, axis=1) - (1e-4 * np.max(np.abs(d_o)) + 4.0 * ulp)
        assert np.mean(excess > 0) < 0.1, (step, np.mean(excess > 0))
    g2, o2 = make_pair(sc)
    for _ in range(60):
        g2.update(sc.dt)
        o2.update(sc.dt)
    check_granular(g2.positions(), o2.positions(), 0.05)


def _small_mixed():
    return W.mixed_scene(cloth=24, ropes=12, rope_particles=16, bodies=24, rope_lift=0.55, layer_gap=0.55,
                         body_lift=1.4)


def test_mixed_scene_stages():
    """Cloth (stretch/shear/bend), ropes and shape-matched boxes pressed
    together: every projector of one iteration against the FP64 oracle."""
    sc = _small_mixed()
    g, o = make_pair(sc)
    pos = sc.pos_w.copy()
    pos[:, 1] = 10.0 + (pos[:, 1] - 10.0) * 0.6  # overlap rope and box layers
    g.set_positions(pos)
    o.set_positions(pos.astype(np.float64))
    g.build_grid()
    o.build_grid()
    for stage in ("collide", "collide_world", "solve_distance_constraints", "solve_point_constraints",
                  "solve_shapes"):
        before = g.positions()
        getattr(g, stage)()
        getattr(o, stage)()
        assert_projection(g.positions(), o.positions(), before, TOL_STAGE)
        sync_positions(g, o)


def test_mixed_scene_trajectory_invariants():
    """Ropes fall onto the pinned cloth and boxes onto the ropes: positions
    by invariants, plus the distance-constraint residual and the rigid
    bodies' RMS deviation from their rest shape, against the oracle."""
    sc = _small_mixed()
    g, o = make_pair(sc)
    for _ in range(12):
        g.update(sc.dt)
        o.update(sc.dt)
    pg, po = g.positions().astype(np.float64), o.positions()
    check_trajectory(pg, po, sc.pos_w)
    a, b = sc.pairs[:, 0], sc.pairs[:, 1]

    def residual(p):
        return np.abs(np.linalg.norm(p[a, :3] - p[b, :3], axis=1) - sc.rest)

    assert abs(residual(pg).mean() - residual(po).mean()) <= 1e-3 * sc.rest.mean()

    def rigid_rms(p):
        dev = []
        for f, c, _ in sc.bodies:
            x = p[f:f + c, :3] - p[f:f + c, :3].mean(0)
            r = sc.pos_w[f:f + c, :3].astype(np.float64)
            r = r - r.mean(0)
            u, _, vt = np.linalg.svd(x.T @ r)
            rot = u @ np.diag([1.0, 1.0, np.sign(np.linalg.det(u @ vt))]) @ vt
            dev.append(np.mean(np.sum((x - r @ rot.T) ** 2, 1)))
        return np.sqrt(np.mean(dev))

    assert abs(rigid_rms(pg) - rigid_rms(po)) <= 1e-3 * 2 * sc.params["particle_radius"]
    np.testing.assert_array_equal(g.positions()[sc.pins, :3], sc.pin_points)


def test_graph_replay_matches_eager_bitwise():
    sc = W.dam_break(16, 16, 8)
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    for _ in range(5):
        a.update(sc.dt)
    b.update_graph(sc.dt, 5)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


def test_deterministic_runs():
    sc = W.reference_granular()
    runs = []
    for _ in range(2):
        g = ParticleSystem(default_params(**sc.params), sc.n)
        W.apply_to(sc, g)
        for _ in range(5):
            g.update(sc.dt)
        runs.append(g.positions())
    np.testing.assert_array_equal(runs[0], runs[1])


def test_save_load_state_roundtrip():
    sc = W.rigid_boxes(count=3)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    g.update(sc.dt)
    blob = g.save_state()
    g.update(sc.dt)
    after = g.positions()
    g.load_state(blob)
    g.update(sc.dt)
    np.testing.assert_array_equal(g.positions(), after)


# --------------------------------------------- golden (reference) fixtures

FIXTURES = sorted(GOLDEN.glob("ref_*.npz"))


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_stages_match_reference_golden(path):
    data = np.load(path)
    sc = golden_scene(data)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    out = run_stages(g)
    check_against_golden(out, data, sc.pos_w)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_updates_match_reference_golden(path):
    data = np.load(path)
    sc = golden_scene(data)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    for k in range(3):
        g.update(sc.dt)
        check_trajectory(g.positions(), data[f"update{k + 1}_pos"], sc.pos_w)


# ------------------------------------------------------ launch shapes

@pytest.mark.parametrize("tpp", [1, 2, 4, 8, 16, 32])
def test_every_group_size_matches_oracle(tpp):
    sc = W.reference_granular(ll=(-2, 0, -2), ur=(2, 3, 2))
    fl = W.reference_fluid(ll=(-4, 0, 3), ur=(4, 4, 7))
    mix = W.Scene("mix", fl.params, np.concatenate([fl.pos_w, sc.pos_w]), np.concatenate([fl.phase, sc.phase]),
                  rest_density=np.concatenate([fl.rest_density, np.ones(sc.n, np.float32)]))
    g, o = make_pair(mix)
    g.set_threads_per_particle(tpp)
    assert g.threads_per_particle == tpp
    g.build_grid()
    o.build_grid()
    g.collide()
    o.collide()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
    assert_projection(g.positions(), o.positions(), mix.pos_w, TOL_STAGE)


def test_neighbor_cap_keeps_first_in_visiting_order():
    sc = W.reference_fluid(ll=(-2, 0, -2), ur=(2, 3, 2))
    for tpp in (1, 8):
        g, o = make_pair(sc, max_neighbors=7)
        g.set_threads_per_particle(tpp)
        g.build_grid()
        o.build_grid()
        g.solve_fluids()
        o.solve_fluids()
        assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
        assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)


def test_autotune_restores_state():
    sc = W.dam_break(16, 16, 8)
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    a.update(sc.dt)
    b.update(sc.dt)
    chosen = a.autotune(sc.dt, 2)
    assert chosen in (1, 2, 4, 8, 16, 32)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


def test_autotune_cell_size():
    """A fluid system may come out of the autotuner with cells of half the
    size (grid doubled per axis) or with its cells on half the grid; its
    step still matches the oracle on the given grid (neighbour sets do not
    depend on the grid).  A system with contacts keeps its cell size."""
    sc = W.dam_break(16, 16, 8)
    g, o = make_pair(sc)
    g.autotune(sc.dt, 2)
    p = g.get_params()
    given = sc.params["grid_size"]
    assert p.cell_size in (np.float32(sc.params["cell_size"]), np.float32(sc.params["cell_size"] / 2))
    div = round(sc.params["cell_size"] / p.cell_size)
    assert list(p.grid_size) in ([v * div for v in given], [v // 2 for v in given])
    g.update(sc.dt)
    o.update(sc.dt)
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)
    gc = W.granular_column(200, seed=3)
    c = ParticleSystem(default_params(**gc.params), gc.n)
    W.apply_to(gc, c)
    c.autotune(gc.dt, 2)
    assert c.get_params().cell_size == np.float32(gc.params["cell_size"])


def test_halved_grid_matches_the_oracle():
    """The same cells on half the grid per axis (what the autotuner may
    pick for a sparse scene): particles wrap onto it, the walks reject the
    far ones, and a step of a mixed rope/cloth/grain scene and of a dam
    break still matches the oracle on the given grid."""
    dam = W.dam_break(16, 16, 8)
    dam.params["grid_size"] = [64, 16, 16]
    for sc in (dam, W.rope_and_cloth()):
        g, o = make_pair(sc)
        p = default_params(**sc.params)
        for a in range(3):
            p.grid_size[a] = max(1, sc.params["grid_size"][a] // 2)
        g.set_params(p)
        before = g.positions()
        g.update(sc.dt)
        o.update(sc.dt)
        assert_projection(g.positions(), o.positions(), before, TOL_STAGE)


@pytest.mark.parametrize("capacity", [0, 4, 16, 64])
def test_neighbor_list_capacity_and_fallback(capacity):
    """Small list capacities force the exact stencil-walk fallback for some
    or all particles; every capacity gives the oracle's result."""
    sc = W.dam_break(20, 16, 12, cell_div=2)
    g, o = make_pair(sc)
    g.set_tuning(threads_per_particle=1, neighbor_list_capacity=capacity)
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    sync_positions(g, o)
    g.build_grid()
    o.build_grid()
    before = g.positions()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas(), o.lambdas()) < TOL_STAGE
    assert_projection(g.positions(), o.positions(), before, TOL_STAGE)
    g.calc_velocity(sc.dt)
    o.calc_velocity(sc.dt)
    g.apply_xsph()
    o.apply_xsph()
    assert norm_err(g.velocities()[:, :3], o.velocities()[:, :3]) < TOL_STAGE


@pytest.mark.parametrize("capacity,skin,squeeze", [(64, 0.0, 1.0), (24, 0.0, 1.0), (48, 0.0, 1.0), (92, 0.0, 1.0),
                                                   (92, 0.0, 0.8), (44, 0.0, 0.8), (80, 0.2, 1.0), (128, 0.5, 1.0)])
def test_list_assembly_shared_equals_registers(capacity, skin, squeeze):
    """The lambda pass keeps the first row chunks of a particle's walk in
    shared memory (list_assembly 0) or stores every chunk to the global
    chunk buffer (1): the same neighbours in the same order with the same
    arithmetic, so updates agree bit for bit, also when particles overflow
    the list (24 entries, 6 chunks), when the chunk buffer is as large as
    the shared columns (48 entries: 12 chunks), and when particles have
    more chunks than the shared columns hold and continue in global memory:
    a fluid squeezed to 0.8 of its lattice spacing (~70 neighbours, rows of
    more than 32 candidates; with a list of 92, and of 44 where they
    overflow) and a skin list of 1.5 h (a 25-row stencil against 20 skin
    columns)."""
    mode = 0
    sc = W.dam_break(24, 20, 12)
    sc.pos_w[:, :3] *= squeeze
    sc.params["grid_size"] = [64, 16, 16]
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    a.set_tuning(threads_per_particle=1, neighbor_list_capacity=capacity, neighbor_skin=skin, list_assembly=mode)
    b.set_tuning(threads_per_particle=1, neighbor_list_capacity=capacity, neighbor_skin=skin, list_assembly=1)
    assert a.tuning().list_assembly == mode and b.tuning().list_assembly == 1
    for _ in range(4):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


@pytest.mark.parametrize("squeeze", [1.0, 0.8, 0.6])
def test_chunk_list_equals_the_exact_walk(squeeze):
    """The list path (row chunks of whole three-cell rows, the index list
    written by lambda's sums) against the exact trimmed stencil walk of a
    system without lists (capacity 0): the same neighbours in the same
    order, so updates agree bit for bit -- at rest density, and squeezed to
    0.8 and 0.6 of the lattice spacing (rows of more than 32 candidates,
    several chunks per row)."""
    sc = W.dam_break(24, 20, 12)
    sc.pos_w[:, :3] *= squeeze
    sc.params["grid_size"] = [64, 16, 16]
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    a.set_tuning(threads_per_particle=1, neighbor_list_capacity=512)
    b.set_tuning(threads_per_particle=1, neighbor_list_capacity=0)
    for _ in range(3):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.lambdas(), b.lambdas())
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


def test_list_build_with_a_coincident_pile():
    """600 particles stacked on one point (as a clamped corner collects
    them in a long run): every one has more neighbours than the list holds
    and than the 500-neighbour cap, so the list builds stop walking early
    and the exact walk takes the first 500.  Both builds agree bit for bit
    and the state stays finite."""
    sc = W.dam_break(24, 20, 12)
    sc.params["grid_size"] = [64, 16, 16]
    sc.pos_w[:600, :3] = sc.pos_w[700, :3]
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    a.set_tuning(threads_per_particle=1, list_assembly=0)
    b.set_tuning(threads_per_particle=1, list_assembly=1)
    for _ in range(3):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())
    a.check_finite()


# ------------------------------------------------------------ skin lists

def test_skin_list_forced_rebuild_is_bitwise_the_plain_schedule():
    """A skin of 1e-6 h forces the grid and list rebuild every iteration
    (every particle moves farther than 0.49e-6 h): the filtered skin list
    then visits the same neighbours in the same order, so the result is
    bit for bit the plain schedule's."""
    sc = W.dam_break(16, 16, 8)
    sc.params["grid_size"] = [32, 8, 8]  # room for the skin list's 5-cell stencil
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    b.set_tuning(neighbor_skin=1e-6)
    for _ in range(3):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


@pytest.mark.parametrize("skin", [0.1, 0.2])
def test_skin_list_matches_oracle(skin):
    """Skin lists reused across iterations: one update against the FP64
    oracle (summation order differs from the rebuild schedule, the
    neighbour sets do not), then several updates by invariants."""
    sc = W.dam_break(16, 16, 8)
    sc.params["grid_size"] = [32, 8, 8]
    g, o = make_pair(sc)
    g.set_tuning(neighbor_skin=skin, neighbor_list_capacity=128)
    g.update(sc.dt)
    o.update(sc.dt)
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL_STAGE)
    for _ in range(5):
        g.update(sc.dt)
        o.update(sc.dt)
    check_trajectory(g.positions(), o.positions(), sc.pos_w)


def test_skin_list_reuse_happens_and_agrees_with_rebuild():
    """With a skin wide enough for the step's motion (1.0 h: reuse while
    every particle stays within 0.49 h of its build position; the dam
    break's iterations move particles up to ~0.4 h) later iterations reuse
    the list; the result agrees with the rebuild schedule to FP32
    summation-order noise."""
    sc = W.dam_break(24, 20, 12)
    sc.params["grid_size"] = [64, 16, 16]  # the 2 h list's 7-cell stencil must not alias
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    b.set_tuning(neighbor_skin=1.0, neighbor_list_capacity=512)
    a.update(sc.dt)
    b.update(sc.dt)
    assert_projection(b.positions(), a.positions().astype(np.float64), sc.pos_w, TOL_STAGE)
    assert b.list_reuses() >= 1
    assert a.list_reuses() == 0


def test_skin_list_on_an_aliasing_grid_stays_exact():
    """A skin whose stencil would alias on the grid (7 cells over a 4-cell
    z axis) is not used: the plain schedule's result, bit for bit."""
    sc = W.dam_break(16, 16, 8)
    a = ParticleSystem(default_params(**sc.params), sc.n)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, a)
    W.apply_to(sc, b)
    b.set_tuning(neighbor_skin=1.0, neighbor_list_capacity=512)
    for _ in range(2):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_dam_break_density_invariant():
    """The density invariant over a free-running dam break (30 steps): the
    mean compression (rho above rho0) stays within 2 % and matches the FP64
    oracle's to 0.5 %, and the mean signed error matches it to 1 %."""
    sc = W.dam_break(16, 16, 8)
    g, o = make_pair(sc)
    for _ in range(30):
        g.update(sc.dt)
        o.update(sc.dt)
    g.check_finite()
    h = sc.params["kernel_radius"]
    eg = density_error(g.positions(), sc.rest_density, h)
    eo = density_error(o.positions(), sc.rest_density, h)
    cg, co = np.mean(np.clip(eg, 0, None)), np.mean(np.clip(eo, 0, None))
    assert cg < 0.02 and abs(cg - co) < 0.005, (cg, co)
    assert abs(np.mean(eg) - np.mean(eo)) < 0.01, (np.mean(eg), np.mean(eo))
