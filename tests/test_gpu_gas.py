"""The gas phase on the CUDA path, through the C ABI, against the FP64
oracle, whose gas formulas are pinned to the reference's own
GasConstraint::project (tests/test_golden_oracle.py,
tests/test_oracle_vs_reference.py).

Tolerances: grids bit-exact; one gas iteration (lambda, correction, and
the force it adds: vorticity and open drag) to 1e-5 of the largest value,
corrections plus one FP32 ulp of the stored coordinate; several full
updates by the invariants of the other trajectory tests."""
import numpy as np
import pytest

from helpers import assert_projection, check_trajectory, norm_err
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-5


def smoke(twod=False, open_=True, seed=1096):
    sc = W.smoke_box(twod=twod, open_gas=open_, solid_floor=True, seed=seed)
    vel = np.zeros((sc.n, 4), np.float32)
    vel[:, :3] = W.uniform(seed + 7, (sc.n, 3), -1.0, 1.0)
    if twod:
        vel[:, 2] = 0.0
    vel[sc.pos_w[:, 3] == 0.0] = 0.0
    sc.vel = vel
    return sc


def make_pair(sc):
    p = default_params(**sc.params)
    g = ParticleSystem(p, sc.n)
    W.apply_to(sc, g)
    o = Oracle(p, sc.n)
    W.apply_to(sc, o)
    return g, o


@pytest.mark.parametrize("twod", [False, True])
@pytest.mark.parametrize("open_", [False, True])
def test_gas_iteration_matches_oracle(twod, open_):
    """After one full update (which leaves every gas particle a force), both
    sides start from the CUDA state: the prediction (gas gravity x ALPHA,
    the carried force, v' kept), the grid, then one gas pass -- lambda, the
    correction and the new force -- agree with the FP64 replay."""
    sc = smoke(twod, open_)
    g, o = make_pair(sc)
    g.update(sc.dt)
    o.update(sc.dt)
    f_carry = g.forces()
    gas = sc.phase == W.PHASE_GAS
    assert np.max(np.abs(f_carry[gas, :2])) > 0.0
    o.set_positions(g.positions().astype(np.float64))
    o.set_velocities(g.velocities().astype(np.float64))
    o.set_forces(f_carry.astype(np.float64))
    x0 = g.positions()
    g.integrate(sc.dt)
    o.integrate(sc.dt)
    assert_projection(g.positions(), o.positions(), x0, TOL)
    assert norm_err(g.velocities()[:, :3], o.velocities()[:, :3]) < TOL
    assert np.max(np.abs(g.forces())) == 0.0  # the prediction consumed the force
    o.set_positions(g.positions().astype(np.float64))
    o.set_velocities(g.velocities().astype(np.float64))
    g.build_grid()
    o.build_grid()
    for a, b in zip(g.grid(), o.grid()):
        np.testing.assert_array_equal(a, b)
    before = g.positions()
    g.solve_fluids()
    o.solve_fluids()
    assert norm_err(g.lambdas()[gas], o.lambdas()[gas]) < TOL
    assert_projection(g.positions(), o.positions(), before, TOL)
    assert norm_err(g.forces()[gas, :3], o.forces()[gas, :3]) < TOL
    assert np.array_equal(g.positions()[~gas], before[~gas])  # solids: no gas pass


@pytest.mark.parametrize("twod,open_", [(False, False), (True, True)])
def test_gas_trajectory_matches_oracle(twod, open_):
    """Five full updates of the smoke box with its solid floor: closed in
    3-D, open in 2-D (the reference's SMOKE_OPEN_TEST)."""
    sc = smoke(twod, open_)
    g, o = make_pair(sc)
    for _ in range(5):
        g.update(sc.dt)
        o.update(sc.dt)
    gas = sc.phase == W.PHASE_GAS
    check_trajectory(g.positions()[gas], o.positions()[gas], sc.pos_w[gas])
    g.check_finite()


@pytest.mark.parametrize("twod,open_,rise", [(False, False, 0.5), (True, True, 0.1)])
def test_gas_rises_and_stays_finite(twod, open_, rise):
    """With gravity times ALPHA = -0.2 the gas rises over one second (the
    oracle's replay: 0.74 for the closed 3-D box, 0.20 for the open 2-D
    box of the reference's SMOKE_OPEN_TEST).  (The open drag feeds back on
    compressed gas -- force along v' times (rho / rho0 - 1) -- and a 3-D
    open box runs away within a second; the reference tuned it in 2-D.)"""
    sc = smoke(twod, open_)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    gas = sc.phase == W.PHASE_GAS
    y0 = sc.pos_w[gas, 1].mean()
    for _ in range(60):
        g.update_graph(sc.dt, 1)
    g.check_finite()
    assert g.positions()[gas, 1].mean() > y0 + rise


def test_gas_scene_in_a_batch_equals_its_solo_run():
    from test_gpu_batch import assert_same_state, load_alone, load_batch

    scenes = [W.pbf_block(1200, seed=9), smoke(open_=True, seed=31), W.granular_column(400, seed=4),
              smoke(twod=True, open_=False, seed=32)]
    batch, firsts = load_batch(scenes)
    alone = [load_alone(sc) for sc in scenes]
    for _ in range(3):  # each scene clamps the step to its own max_dt
        batch.update(1.0 / 60.0)
        for a in alone:
            a.update(1.0 / 60.0)
    pos = batch.positions()
    for sc, a, f in zip(scenes, alone, firsts):
        assert_same_state(pos[f:f + sc.n], a.positions(), sc.name)


def test_state_blob_carries_the_gas_force():
    sc = smoke()
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    for _ in range(2):
        g.update(sc.dt)
    blob = g.save_state()
    for _ in range(2):
        g.update(sc.dt)
    a = g.positions()
    g.load_state(blob)
    for _ in range(2):
        g.update(sc.dt)
    np.testing.assert_array_equal(g.positions(), a)


def test_adjoint_refuses_gas():
    sc = smoke()
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    with pytest.raises(PbdError, match="gas"):
        g.rollout(sc.dt, 2, 1)


def test_gas_params_validated():
    sc = smoke()
    with pytest.raises(PbdError):
        ParticleSystem(default_params(**sc.params, gas_scorr_dq=1.5), sc.n)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    bad = sc.pos_w[:1].copy()
    bad[0, 3] = 0.0
    with pytest.raises(PbdError, match="gas particle"):
        g.add_particles(bad, phase=[W.PHASE_GAS])
