"""The oracle against the golden fixtures made from the reference's own
kernels (tests/golden/make_golden.py).  Runs anywhere (no reference tree,
no GPU needed)."""
import numpy as np
import pytest

from helpers import check_against_golden, check_trajectory, golden_scene, params_nolib, run_stages
from conftest import GOLDEN
from oracle import Oracle
from particlesolver_gb300 import workloads as W

FIXTURES = sorted(GOLDEN.glob("ref_*.npz"))


class OracleSystem(Oracle):
    """Oracle with the CUDA system's method names for run_stages."""

    def grid(self):
        return super().grid()


def load_oracle(data):
    sc = golden_scene(data)
    o = OracleSystem(params_nolib(sc.params), sc.n)
    W.apply_to(sc, o)
    return sc, o


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_stages_match_reference_golden(path):
    data = np.load(path)
    sc, o = load_oracle(data)
    out = run_stages(o)
    check_against_golden(out, data, sc.pos_w)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_updates_match_reference_golden(path):
    data = np.load(path)
    sc, o = load_oracle(data)
    for k in range(3):
        o.update(sc.dt)
        check_trajectory(o.positions(), data[f"update{k + 1}_pos"], sc.pos_w)


def test_fixtures_present():
    assert len(FIXTURES) >= 3


GAS = GOLDEN / "gas_project.npz"


@pytest.mark.parametrize("open_", [0, 1])
@pytest.mark.parametrize("calls", [1, 3])
def test_gas_projection_matches_reference_golden(open_, calls):
    """The oracle's gas passes against the reference's own
    GasConstraint::project (gasconstraint.cpp:34-134) on a 2-D smoke box
    with solid (S_SOLID-weighted) and fixed (ignored) neighbours: estimates
    and forces (vorticity, open drag) after 1 and 3 calls, to 1e-7 of the
    largest displacement / force (FP64 on both sides; the two differ in
    summation order only)."""
    from helpers import assert_gas_projection, oracle_gas_projection

    data = np.load(GAS)
    params = W.smoke_box(twod=True, solid_floor=True).params
    pos, force = oracle_gas_projection(data["pos_w"], data["phase"], data["rest_density"], data["vel"], params,
                                       bool(open_), calls)
    gas = data["phase"] == W.PHASE_GAS
    assert_gas_projection(pos, force, data[f"open{open_}_k{calls}_pos"], data[f"open{open_}_k{calls}_force"],
                          data["pos_w"][:, :2].astype(np.float64), gas, 1e-7)


def test_sdf_rigid_contact_matches_reference_golden():
    """The oracle's signed-distance rigid contact against the reference's own
    RigidContactConstraint::project (rigidcontactconstraint.cpp:30-96): 24
    pairs of rotated 2-D boxes touching at one corner each (so the
    reference's sequential projections and the Jacobi pass coincide), with
    height-scaled masses and friction, to 1e-6 of the largest correction
    (the body rotations come from one shape-matching pass)."""
    from helpers import SDF_PIN_PARAMS, load_sdf_pin, norm_err

    data = dict(np.load(GOLDEN / "sdf_contacts.npz"))
    n = len(data["start"])
    o = Oracle(params_nolib(SDF_PIN_PARAMS), n)
    pos = load_sdf_pin(o, data)
    d_ref = data["reference"] - data["estimate"]
    assert np.max(np.abs(d_ref)) > 1e-3
    assert norm_err(pos - data["estimate"], d_ref) < 1e-6


def test_oracle_2d_grid_depth_does_not_matter():
    """In 2-D mode every particle sits in twod_z's layer and the stencils
    walk only that layer, so a granular column steps identically on a grid
    one cell deep and on one four cells deep (where a three-layer stencil
    would have found the same neighbours in empty layers)."""
    import numpy as np

    from oracle import Oracle
    from particlesolver_gb300 import default_params
    from particlesolver_gb300 import workloads as W

    sc = W.granular_column(300, seed=7)
    out = []
    for depth in (1, 4):
        params = dict(sc.params)
        params["grid_size"] = [sc.params["grid_size"][0], sc.params["grid_size"][1], depth]
        o = Oracle(default_params(**params), sc.n, threads=1)
        W.apply_to(sc, o)
        for _ in range(5):
            o.update(sc.dt)
        out.append(o.positions())
        assert np.all(o.positions()[:, 2] == 0.0)
    np.testing.assert_array_equal(out[0], out[1])


def test_cpu_fluid_formulas_match_reference_golden():
    """The oracle's CPU fluid formulas (neighbour masses, fixed neighbours
    left out, correction over rho0 (n + 1), S_SOLID 0) against the
    reference's own TotalFluidConstraint::project
    (totalfluidconstraint.cpp:41-116) on a 2-D fluid box over a fixed plate
    and movable grains: displacements and lambdas after 1 and 3 calls, to
    1e-7 (FP64 on both sides)."""
    from helpers import fluid_projection, norm_err

    data = np.load(GOLDEN / "fluid_project.npz")
    sc = W.cpu_fluid_box(seed=890)
    np.testing.assert_array_equal(sc.pos_w, data["pos_w"])
    fluid = sc.phase == W.PHASE_FLUID
    start = sc.pos_w[:, :2].astype(np.float64)
    for k in (1, 3):
        o = Oracle(params_nolib(sc.params), sc.n)
        W.apply_to(sc, o)
        pos, lam = fluid_projection(o, k)
        ref = data[f"k{k}_pos"]
        assert np.max(np.abs(ref[fluid] - start[fluid])) > 0.05
        assert norm_err(pos[fluid] - start[fluid], ref[fluid] - start[fluid]) < 1e-7
        assert norm_err(lam[fluid], data[f"k{k}_lambda"][fluid]) < 1e-7


def test_emitter_rules_match_reference_golden():
    """The emitter rules the CUDA path is tested against (emission per tick,
    solidification) against the reference's own FluidEmitter::tick
    (fluidemitter.cpp:13-77): emission counts of 40 ticks and one
    solidification tick of 400 fluid members, exactly."""
    from helpers import emitter_counts, solidify_rule

    d = np.load(GOLDEN / "fluid_emitter.npz")
    assert list(d["counts"]) == emitter_counts(float(d["rate"]), 5.0, float(d["dt"]), len(d["counts"]))
    m = int(d["members"])
    n = len(d["t"])
    fluid = np.arange(n) < m
    lam = np.concatenate([d["lam"], np.zeros(n - m)])
    t, turn = solidify_rule(d["p"][:, 1], np.linalg.norm(d["v"], axis=1), lam, d["t"], fluid, float(d["dt"]))
    assert turn.any()
    np.testing.assert_array_equal(d["fluid_out"], fluid & ~turn)
    np.testing.assert_allclose(d["t_out"][fluid], t[fluid], rtol=0, atol=1e-12)
    assert np.all(d["imass_out"][turn] == 0.0) and np.all(d["v_out"][turn] == 0.0)



def test_smoke_emitter_rule_matches_reference_golden():
    """The gas emitter's emission rule (emitter_counts with no time limit)
    against the reference's own OpenSmokeEmitter::tick
    (opensmokeemitter.cpp:17-43, tests/golden/smoke_emitter.npz): 6 s of
    ticks at three rates, each particle a gas particle of inverse mass 1."""
    from helpers import emitter_counts

    d = np.load(GOLDEN / "smoke_emitter.npz")
    for k in range(3):
        counts = list(d[f"counts{k}"])
        assert counts == emitter_counts(float(d[f"rate{k}"]), 0.0, float(d[f"dt{k}"]), len(counts))
        assert np.all(d[f"imass{k}"] == 1.0) and np.all(d[f"gas{k}"])

@pytest.mark.parametrize("tag,friction", [("f1", (0.4, 0.3)), ("f2", (0.01, 0.005))])
def test_cpu_contacts_match_reference_golden(tag, friction):
    """The oracle's CPU contact projectors against the reference's own
    RigidContactConstraint (plain branch), ContactConstraint and
    BoundaryConstraint (tests/golden/cpu_contacts.npz): grains in one
    constraint each, static and kinetic friction, to 1e-7."""
    from helpers import cpu_contact_params, load_cpu_contact_pin, norm_err

    d = dict(np.load(GOLDEN / "cpu_contacts.npz"))
    o = Oracle(params_nolib(cpu_contact_params(*friction)), len(d["start"]))
    pos = load_cpu_contact_pin(o, d)
    grain = d["solid"] != 0
    d_ref = d[f"reference_{tag}"] - d["estimate"]
    assert np.max(np.abs(d_ref[grain])) > 0.05
    assert norm_err(pos[grain] - d["estimate"][grain], d_ref[grain]) < 1e-7
