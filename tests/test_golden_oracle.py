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
