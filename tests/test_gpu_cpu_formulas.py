"""The CPU reference's fluid formulas on the CUDA path, through the C ABI.

TotalFluidConstraint::project (cpu/src/constraint/totalfluidconstraint.cpp:
41-116) differs from the GPU reference's fluid passes in four places; the
flags PBD_FLAG_DENSITY_NEIGHBOR_MASS, PBD_FLAG_SKIP_FIXED_NEIGHBORS,
PBD_FLAG_DELTA_OVER_COUNT and solid_density_weight = 0 select them
(workloads.cpu_fluid_box).  The oracle's restatement of them is pinned to
the reference's own code (tests/test_oracle_vs_reference.py,
tests/test_golden_oracle.py); here the CUDA passes are checked against the
oracle and against the reference's golden outputs.

Tolerances: lambda within 1e-5 (normalised max error); displacements
within 1e-5 of the largest displacement plus one FP32 ulp of the
coordinate (FP32 against FP64).
"""
import numpy as np
import pytest

from conftest import GOLDEN
from helpers import assert_projection, check_trajectory, fluid_projection, norm_err
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def pair(sc):
    p = default_params(**sc.params)
    g = ParticleSystem(p, sc.n)
    W.apply_to(sc, g)
    o = Oracle(p, sc.n)
    W.apply_to(sc, o)
    return g, o


def to_pos_w(sc, xy):
    out = sc.pos_w.astype(np.float64).copy()
    out[:, :2] = xy
    return out


@pytest.mark.parametrize("seed", [890, 893])
@pytest.mark.parametrize("calls", [1, 3])
def test_cpu_fluid_formulas_against_oracle(seed, calls):
    sc = W.cpu_fluid_box(seed=seed)
    g, o = pair(sc)
    fluid = sc.phase == W.PHASE_FLUID
    pg, lg = fluid_projection(g, calls)
    po, lo = fluid_projection(o, calls)
    assert norm_err(lg[fluid], lo[fluid]) < 1e-5
    assert_projection(to_pos_w(sc, pg), to_pos_w(sc, po), sc.pos_w, 1e-5)
    assert np.max(np.abs(pg[~fluid] - sc.pos_w[~fluid, :2])) == 0.0


@pytest.mark.parametrize("calls", [1, 3])
def test_cpu_fluid_formulas_against_reference_golden(calls):
    """Against the reference's own TotalFluidConstraint::project outputs
    (tests/golden/fluid_project.npz)."""
    data = np.load(GOLDEN / "fluid_project.npz")
    sc = W.cpu_fluid_box(seed=890)
    np.testing.assert_array_equal(sc.pos_w, data["pos_w"])
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    fluid = sc.phase == W.PHASE_FLUID
    pg, lg = fluid_projection(g, calls)
    assert norm_err(lg[fluid], data[f"k{calls}_lambda"][fluid]) < 1e-5
    assert_projection(to_pos_w(sc, pg), to_pos_w(sc, data[f"k{calls}_pos"]), sc.pos_w, 1e-5)


def test_cpu_fluid_formulas_full_steps_and_batch():
    """Whole steps with the CPU formulas: the CUDA path against the oracle by
    invariants over 10 steps, and the same scene inside a batch (next to a
    scene with the GPU formulas) equal to its solo run."""
    sc = W.cpu_fluid_box(seed=894)
    g, o = pair(sc)
    for _ in range(10):
        g.update(sc.dt)
        o.update(sc.dt)
    check_trajectory(g.positions(), o.positions(), sc.pos_w)
    other = W.pbf_block(900, seed=5)
    b = ParticleSystem(default_params(**other.params), other.n + sc.n)
    W.apply_to(other, b)
    b.begin_scene(default_params(**sc.params))
    W.apply_to(sc, b)
    solo = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, solo)
    for _ in range(3):
        b.update(sc.dt)
        solo.update(sc.dt)
    a = b.positions()[other.n:].astype(np.float64)
    s = solo.positions().astype(np.float64)
    ulp = np.spacing(np.maximum(np.abs(a), np.abs(s)).astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(a - s)[:, :3] / ulp[:, :3]) <= 2.0


def test_divisor_flags_exclude_each_other():
    from particlesolver_gb300 import FLAG_DELTA_OVER_COUNT, FLAG_DELTA_OVER_RHO0

    with pytest.raises(PbdError):
        ParticleSystem(default_params(flags=FLAG_DELTA_OVER_COUNT | FLAG_DELTA_OVER_RHO0), 16)
