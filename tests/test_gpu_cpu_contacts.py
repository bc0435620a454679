"""The CPU reference's contact and boundary projectors on the CUDA path
(PBD_FLAG_CPU_CONTACTS), through the C ABI.

RigidContactConstraint's plain branch, ContactConstraint and
BoundaryConstraint (cpu/src/constraint/rigidcontactconstraint.cpp:30-96,
contactconstraint.cpp:13-42, boundaryconstraint.cpp:14-93) as restated in
the oracle are pinned to the reference's own code
(tests/test_oracle_vs_reference.py, tests/test_golden_oracle.py).  Here the
CUDA contact and wall passes are checked against the oracle and the
reference's golden outputs, and the 2-D granular column -- the CPU
sand-pile path -- against the reference Simulation's settled pile.

Tolerances: one pass within 1e-5 of the largest correction plus one FP32
ulp of the coordinate; the pile by invariants (mean height, spread and
99th-percentile height within 10 %, runout within 2 %: the trajectories
are chaotic, and the reference projects in sequence where the CUDA pass is
Jacobi).
"""
import numpy as np
import pytest

from conftest import GOLDEN
from helpers import (assert_projection, check_granular, cpu_contact_params, load_cpu_contact_pin, params_nolib,
                     pile_invariants)
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def as_pos_w(xy):
    out = np.zeros((len(xy), 4))
    out[:, :2] = xy
    return out


@pytest.mark.parametrize("seed,friction", [(31, (0.4, 0.3)), (35, (0.01, 0.005))])
def test_cpu_contact_pass_against_oracle(seed, friction):
    case = W.cpu_contact_case(seed=seed)
    n = len(case["start"])
    g = ParticleSystem(default_params(**cpu_contact_params(*friction)), n)
    o = Oracle(params_nolib(cpu_contact_params(*friction)), n)
    pg = load_cpu_contact_pin(g, case, fp32_inputs=True)
    po = load_cpu_contact_pin(o, case, fp32_inputs=True)
    est = case["estimate"].astype(np.float32).astype(np.float64)
    assert np.max(np.abs(po - est)) > 0.05
    assert_projection(as_pos_w(pg), as_pos_w(po), as_pos_w(est), 1e-5)


@pytest.mark.parametrize("tag,friction", [("f1", (0.4, 0.3)), ("f2", (0.01, 0.005))])
def test_cpu_contact_pass_against_reference_golden(tag, friction):
    d = dict(np.load(GOLDEN / "cpu_contacts.npz"))
    n = len(d["start"])
    g = ParticleSystem(default_params(**cpu_contact_params(*friction)), n)
    pg = load_cpu_contact_pin(g, d)
    grain = d["solid"] != 0
    ref = d[f"reference_{tag}"]
    assert_projection(as_pos_w(pg[grain]), as_pos_w(ref[grain]), as_pos_w(d["estimate"][grain]), 1e-5)
    np.testing.assert_allclose(pg[~grain], d["estimate"][~grain], rtol=0, atol=1e-5)


def test_granular_column_settles_like_the_reference():
    """600 steps of the 2-D column with the CPU projectors: the settled pile
    against the reference Simulation's (tests/golden/granular_pile.npz)."""
    sc = W.granular_column(cpu_contacts=True)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    for _ in range(600):
        g.update(sc.dt)
    g.check_finite()
    got = pile_invariants(g.positions()[:, :2])
    ref = pile_invariants(np.load(GOLDEN / "granular_pile.npz")["positions"])
    for key, tol in (("mean_height", 0.1), ("spread", 0.1), ("top", 0.1), ("runout", 0.02)):
        assert abs(got[key] - ref[key]) <= tol * ref[key], (key, got, ref)


def test_cpu_contact_column_short_run_and_batch():
    """30 steps of a 400-grain column: the CUDA path against the oracle by
    the pile invariants, and the same scene in a batch (beside a scene with
    the GPU contact model) equal to its solo run."""
    sc = W.granular_column(400, seed=9, cpu_contacts=True)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    o = Oracle(params_nolib(sc.params), sc.n)
    W.apply_to(sc, o)
    for _ in range(30):
        g.update(sc.dt)
        o.update(sc.dt)
    check_granular(g.positions(), o.positions(), 0.03)
    other = W.granular_column(300, seed=10)
    b = ParticleSystem(default_params(**other.params), other.n + sc.n)
    W.apply_to(other, b)
    b.begin_scene(default_params(**sc.params))
    W.apply_to(sc, b)
    solo = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, solo)
    for _ in range(3):
        b.update(sc.dt)
        solo.update(sc.dt)
    a = b.positions()[other.n:].astype(np.float64)[:, :3]
    s = solo.positions().astype(np.float64)[:, :3]
    ulp = np.spacing(np.maximum(np.abs(a), np.abs(s)).astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(a - s) / ulp) <= 2.0
