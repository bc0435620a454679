"""The signed-distance rigid contact on the CUDA path, through the C ABI,
against the FP64 oracle, whose formulas are pinned to the reference's own
RigidContactConstraint::project (tests/test_golden_oracle.py,
tests/test_oracle_vs_reference.py).

Tolerance: one contact pass to 1e-5 of the largest correction plus one FP32
ulp of the stored coordinate (assert_projection); longer runs by
invariants."""
import numpy as np
import pytest

from helpers import SDF_PIN_PARAMS, assert_projection, load_sdf_pin, params_nolib
from oracle import Oracle
from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-5


def pad4(xy):
    out = np.zeros((len(xy), 4))
    out[:, :2] = xy
    return out


@pytest.mark.parametrize("seed", [9, 10])
def test_sdf_pin_case_matches_oracle(seed):
    """2-D body pairs touching at one corner: normals rotated by the stored
    body rotation, initBoundary reflection, height-scaled masses, friction."""
    case = W.sdf_contact_pairs(24, seed=seed)
    n = len(case["start"])
    g = ParticleSystem(default_params(**SDF_PIN_PARAMS), n)
    o = Oracle(params_nolib(SDF_PIN_PARAMS), n)
    pg = load_sdf_pin(g, case, fp32_inputs=True)
    po = load_sdf_pin(o, case, fp32_inputs=True)
    est = pad4(case["estimate"]).astype(np.float32)
    assert np.max(np.abs(po - case["estimate"])) > 1e-3
    assert_projection(pad4(pg), pad4(po), est, TOL)


def sdf_box_row(count=6, side=3, radius=0.25, seed=4, overlap=0.3):
    """count side^3 SDF boxes at seeded random orientations on a line, each
    centre `side * 2r - overlap` from the next, so that neighbours
    interpenetrate: contacts between face, edge, corner and interior
    particles of different bodies."""
    d = 2.0 * radius
    g = (np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3) - (side - 1) / 2.0) * d
    qs = W.random_quaternions(seed, count)
    lat_sdf = W.box_sdf([side] * 3, radius)
    pos, ph, bodies, sdfs = [], [], [], []
    for b in range(count):
        qb = np.broadcast_to(qs[b], (g.shape[0], 4))
        pts = W.quat_rotate(qb, g) + [b * (side * d - overlap), 5.0, 0.0]
        bodies.append((len(pos), g.shape[0], 1.0))
        e = lat_sdf.copy()
        e[:, :3] = W.quat_rotate(qb, lat_sdf[:, :3])
        sdfs.append(e)
        for p in pts:
            pos.append([*p, 1.0])
            ph.append(W.PHASE_RIGID + b)
    params = W.reference_scene_params(radius, iterations=4)
    params.update(contact_static_friction=0.4, contact_kinetic_friction=0.3)
    return W.Scene("sdf_row", params, np.asarray(pos, np.float32), np.asarray(ph, np.int32), bodies=bodies,
                   sdf=sdfs)


def test_sdf_box_row_contact_pass_matches_oracle():
    sc = sdf_box_row()
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    o = Oracle(default_params(**sc.params), sc.n)
    W.apply_to(sc, o)
    g.build_grid()
    o.build_grid()
    g.collide()
    o.collide()
    d = o.positions()[:, :3] - sc.pos_w[:, :3]
    assert np.max(np.abs(d)) > 1e-3
    assert_projection(g.positions(), o.positions(), sc.pos_w, TOL)


def test_sdf_changes_the_contact_only_where_both_have_data():
    """Without sdf data the same row takes the particle-particle contact;
    with data on every body the result differs."""
    sc = sdf_box_row()
    plain = W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, bodies=sc.bodies)
    out = []
    for scene in (sc, plain):
        g = ParticleSystem(default_params(**scene.params), scene.n)
        W.apply_to(scene, g)
        g.build_grid()
        g.collide()
        out.append(g.positions())
    assert np.max(np.abs(out[0] - out[1])) > 1e-3


def test_sdf_boxes_fall_and_stay_rigid():
    """Sixteen SDF boxes dropped on the floor for two seconds: finite, every
    box keeps its shape (RMS deviation from its rest shape after shape
    matching) and rests above the floor."""
    sc = W.rigid_boxes(count=16, sdf=True)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    y0 = sc.pos_w[:, 1].mean()
    for _ in range(120):
        g.update_graph(sc.dt, 1)
    g.check_finite()
    x = g.positions()
    assert x[:, 1].mean() < y0 - 1.0
    assert x[:, 1].min() > sc.params["box_min"][1] - 1e-3
    for first, count, _ in sc.bodies:
        p = x[first:first + count, :3].astype(np.float64)
        r = sc.pos_w[first:first + count, :3].astype(np.float64)
        pc, rc = p - p.mean(0), r - r.mean(0)
        u, _, vt = np.linalg.svd(rc.T @ pc)
        rot = (u @ vt).T
        rms = np.sqrt(np.mean(np.sum((pc - rc @ rot.T) ** 2, 1)))
        assert rms < 0.05 * sc.params["particle_radius"]


def test_sdf_scene_in_a_batch_equals_its_solo_run():
    from test_gpu_batch import assert_same_state, load_alone, load_batch

    scenes = [W.rigid_boxes(count=6, sdf=True, seed=3), W.pbf_block(900, seed=6), sdf_box_row(seed=8)]
    batch, firsts = load_batch(scenes)
    alone = [load_alone(sc) for sc in scenes]
    for _ in range(3):
        batch.update(1.0 / 60.0)
        for a in alone:
            a.update(1.0 / 60.0)
    pos = batch.positions()
    for sc, a, f in zip(scenes, alone, firsts):
        assert_same_state(pos[f:f + sc.n], a.positions(), sc.name)


def test_adjoint_refuses_sdf_contact():
    sc = sdf_box_row()
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    with pytest.raises(PbdError, match="signed-distance"):
        g.rollout(1.0 / 60.0, 2, 1)


def test_sdf_arguments_validated():
    sc = sdf_box_row(count=2)
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, bodies=sc.bodies), g)
    with pytest.raises(PbdError):
        g.set_rigid_sdf(5, sc.sdf[0])
    bad = np.array(sc.sdf[0], np.float32)
    bad[0, :3] = 0.0
    with pytest.raises(PbdError, match="zero normal"):
        g.set_rigid_sdf(0, bad)
