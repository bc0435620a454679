"""The entry points named by the hot-path contract (pbd_tick,
pbd_batch_create, pbd_batch_tick, pbd_add_fluid_group, pbd_add_rigid_group,
pbd_set_box, pbd_record) give exactly what the calls they stand for give."""
import ctypes

import numpy as np
import pytest

from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def load(sc):
    g = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, g)
    return g


def test_tick_is_update():
    sc = W.dam_break(16, 12, 8)
    a, b = load(sc), load(sc)
    for _ in range(3):
        a.update(sc.dt)
        assert b.lib.pbd_tick(b.h, ctypes.c_float(sc.dt), None) == 0
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_batch_tick_is_update_graph():
    scenes = [W.pbf_block(800, seed=2), W.granular_column(300, seed=3)]
    from test_gpu_batch import load_batch

    a, _ = load_batch(scenes)
    b, _ = load_batch(scenes)
    a.update_graph(1.0 / 60.0, 3)
    assert b.lib.pbd_batch_tick(b.h, ctypes.c_float(1.0 / 60.0), 3, None) == 0
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_batch_create_is_begin_scene_and_add():
    """One pbd_batch_create call equals pbd_create + pbd_begin_scene +
    pbd_add_particles per scene: same scenes, same slots, same steps."""
    scenes = [W.pbf_block(800, seed=2), W.granular_column(300, seed=3), W.pbf_block(500, seed=4, iterations=3)]
    from test_gpu_batch import load_batch

    a, firsts = load_batch(scenes)
    pos = np.concatenate([sc.pos_w for sc in scenes])
    vel = np.concatenate([sc.vel if sc.vel is not None else np.zeros((sc.n, 4), np.float32) for sc in scenes])
    phase = np.concatenate([sc.phase for sc in scenes])
    rho = np.concatenate([sc.rest_density if sc.rest_density is not None else np.ones(sc.n, np.float32)
                          for sc in scenes])
    b = ParticleSystem.batch([default_params(**sc.params) for sc in scenes], [sc.n for sc in scenes], pos, vel,
                             phase, rho)
    assert b.num_scenes == len(scenes)
    for k in range(len(scenes)):
        assert b.scene(k)[:2] == a.scene(k)[:2] == (firsts[k], scenes[k].n)
    a.update_graph(1.0 / 60.0, 4)
    b.update_graph(1.0 / 60.0, 4)
    np.testing.assert_array_equal(a.positions(), b.positions())
    np.testing.assert_array_equal(a.velocities(), b.velocities())


def test_batch_create_rejects_bad_input():
    sc = W.pbf_block(100, seed=1)
    p = default_params(**sc.params)
    with pytest.raises(PbdError):
        ParticleSystem.batch([p], [sc.n], sc.pos_w, max_particles=sc.n - 1)
    with pytest.raises(PbdError):
        ParticleSystem.batch([], [], sc.pos_w)
    bad = default_params(**sc.params)
    bad.kernel_radius = -1.0
    with pytest.raises(PbdError):
        ParticleSystem.batch([p, bad], [50, 50], sc.pos_w)


def test_add_fluid_group_equals_fluid_particles():
    """Particles added as solid grains, then made fluid of rest density 3,
    step exactly as particles added as fluid of that density."""
    sc = W.dam_break(12, 12, 8)
    rho = np.full(sc.n, 3.0, np.float32)
    a = ParticleSystem(default_params(**sc.params), sc.n)
    a.add_particles(sc.pos_w, None, np.full(sc.n, W.PHASE_FLUID, np.int32), rho)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    b.add_particles(sc.pos_w, None, np.full(sc.n, W.PHASE_SOLID, np.int32), None)
    b.add_fluid_group(0, sc.n, 3.0)
    np.testing.assert_array_equal(b.phases(), a.phases())
    for _ in range(3):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())
    with pytest.raises(PbdError):
        b.add_fluid_group(0, sc.n, -1.0)


def test_add_rigid_group_is_add_rigid_body():
    sc = W.rigid_boxes(count=4)
    a = load(sc)
    b = ParticleSystem(default_params(**sc.params), sc.n)
    b.add_particles(sc.pos_w, sc.vel, sc.phase, sc.rest_density)
    for first, count, st in sc.bodies:
        assert b.lib.pbd_add_rigid_group(b.h, first, count, ctypes.c_float(st)) == 0
    for _ in range(5):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_set_box_is_the_params_box():
    sc = W.reference_granular()
    lo, hi = [-3.0, 0.5, -3.0], [3.0, 100.0, 3.0]
    a = ParticleSystem(default_params(**{**sc.params, "box_min": lo, "box_max": hi}), sc.n)
    W.apply_to(sc, a)
    b = load(sc)
    b.set_box(lo, hi)
    for _ in range(5):
        a.update(sc.dt)
        b.update(sc.dt)
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_record_is_rollout():
    sc = W.cloth_ropes_grains(cloth=8, ropes=2, rope_particles=6, grains=10)
    a, b = load(sc), load(sc)
    a.rollout(sc.dt, 6, 3)
    assert b.lib.pbd_record(b.h, ctypes.c_float(sc.dt), 6, 3, None) == 0
    np.testing.assert_array_equal(a.positions(), b.positions())


def test_vbo_is_the_reference_render_layout():
    """pbd_get_vbo gives the reference's render buffer: each particle's
    position with w = 1 (integration_kernel.cuh:461), to host memory or to
    a device buffer, for any subrange."""
    import torch

    sc = W.dam_break(16, 12, 8)
    g = load(sc)
    for _ in range(2):
        g.update(sc.dt)
    x = g.positions()
    v = g.vbo()
    np.testing.assert_array_equal(v[:, :3], x[:, :3])
    assert np.all(v[:, 3] == 1.0)
    np.testing.assert_array_equal(g.vbo(5, 10), v[5:15])
    t = torch.zeros((sc.n, 4), dtype=torch.float32, device="cuda")
    g.vbo(device_ptr=t.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t.cpu().numpy(), v)
    with pytest.raises(PbdError):
        g.vbo(sc.n - 2, 5)


def test_paired_state_copies_equal_the_single_ones():
    """pbd_set/get_positions_velocities (the two copies run concurrently)
    move exactly what pbd_set/get_positions and _velocities move, from host
    and from device memory, and a step after either gives the same state."""
    torch = pytest.importorskip("torch")
    sc = W.dam_break(16, 12, 8)
    a, b = load(sc), load(sc)
    a.update(sc.dt)
    b.update(sc.dt)
    n = sc.n
    rng = np.random.default_rng(3)
    x = (a.positions() + rng.uniform(-1e-3, 1e-3, (n, 4)).astype(np.float32) * [1, 1, 1, 0]).astype(np.float32)
    v = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    a.set_positions(x)
    a.set_velocities(v)
    assert b.lib.pbd_set_positions_velocities(b.h, 0, n, x.ctypes.data, v.ctypes.data, 0, None) == 0
    xo, vo = np.empty_like(x), np.empty_like(v)
    assert b.lib.pbd_get_positions_velocities(b.h, 0, n, xo.ctypes.data, vo.ctypes.data, 0, None) == 0
    np.testing.assert_array_equal(xo, a.positions())
    np.testing.assert_array_equal(vo, a.velocities())
    # device pointers, a sub-range and one of the two alone
    xd = torch.tensor(x[5:40], device="cuda")
    vd = torch.tensor(v[5:40] * 2, device="cuda")
    assert b.lib.pbd_set_positions_velocities(b.h, 5, 35, xd.data_ptr(), vd.data_ptr(), 1, None) == 0
    a.set_velocities(v[5:40] * 2, first=5)
    assert b.lib.pbd_set_positions_velocities(b.h, 0, n, None, None, 0, None) == 0
    a.update(sc.dt)
    assert b.lib.pbd_update(b.h, ctypes.c_float(sc.dt), None) == 0
    xs = torch.empty((n, 4), device="cuda")
    assert b.lib.pbd_get_positions_velocities(b.h, 0, n, xs.data_ptr(), None, 1, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(xs.cpu().numpy(), a.positions())
    assert b.lib.pbd_get_positions_velocities(b.h, 0, n + 1, xo.ctypes.data, vo.ctypes.data, 0, None) != 0
