"""Adjoint (reverse-mode) gradients of rollouts, through the C ABI and the
torch.autograd bridge, against central finite differences of the FP64
oracle and against the forward-mode dual-number derivative of the same
FP64 replay.

Loss L = sum_i c_i . x_T,i with fixed random c.  The FP32 adjoint's
directional derivative along a random direction d in (stiffness, x0, v0)
must match, to 1e-3 relative, both the oracle's
(L(p + eps d) - L(p - eps d)) / (2 eps) (eps = 1e-5 is far inside the range
where the oracle's central difference has converged and no contact switches
on or off) and sum_i c_i . dx_T,i of the dual-number oracle seeded with d
(exact for the branches the FP64 replay takes, no step size)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import Oracle, OracleDual  # noqa: E402
from particlesolver_gb300 import ParticleSystem, PbdError, default_params  # noqa: E402
from particlesolver_gb300 import workloads as W  # noqa: E402
from particlesolver_gb300.autograd import rollout  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 1e-3


def small_scene(seed=5, stiffness_seed=9):
    return W.cloth_ropes_grains(cloth=8, ropes=2, rope_particles=8, grains=12, drop=0.8, seed=seed,
                                stiffness_seed=stiffness_seed)


def sliding_grains():
    """Grains sliding on the floor into a side wall: wall clamps and wall
    friction (static and kinetic), no particle contacts."""
    sc = W.granular_column(16, width=4, seed=3)
    sc.params.update(contact_static_friction=0.3, contact_kinetic_friction=0.2, wall_static_friction=0.3,
                     wall_kinetic_friction=0.2, flags=0, box_min=[-2.0, 0.0, -2.0], box_max=[2.0, 40.0, 2.0],
                     grid_size=[16, 32, 16], world_origin=[-2.0, 0.0, -2.0])
    pos = sc.pos_w.copy()
    pos[:, 0] *= 1.3  # spacing 0.65: no contacts
    pos[:, 1] = 0.3 + 0.65 * (np.arange(16) // 4) * 0.0
    pos[:, 2] = np.repeat(np.arange(4), 4) * 0.65 - 1.0
    sc.pos_w = pos
    vel = np.zeros((16, 4), np.float32)
    vel[:, 0] = 1.5
    vel[:, 1] = -0.5
    vel[:, 2] = np.linspace(-0.4, 0.4, 16)
    sc.vel = vel
    return sc


def gpu_gradients(sc, stiffness, steps, every, c):
    sys = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, sys)
    dev = torch.device("cuda", 0)
    st = torch.tensor(stiffness if stiffness is not None else np.zeros(0), dtype=torch.float32, device=dev,
                      requires_grad=True)
    x0 = torch.tensor(sc.pos_w, device=dev, requires_grad=True)
    v0 = torch.tensor(sc.vel if sc.vel is not None else np.zeros((sc.n, 4), np.float32), device=dev,
                      requires_grad=True)
    xT, _ = rollout(sys, st, x0, v0, sc.dt, steps, every)
    loss = (xT[:, :3] * torch.tensor(c, dtype=torch.float32, device=dev)).sum()
    loss.backward()
    torch.cuda.synchronize()
    gs = st.grad.cpu().numpy() if st.grad is not None else np.zeros(0)
    return gs, x0.grad.cpu().numpy()[:, :3], v0.grad.cpu().numpy()[:, :3], xT.detach().cpu().numpy()


def oracle_loss(sc, stiffness, x0, v0, steps, c, tangent=None):
    """L of the FP64 oracle from (x0, v0): the scene is loaded as given
    (rigid bodies take their rest shapes from the scene's positions, as in
    the differentiated rollout), then the state is set.  With
    tangent = (ds, dx, dv) the dual-number oracle runs instead and the
    directional derivative of L along that direction is returned."""
    o = (Oracle if tangent is None else OracleDual)(default_params(**sc.params), sc.n)
    W.apply_to(W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, rest_density=sc.rest_density, pairs=sc.pairs,
                       rest=sc.rest, stiffness=None if stiffness is None else np.asarray(stiffness),
                       pins=sc.pins, pin_points=sc.pin_points, bodies=sc.bodies), o)
    pos = np.asarray(sc.pos_w, np.float64).copy()
    pos[:, :3] = x0
    vel = np.zeros((sc.n, 4))
    vel[:, :3] = v0
    o.set_positions(pos)
    o.set_velocities(vel)
    if tangent is not None:
        o.seed_tangents(tangent[1], tangent[2], tangent[0])
    for _ in range(steps):
        o.update(sc.dt)
    if tangent is not None:
        return float(np.sum(o.tangents()[0][:, :3] * c))
    return float(np.sum(o.positions()[:, :3] * c))


def dual_directional(sc, stiffness, x0, v0, steps, c, ds, dx, dv):
    return oracle_loss(sc, stiffness, x0, v0, steps, c, tangent=(ds, dx, dv))


def check_directional(sc, steps, every, seed, eps=1e-5):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((sc.n, 3))
    m = 0 if sc.pairs is None else len(sc.pairs)
    stiff = None if not m else (sc.stiffness if sc.stiffness is not None else np.ones(m, np.float32))
    gs, gx, gv, _ = gpu_gradients(sc, stiff, steps, every, c)
    ds = rng.uniform(-1, 1, m)
    dx = rng.standard_normal((sc.n, 3)) * 0.1
    dv = rng.standard_normal((sc.n, 3))
    ad = float(np.dot(gs, ds) + np.sum(gx * dx) + np.sum(gv * dv))
    s0 = None if not m else np.asarray(stiff, np.float64)
    x0 = np.asarray(sc.pos_w[:, :3], np.float64)
    v0 = np.zeros((sc.n, 3)) if sc.vel is None else np.asarray(sc.vel[:, :3], np.float64)
    lp = oracle_loss(sc, None if s0 is None else s0 + eps * ds, x0 + eps * dx, v0 + eps * dv, steps, c)
    lm = oracle_loss(sc, None if s0 is None else s0 - eps * ds, x0 - eps * dx, v0 - eps * dv, steps, c)
    fd = (lp - lm) / (2 * eps)
    dual = dual_directional(sc, s0, x0, v0, steps, c, ds if m else None, dx, dv)
    assert abs(ad - fd) <= TOL * abs(fd), (ad, fd)
    assert abs(ad - dual) <= TOL * abs(dual), (ad, dual)
    return ad, fd


@pytest.mark.parametrize("steps,every", [(6, 6), (12, 5)])
def test_cloth_ropes_grains_gradient_matches_fd(steps, every):
    """Distance constraints with per-constraint stiffness, pins, contacts
    with friction between grains and cloth / ropes, the integrator."""
    check_directional(small_scene(), steps, every, seed=steps)


def test_each_parameter_block_matches_fd():
    """Stiffness, x0 and v0 directions checked one at a time."""
    sc = small_scene(seed=6, stiffness_seed=10)
    steps, every = 10, 4
    rng = np.random.default_rng(1)
    c = rng.standard_normal((sc.n, 3))
    gs, gx, gv, _ = gpu_gradients(sc, sc.stiffness, steps, every, c)
    eps = 1e-5
    s0 = sc.stiffness.astype(np.float64)
    x0 = sc.pos_w[:, :3].astype(np.float64)
    v0 = sc.vel[:, :3].astype(np.float64)
    for which in ("stiffness", "x0", "v0"):
        ds = rng.uniform(-1, 1, len(s0)) if which == "stiffness" else np.zeros(len(s0))
        dx = rng.standard_normal(x0.shape) * 0.1 if which == "x0" else np.zeros_like(x0)
        dv = rng.standard_normal(v0.shape) if which == "v0" else np.zeros_like(v0)
        ad = float(np.dot(gs, ds) + np.sum(gx * dx) + np.sum(gv * dv))
        fd = (oracle_loss(sc, s0 + eps * ds, x0 + eps * dx, v0 + eps * dv, steps, c)
              - oracle_loss(sc, s0 - eps * ds, x0 - eps * dx, v0 - eps * dv, steps, c)) / (2 * eps)
        dual = dual_directional(sc, s0, x0, v0, steps, c, ds, dx, dv)
        assert abs(ad - fd) <= TOL * abs(fd), (which, ad, fd)
        assert abs(ad - dual) <= TOL * abs(dual), (which, ad, dual)


def test_wall_clamps_and_friction_gradient():
    check_directional(sliding_grains(), 8, 3, seed=4)


def test_gradient_independent_of_checkpoint_interval():
    """The backward pass recomputes segments from checkpoints; any
    interval gives the same result bit for bit."""
    sc = small_scene()
    c = np.random.default_rng(2).standard_normal((sc.n, 3))
    ref = gpu_gradients(sc, sc.stiffness, 9, 9, c)
    for every in (1, 2, 4):
        got = gpu_gradients(sc, sc.stiffness, 9, every, c)
        for a, b in zip(ref, got):
            np.testing.assert_array_equal(a, b)


def test_batched_gradients_equal_each_scene_alone():
    scenes = [small_scene(seed=5, stiffness_seed=9), small_scene(seed=8, stiffness_seed=11)]
    rng = np.random.default_rng(3)
    cs = [rng.standard_normal((sc.n, 3)) for sc in scenes]
    alone = [gpu_gradients(sc, sc.stiffness, 8, 3, c) for sc, c in zip(scenes, cs)]
    total = sum(sc.n for sc in scenes)
    sys = ParticleSystem(default_params(**scenes[0].params), total)
    off = [0, scenes[0].n]
    for k, sc in enumerate(scenes):
        if k:
            sys.begin_scene(default_params(**sc.params))
        W.apply_to(W.Scene(sc.name, sc.params, sc.pos_w, sc.phase, vel=sc.vel, pairs=sc.pairs + off[k],
                           rest=sc.rest, stiffness=sc.stiffness, pins=sc.pins + off[k], pin_points=sc.pin_points),
                   sys)
    dev = torch.device("cuda", 0)
    st = torch.tensor(np.concatenate([sc.stiffness for sc in scenes]), device=dev, requires_grad=True)
    x0 = torch.tensor(np.concatenate([sc.pos_w for sc in scenes]), device=dev, requires_grad=True)
    v0 = torch.tensor(np.concatenate([sc.vel for sc in scenes]), device=dev, requires_grad=True)
    xT, _ = rollout(sys, st, x0, v0, 1.0 / 60.0, 8, 3)
    (xT[:, :3] * torch.tensor(np.concatenate(cs), dtype=torch.float32, device=dev)).sum().backward()
    m0 = len(scenes[0].pairs)
    gs, gx, gv = st.grad.cpu().numpy(), x0.grad.cpu().numpy()[:, :3], v0.grad.cpu().numpy()[:, :3]
    for k, sc in enumerate(scenes):
        sl = slice(off[k], off[k] + sc.n)
        ss = slice(0, m0) if k == 0 else slice(m0, None)
        for a, b in ((gs[ss], alone[k][0]), (gx[sl], alone[k][1]), (gv[sl], alone[k][2])):
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5 * np.max(np.abs(b)))


def test_backward_is_deterministic_and_restores_state():
    sc = small_scene()
    sys = ParticleSystem(default_params(**sc.params), sc.n)
    W.apply_to(sc, sys)
    sys.rollout(sc.dt, 7, 3)
    end = sys.positions()
    dev = torch.device("cuda", 0)
    g = torch.randn((sc.n, 4), device=dev)
    outs = []
    for _ in range(2):
        dx0 = torch.empty((sc.n, 4), device=dev)
        dv0 = torch.empty((sc.n, 4), device=dev)
        ds = torch.empty(len(sc.pairs), device=dev)
        sys.backward_device(g.data_ptr(), None, dx0.data_ptr(), dv0.data_ptr(), ds.data_ptr())
        torch.cuda.synchronize()
        outs.append((dx0.cpu().numpy(), dv0.cpu().numpy(), ds.cpu().numpy()))
        np.testing.assert_array_equal(sys.positions(), end)
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)


def fluid_scene(xsph):
    """A PBF block with the smooth delta divisor (PBD_FLAG_DELTA_OVER_RHO0:
    the reference's rho0 + n jumps whenever a neighbour count changes, so
    central differences of a fluid step only converge without it)."""
    from particlesolver_gb300 import FLAG_DELTA_OVER_RHO0

    sc = W.dam_break(8, 8, 6, xsph=xsph)
    sc.params["flags"] = sc.params["flags"] | FLAG_DELTA_OVER_RHO0
    return sc


@pytest.mark.parametrize("xsph,steps,every", [(0.0, 1, 1), (0.0, 3, 2), (0.01, 3, 2)])
def test_fluid_gradient_matches_fd(xsph, steps, every):
    """PBF density / lambda, the fluid delta with s_corr, walls, XSPH and
    the integrator (eps 1e-6: the oracle's central differences agree to 6
    digits from 1e-6 down)."""
    check_directional(fluid_scene(xsph), steps, every, seed=7 + steps, eps=1e-6)


def test_fluid_on_solid_gradient_matches_fd():
    """Fluid falling onto solid grains: lambda and delta over neighbours of
    both phases, contacts of the grains with the fluid."""
    from particlesolver_gb300 import FLAG_DELTA_OVER_RHO0

    sc = W.dam_break(8, 8, 4, xsph=0.01)
    sc.params["flags"] = sc.params["flags"] | FLAG_DELTA_OVER_RHO0
    n = sc.n
    pos = sc.pos_w.copy()
    pos[:, 1] += 0.06
    grains = np.stack(np.meshgrid(np.arange(8), np.arange(4), indexing="ij"), -1).reshape(-1, 2)
    gpos = np.zeros((len(grains), 4), np.float32)
    gpos[:, 0] = 0.03 + grains[:, 0] * 0.055  # apart (contact at 2.001 r = 0.050025)
    gpos[:, 1] = 0.026                         # just above the floor clamp (r = 0.025)
    gpos[:, 2] = 0.03 + grains[:, 1] * 0.055
    gpos[:, 3] = 1.0
    sc = W.Scene("fluid_on_grains", sc.params, np.concatenate([pos, gpos]),
                 np.concatenate([sc.phase, np.full(len(gpos), W.PHASE_SOLID, np.int32)]),
                 rest_density=np.concatenate([sc.rest_density, np.ones(len(gpos), np.float32)]), dt=sc.dt)
    assert sc.n == n + len(gpos)
    check_directional(sc, 3, 2, seed=21, eps=1e-6)
    sc.params["solid_density_weight"] = 0.5  # fluid-solid coupling weight
    # (the oracle's central difference crosses a neighbour switch at 1e-6 here
    # and has converged at 1e-7 and 1e-8: 18.25987 both)
    check_directional(sc, 3, 2, seed=22, eps=1e-7)


def spinning_boxes(stiffness, seed=5):
    sc = W.rigid_boxes(count=3, stiffness=stiffness)
    rng = np.random.default_rng(seed)
    vel = np.zeros((sc.n, 4), np.float32)
    for f, cnt, _ in sc.bodies:
        w = rng.standard_normal(3) * 2.0
        r = sc.pos_w[f:f + cnt, :3] - sc.pos_w[f:f + cnt, :3].mean(0)
        vel[f:f + cnt, :3] = rng.standard_normal(3) + np.cross(w, r)
    sc.vel = vel
    return sc


@pytest.mark.parametrize("stiffness,steps", [(1.0, 1), (1.0, 4), (0.6, 4)])
def test_shape_matching_gradient_matches_fd(stiffness, steps):
    """Shape matching of spinning boxes: the adjoint of the centre of mass
    and of the polar rotation (tr S I - S) y = vee(R^T Rbar - Rbar^T R)."""
    check_directional(spinning_boxes(stiffness), steps, 2, seed=30 + steps)


def test_unsupported_and_state_errors():
    sys2 = ParticleSystem(default_params(**small_scene().params), 10)
    with pytest.raises(PbdError):
        sys2.backward_device(None, None, None, None, None)  # no rollout yet
