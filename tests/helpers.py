"""Shared helpers of the test suite (parameter structs, error metrics)."""
from __future__ import annotations

import numpy as np

REF_BASE = dict(particle_radius=0.25, kernel_radius=2.0, cell_size=0.5, grid_size=[64, 64, 64],
                world_origin=[0, 0, 0], gravity=[0, -9.8, 0], box_min=[-50, 0, -50], box_max=[50, 200, 50],
                iterations=5, max_dt=0.05, relaxation=0.01, scorr_k=0.1, scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0,
                contact_static_friction=0.005, contact_kinetic_friction=0.0002, wall_static_friction=0.005,
                wall_kinetic_friction=0.0002, max_neighbors=500, twod_z=0.0, flags=0)


def params_nolib(d: dict | None = None):
    """pbd_params filled without loading the CUDA library (CPU tests)."""
    from particlesolver_gb300 import PbdParams

    base = dict(REF_BASE)
    base.update(d or {})
    return PbdParams().update(**base)


def norm_err(a, b) -> float:
    """max_i |a_i - b_i| / max_i |b_i| over all components (vectors flattened)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / scale)


def displacement(after, before) -> np.ndarray:
    return np.asarray(after, np.float64)[:, :3] - np.asarray(before, np.float64)[:, :3]


def assert_projection(after_gpu, after_64, before, rel: float = 1e-5):
    """One projection of the FP32 path against the FP64 replay: every
    component of the correction agrees to rel * max|correction| plus one
    FP32 ulp of the stored coordinate (the FP32 result is a rounded
    position; the replay's is exact)."""
    d_g = displacement(after_gpu, before)
    d_o = displacement(after_64, before)
    coord = np.abs(np.asarray(after_64, np.float64)[:, :3]).astype(np.float32)
    ulp = np.spacing(coord).astype(np.float64)
    bound = rel * np.max(np.abs(d_o)) + ulp
    excess = np.abs(d_g - d_o) - bound
    worst = np.unravel_index(np.argmax(excess), excess.shape)
    assert np.max(excess) <= 0.0, (
        f"correction error {np.abs(d_g - d_o)[worst]:.3e} at {worst} exceeds {bound[worst]:.3e} "
        f"(max correction {np.max(np.abs(d_o)):.3e}, normalised error {norm_err(d_g, d_o):.3e})")
    return norm_err(d_g, d_o)


def golden_scene(data):
    """Rebuild the Scene stored in a golden fixture."""
    from particlesolver_gb300 import workloads as W

    pos_w = data["pos_w"]
    params = dict(W.reference_scene_params(iterations=int(data["iterations"])))
    return W.Scene("golden", params, pos_w, data["phase"],
                   rest_density=data["rest_density"] if "rest_density" in data else None,
                   pairs=data["pairs"] if "pairs" in data else None,
                   rest=data["rest"] if "rest" in data else None,
                   pins=data["pins"] if "pins" in data else None,
                   pin_points=data["pin_points"] if "pin_points" in data else None,
                   dt=float(data["dt"]))


def run_stages(system) -> dict:
    """One iteration stage by stage on a freshly loaded system (x_old = the
    start positions), in the reference's order (particlesystem.cpp:171-232)."""
    out = {}
    system.build_grid()
    sh, si, cs, ce = system.grid()
    out.update(grid_hash=sh, grid_index=si, cell_start=cs, cell_end=ce)
    system.collide()
    out["after_collide"] = system.positions()
    system.solve_fluids()
    out["after_fluids"] = system.positions()
    out["lambda"] = system.lambdas()
    system.collide_world()
    out["after_world"] = system.positions()
    system.solve_distance_constraints()
    out["after_distance"] = system.positions()
    system.solve_point_constraints()
    out["after_points"] = system.positions()
    return out


STAGE_KEYS = ["after_collide", "after_fluids", "after_world", "after_distance", "after_points"]


def check_against_golden(out: dict, gold, start, tol: float = 5e-5):
    """Compare stage outputs of a system with a golden fixture: grid
    bit-exact, lambda and each stage's displacement within tol (normalised)."""
    np.testing.assert_array_equal(out["grid_hash"], gold["grid_hash"])
    np.testing.assert_array_equal(out["grid_index"], gold["grid_index"])
    np.testing.assert_array_equal(out["cell_start"], gold["cell_start"])
    np.testing.assert_array_equal(out["cell_end"], gold["cell_end"])
    assert norm_err(out["lambda"], gold["lambda"]) < max(tol, 1e-5) or np.max(np.abs(gold["lambda"])) == 0
    prev = start
    for k in STAGE_KEYS:
        d_out = displacement(out[k], prev)
        d_gold = displacement(gold[k], prev)
        if np.max(np.abs(d_gold)) > 0:
            assert norm_err(d_out, d_gold) < tol, k
        else:
            assert np.max(np.abs(d_out)) < 1e-6, k
        prev = gold[k]


def check_trajectory(pos, gold_pos, start, pct_tol=1e-3):
    """Invariant-style comparison of positions after full updates."""
    d = displacement(pos, start)
    g = displacement(gold_pos, start)
    scale = np.max(np.abs(g))
    per = np.linalg.norm(d - g, axis=1) / scale
    assert np.percentile(per, 90) < pct_tol
    assert np.max(np.abs(d.mean(0) - g.mean(0))) / scale < pct_tol


def check_granular(pos, gold_pos, rel: float):
    """Invariants of a granular pile, whose particle trajectories are
    chaotic (contacts switch at the 2.001 r threshold, friction switches
    static / kinetic): the mean height and the horizontal spread agree to
    rel, and every particle is finite."""
    p = np.asarray(pos, np.float64)[:, :3]
    g = np.asarray(gold_pos, np.float64)[:, :3]
    assert np.all(np.isfinite(p))
    mean_y, gmean_y = p[:, 1].mean(), g[:, 1].mean()
    assert abs(mean_y - gmean_y) <= rel * abs(gmean_y), (mean_y, gmean_y)
    sx, gsx = p[:, 0].std(), g[:, 0].std()
    assert abs(sx - gsx) <= rel * gsx, (sx, gsx)


def oracle_gas_projection(pos_w, phase, rest_density, vel, params: dict, open_: bool, calls: int):
    """The oracle's gas passes run `calls` times from the given positions
    and step velocities (grid build + lambda / delta, no prediction and no
    walls): the counterpart of one GasConstraint::project per call.  Returns
    the positions and forces, (n, 2) each."""
    from oracle import Oracle

    p = params_nolib(params)
    n = len(pos_w)
    o = Oracle(p, n)
    o.add_particles(pos_w, vel, phase, rest_density)
    if open_:
        o.set_gas_open(0, n, True)
    for _ in range(calls):
        o.build_grid()
        o.solve_fluids()
    return o.positions()[:, :2], o.forces()[:, :2]


def fluid_projection(system, calls: int):
    """The fluid passes of a loaded system (oracle or CUDA) run `calls`
    times (grid build + lambda / delta, no prediction and no walls): the
    counterpart of one TotalFluidConstraint::project per call.  Returns the
    positions (n, 2) and the last call's lambdas."""
    for _ in range(calls):
        system.build_grid()
        system.solve_fluids()
    return np.asarray(system.positions(), np.float64)[:, :2], np.asarray(system.lambdas(), np.float64)


def assert_gas_projection(pos, force, ref_pos, ref_force, start, gas, tol):
    """Gas displacements and forces within tol of the reference, relative to
    the largest of each; particles that are not gas stay where they were."""
    d_ref = ref_pos[gas] - start[gas]
    assert norm_err(pos[gas] - start[gas], d_ref) < tol
    assert norm_err(force[gas], ref_force[gas]) < tol
    assert np.max(np.abs(pos[~gas] - start[~gas])) == 0.0


SDF_PIN_PARAMS = dict(particle_radius=0.25, kernel_radius=1.0, cell_size=0.5, grid_size=[1024, 32, 4],
                      world_origin=[-5.0, 0.0, -1.0], gravity=[0.0, 0.0, 0.0], box_min=[-100.0, -100.0, -1.0],
                      box_max=[1000.0, 100.0, 1.0], iterations=1, max_dt=1.0, contact_static_friction=0.4,
                      contact_kinetic_friction=0.3, twod_z=0.0, max_neighbors=500, flags=1)


def load_sdf_pin(system, case, fp32_inputs: bool = False):
    """One contact pass of the 2-D signed-distance pinning case
    (workloads.sdf_contact_pairs) on `system` (the CUDA system or the
    oracle: same methods).  Each body is added in a rest frame within 0.7
    rad of its target angle (its sdf normals rotated with it) and posed at
    its target angle, every body centred at the origin -- one
    shape-matching pass there stores the remaining rotation, the pose
    being rigid and the coordinates small (FP32 shape matching far from
    the origin loses digits in the centred offsets); then the start
    positions are set and become x_old by a prediction at rest, the
    estimates are set and the grid and the contact pass run.  fp32_inputs
    rounds start and estimates to FP32 first, so that the CUDA path and the
    oracle see the same inputs.  Returns the positions (n, 2)."""
    from particlesolver_gb300 import workloads as W

    n = len(case["start"])
    nb = n // 4
    rot = lambda a, v: np.stack([np.cos(a) * v[:, 0] - np.sin(a) * v[:, 1],  # noqa: E731
                                 np.sin(a) * v[:, 0] + np.cos(a) * v[:, 1]], 1)
    phi = case["angles"] - W.uniform(77, (nb,), -0.7, 0.7)
    pos = np.zeros((n, 4))
    pos[:, 3] = case["imass"]
    sdf = np.zeros((n, 4))
    posed = pos.copy()
    for b in range(nb):
        k = slice(4 * b, 4 * b + 4)
        pos[k, :2] = rot(phi[b], case["lattice"][k])
        posed[k, :2] = rot(case["angles"][b], case["lattice"][k])
        sdf[k, :2] = rot(phi[b], case["sdf"][k, :2])
        sdf[k, 3] = case["sdf"][k, 3]
    system.add_particles(pos, None, (W.PHASE_RIGID + case["body"]).astype(np.int32), None)
    for b in range(nb):
        system.add_rigid_body(4 * b, 4, 1.0)
        system.set_rigid_sdf(b, sdf[4 * b:4 * b + 4])
    system.set_positions(posed)
    system.solve_shapes()
    rnd = (lambda a: a.astype(np.float32).astype(np.float64)) if fp32_inputs else (lambda a: a)  # noqa: E731
    st = pos.copy()
    st[:, :2] = case["start"]
    st = rnd(st)
    system.set_positions(st)
    system.set_velocities(np.zeros((n, 4)))
    system.integrate(1.0 / 60.0)
    est = st.copy()
    est[:, :2] = case["estimate"]
    est = rnd(est)
    system.set_positions(est)
    system.build_grid()
    system.collide()
    return np.asarray(system.positions(), np.float64)[:, :2]


def density_error(pos, rho0, h: float, sample=None, mass: float = 1.0):
    """Per-particle density error rho / rho0 - 1 (rho = sum of poly6 over
    the particles within h, the particle itself included, unit mass) for
    the particles `sample` (all if None), FP64 on the host."""
    from scipy.spatial import cKDTree

    x = np.asarray(pos, np.float64)[:, :3]
    idx = np.arange(len(x)) if sample is None else np.asarray(sample)
    c6 = 315.0 / (64.0 * np.pi * h ** 9)
    nb = cKDTree(x).query_ball_point(x[idx], r=h)
    rho = np.array([mass * np.sum(c6 * np.clip(h * h - np.sum((x[p] - x[i]) ** 2, 1), 0.0, None) ** 3)
                    for i, p in zip(idx, nb)])
    return rho / np.asarray(rho0, np.float64)[idx] - 1.0


def emitter_counts(rate: float, duration: float, dt: float, ticks: int) -> list:
    """Particles FluidEmitter::tick emits per tick (fluidemitter.cpp:69-76):
    a timer advanced by dt releases one particle per 1 / rate while the
    emitter's total time is below `duration` (the reference's 5 s; 0 = no
    limit, as OpenSmokeEmitter::tick, opensmokeemitter.cpp:17-28)."""
    timer = elapsed = 0.0
    out = []
    for _ in range(ticks):
        timer += dt
        elapsed += dt
        k = 0
        while (duration <= 0 or elapsed < duration) and timer >= 1.0 / rate:
            timer -= 1.0 / rate
            k += 1
        out.append(k)
    return out


def solidify_rule(y, speed_of, lam, timer, fluid, dt: float, speed: float = 0.06, height: float = 5.0):
    """FluidEmitter::tick's solidification (fluidemitter.cpp:14-51) for one
    tick: a fluid particle slower than `speed` at a height <= `height`
    counts its timer down by 1 while its lambda <= 0, else up by dt (to 3);
    at <= 0 (then set to 0) it turns solid.  Returns the new timers and the
    converted particles."""
    t = np.array(timer, np.float64, copy=True)
    act = np.asarray(fluid, bool) & (np.asarray(speed_of) < speed) & (np.asarray(y) <= height)
    down = act & (np.asarray(lam) <= 0)
    up = act & (np.asarray(lam) > 0)
    t[down] -= 1.0
    t[up] = np.minimum(t[up] + dt, 3.0)
    turn = down & (t <= 0)
    t[turn] = 0.0
    return t, turn


def cpu_contact_params(static_friction: float = 0.4, kinetic_friction: float = 0.3) -> dict:
    """Parameters of the CPU-contact pinning case (workloads.cpu_contact_case):
    2-D, PBD_FLAG_CPU_CONTACTS, its box, no gravity, r = 0.25."""
    from particlesolver_gb300 import workloads as W

    xmin, xmax, ymin, ymax = W.CPU_CONTACT_BOX
    return dict(particle_radius=0.25, kernel_radius=1.0, cell_size=0.5, grid_size=[1024, 128, 1],
                world_origin=[xmin, ymin, -1.0], gravity=[0.0, 0.0, 0.0], box_min=[xmin, ymin, -1.0],
                box_max=[xmax, ymax, 1.0], iterations=1, max_dt=1.0, contact_static_friction=static_friction,
                contact_kinetic_friction=kinetic_friction, wall_static_friction=static_friction,
                wall_kinetic_friction=kinetic_friction, twod_z=0.0, max_neighbors=500,
                flags=W.FLAG_TWOD | W.FLAG_CPU_CONTACTS)


def load_cpu_contact_pin(system, case, fp32_inputs: bool = False):
    """One contact and wall pass of the CPU-contact pinning case on `system`
    (the CUDA system or the oracle): the start positions become x_old by a
    prediction at rest, then the estimates are set and the grid, the
    contact pass and the wall pass run.  fp32_inputs rounds the inputs to
    FP32 first.  Returns the positions (n, 2)."""
    from particlesolver_gb300 import workloads as W

    n = len(case["start"])
    rnd = (lambda a: a.astype(np.float32).astype(np.float64)) if fp32_inputs else (lambda a: a)  # noqa: E731
    st = np.zeros((n, 4))
    st[:, :2] = case["start"]
    st[:, 3] = case["imass"]
    st = rnd(st)
    phase = np.where(case["solid"] != 0, W.PHASE_SOLID, W.PHASE_FLUID).astype(np.int32)
    system.add_particles(st, None, phase, None)
    system.set_velocities(np.zeros((n, 4)))
    system.integrate(1.0 / 60.0)
    est = st.copy()
    est[:, :2] = case["estimate"]
    est = rnd(est)
    system.set_positions(est)
    system.build_grid()
    system.collide()
    system.collide_world()
    return np.asarray(system.positions(), np.float64)[:, :2]


def pile_invariants(xy) -> dict:
    """Invariants of a 2-D granular pile, whose particle trajectories are
    chaotic: mean height, horizontal spread (standard deviation of x),
    runout (largest |x|) and the 99th percentile of the height."""
    xy = np.asarray(xy, np.float64)
    return {"mean_height": float(xy[:, 1].mean()), "spread": float(xy[:, 0].std()),
            "runout": float(np.abs(xy[:, 0]).max()), "top": float(np.percentile(xy[:, 1], 99))}
