"""Generates the golden fixtures of tests/golden/ from the reference's own
code: the reference GPU kernels and thrust functors compiled for the CPU
(oracle/_ref/librefgpu.so, built from gpu/src/cuda/*.cuh in the reference
tree), and the reference's 2-D CPU solver (oracle/_ref/librefcpu.so, built
from cpu/src).  Run where the reference sources exist:

    python tests/golden/make_golden.py

Each ref_*.npz fixture holds the seeded inputs of one small scene and the
reference's outputs after the grid build, each solver stage and full
updates.  gas_project.npz holds a 2-D smoke box with solid and fixed
neighbours and the outputs of the reference's GasConstraint::project
(gasconstraint.cpp:34-134) after 1 and 3 calls, open and closed: the
estimates and each particle's force.  sdf_contacts.npz holds 2-D body
pairs touching at one corner each and the reference's
RigidContactConstraint::project (rigidcontactconstraint.cpp:30-96) result.
fluid_project.npz holds a 2-D fluid box over a fixed plate and movable
grains and the reference's TotalFluidConstraint::project
(totalfluidconstraint.cpp:41-116) estimates and lambdas after 1 and 3
calls.  fluid_emitter.npz holds FluidEmitter::tick (fluidemitter.cpp:13-77)
emission counts over 40 ticks and one solidification tick of a seeded
state; smoke_emitter.npz OpenSmokeEmitter::tick (opensmokeemitter.cpp:
17-43) emission counts over 6 s of ticks at three rates.  cpu_contacts.npz holds 2-D grains each in one contact or wall
constraint and the reference's RigidContactConstraint / ContactConstraint /
BoundaryConstraint results; granular_pile.npz the reference Simulation's
granular column after 600 steps.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import refgpu  # noqa: E402
from particlesolver_gb300 import workloads as W  # noqa: E402


def ref_for(scene):
    p = scene.params
    r = refgpu.RefGPU(p["particle_radius"], p["grid_size"], [int(v) for v in p["box_min"]],
                      [int(v) for v in p["box_max"]], p["iterations"])
    r.add_particles(scene.pos_w, scene.vel, scene.phase, scene.rest_density)
    if scene.pairs is not None:
        r.add_distance_constraints(scene.pairs, scene.rest)
    if scene.pins is not None:
        r.add_point_constraints(scene.pins, scene.pin_points)
    return r


def scene_inputs(scene) -> dict:
    d = dict(pos_w=scene.pos_w, phase=scene.phase, dt=np.float32(scene.dt),
             iterations=np.int32(scene.params["iterations"]))
    if scene.rest_density is not None:
        d["rest_density"] = scene.rest_density
    if scene.pairs is not None:
        d.update(pairs=scene.pairs, rest=scene.rest)
    if scene.pins is not None:
        d.update(pins=scene.pins, pin_points=scene.pin_points)
    return d


def stage_outputs(scene) -> dict:
    """Reference outputs of one iteration, stage by stage, starting from the
    scene's positions (no prediction, so both sides share FP32 inputs)."""
    r = ref_for(scene)
    r.integrate(np.float32(1e-30))  # records x_old = start positions (no motion at dt ~ 0)
    r.lib.refgpu_set_positions(r.s, np.ascontiguousarray(
        np.where(np.arange(4) < 3, scene.pos_w, 1.0).astype(np.float32)).ctypes.data_as(
        refgpu.ctypes.POINTER(refgpu.ctypes.c_float)))
    out = {}
    r.build_grid()
    sh, si, cs, ce = r.grid()
    out.update(grid_hash=sh, grid_index=si, cell_start=cs, cell_end=np.where(cs != 0xFFFFFFFF, ce, 0))
    r.collide()
    out["after_collide"] = r.positions()
    r.solve_fluids()
    out["after_fluids"] = r.positions()
    out["lambda"] = r.lambdas()
    r.collide_world()
    out["after_world"] = r.positions()
    r.solve_distances()
    out["after_distance"] = r.positions()
    r.solve_points()
    out["after_points"] = r.positions()
    return out


def update_outputs(scene, steps: int) -> dict:
    r = ref_for(scene)
    out = {}
    for k in range(steps):
        r.update(np.float32(scene.dt))
        out[f"update{k + 1}_pos"] = r.positions()
        out[f"update{k + 1}_vel"] = r.velocities()
    return out


def scenes():
    return {
        "fluid": W.reference_fluid(ll=(-3, 0, -3), ur=(3, 5, 3), seed=21),
        "granular": W.reference_granular(ll=(-2, 0, -2), ur=(2, 4, 2), seed=22),
        "rope_cloth": W.rope_and_cloth(seed=23, cloth=(8, 6), ropes=3, links=10),
    }


def gas_fixture() -> dict:
    """Inputs and the reference's gas projection outputs (see the module
    docstring); velocities are seeded U(-1, 1) per axis."""
    from oracle import refcpu

    sc = W.smoke_box(twod=True, solid_floor=True, seed=1097)
    n = sc.n
    xy = sc.pos_w[:, :2].astype(np.float64)
    vel = np.zeros((n, 4), np.float32)
    vel[:, :2] = W.uniform(1098, (n, 2), -1.0, 1.0)
    imass = sc.pos_w[:, 3].astype(np.float64)
    solid = (sc.phase != W.PHASE_GAS).astype(np.int32)
    out = dict(pos_w=sc.pos_w, phase=sc.phase, rest_density=sc.rest_density, vel=vel)
    for open_ in (0, 1):
        for k in (1, 3):
            ex, f = refcpu.gas_project(xy, vel[:, :2].astype(np.float64), imass, solid, 1.5, bool(open_), k)
            out[f"open{open_}_k{k}_pos"] = ex
            out[f"open{open_}_k{k}_force"] = f
    return out


def sdf_fixture() -> dict:
    """The 2-D signed-distance pinning case (workloads.sdf_contact_pairs)
    and the reference's RigidContactConstraint::project estimates (static
    friction 0.4, kinetic 0.3)."""
    from oracle import refcpu

    case = W.sdf_contact_pairs(24)
    out = refcpu.rigid_contacts(case["start"], case["estimate"], case["imass"], case["body"],
                                case["sdf"][:, [0, 1, 3]], case["angles"], case["pairs"], 0.4, 0.3)
    return dict(case, reference=out)


def fluid_fixture() -> dict:
    """A 2-D fluid box over a fixed plate and movable grains
    (workloads.cpu_fluid_box) and the reference's
    TotalFluidConstraint::project estimates and lambdas after 1 and 3
    calls."""
    from oracle import refcpu

    sc = W.cpu_fluid_box(seed=890)
    fluid = (sc.phase == W.PHASE_FLUID).astype(np.int32)
    xy = sc.pos_w[:, :2].astype(np.float64)
    out = dict(pos_w=sc.pos_w, phase=sc.phase, rest_density=sc.rest_density)
    for k in (1, 3):
        ex, lam = refcpu.fluid_project(xy, sc.pos_w[:, 3].astype(np.float64), fluid, 1.75, k)
        out[f"k{k}_pos"] = ex
        out[f"k{k}_lambda"] = lam
    return out


def emitter_fixture() -> dict:
    """FluidEmitter::tick of the reference: the emission counts of 40 ticks
    (rate 33/s, dt 1/60) and the solidification of a seeded state of 400
    fluid members and 20 solids (velocities, timers, phases, inverse masses
    after the tick)."""
    from oracle import refcpu

    dt, rate = 1.0 / 60.0, 33.0
    clocks = np.zeros(2)
    counts = []
    for k in range(40):
        o = refcpu.fluid_emitter_tick(np.zeros((1, 2)), np.zeros((1, 2)), np.ones(1), np.full(1, 4.0), np.zeros(0),
                                      0, (0.5, 2.0), rate, clocks, dt, seed=k + 1)
        clocks = o["clocks"]
        counts.append(len(o["new_p"]))
    m, n = 400, 420
    p = np.stack([W.uniform(11, (n,), -5.0, 5.0), W.uniform(21, (n,), 3.0, 7.0)], 1)
    v = W.uniform(31, (n, 2), -0.06, 0.06)
    lam = W.uniform(41, (m,), -1.0, 1.0)
    t = W.uniform(51, (n,), 0.5, 4.0)
    o = refcpu.fluid_emitter_tick(p, v, np.ones(n), t, lam, m, (0.0, 100.0), 1.0, np.zeros(2), dt)
    return dict(dt=dt, rate=rate, counts=np.array(counts), members=m, p=p, v=v, lam=lam, t=t, t_out=o["t"],
                v_out=o["v"], imass_out=o["imass"], fluid_out=o["fluid"])


def smoke_fixture() -> dict:
    """OpenSmokeEmitter::tick of the reference: emission counts over 6 s of
    ticks at three rates and steps, and the emitted particles' inverse
    masses."""
    from oracle import refcpu

    out = {}
    for k, (rate, dt) in enumerate(((15.0, 1.0 / 60.0), (40.0, 1.0 / 120.0), (7.0, 0.05))):
        o = refcpu.smoke_emitter_ticks(5, (0.5, -2.0), rate, dt, int(np.ceil(6.0 / dt)))
        out[f"rate{k}"], out[f"dt{k}"], out[f"counts{k}"] = rate, dt, o["counts"]
        out[f"imass{k}"], out[f"gas{k}"] = o["new_imass"], o["gas"] & o["member"]
    return out


def contact_fixture() -> dict:
    """The CPU-contact pinning case (workloads.cpu_contact_case, seed 31,
    inputs rounded to FP32) and the reference's RigidContactConstraint /
    ContactConstraint / BoundaryConstraint estimates, with mu 0.4 / 0.3 and
    0.01 / 0.005."""
    from oracle import refcpu

    case = W.cpu_contact_case(seed=31)
    # inputs rounded to FP32 first, so that the CUDA path sees them exactly
    for key in ("start", "estimate", "imass"):
        case[key] = case[key].astype(np.float32).astype(np.float64)
    out = dict(case)
    for tag, fr in (("f1", (0.4, 0.3)), ("f2", (0.01, 0.005))):
        out[f"reference_{tag}"] = refcpu.contacts(case["start"], case["estimate"], case["imass"], case["solid"],
                                                  case["pairs"], case["walls"], W.CPU_CONTACT_BOX, *fr)
    return out


def pile_fixture() -> dict:
    """The 2-D granular column (1,600 grains) after 600 steps of the
    reference's own Simulation: positions."""
    from oracle import refcpu

    sc = W.granular_column(cpu_contacts=True)
    r = refcpu.RefCPU(sc.pos_w[:, :2], mass=1.0, s_friction=0.5, k_friction=0.3)
    r.tick(sc.dt, 600)
    return dict(start=sc.pos_w[:, :2], steps=600, positions=r.state()[0])


def main():
    if not refgpu.available():
        raise SystemExit("reference sources not found")
    from oracle import refcpu

    if refcpu.available():
        for name, fix in (("gas_project", gas_fixture), ("sdf_contacts", sdf_fixture),
                          ("fluid_project", fluid_fixture), ("fluid_emitter", emitter_fixture),
                          ("smoke_emitter", smoke_fixture),
                          ("cpu_contacts", contact_fixture), ("granular_pile", pile_fixture)):
            path = HERE / f"{name}.npz"
            np.savez_compressed(path, **fix())
            print(path, path.stat().st_size, "bytes")
    for name, sc in scenes().items():
        data = scene_inputs(sc)
        data.update(stage_outputs(sc))
        data.update(update_outputs(sc, 3))
        path = HERE / f"ref_{name}.npz"
        np.savez_compressed(path, **data)
        print(path, path.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
