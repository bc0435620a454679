"""ctypes wrapper of oracle/_ref/librefcpu.so: the reference's own 2-D CPU
solver (cpu/src, built headless by oracle/ref_build.py where the reference
tree exists).  Test infrastructure only: a timed CPU baseline and an
invariant comparison for the 2-D granular column.  The reference's
sources do not travel to machines without the tree, so it is absent
there and callers skip."""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_ref" / "librefcpu.so"
_lib = None


def available() -> bool:
    if not LIB.exists():
        return False
    try:
        load()
        return True
    except OSError:
        return False


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(LIB))
        D, P, I = ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        PD = ctypes.POINTER(ctypes.c_double)
        lib.refcpu_create.argtypes = [D, D, D, D, D, D]
        lib.refcpu_create.restype = P
        lib.refcpu_add_particles.argtypes = [P, I, PD, PD, D, D, D]
        lib.refcpu_finalize.argtypes = [P]
        lib.refcpu_tick.argtypes = [P, D, I]
        lib.refcpu_num.argtypes = [P]
        lib.refcpu_num.restype = I
        lib.refcpu_get.argtypes = [P, PD, PD]
        lib.refcpu_destroy.argtypes = [P]
        lib.refcpu_gas_project.argtypes = [I, PD, PD, PD, ctypes.POINTER(ctypes.c_int), D, I, I, PD, PD]
        PI = ctypes.POINTER(ctypes.c_int)
        lib.refcpu_rigid_contacts.argtypes = [I, PD, PD, PD, PI, PD, I, PD, I, PI, D, D, PD]
        lib.refcpu_fluid_project.argtypes = [I, PD, PD, PI, PI, D, I, PD, PD]
        lib.refcpu_fluid_emitter_tick.argtypes = [I, I, PD, PD, PD, PD, PD, D, D, D, PD, D, ctypes.c_uint, PD, PD,
                                                  PD, PI, I, PD, PD]
        lib.refcpu_fluid_emitter_tick.restype = I
        lib.refcpu_contacts.argtypes = [I, PD, PD, PD, PI, I, PI, I, PI, D, D, D, D, D, D, PD]
        lib.refcpu_smoke_emitter_tick.argtypes = [I, D, D, D, D, I, PI, I, PD, PD, PI, PI]
        lib.refcpu_smoke_emitter_tick.restype = I
        _lib = lib
    return _lib


class RefCPU:
    """The reference's Simulation with a scene of solid particles (x, y);
    particle radius fixed at 0.25 and 3 solver iterations, as compiled."""

    def __init__(self, xy, v=None, mass=1.0, s_friction=0.5, k_friction=0.3, x_bounds=(-20.0, 20.0),
                 y_bounds=(0.0, 1e6), gravity=(0.0, -9.8)):
        self.lib = load()
        self.h = self.lib.refcpu_create(x_bounds[0], x_bounds[1], y_bounds[0], y_bounds[1], *gravity)
        xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
        vv = None if v is None else np.ascontiguousarray(v, np.float64).reshape(-1, 2)
        pd = ctypes.POINTER(ctypes.c_double)
        self.lib.refcpu_add_particles(self.h, xy.shape[0], xy.ctypes.data_as(pd),
                                      None if vv is None else vv.ctypes.data_as(pd), mass, s_friction, k_friction)
        self.lib.refcpu_finalize(self.h)

    def tick(self, dt: float, steps: int = 1):
        self.lib.refcpu_tick(self.h, dt, steps)

    def state(self):
        n = self.lib.refcpu_num(self.h)
        xy = np.empty((n, 2))
        v = np.empty((n, 2))
        pd = ctypes.POINTER(ctypes.c_double)
        self.lib.refcpu_get(self.h, xy.ctypes.data_as(pd), v.ctypes.data_as(pd))
        return xy, v

    def close(self):
        if getattr(self, "h", None):
            self.lib.refcpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gas_project(xy, v, imass, solid, density: float, open_: bool, iterations: int):
    """The reference's GasConstraint::project run `iterations` times on 2-D
    particles (solid[i] != 0: SOLID neighbour, else gas); returns the
    estimates and forces, (n, 2) each."""
    lib = load()
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
    n = xy.shape[0]
    v = np.ascontiguousarray(v, np.float64).reshape(n, 2)
    imass = np.ascontiguousarray(imass, np.float64).reshape(n)
    solid = np.ascontiguousarray(solid, np.int32).reshape(n)
    out_x = np.empty((n, 2))
    out_f = np.empty((n, 2))
    pd = ctypes.POINTER(ctypes.c_double)
    lib.refcpu_gas_project(n, xy.ctypes.data_as(pd), v.ctypes.data_as(pd), imass.ctypes.data_as(pd),
                           solid.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), float(density), int(bool(open_)),
                           int(iterations), out_x.ctypes.data_as(pd), out_f.ctypes.data_as(pd))
    return out_x, out_f


def rigid_contacts(p, ep, imass, body, sdf, angles, pairs, s_friction: float, k_friction: float):
    """The reference's RigidContactConstraint::project, once per listed pair
    (i1 < i2), on 2-D SOLID particles with start positions p and estimates
    ep, (n, 2) each; body[i] (-1 = none) with signed-distance data sdf (n, 3:
    rest-frame normal x, y, depth) and body angles.  Returns the estimates."""
    lib = load()
    p = np.ascontiguousarray(p, np.float64).reshape(-1, 2)
    n = p.shape[0]
    ep = np.ascontiguousarray(ep, np.float64).reshape(n, 2)
    imass = np.ascontiguousarray(imass, np.float64).reshape(n)
    body = np.ascontiguousarray(body, np.int32).reshape(n)
    sdf = np.ascontiguousarray(sdf, np.float64).reshape(n, 3)
    angles = np.ascontiguousarray(angles, np.float64).reshape(-1)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    out = np.empty((n, 2))
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int)
    lib.refcpu_rigid_contacts(n, p.ctypes.data_as(pd), ep.ctypes.data_as(pd), imass.ctypes.data_as(pd),
                              body.ctypes.data_as(pi), sdf.ctypes.data_as(pd), angles.shape[0],
                              angles.ctypes.data_as(pd), pairs.shape[0], pairs.ctypes.data_as(pi),
                              float(s_friction), float(k_friction), out.ctypes.data_as(pd))
    return out


def fluid_project(xy, imass, fluid, density: float, iterations: int, counts=None):
    """The reference's TotalFluidConstraint::project run `iterations` times
    on 2-D particles (fluid[i] != 0: member of one fluid of rest density
    `density`, else SOLID; imass 0 = fixed; counts: other constraints per
    particle, default zero).  Returns the estimates (n, 2) and the last
    call's lambdas (n,)."""
    lib = load()
    xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
    n = xy.shape[0]
    imass = np.ascontiguousarray(imass, np.float64).reshape(n)
    fluid = np.ascontiguousarray(fluid, np.int32).reshape(n)
    cnt = None if counts is None else np.ascontiguousarray(counts, np.int32).reshape(n)
    out_x = np.empty((n, 2))
    out_l = np.empty(n)
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int)
    lib.refcpu_fluid_project(n, xy.ctypes.data_as(pd), imass.ctypes.data_as(pd), fluid.ctypes.data_as(pi),
                             None if cnt is None else cnt.ctypes.data_as(pi), float(density), int(iterations),
                             out_x.ctypes.data_as(pd), out_l.ctypes.data_as(pd))
    return out_x, out_l


def fluid_emitter_tick(p, v, imass, t, lambdas, members: int, position, rate: float, clocks, secs: float,
                       seed: int = 1, max_new: int = 1024):
    """One FluidEmitter::tick of the reference on 2-D particles (the first
    `members` are the emitter fluid's members, in order, with the given
    lambdas).  Returns a dict: v, imass, t, fluid (after the tick), clocks
    (timer, totalTimer) and the emitted particles' p and v."""
    lib = load()
    p = np.ascontiguousarray(p, np.float64).reshape(-1, 2)
    n = p.shape[0]
    v = np.ascontiguousarray(v, np.float64).reshape(n, 2)
    imass = np.ascontiguousarray(imass, np.float64).reshape(n)
    t = np.ascontiguousarray(t, np.float64).reshape(n)
    lam = np.ascontiguousarray(lambdas, np.float64).reshape(-1)
    clk = np.ascontiguousarray(clocks, np.float64).reshape(2).copy()
    v_out, im_out, t_out = np.empty((n, 2)), np.empty(n), np.empty(n)
    ph_out = np.empty(n, np.int32)
    new_p, new_v = np.empty((max_new, 2)), np.empty((max_new, 2))
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int)
    k = lib.refcpu_fluid_emitter_tick(n, int(members), p.ctypes.data_as(pd), v.ctypes.data_as(pd),
                                      imass.ctypes.data_as(pd), t.ctypes.data_as(pd), lam.ctypes.data_as(pd),
                                      float(position[0]), float(position[1]), float(rate), clk.ctypes.data_as(pd),
                                      float(secs), int(seed), v_out.ctypes.data_as(pd), im_out.ctypes.data_as(pd),
                                      t_out.ctypes.data_as(pd), ph_out.ctypes.data_as(pi), int(max_new),
                                      new_p.ctypes.data_as(pd), new_v.ctypes.data_as(pd))
    k = min(k, max_new)
    return {"v": v_out, "imass": im_out, "t": t_out, "fluid": ph_out == 1, "clocks": clk,
            "new_p": new_p[:k], "new_v": new_v[:k]}


def smoke_emitter_ticks(n: int, position, rate: float, secs: float, ticks: int, max_new: int = 4096):
    """`ticks` OpenSmokeEmitter::tick calls of the reference (with its gas
    constraint) after an estimates list of n particles.  Returns a dict:
    counts per tick, and the appended particles' p, imass, gas (phase GAS)
    and member (index taken by the gas constraint)."""
    lib = load()
    counts = np.zeros(ticks, np.int32)
    new_p, new_im = np.empty((max_new, 2)), np.empty(max_new)
    gas, member = np.empty(max_new, np.int32), np.empty(max_new, np.int32)
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int)
    k = lib.refcpu_smoke_emitter_tick(int(n), ctypes.c_double(position[0]), ctypes.c_double(position[1]),
                                      ctypes.c_double(rate), ctypes.c_double(secs), int(ticks),
                                      counts.ctypes.data_as(pi), int(max_new), new_p.ctypes.data_as(pd),
                                      new_im.ctypes.data_as(pd), gas.ctypes.data_as(pi), member.ctypes.data_as(pi))
    k = min(k, max_new)
    return {"counts": counts, "new_p": new_p[:k], "new_imass": new_im[:k], "gas": gas[:k] == 1,
            "member": member[:k] == 1}


def contacts(p, ep, imass, solid, pairs, walls, box, s_friction: float, k_friction: float):
    """The reference's contact projectors once each, in order: the listed
    pairs (i1 < i2; RigidContactConstraint between two SOLID particles,
    else ContactConstraint), then the listed walls (idx, is_x, lower) as
    BoundaryConstraint of the box (xmin, xmax, ymin, ymax); start positions
    p and estimates ep (n, 2).  Returns the estimates."""
    lib = load()
    p = np.ascontiguousarray(p, np.float64).reshape(-1, 2)
    n = p.shape[0]
    ep = np.ascontiguousarray(ep, np.float64).reshape(n, 2)
    imass = np.ascontiguousarray(imass, np.float64).reshape(n)
    solid = np.ascontiguousarray(solid, np.int32).reshape(n)
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    walls = np.ascontiguousarray(walls, np.int32).reshape(-1, 3)
    out = np.empty((n, 2))
    pd = ctypes.POINTER(ctypes.c_double)
    pi = ctypes.POINTER(ctypes.c_int)
    lib.refcpu_contacts(n, p.ctypes.data_as(pd), ep.ctypes.data_as(pd), imass.ctypes.data_as(pd),
                        solid.ctypes.data_as(pi), pairs.shape[0], pairs.ctypes.data_as(pi), walls.shape[0],
                        walls.ctypes.data_as(pi), float(box[0]), float(box[1]), float(box[2]), float(box[3]),
                        float(s_friction), float(k_friction), out.ctypes.data_as(pd))
    return out
