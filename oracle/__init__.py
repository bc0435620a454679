"""Oracle package: CPU restatement of the reference PBD step.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py, as the checker.  The product path
(particlesolver_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _buildmod

_LIB = None


def _pbd_params_type():
    from particlesolver_gb300 import PbdParams  # the shared parameter struct layout

    return PbdParams


_LIB_DUAL = None


def load(dual: bool = False):
    """The FP64 oracle, or (dual=True) the same source on dual numbers."""
    global _LIB, _LIB_DUAL
    if dual and _LIB_DUAL is not None:
        return _LIB_DUAL
    if not dual and _LIB is not None:
        return _LIB
    if True:
        path = _buildmod.build_oracle_dual() if dual else _buildmod.build_oracle()
        lib = ctypes.CDLL(str(path))
        P = ctypes.c_void_p
        PD = ctypes.POINTER(ctypes.c_double)
        PU = ctypes.POINTER(ctypes.c_uint32)
        PI = ctypes.POINTER(ctypes.c_int32)
        U = ctypes.c_uint32
        sig = {
            "orc_create": ([ctypes.POINTER(_pbd_params_type()), U], P),
            "orc_destroy": ([P], None),
            "orc_set_threads": ([ctypes.c_int], None),
            "orc_add_particles": ([P, U, PD, PD, PI, PD], ctypes.c_int),
            "orc_add_distance_constraints": ([P, U, PU, PD, PD], ctypes.c_int),
            "orc_add_point_constraints": ([P, U, PU, PD], ctypes.c_int),
            "orc_add_rigid_body": ([P, U, U, ctypes.c_double], ctypes.c_int),
            "orc_set_wall_jitter": ([P, PD], None),
            "orc_integrate": ([P, ctypes.c_double], None),
            "orc_build_grid": ([P], None),
            "orc_collide": ([P], None),
            "orc_solve_fluids": ([P], None),
            "orc_collide_world": ([P], None),
            "orc_solve_distance_constraints": ([P], None),
            "orc_solve_point_constraints": ([P], None),
            "orc_solve_shapes": ([P], None),
            "orc_calc_velocity": ([P, ctypes.c_double], None),
            "orc_apply_xsph": ([P], None),
            "orc_update": ([P, ctypes.c_double], None),
            "orc_num_particles": ([P], U),
            "orc_get_positions": ([P, PD], None),
            "orc_get_velocities": ([P, PD], None),
            "orc_set_positions": ([P, PD], None),
            "orc_set_velocities": ([P, PD], None),
            "orc_get_grid": ([P, PU, PU, PU, PU], None),
            "orc_get_lambdas": ([P, PD], None),
            "orc_get_neighbor_counts": ([P, PU, PU], None),
            "orc_set_gas_open": ([P, U, U, ctypes.c_int], None),
            "orc_get_forces": ([P, PD], None),
            "orc_set_forces": ([P, PD], None),
            "orc_set_rigid_sdf": ([P, U, PD], None),
        }
        if dual:
            sig["orc_seed_tangents"] = ([P, PD, PD, PD], None)
            sig["orc_get_tangents"] = ([P, PD, PD], None)
        for name, (a, r) in sig.items():
            f = getattr(lib, name)
            f.argtypes = a
            f.restype = r
        if dual:
            _LIB_DUAL = lib
        else:
            _LIB = lib
    return lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """FP64 replay of the reference step with the same stage API as the CUDA system."""

    _dual = False

    def __init__(self, params, capacity: int, threads: int = 0):
        self.lib = load(self._dual)
        self.lib.orc_set_threads(int(threads))
        self.params = params
        self.s = self.lib.orc_create(ctypes.byref(params), int(capacity))
        self.cells = params.grid_size[0] * params.grid_size[1] * params.grid_size[2]

    def close(self):
        if self.s:
            self.lib.orc_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_particles(self) -> int:
        return int(self.lib.orc_num_particles(self.s))

    def add_particles(self, pos_w, vel=None, phase=None, rest_density=None):
        pos, pp = _d(np.asarray(pos_w, np.float64).reshape(-1, 4))
        n = pos.shape[0]
        vp = None
        if vel is not None:
            vel, vp = _d(np.asarray(vel).reshape(n, 4))
        ph = np.ascontiguousarray(np.zeros(n) if phase is None else phase, dtype=np.int32)
        rp = None
        if rest_density is not None:
            rest_density, rp = _d(np.asarray(rest_density).reshape(n))
        rc = self.lib.orc_add_particles(self.s, n, pp, vp, ph.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), rp)
        if rc:
            raise RuntimeError(f"oracle add_particles failed ({rc})")

    def add_distance_constraints(self, pairs, rest, stiffness=None):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        rest, rp = _d(np.asarray(rest).reshape(-1))
        sp = None
        if stiffness is not None:
            stiffness, sp = _d(np.asarray(stiffness).reshape(-1))
        self.lib.orc_add_distance_constraints(self.s, pairs.shape[0],
                                              pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), rp, sp)

    def add_point_constraints(self, index, points):
        index = np.ascontiguousarray(index, dtype=np.uint32).reshape(-1)
        pts, pp = _d(np.asarray(points).reshape(-1, 3))
        self.lib.orc_add_point_constraints(self.s, index.shape[0],
                                           index.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), pp)

    def add_rigid_body(self, first, count, stiffness=1.0):
        self.lib.orc_add_rigid_body(self.s, first, count, stiffness)
        self._bodies = getattr(self, "_bodies", 0) + 1
        return self._bodies - 1

    def set_rigid_sdf(self, body, sdf):
        sdf, sp = _d(np.asarray(sdf, np.float64).reshape(-1, 4))
        self.lib.orc_set_rigid_sdf(self.s, int(body), sp)

    def set_wall_jitter(self, r):
        r, rp = _d(np.asarray(r).reshape(6))
        self.lib.orc_set_wall_jitter(self.s, rp)

    def integrate(self, dt):
        self.lib.orc_integrate(self.s, dt)

    def build_grid(self):
        self.lib.orc_build_grid(self.s)

    def collide(self):
        self.lib.orc_collide(self.s)

    def solve_fluids(self):
        self.lib.orc_solve_fluids(self.s)

    def collide_world(self):
        self.lib.orc_collide_world(self.s)

    def solve_distance_constraints(self):
        self.lib.orc_solve_distance_constraints(self.s)

    def solve_point_constraints(self):
        self.lib.orc_solve_point_constraints(self.s)

    def solve_shapes(self):
        self.lib.orc_solve_shapes(self.s)

    def calc_velocity(self, dt):
        self.lib.orc_calc_velocity(self.s, dt)

    def apply_xsph(self):
        self.lib.orc_apply_xsph(self.s)

    def update(self, dt):
        self.lib.orc_update(self.s, dt)

    def positions(self) -> np.ndarray:
        out = np.empty((self.num_particles, 4), np.float64)
        self.lib.orc_get_positions(self.s, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def velocities(self) -> np.ndarray:
        out = np.empty((self.num_particles, 4), np.float64)
        self.lib.orc_get_velocities(self.s, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def set_positions(self, pos):
        pos, pp = _d(np.asarray(pos).reshape(-1, 4))
        self.lib.orc_set_positions(self.s, pp)

    def set_velocities(self, vel):
        vel, vp = _d(np.asarray(vel).reshape(-1, 4))
        self.lib.orc_set_velocities(self.s, vp)

    def grid(self):
        n = self.num_particles
        sh, si = np.empty(n, np.uint32), np.empty(n, np.uint32)
        cs, ce = np.empty(self.cells, np.uint32), np.empty(self.cells, np.uint32)
        pu = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))  # noqa: E731
        self.lib.orc_get_grid(self.s, pu(sh), pu(si), pu(cs), pu(ce))
        return sh, si, cs, ce

    def lambdas(self) -> np.ndarray:
        out = np.empty(self.num_particles, np.float64)
        self.lib.orc_get_lambdas(self.s, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def set_gas_open(self, first: int, count: int, open_: bool = True):
        self.lib.orc_set_gas_open(self.s, int(first), int(count), int(bool(open_)))

    def forces(self) -> np.ndarray:
        out = np.empty((self.num_particles, 4), np.float64)
        self.lib.orc_get_forces(self.s, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def set_forces(self, f):
        f, fp = _d(np.asarray(f, np.float64).reshape(-1, 4))
        self.lib.orc_set_forces(self.s, fp)

    def neighbor_counts(self):
        n = self.num_particles
        f, c = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        pu = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))  # noqa: E731
        self.lib.orc_get_neighbor_counts(self.s, pu(f), pu(c))
        return f, c


class OracleDual(Oracle):
    """The oracle on forward-mode dual numbers: seed a direction in
    (positions, velocities, stiffness), run the same stages, read the exact
    directional derivative of the FP64 replay (branches as in the values)."""

    _dual = True

    def seed_tangents(self, dx=None, dv=None, dstiffness=None):
        n = self.num_particles
        args = []
        for a, shape in ((dx, (n, 4)), (dv, (n, 4))):
            if a is None:
                args.append(None)
                continue
            a = np.asarray(a, np.float64)
            if a.shape[-1] == 3:
                a = np.concatenate([a, np.zeros((n, 1))], 1)
            args.append(_d(a.reshape(shape))[0])
        st = None if dstiffness is None else _d(dstiffness)[0]
        ptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        self.lib.orc_seed_tangents(self.s, ptr(args[0]), ptr(args[1]), ptr(st))

    def tangents(self):
        n = self.num_particles
        dx = np.empty((n, 4))
        dv = np.empty((n, 4))
        self.lib.orc_get_tangents(self.s, _d(dx)[1], _d(dv)[1])
        return dx, dv
