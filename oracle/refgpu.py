"""ctypes wrapper of oracle/_ref/librefgpu.so: the reference's own GPU kernels
run on the CPU (test infrastructure; only where the reference tree exists)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _b

_LIB = None


def available() -> bool:
    return _b.reference_available()


def load():
    global _LIB
    if _LIB is None:
        paths = _b.build_reference()
        lib = ctypes.CDLL(str(paths["refgpu"]))
        P, U = ctypes.c_void_p, ctypes.c_uint32
        PF = ctypes.POINTER(ctypes.c_float)
        PU = ctypes.POINTER(ctypes.c_uint32)
        PI = ctypes.POINTER(ctypes.c_int32)
        sig = {
            "refgpu_create": ([ctypes.c_float, U, U, U, PI, PI, ctypes.c_int], P),
            "refgpu_destroy": ([P], None),
            "refgpu_add_particles": ([P, U, PF, PF, PF, PF, PI], None),
            "refgpu_add_points": ([P, U, PU, PF], None),
            "refgpu_add_distances": ([P, U, PU, PF], None),
            "refgpu_set_rands": ([P, PF], None),
            "refgpu_integrate": ([P, ctypes.c_float], None),
            "refgpu_grid": ([P], None),
            "refgpu_collide": ([P], None),
            "refgpu_solve_fluids": ([P], None),
            "refgpu_collide_world": ([P], None),
            "refgpu_solve_distances": ([P], None),
            "refgpu_solve_points": ([P], None),
            "refgpu_calc_velocity": ([P, ctypes.c_float], None),
            "refgpu_update": ([P, ctypes.c_float], None),
            "refgpu_num_particles": ([P], U),
            "refgpu_get_positions": ([P, PF], None),
            "refgpu_get_velocities": ([P, PF], None),
            "refgpu_set_positions": ([P, PF], None),
            "refgpu_get_grid": ([P, PU, PU, PU, PU], None),
            "refgpu_get_lambdas_sorted": ([P, PF], None),
            "refgpu_get_num_neighbors_sorted": ([P, PU], None),
        }
        for name, (a, r) in sig.items():
            f = getattr(lib, name)
            f.argtypes = a
            f.restype = r
        _LIB = lib
    return _LIB


def _pf(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _pu(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


class RefGPU:
    """The reference ParticleSystem step (GPU kernels on the CPU, FP32)."""

    def __init__(self, radius, grid_size, min_bounds, max_bounds, iterations):
        self.lib = load()
        mn = (ctypes.c_int32 * 3)(*min_bounds)
        mx = (ctypes.c_int32 * 3)(*max_bounds)
        self.s = self.lib.refgpu_create(radius, grid_size[0], grid_size[1], grid_size[2], mn, mx, iterations)
        self.cells = int(np.prod(grid_size))

    def close(self):
        if self.s:
            self.lib.refgpu_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        return int(self.lib.refgpu_num_particles(self.s))

    def add_particles(self, pos_w, vel=None, phase=None, rest_density=None):
        """pos_w carries the inverse mass in w, as the pbd ABI does; the
        reference keeps w = 1 in its position buffer and W separately."""
        pos_w = np.asarray(pos_w, np.float32).reshape(-1, 4)
        n = pos_w.shape[0]
        pos = np.ascontiguousarray(pos_w.copy())
        w = np.ascontiguousarray(pos[:, 3].copy())
        pos[:, 3] = 1.0
        vel = np.zeros((n, 4), np.float32) if vel is None else np.ascontiguousarray(vel, np.float32).reshape(n, 4)
        ph = np.ascontiguousarray(np.zeros(n) if phase is None else phase, np.int32)
        ro = np.ascontiguousarray(np.ones(n) if rest_density is None else rest_density, np.float32)
        self.lib.refgpu_add_particles(self.s, n, _pf(pos), _pf(vel), _pf(w), _pf(ro),
                                      ph.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))

    def add_distance_constraints(self, pairs, rest):
        pairs = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
        rest = np.ascontiguousarray(rest, np.float32).reshape(-1)
        self.lib.refgpu_add_distances(self.s, pairs.shape[0], _pu(pairs), _pf(rest))

    def add_point_constraints(self, index, points):
        index = np.ascontiguousarray(index, np.uint32).reshape(-1)
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        self.lib.refgpu_add_points(self.s, index.shape[0], _pu(index), _pf(pts))

    def set_rands(self, r):
        r = np.ascontiguousarray(r, np.float32).reshape(6)
        self.lib.refgpu_set_rands(self.s, _pf(r))

    def __getattr__(self, name):
        stage = {"integrate": "refgpu_integrate", "build_grid": "refgpu_grid", "collide": "refgpu_collide",
                 "solve_fluids": "refgpu_solve_fluids", "collide_world": "refgpu_collide_world",
                 "solve_distances": "refgpu_solve_distances", "solve_points": "refgpu_solve_points",
                 "calc_velocity": "refgpu_calc_velocity", "update": "refgpu_update"}.get(name)
        if stage is None:
            raise AttributeError(name)
        fn = getattr(self.lib, stage)
        return lambda *a: fn(self.s, *a)

    def positions(self):
        out = np.empty((self.n, 4), np.float32)
        self.lib.refgpu_get_positions(self.s, _pf(out))
        return out

    def velocities(self):
        out = np.empty((self.n, 4), np.float32)
        self.lib.refgpu_get_velocities(self.s, _pf(out))
        return out

    def grid(self):
        n = self.n
        sh, si = np.empty(n, np.uint32), np.empty(n, np.uint32)
        cs, ce = np.empty(self.cells, np.uint32), np.empty(self.cells, np.uint32)
        self.lib.refgpu_get_grid(self.s, _pu(sh), _pu(si), _pu(cs), _pu(ce))
        return sh, si, cs, ce

    def lambdas(self):
        """lambda per particle (original order)."""
        n = self.n
        lam = np.empty(n, np.float32)
        self.lib.refgpu_get_lambdas_sorted(self.s, _pf(lam))
        _, si, _, _ = self.grid()
        out = np.empty(n, np.float32)
        out[si] = lam
        return out
