"""GB300-native unified position-based-dynamics step (Python host binding).

Thin ctypes layer over ``libpbd_gb300.so`` (the C ABI in ``include/pbd.h``).
``ParticleSystem`` mirrors the reference class ``ParticleSystem``
(gpu/src/particlesystem.h:22-53): create with radius / grid / capacity /
bounds / iterations, add fluids, particle grids, cloths, ropes and static
spheres, ``update(dt)``, and read positions back.  There is no CPU fallback:
every call goes to the CUDA library, and importing the binding without it
raises.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np

from . import _build

__all__ = [
    "PbdParams", "PbdError", "ParticleSystem", "load_library", "default_params", "header_functions",
    "PHASE_FLUID", "PHASE_GAS", "PHASE_CLOTH", "PHASE_SOLID", "PHASE_RIGID",
    "FLAG_TWOD", "FLAG_DENSITY_NEIGHBOR_MASS", "FLAG_DELTA_OVER_RHO0", "FLAG_DISTANCE_MASS_WEIGHTED",
    "FLAG_KERNEL_UNITS", "FLAG_SKIP_FIXED_NEIGHBORS", "FLAG_DELTA_OVER_COUNT", "FLAG_CPU_CONTACTS", "PARAM_DEFAULTS", "host_params",
]

PHASE_FLUID, PHASE_GAS, PHASE_CLOTH, PHASE_SOLID, PHASE_RIGID = 0, 1, 2, 3, 4
FLAG_TWOD = 1 << 0
FLAG_DENSITY_NEIGHBOR_MASS = 1 << 1
FLAG_DELTA_OVER_RHO0 = 1 << 2
FLAG_DISTANCE_MASS_WEIGHTED = 1 << 3
FLAG_KERNEL_UNITS = 1 << 4
FLAG_SKIP_FIXED_NEIGHBORS = 1 << 5
FLAG_DELTA_OVER_COUNT = 1 << 6
FLAG_CPU_CONTACTS = 1 << 7

HEADER = _build.ROOT / "include" / "pbd.h"


ABI_VERSION = 3  # PBD_ABI_VERSION of include/pbd.h that these mirrors follow


class PbdParams(ctypes.Structure):
    """Mirror of ``pbd_params`` (include/pbd.h)."""

    _fields_ = [
        ("particle_radius", ctypes.c_float),
        ("kernel_radius", ctypes.c_float),
        ("cell_size", ctypes.c_float),
        ("grid_size", ctypes.c_uint32 * 3),
        ("world_origin", ctypes.c_float * 3),
        ("gravity", ctypes.c_float * 3),
        ("box_min", ctypes.c_float * 3),
        ("box_max", ctypes.c_float * 3),
        ("iterations", ctypes.c_uint32),
        ("max_dt", ctypes.c_float),
        ("relaxation", ctypes.c_float),
        ("scorr_k", ctypes.c_float),
        ("scorr_n", ctypes.c_float),
        ("scorr_dq", ctypes.c_float),
        ("xsph_c", ctypes.c_float),
        ("contact_static_friction", ctypes.c_float),
        ("contact_kinetic_friction", ctypes.c_float),
        ("wall_static_friction", ctypes.c_float),
        ("wall_kinetic_friction", ctypes.c_float),
        ("max_neighbors", ctypes.c_uint32),
        ("twod_z", ctypes.c_float),
        ("flags", ctypes.c_uint32),
        ("solid_density_weight", ctypes.c_float),
        ("gas_gravity_scale", ctypes.c_float),
        ("gas_scorr_k", ctypes.c_float),
        ("gas_scorr_dq", ctypes.c_float),
        ("gas_solid_density_weight", ctypes.c_float),
        ("gas_drag", ctypes.c_float),
    ]

    def __init__(self, **kw):
        super().__init__()
        # pbd_default_params' values of the fields whose zero means something
        self.solid_density_weight = 1.0
        self.gas_gravity_scale = -0.2
        self.gas_scorr_k = 0.2
        self.gas_scorr_dq = 0.25
        self.gas_solid_density_weight = 0.5
        self.gas_drag = 50.0
        self.update(**kw)

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, ctypes.Array) else v
        return out

    def update(self, **kw) -> "PbdParams":
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            cur = getattr(self, k)
            if isinstance(cur, ctypes.Array):
                for i, x in enumerate(v):
                    cur[i] = x
            else:
                setattr(self, k, v)
        return self


class PbdDeviceBuffers(ctypes.Structure):
    _fields_ = [
        ("positions", ctypes.c_void_p),
        ("velocities", ctypes.c_void_p),
        ("phases", ctypes.c_void_p),
        ("num_particles", ctypes.c_uint32),
        ("capacity", ctypes.c_uint32),
    ]


STAGES = ["predict", "grid", "lambda", "solve", "distance", "shapes", "velocity", "xsph"]


class PbdTuning(ctypes.Structure):
    _fields_ = [("threads_per_particle", ctypes.c_uint32), ("neighbor_list_capacity", ctypes.c_uint32),
                ("neighbor_skin", ctypes.c_float), ("list_assembly", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32 * 4)]


class PbdEmitter(ctypes.Structure):
    """Mirror of ``pbd_emitter`` (include/pbd.h)."""

    _fields_ = [("position", ctypes.c_float * 3), ("rate", ctypes.c_float), ("duration", ctypes.c_float),
                ("phase", ctypes.c_int32), ("inverse_mass", ctypes.c_float), ("rest_density", ctypes.c_float),
                ("open_gas", ctypes.c_int32), ("velocity", ctypes.c_float * 3),
                ("velocity_jitter", ctypes.c_float * 3), ("seed", ctypes.c_uint64), ("solidify", ctypes.c_int32),
                ("solidify_speed", ctypes.c_float), ("solidify_height", ctypes.c_float),
                ("group_first", ctypes.c_uint32), ("group_count", ctypes.c_uint32)]

    def __init__(self, **kw):
        super().__init__()
        self.inverse_mass = 1.0
        self.rest_density = 1.0
        self.solidify_speed = 0.06  # FluidEmitter's thresholds
        self.solidify_height = 5.0
        for k, v in kw.items():
            cur = getattr(self, k)
            if isinstance(cur, ctypes.Array):
                for i, x in enumerate(v):
                    cur[i] = x
            else:
                setattr(self, k, v)


class PbdProfile(ctypes.Structure):
    _fields_ = [
        ("stage_ms", ctypes.c_double * 8),
        ("stage_launches", ctypes.c_uint64 * 8),
        ("kernel_launches", ctypes.c_uint64),
        ("steps", ctypes.c_uint64),
    ]


PBD_OK, PBD_ERR_INVALID_ARGUMENT, PBD_ERR_CAPACITY, PBD_ERR_CUDA, PBD_ERR_STATE, PBD_ERR_NONFINITE, \
    PBD_ERR_UNSUPPORTED = range(7)


class PbdError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"pbd error {code}: {message}")
        self.code = code


_LIB: ctypes.CDLL | None = None

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_F = ctypes.c_float
_I = ctypes.c_int
_PF = ctypes.POINTER(ctypes.c_float)
_PU = ctypes.POINTER(ctypes.c_uint32)
_PI = ctypes.POINTER(ctypes.c_int32)

_SIGNATURES = {
    "pbd_abi_version": ([], _I),
    "pbd_default_params": ([ctypes.POINTER(PbdParams)], None),
    "pbd_create": ([ctypes.POINTER(PbdParams), _U32, ctypes.POINTER(_P)], _I),
    "pbd_destroy": ([_P], _I),
    "pbd_last_error": ([_P], ctypes.c_char_p),
    "pbd_set_params": ([_P, ctypes.POINTER(PbdParams)], _I),
    "pbd_get_params": ([_P, ctypes.POINTER(PbdParams)], _I),
    "pbd_begin_scene": ([_P, ctypes.POINTER(PbdParams), _PU], _I),
    "pbd_get_vbo": ([_P, _U32, _U32, _P, _I, _P], _I),
    "pbd_batch_create": ([_U32, ctypes.POINTER(PbdParams), _PU, _PF, _PF, _PI, _PF, _U32, ctypes.POINTER(_P)], _I),
    "pbd_num_scenes": ([_P], _U32),
    "pbd_get_scene": ([_P, _U32, _PU, _PU, ctypes.POINTER(PbdParams)], _I),
    "pbd_set_scene_params": ([_P, _U32, ctypes.POINTER(PbdParams)], _I),
    "pbd_num_particles": ([_P], _U32),
    "pbd_capacity": ([_P], _U32),
    "pbd_num_cells": ([_P], _U32),
    "pbd_add_particles": ([_P, _U32, _PF, _PF, _PI, _PF, _PU], _I),
    "pbd_add_distance_constraints": ([_P, _U32, _PU, _PF, _PF], _I),
    "pbd_add_point_constraints": ([_P, _U32, _PU, _PF], _I),
    "pbd_add_rigid_body": ([_P, _U32, _U32, _F, _PU], _I),
    "pbd_set_wall_jitter": ([_P, _PF], _I),
    "pbd_set_positions": ([_P, _U32, _U32, _P, _I, _P], _I),
    "pbd_set_velocities": ([_P, _U32, _U32, _P, _I, _P], _I),
    "pbd_get_positions": ([_P, _U32, _U32, _P, _I, _P], _I),
    "pbd_get_velocities": ([_P, _U32, _U32, _P, _I, _P], _I),
    "pbd_get_phases": ([_P, _PI], _I),
    "pbd_set_gas_open": ([_P, _U32, _U32, _I], _I),
    "pbd_set_rigid_sdf": ([_P, _U32, _PF], _I),
    "pbd_add_fluid_group": ([_P, _U32, _U32, _F], _I),
    "pbd_add_emitter": ([_P, ctypes.POINTER(PbdEmitter), _PU], _I),
    "pbd_emit": ([_P, _F, _PU, _P], _I),
    "pbd_add_rigid_group": ([_P, _U32, _U32, _F], _I),
    "pbd_set_box": ([_P, _PF, _PF], _I),
    "pbd_tick": ([_P, _F, _P], _I),
    "pbd_batch_tick": ([_P, _F, _U32, _P], _I),
    "pbd_record": ([_P, _F, _U32, _U32, _P], _I),
    "pbd_get_forces": ([_P, _PF], _I),
    "pbd_get_device_buffers": ([_P, ctypes.POINTER(PbdDeviceBuffers)], _I),
    "pbd_add_fluid": ([_P, _PI, _PI, _F, _F, ctypes.c_uint64], _I),
    "pbd_add_particle_grid": ([_P, _PI, _PI, _F, _I, ctypes.c_uint64], _I),
    "pbd_add_horiz_cloth": ([_P, _PI, _PI, _PF, _PF, _F, _I], _I),
    "pbd_add_rope": ([_P, _PF, _PF, _F, ctypes.c_int32, _F, _I], _I),
    "pbd_add_static_sphere": ([_P, _PI, _PI, _F], _I),
    "pbd_update": ([_P, _F, _P], _I),
    "pbd_update_graph": ([_P, _F, _U32, _P], _I),
    "pbd_integrate": ([_P, _F, _P], _I),
    "pbd_build_grid": ([_P, _P], _I),
    "pbd_collide": ([_P, _P], _I),
    "pbd_solve_fluids": ([_P, _P], _I),
    "pbd_collide_world": ([_P, _P], _I),
    "pbd_solve_distance_constraints": ([_P, _P], _I),
    "pbd_solve_point_constraints": ([_P, _P], _I),
    "pbd_solve_shapes": ([_P, _P], _I),
    "pbd_calc_velocity": ([_P, _F, _P], _I),
    "pbd_apply_xsph": ([_P, _P], _I),
    "pbd_get_grid": ([_P, _PU, _PU, _PU, _PU], _I),
    "pbd_get_lambdas": ([_P, _PF], _I),
    "pbd_check_finite": ([_P, _P], _I),
    "pbd_synchronize": ([_P, _P], _I),
    "pbd_set_tuning": ([_P, ctypes.POINTER(PbdTuning)], _I),
    "pbd_get_tuning": ([_P, ctypes.POINTER(PbdTuning)], _I),
    "pbd_autotune": ([_P, _F, _U32, _P, ctypes.POINTER(PbdTuning)], _I),
    "pbd_set_profiling": ([_P, _I], _I),
    "pbd_get_profile": ([_P, ctypes.POINTER(PbdProfile)], _I),
    "pbd_reset_profile": ([_P], _I),
    "pbd_build_grid_noalloc": ([ctypes.POINTER(PbdParams), _P, _U32, _P, _P, _P, _P], _I),
    "pbd_state_size": ([_P], ctypes.c_uint64),
    "pbd_save_state": ([_P, _P, ctypes.c_uint64], _I),
    "pbd_set_distance_stiffness": ([_P, _U32, _P, _I, _P], _I),
    "pbd_rollout": ([_P, _F, _U32, _U32, _P], _I),
    "pbd_list_reuses": ([_P, _PU], _I),
    "pbd_num_distance_constraints": ([_P], _U32),
    "pbd_set_positions_velocities": ([_P, _U32, _U32, _P, _P, _I, _P], _I),
    "pbd_get_positions_velocities": ([_P, _U32, _U32, _P, _P, _I, _P], _I),
    "pbd_backward": ([_P, _P, _P, _P, _P, _P, _P], _I),
    "pbd_load_state": ([_P, _P, ctypes.c_uint64], _I),
}


def header_functions() -> list[str]:
    """Names of every function declared in include/pbd.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pbd_[a-z0-9_]+)\s*\(", text)))


def load_library(build: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library; raise if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build else _build.lib_path()
    if not Path(path).exists():
        raise RuntimeError(f"{path} is missing: build it with particlesolver_gb300._build.build()")
    lib = ctypes.CDLL(str(path))
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.pbd_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path} has ABI {lib.pbd_abi_version()}, this binding expects {ABI_VERSION}: rebuild it")
    _LIB = lib
    return lib


def default_params(**kw) -> PbdParams:
    p = PbdParams()
    load_library().pbd_default_params(ctypes.byref(p))
    return p.update(**kw)


# pbd_default_params' values (the reference's compile-time constants and
# scene defaults, integration_kernel.cuh:20-42, particleapp.cpp:23-38), for
# host-only users that do not load the CUDA library (a CPU checker, the
# benchmark's reference arm); a CPU test keeps the two equal.
PARAM_DEFAULTS = dict(
    particle_radius=0.25, kernel_radius=2.0, cell_size=0.5, grid_size=[64, 64, 64], world_origin=[0.0, 0.0, 0.0],
    gravity=[0.0, -9.8, 0.0], box_min=[-50.0, 0.0, -50.0], box_max=[50.0, 200.0, 50.0], iterations=5, max_dt=0.05,
    relaxation=0.01, scorr_k=0.1, scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, contact_static_friction=0.005,
    contact_kinetic_friction=0.0002, wall_static_friction=0.005, wall_kinetic_friction=0.0002, max_neighbors=500,
    twod_z=0.0, flags=0, solid_density_weight=1.0, gas_gravity_scale=-0.2, gas_scorr_k=0.2, gas_scorr_dq=0.25,
    gas_solid_density_weight=0.5, gas_drag=50.0)


def host_params(**kw) -> PbdParams:
    """default_params(**kw) without loading the CUDA library."""
    return PbdParams().update(**{**PARAM_DEFAULTS, **kw})


def _fptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_PF)


def _f32(a, shape_last=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape_last is not None and a.shape[-1] != shape_last:
        raise ValueError(f"expected trailing dimension {shape_last}, got {a.shape}")
    return a


class ParticleSystem:
    """One pbd_system handle (the reference's ParticleSystem, headless)."""

    def __init__(self, params: PbdParams, max_particles: int):
        self.lib = load_library()
        self.params = params
        h = ctypes.c_void_p()
        rc = self.lib.pbd_create(ctypes.byref(params), int(max_particles), ctypes.byref(h))
        if rc:
            raise PbdError(rc, self.lib.pbd_last_error(None).decode())
        self.h = h

    @classmethod
    def reference(cls, particle_radius: float, grid_size, max_particles: int, min_bounds, max_bounds,
                  iterations: int) -> "ParticleSystem":
        """The reference constructor (particlesystem.cpp:36-69)."""
        p = default_params(particle_radius=particle_radius, cell_size=particle_radius * 2.0,
                           grid_size=grid_size, box_min=[float(v) for v in min_bounds],
                           box_max=[float(v) for v in max_bounds], iterations=iterations)
        return cls(p, max_particles)

    @classmethod
    def batch(cls, params, counts, pos_w, vel=None, phase=None, rest_density=None,
              max_particles: int = 0) -> "ParticleSystem":
        """pbd_batch_create: scene k takes params[k] and the next counts[k]
        particles of the arrays (pos_w (N, 4); vel (N, 4), phase (N,) and
        rest_density (N,) optional)."""
        self = cls.__new__(cls)
        self.lib = load_library()
        S = len(params)
        self.params = params[0] if S else None
        par = (PbdParams * max(S, 1))(*params)
        cnt = np.ascontiguousarray(counts, dtype=np.uint32)
        pos = np.ascontiguousarray(pos_w, dtype=np.float32).reshape(-1, 4)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 4)
        ph = None if phase is None else np.ascontiguousarray(phase, dtype=np.int32)
        ro = None if rest_density is None else np.ascontiguousarray(rest_density, dtype=np.float32)
        h = ctypes.c_void_p()
        rc = self.lib.pbd_batch_create(S, par, cnt.ctypes.data_as(_PU), _fptr(pos), _fptr(v),
                                       None if ph is None else ph.ctypes.data_as(_PI), _fptr(ro),
                                       int(max_particles), ctypes.byref(h))
        if rc:
            raise PbdError(rc, self.lib.pbd_last_error(None).decode())
        self.h = h
        return self

    # -- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.pbd_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc:
            raise PbdError(rc, self.lib.pbd_last_error(self.h).decode())

    # -- content --------------------------------------------------------
    @property
    def num_particles(self) -> int:
        return int(self.lib.pbd_num_particles(self.h))

    @property
    def num_cells(self) -> int:
        return int(self.lib.pbd_num_cells(self.h))

    def add_particles(self, pos_w, vel=None, phase=None, rest_density=None) -> int:
        pos_w = _f32(pos_w, 4).reshape(-1, 4)
        n = pos_w.shape[0]
        vel = None if vel is None else _f32(vel, 4).reshape(n, 4)
        phase = np.ascontiguousarray(np.zeros(n) if phase is None else phase, dtype=np.int32)
        rd = None if rest_density is None else _f32(rest_density).reshape(n)
        first = ctypes.c_uint32()
        self._check(self.lib.pbd_add_particles(self.h, n, _fptr(pos_w), _fptr(vel),
                                               phase.ctypes.data_as(_PI), _fptr(rd), ctypes.byref(first)))
        return first.value

    def add_distance_constraints(self, pairs, rest, stiffness=None):
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1, 2)
        rest = _f32(rest).reshape(-1)
        st = None if stiffness is None else _f32(stiffness).reshape(-1)
        self._check(self.lib.pbd_add_distance_constraints(self.h, pairs.shape[0], pairs.ctypes.data_as(_PU),
                                                          _fptr(rest), _fptr(st)))


    def add_point_constraints(self, index, points):
        index = np.ascontiguousarray(index, dtype=np.uint32).reshape(-1)
        points = _f32(points).reshape(-1, 3)
        self._check(self.lib.pbd_add_point_constraints(self.h, index.shape[0], index.ctypes.data_as(_PU),
                                                       _fptr(points)))

    def add_rigid_body(self, first: int, count: int, stiffness: float = 1.0) -> int:
        b = ctypes.c_uint32()
        self._check(self.lib.pbd_add_rigid_body(self.h, first, count, stiffness, ctypes.byref(b)))
        return b.value

    def add_fluid_group(self, first: int, count: int, rest_density: float):
        """Make [first, first + count) fluid with this rest density."""
        self._check(self.lib.pbd_add_fluid_group(self.h, int(first), int(count), float(rest_density)))

    def add_emitter(self, **kw) -> int:
        """pbd_add_emitter with the fields of PbdEmitter; returns its id."""
        e = PbdEmitter(**kw)
        i = ctypes.c_uint32()
        self._check(self.lib.pbd_add_emitter(self.h, ctypes.byref(e), ctypes.byref(i)))
        return i.value

    def emit(self, dt: float, stream=None) -> int:
        """Advance every emitter by dt; returns the particles appended."""
        c = ctypes.c_uint32()
        self._check(self.lib.pbd_emit(self.h, dt, ctypes.byref(c), stream))
        return c.value

    def set_box(self, box_min, box_max):
        lo, hi = _f32(box_min).reshape(3), _f32(box_max).reshape(3)
        self._check(self.lib.pbd_set_box(self.h, _fptr(lo), _fptr(hi)))

    def set_rigid_sdf(self, body: int, sdf):
        """Signed-distance data of a rigid body's particles: (count, 4)
        rest-frame normal xyz and depth (< 0 = none)."""
        a = _f32(sdf, 4).reshape(-1, 4)
        self._check(self.lib.pbd_set_rigid_sdf(self.h, int(body), _fptr(a)))

    def set_wall_jitter(self, rands):
        r = _f32(rands).reshape(6)
        self._check(self.lib.pbd_set_wall_jitter(self.h, _fptr(r)))

    def set_params(self, params: PbdParams):
        self._check(self.lib.pbd_set_params(self.h, ctypes.byref(params)))
        self.params = params

    def get_params(self) -> PbdParams:
        """Scene 0's parameters as the system holds them (the autotuner may
        have changed cell_size and grid_size)."""
        p = PbdParams()
        self._check(self.lib.pbd_get_params(self.h, ctypes.byref(p)))
        return p

    # -- scenes ---------------------------------------------------------
    def begin_scene(self, params: PbdParams) -> int:
        """Open the next independent scene; later add_* calls fill it."""
        k = ctypes.c_uint32()
        self._check(self.lib.pbd_begin_scene(self.h, ctypes.byref(params), ctypes.byref(k)))
        return k.value

    @property
    def num_scenes(self) -> int:
        return int(self.lib.pbd_num_scenes(self.h))

    def scene(self, k: int):
        """(first slot, particle count, params) of scene k."""
        first, count, p = ctypes.c_uint32(), ctypes.c_uint32(), PbdParams()
        self._check(self.lib.pbd_get_scene(self.h, k, ctypes.byref(first), ctypes.byref(count), ctypes.byref(p)))
        return first.value, count.value, p

    def set_scene_params(self, k: int, params: PbdParams):
        self._check(self.lib.pbd_set_scene_params(self.h, k, ctypes.byref(params)))

    # reference scene builders
    def add_fluid(self, ll, ur, mass, density, seed=1):
        a = (ctypes.c_int32 * 3)(*ll)
        b = (ctypes.c_int32 * 3)(*ur)
        self._check(self.lib.pbd_add_fluid(self.h, a, b, mass, density, seed))

    def add_particle_grid(self, ll, ur, mass, jitter=False, seed=1):
        a = (ctypes.c_int32 * 3)(*ll)
        b = (ctypes.c_int32 * 3)(*ur)
        self._check(self.lib.pbd_add_particle_grid(self.h, a, b, mass, int(jitter), seed))

    def add_horiz_cloth(self, ll, ur, spacing, dist, mass, hold_edges):
        self._check(self.lib.pbd_add_horiz_cloth(self.h, (ctypes.c_int32 * 2)(*ll), (ctypes.c_int32 * 2)(*ur),
                                                 (ctypes.c_float * 3)(*spacing), (ctypes.c_float * 2)(*dist),
                                                 mass, int(hold_edges)))

    def add_rope(self, start, spacing, dist, links, mass, pin_start):
        self._check(self.lib.pbd_add_rope(self.h, (ctypes.c_float * 3)(*start), (ctypes.c_float * 3)(*spacing),
                                          dist, links, mass, int(pin_start)))

    def add_static_sphere(self, ll, ur, spacing):
        self._check(self.lib.pbd_add_static_sphere(self.h, (ctypes.c_int32 * 3)(*ll), (ctypes.c_int32 * 3)(*ur),
                                                   spacing))

    # -- stepping ---------------------------------------------------------
    def update(self, dt: float, stream: int | None = None):
        self._check(self.lib.pbd_update(self.h, dt, stream))

    def update_graph(self, dt: float, nsteps: int = 1, stream: int | None = None):
        self._check(self.lib.pbd_update_graph(self.h, dt, nsteps, stream))

    def integrate(self, dt, stream=None):
        self._check(self.lib.pbd_integrate(self.h, dt, stream))

    def build_grid(self, stream=None):
        self._check(self.lib.pbd_build_grid(self.h, stream))

    def collide(self, stream=None):
        self._check(self.lib.pbd_collide(self.h, stream))

    def solve_fluids(self, stream=None):
        self._check(self.lib.pbd_solve_fluids(self.h, stream))

    def collide_world(self, stream=None):
        self._check(self.lib.pbd_collide_world(self.h, stream))

    def solve_distance_constraints(self, stream=None):
        self._check(self.lib.pbd_solve_distance_constraints(self.h, stream))

    def solve_point_constraints(self, stream=None):
        self._check(self.lib.pbd_solve_point_constraints(self.h, stream))

    def solve_shapes(self, stream=None):
        self._check(self.lib.pbd_solve_shapes(self.h, stream))

    def calc_velocity(self, dt, stream=None):
        self._check(self.lib.pbd_calc_velocity(self.h, dt, stream))

    def apply_xsph(self, stream=None):
        self._check(self.lib.pbd_apply_xsph(self.h, stream))

    def synchronize(self, stream=None):
        self._check(self.lib.pbd_synchronize(self.h, stream))

    def check_finite(self, stream=None):
        self._check(self.lib.pbd_check_finite(self.h, stream))

    # -- state ------------------------------------------------------------
    def positions(self) -> np.ndarray:
        n = self.num_particles
        out = np.empty((n, 4), np.float32)
        if n:
            self._check(self.lib.pbd_get_positions(self.h, 0, n, out.ctypes.data, 0, None))
        return out

    def velocities(self) -> np.ndarray:
        n = self.num_particles
        out = np.empty((n, 4), np.float32)
        if n:
            self._check(self.lib.pbd_get_velocities(self.h, 0, n, out.ctypes.data, 0, None))
        return out

    def set_positions(self, pos_w, first=0):
        a = _f32(pos_w, 4).reshape(-1, 4)
        self._check(self.lib.pbd_set_positions(self.h, first, a.shape[0], a.ctypes.data, 0, None))

    def set_velocities(self, vel, first=0):
        a = _f32(vel, 4).reshape(-1, 4)
        self._check(self.lib.pbd_set_velocities(self.h, first, a.shape[0], a.ctypes.data, 0, None))

    def vbo(self, first: int = 0, count: int | None = None, device_ptr: int | None = None, stream=None):
        """The reference's render buffer content (xyz, w = 1) of particles
        [first, first + count): into device memory at device_ptr (on the
        stream), or returned as an (count, 4) array."""
        count = self.num_particles - first if count is None else int(count)
        if device_ptr is not None:
            self._check(self.lib.pbd_get_vbo(self.h, first, count, device_ptr, 1, stream))
            return None
        out = np.empty((count, 4), np.float32)
        self._check(self.lib.pbd_get_vbo(self.h, first, count, out.ctypes.data, 0, stream))
        return out

    def phases(self) -> np.ndarray:
        out = np.empty(self.num_particles, np.int32)
        self._check(self.lib.pbd_get_phases(self.h, out.ctypes.data_as(_PI)))
        return out

    def set_gas_open(self, first: int, count: int, open_: bool = True):
        """Open (or close) the gas particles of [first, first + count)."""
        self._check(self.lib.pbd_set_gas_open(self.h, int(first), int(count), int(bool(open_))))

    def forces(self) -> np.ndarray:
        """(n, 4) force each particle carries into the next prediction."""
        out = np.empty((self.num_particles, 4), np.float32)
        self._check(self.lib.pbd_get_forces(self.h, out.ctypes.data_as(_PF)))
        return out

    def device_buffers(self) -> PbdDeviceBuffers:
        b = PbdDeviceBuffers()
        self._check(self.lib.pbd_get_device_buffers(self.h, ctypes.byref(b)))
        return b

    def grid(self):
        """(sorted_hash, sorted_index, cell_start, cell_end) of the last grid build."""
        n, c = self.num_particles, self.num_cells
        sh = np.empty(n, np.uint32)
        si = np.empty(n, np.uint32)
        cs = np.empty(c, np.uint32)
        ce = np.empty(c, np.uint32)
        self._check(self.lib.pbd_get_grid(self.h, sh.ctypes.data_as(_PU), si.ctypes.data_as(_PU),
                                          cs.ctypes.data_as(_PU), ce.ctypes.data_as(_PU)))
        return sh, si, cs, ce

    def lambdas(self) -> np.ndarray:
        out = np.empty(self.num_particles, np.float32)
        self._check(self.lib.pbd_get_lambdas(self.h, out.ctypes.data_as(_PF)))
        return out

    def tuning(self) -> PbdTuning:
        t = PbdTuning()
        self._check(self.lib.pbd_get_tuning(self.h, ctypes.byref(t)))
        return t

    def set_tuning(self, threads_per_particle: int | None = None, neighbor_list_capacity: int | None = None,
                   neighbor_skin: float | None = None, list_assembly: int | None = None):
        t = self.tuning()
        if list_assembly is not None:
            t.list_assembly = int(list_assembly)
        if threads_per_particle is not None:
            t.threads_per_particle = int(threads_per_particle)
        if neighbor_list_capacity is not None:
            t.neighbor_list_capacity = int(neighbor_list_capacity)
        if neighbor_skin is not None:
            t.neighbor_skin = float(neighbor_skin)
        self._check(self.lib.pbd_set_tuning(self.h, ctypes.byref(t)))

    def list_reuses(self) -> int:
        """Iterations of the last step that reused a skin list."""
        c = ctypes.c_uint32()
        self._check(self.lib.pbd_list_reuses(self.h, ctypes.byref(c)))
        return c.value

    def set_threads_per_particle(self, tpp: int):
        self.set_tuning(threads_per_particle=tpp)

    def autotune(self, dt: float, steps: int = 2, stream: int | None = None) -> int:
        """Pick the fastest launch shape / list schedule (lanes per
        particle, skin) for the current scene (state is restored
        afterwards); returns the lanes per particle chosen."""
        t = PbdTuning()
        self._check(self.lib.pbd_autotune(self.h, dt, steps, stream, ctypes.byref(t)))
        return int(t.threads_per_particle)

    @property
    def threads_per_particle(self) -> int:
        t = PbdTuning()
        self._check(self.lib.pbd_get_tuning(self.h, ctypes.byref(t)))
        return int(t.threads_per_particle)

    def set_profiling(self, enable: bool = True):
        self._check(self.lib.pbd_set_profiling(self.h, int(enable)))

    def profile(self) -> dict:
        p = PbdProfile()
        self._check(self.lib.pbd_get_profile(self.h, ctypes.byref(p)))
        return dict(stage_ms={k: p.stage_ms[i] for i, k in enumerate(STAGES)},
                    stage_launches={k: int(p.stage_launches[i]) for i, k in enumerate(STAGES)},
                    kernel_launches=int(p.kernel_launches), steps=int(p.steps))

    def reset_profile(self):
        self._check(self.lib.pbd_reset_profile(self.h))

    # -- differentiation ---------------------------------------------------
    @property
    def num_distance_constraints(self) -> int:
        return int(self.lib.pbd_num_distance_constraints(self.h))

    def set_distance_stiffness(self, stiffness, device_ptr: int | None = None, stream=None):
        """Stiffness of every distance constraint (add order): a host array,
        or `device_ptr` to `num_distance_constraints` device floats."""
        if device_ptr is not None:
            self._check(self.lib.pbd_set_distance_stiffness(self.h, self.num_distance_constraints, device_ptr, 1,
                                                            stream))
            return
        a = _f32(stiffness).reshape(-1)
        self._check(self.lib.pbd_set_distance_stiffness(self.h, a.shape[0], a.ctypes.data, 0, stream))

    def rollout(self, dt: float, steps: int, checkpoint_every: int = 10, stream=None):
        """`steps` updates with checkpoints every `checkpoint_every` steps
        (the forward pass of pbd_backward)."""
        self._check(self.lib.pbd_rollout(self.h, dt, steps, checkpoint_every, stream))

    def backward_device(self, dL_dx: int | None, dL_dv: int | None, dL_dx0: int | None, dL_dv0: int | None,
                        dL_dstiffness: int | None, stream=None):
        """pbd_backward on raw device pointers (float4[n] / float[m])."""
        self._check(self.lib.pbd_backward(self.h, dL_dx, dL_dv, dL_dx0, dL_dv0, dL_dstiffness, stream))

    def save_state(self) -> bytes:
        size = int(self.lib.pbd_state_size(self.h))
        buf = ctypes.create_string_buffer(size)
        self._check(self.lib.pbd_save_state(self.h, ctypes.cast(buf, ctypes.c_void_p), size))
        return buf.raw

    def load_state(self, blob: bytes):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._check(self.lib.pbd_load_state(self.h, ctypes.cast(buf, ctypes.c_void_p), len(blob)))
