"""The C ABI library builds for sm_103a, loads and exports every symbol
include/pbd.h declares; the ctypes mirror of pbd_params matches the C
layout.  No GPU needed (nothing here launches work)."""
import ctypes
import subprocess
import textwrap
from pathlib import Path

import pytest

import particlesolver_gb300 as pbd
from particlesolver_gb300 import _build


def test_library_builds_and_loads():
    path = _build.build()
    assert path.exists()
    lib = pbd.load_library()
    from particlesolver_gb300 import ABI_VERSION

    assert lib.pbd_abi_version() == ABI_VERSION


def test_every_header_symbol_is_exported():
    lib = pbd.load_library()
    names = pbd.header_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the binding declares a signature for each
    assert set(names) <= set(pbd._SIGNATURES), set(names) - set(pbd._SIGNATURES)


def test_kernels_are_built_for_sm103a_only():
    """Every translation unit is compiled with the one -gencode for sm_103a
    (a kernel launch on another architecture then fails loudly with "no
    kernel image"; the GPU tests launch every kernel family)."""
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.parametrize("mirror,ctype", [(pbd.PbdParams, "pbd_params"), (pbd.PbdEmitter, "pbd_emitter"),
                                           (pbd.PbdTuning, "pbd_tuning")])
def test_struct_layout_matches_c(tmp_path, mirror, ctype):
    src = tmp_path / "layout.c"
    fields = [f for f, _ in mirror._fields_]
    body = "\n".join(f'printf("%zu\\n", offsetof({ctype}, {f}));' for f in fields)
    src.write_text(textwrap.dedent(f"""
        #include <stddef.h>
        #include <stdio.h>
        #include "pbd.h"
        int main(void) {{ printf("%zu\\n", sizeof({ctype})); {body} return 0; }}
    """))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(_build.ROOT / "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(mirror)
    for (name, _), off in zip(mirror._fields_, vals[1:]):
        assert getattr(mirror, name).offset == off, name


def test_default_params_are_reference_values():
    p = pbd.default_params()
    assert p.particle_radius == 0.25 and p.kernel_radius == 2.0 and p.cell_size == 0.5
    assert list(p.grid_size) == [64, 64, 64] and p.iterations == 5
    assert abs(p.relaxation - 0.01) < 1e-9 and p.max_neighbors == 500
    assert list(p.box_min) == [-50, 0, -50] and list(p.box_max) == [50, 200, 50]
    assert p.solid_density_weight == 1.0  # the GPU reference: every neighbour counts


def test_host_param_defaults_match_the_library():
    """PARAM_DEFAULTS (used where the CUDA library is not loaded, e.g. the
    benchmark's reference arm) equals pbd_default_params field by field."""
    a = pbd.host_params().as_dict()
    b = pbd.default_params().as_dict()
    assert a.keys() == b.keys()
    for k in a:
        assert a[k] == b[k], k
    assert pbd.host_params(iterations=4).iterations == 4


def test_create_without_gpu_fails_cleanly():
    """pbd_create reports a CUDA error instead of exiting when no device
    is present (skipped on a GPU machine)."""
    from conftest import cuda_available

    if cuda_available():
        pytest.skip("GPU present")
    lib = pbd.load_library()
    h = ctypes.c_void_p()
    rc = lib.pbd_create(ctypes.byref(pbd.default_params()), 16, ctypes.byref(h))
    assert rc == 3  # PBD_ERR_CUDA
    assert b"CUDA" in lib.pbd_last_error(None) or b"device" in lib.pbd_last_error(None)


def test_batch_create_checks_its_arguments_first():
    """pbd_batch_create rejects a bad batch before it touches a device:
    no scenes, a capacity below the particles, a missing pos_w or out."""
    lib = pbd.load_library()
    h = ctypes.c_void_p(123)
    par = (pbd.PbdParams * 2)(pbd.default_params(), pbd.default_params())
    counts = (ctypes.c_uint32 * 2)(10, 20)
    pos = (ctypes.c_float * 120)()
    pf = ctypes.cast(pos, ctypes.POINTER(ctypes.c_float))
    assert lib.pbd_batch_create(0, par, counts, pf, None, None, None, 0, ctypes.byref(h)) == 1
    assert not h.value
    assert lib.pbd_batch_create(2, par, counts, pf, None, None, None, 29, ctypes.byref(h)) == 2  # PBD_ERR_CAPACITY
    assert lib.pbd_batch_create(2, par, counts, None, None, None, None, 0, ctypes.byref(h)) == 1
    assert lib.pbd_batch_create(2, par, counts, pf, None, None, None, 0, None) == 1
    assert b"capacity" in lib.pbd_last_error(None) or b"NULL" in lib.pbd_last_error(None)


def test_calls_on_a_null_system_fail_cleanly():
    lib = pbd.load_library()
    buf = (ctypes.c_float * 8)()
    assert lib.pbd_get_vbo(None, 0, 1, ctypes.cast(buf, ctypes.c_void_p), 0, None) == 1
    assert lib.pbd_get_positions(None, 0, 1, ctypes.cast(buf, ctypes.POINTER(ctypes.c_float)), 0, None) == 1


def test_cpp_drop_in_header_compiles(tmp_path):
    """include/particle_system.hpp (the reference-shaped C++ class) compiles
    against the C ABI."""
    src = tmp_path / "use.cpp"
    src.write_text(textwrap.dedent("""
        #include "particle_system.hpp"
        int main() {
            pbd::ParticleSystem ps(0.25f, make_uint3(64, 64, 64), 15000, make_int3(-50, 0, -50),
                                   make_int3(50, 200, 50), 5);
            ps.addRope(make_float3(0, 20, 0), make_float3(0, -.5f, 0), .4f, 32, 1.f, true);
            ps.update(1.f / 60);
            return (int)ps.getNumParticles() == 33 ? 0 : 1;
        }
    """))
    res = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(_build.ROOT / "include"),
                          "-I", "/usr/local/cuda/include", str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
