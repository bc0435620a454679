"""The C++ drop-in (include/particle_system.hpp) in a real host program:
compiled against libpbd_gb300.so and run on the GPU (reference
constructor, scene builders, queued runtime insertion, update loop,
errors as exceptions)."""
import shutil
import subprocess
from pathlib import Path

import pytest

from particlesolver_gb300 import _build

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_reference_style_host_program_runs(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = _build.build()
    cuda = Path(_build.nvcc_path()).resolve().parent.parent
    exe = tmp_path / "dropin"
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(ROOT / "tests" / "cpp" / "dropin_main.cpp"), "-o", str(exe), "-L", str(lib.parent), "-lpbd_gb300",
           "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda / 'lib64'}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "bad 0 threw 1" in run.stdout
