"""Headless builds of the reference's own code into oracle/_ref/ (test
infrastructure).  Sources are compiled where they lie in the reference tree;
only project-written shims and drivers live under oracle/.  Nothing here runs
the reference's own build system, and no prebuilt reference binary is read
or linked.

* ``librefgpu.so``: the reference GPU kernels and thrust functors
  (gpu/src/cuda/integration_kernel.cuh, solver_kernel.cuh) compiled as host
  C++ through ``gpu_ref/shim_prelude.h``, driven by
  ``gpu_ref/refgpu_driver.cpp`` in ParticleSystem::update order.  thrust
  and the CUDA runtime headers come from the CUDA toolkit (header-only use).
* ``librefcpu.so``: the reference's 2-D CPU solver (cpu/src) with the
  project-written Qt / GL / UMFPACK stand-ins of ``cpu_ref/``.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _cuda_include() -> list[str]:
    roots = [Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))]
    out = []
    for r in roots:
        inc = r / "include"
        if inc.exists():
            out.append(str(inc))
        for cccl in sorted(r.glob("targets/*/include/cccl")):
            out.append(str(cccl))
        if (inc / "cccl").exists():
            out.append(str(inc / "cccl"))
    return out


def _stale(target: Path, inputs: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.exists() and p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout[-4000:]}\n{res.stderr[-8000:]}")


def build_refgpu(reference: Path, out: Path, cxx: str, force: bool = False) -> Path:
    src_dir = reference / "gpu" / "src" / "cuda"
    target = out / "librefgpu.so"
    inputs = [HERE / "gpu_ref" / "refgpu_driver.cpp", HERE / "gpu_ref" / "shim_prelude.h",
              src_dir / "integration_kernel.cuh", src_dir / "solver_kernel.cuh"]
    if force or _stale(target, inputs):
        out.mkdir(exist_ok=True)
        incs = []
        for d in _cuda_include():
            incs += ["-I", d]
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-ffp-contract=off",
               "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-DTHRUST_HOST_SYSTEM=THRUST_HOST_SYSTEM_CPP",
               *incs, "-I", str(src_dir), "-include", str(HERE / "gpu_ref" / "shim_prelude.h"),
               str(HERE / "gpu_ref" / "refgpu_driver.cpp"), "-o", str(target)]
        _run(cmd)
    return target


def build_refcpu(reference: Path, out: Path, cxx: str, force: bool = False) -> Path | None:
    shim = HERE / "cpu_ref"
    if not (shim / "refcpu_driver.cpp").exists():
        return None
    src = reference / "cpu" / "src"
    target = out / "librefcpu.so"
    sources = [src / "simulation.cpp", src / "fluidemitter.cpp", src / "opensmokeemitter.cpp",
               src / "solver" / "particle.cpp", src / "solver" / "solver.cpp", src / "solver" / "matrix.cpp"]
    sources += sorted((src / "constraint").glob("*.cpp"))
    drivers = [shim / "refcpu_driver.cpp", shim / "lineareq_stub.cpp"]
    inputs = sources + drivers + sorted(shim.rglob("*.h")) + sorted(shim.rglob("*.hpp"))
    if force or _stale(target, inputs):
        out.mkdir(exist_ok=True)
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-w",
               "-I", str(shim / "include"), "-I", str(src), "-I", str(src / "solver"),
               "-I", str(src / "constraint"), "-I", str(reference / "cpu" / "glm"), "-I", str(reference / "cpu"),
               *map(str, sources), *map(str, drivers), "-o", str(target)]
        _run(cmd)
    return target


def build_all(reference: Path, out: Path, cc: str, cxx: str, force: bool = False) -> dict[str, Path]:
    res = {"refgpu": build_refgpu(reference, out, cxx, force)}
    cpu = build_refcpu(reference, out, cxx, force)
    if cpu is not None:
        res["refcpu"] = cpu
    return res
