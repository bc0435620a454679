"""In-tree build of libpbd_gb300.so (hand-written sm_103a CUDA + host C++).

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library next to this file (``_lib/libpbd_gb300.so``).  Rebuilds only
when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_DIR = PKG_DIR / "_lib"
LIB_NAME = "libpbd_gb300.so"
SOURCES = ["pbd_kernels.cu", "pbd_system.cpp", "pbd_scenes.cpp", "pbd_noalloc.cu", "pbd_adjoint.cu"]
# The benchmark's FP32 probe (bench_fp32_peak.cu beside bench.py) is its own
# library: nothing of the product links it.
PROBE_SRC = ROOT / "bench_fp32_peak.cu"
PROBE_NAME = "libpbd_fp32_probe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpbd_gb300.so")


def lib_path() -> Path:
    return LIB_DIR / LIB_NAME


def _inputs() -> list[Path]:
    files = [CSRC / s for s in SOURCES]
    files += sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "pbd.h"]
    return files


def _stale(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(f.stat().st_mtime > t for f in _inputs())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if needed; return its path."""
    target = lib_path()
    if not force and not _stale(target):
        return target
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    common = ARCH + [
        "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3",
        "-I", str(ROOT / "include"), "-I", str(CSRC),
    ]

    def compile_one(src: str) -> Path:
        obj = BUILD_DIR / (src + ".o")
        cmd = [nvcc, *common, "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = target.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, target)
    return target


def build_probe(force: bool = False) -> Path:
    """Compile the benchmark's FP32 throughput probe into its own library."""
    target = LIB_DIR / PROBE_NAME
    if not force and target.exists() and target.stat().st_mtime >= PROBE_SRC.stat().st_mtime:
        return target
    LIB_DIR.mkdir(exist_ok=True)
    tmp = target.with_suffix(".so.tmp")
    cmd = [nvcc_path(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(PROBE_SRC), "-o", str(tmp),
           "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {PROBE_SRC.name}:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, target)
    return target


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
