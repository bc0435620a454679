"""Build recipe of the oracle (test infrastructure; the product never uses it).

* ``oracle/_build/libpbd_oracle.so``: the FP64 C restatement
  (``pbd_oracle.c``), gcc -O2 -fopenmp, FP contraction off so the FP32
  neighbour tests round exactly like the CUDA kernels.
* ``oracle/_ref/`` (only where the reference sources exist): the
  reference's own code compiled headless from its sources in place --
  see ``ref_build`` below and ``cpu_ref/`` / ``gpu_ref/`` for the
  project-written shims.  Outputs go only into ``oracle/_ref/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# The reference tree: PBD_REFERENCE_DIR, else a checkout named "reference"
# beside this repository.  Where neither exists (e.g. on a machine that only
# runs the CUDA path) the reference builds are skipped.
REFERENCE = Path(os.environ.get("PBD_REFERENCE_DIR") or (ROOT.parent / "reference"))
ORACLE_LIB = BUILD / "libpbd_oracle.so"
ORACLE_DUAL_LIB = BUILD / "libpbd_oracle_dual.so"


def _cc() -> str:
    return os.environ.get("CC") or shutil.which("gcc") or "cc"


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "c++"


def _stale(target: Path, inputs: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.exists() and p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "pbd_oracle.c", HERE / "pbd_oracle.h", ROOT / "include" / "pbd.h"]
    if force or _stale(ORACLE_LIB, srcs):
        BUILD.mkdir(exist_ok=True)
        tmp = ORACLE_LIB.with_suffix(".tmp.so")
        _run([_cc(), "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-I", str(ROOT / "include"), str(HERE / "pbd_oracle.c"), "-o", str(tmp), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_oracle_dual(force: bool = False) -> Path:
    """The same restatement compiled as C++ on dual numbers (oracle/dual.hpp):
    forward-mode directional derivatives of the FP64 replay."""
    srcs = [HERE / "pbd_oracle.c", HERE / "pbd_oracle.h", HERE / "dual.hpp", ROOT / "include" / "pbd.h"]
    if force or _stale(ORACLE_DUAL_LIB, srcs):
        BUILD.mkdir(exist_ok=True)
        tmp = ORACLE_DUAL_LIB.with_suffix(".tmp.so")
        _run([_cxx(), "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-DORC_DUAL",
              "-I", str(ROOT / "include"), "-I", str(HERE), "-x", "c++", str(HERE / "pbd_oracle.c"), "-o", str(tmp)])
        os.replace(tmp, ORACLE_DUAL_LIB)
    return ORACLE_DUAL_LIB


def reference_available() -> bool:
    return (REFERENCE / "gpu" / "src" / "cuda" / "integration_kernel.cuh").exists()


def build_reference(force: bool = False) -> dict[str, Path]:
    """Compile the reference's own sources headless into oracle/_ref/."""
    from . import ref_build

    if not reference_available():
        return {}
    return ref_build.build_all(REFERENCE, REF_OUT, _cc(), _cxx(), force=force)


def build_all(force: bool = False) -> dict[str, Path]:
    out = {"oracle": build_oracle(force), "oracle_dual": build_oracle_dual(force)}
    out.update(build_reference(force))
    return out


if __name__ == "__main__":
    import sys

    for k, v in build_all(force="--force" in sys.argv).items():
        print(k, v)
