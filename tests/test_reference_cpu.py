"""The reference's own 2-D CPU solver (cpu/src), built headless from the
reference tree by oracle/ref_build.py: it runs the 2-D granular column
(1,600 particles, 40 x 40 lattice, mu_s 0.5, mu_k 0.3, dt 1/60, its
compiled 3 iterations) deterministically.  It is the CPU baseline of that
configuration, not a parity oracle: its contact model (Gauss-Seidel
groups, contact below 2r - 1e-4, stacking mass scaling,
simulation.cpp:171-271) differs from the GPU step's (Jacobi, 2.001 r).
Skipped where the reference tree is absent."""
import numpy as np
import pytest

from oracle import refcpu
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not refcpu.available(), reason="reference tree not built here")


def run(steps):
    sc = W.granular_column()
    r = refcpu.RefCPU(sc.pos_w[:, :2], mass=1.0, s_friction=0.5, k_friction=0.3)
    r.tick(1.0 / 60.0, steps)
    return sc, r.state()


def test_reference_cpu_granular_column_runs_deterministically():
    sc, (xy, v) = run(30)
    _, (xy2, v2) = run(30)
    np.testing.assert_array_equal(xy, xy2)
    np.testing.assert_array_equal(v, v2)
    assert xy.shape == (1600, 2) and np.all(np.isfinite(xy)) and np.all(np.isfinite(v))
    # inside its box, on or above the floor, spread about the column axis
    assert np.all(np.abs(xy[:, 0]) <= 20.0) and np.all(xy[:, 1] >= 0.0)
    assert abs(xy[:, 0].mean()) < 0.5
