"""pbd_build_grid_noalloc: the neighbour-grid build for callers that cannot
allocate device memory (inside stream capture, real-time loops, or hosts
whose every device buffer comes from their own allocator).

It must give exactly what the allocating path gives -- pbd_build_grid
followed by pbd_get_grid -- through the C ABI, on two calls in a row (the
shared scratch array keeps the previous call's contents, so the second call
checks that everything that must start cleared is cleared).  Integer
outputs, so the tolerance is exact equality.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import particlesolver_gb300 as pbd
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PBD_ERR_INVALID_ARGUMENT = 1


def _noalloc_grid(lib, params, positions_dev, n, cells):
    import torch

    idx = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    cs = torch.zeros(cells, dtype=torch.int32, device="cuda")
    ce = torch.zeros(cells, dtype=torch.int32, device="cuda")
    rc = lib.pbd_build_grid_noalloc(ctypes.byref(params), positions_dev, n, idx.data_ptr(), cs.data_ptr(),
                                    ce.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0, lib.pbd_last_error(None)
    view = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    return view(idx)[:n], view(cs), view(ce)


def test_noalloc_grid_matches_allocating_path_twice():
    pytest.importorskip("torch")
    sc = W.dam_break(24, 20, 12)
    params = pbd.default_params(**sc.params)
    g = pbd.ParticleSystem(params, sc.n)
    W.apply_to(sc, g)
    lib = g.lib
    for _ in range(2):
        g.build_grid()
        _, ref_idx, ref_start, ref_end = g.grid()
        buf = g.device_buffers()
        idx, start, end = _noalloc_grid(lib, params, buf.positions, g.num_particles, g.num_cells)
        np.testing.assert_array_equal(idx, ref_idx)
        np.testing.assert_array_equal(start, ref_start)
        np.testing.assert_array_equal(end, ref_end)
        g.update(sc.dt)  # new positions for the second call


def test_noalloc_grid_rejects_sizes_beyond_its_limits():
    lib = pbd.load_library()
    params = pbd.default_params()
    # too many particles: rejected before any device access
    rc = lib.pbd_build_grid_noalloc(ctypes.byref(params), ctypes.c_void_p(16), (1 << 18) + 1, ctypes.c_void_p(16),
                                    ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == PBD_ERR_INVALID_ARGUMENT
    assert b"exceed the limit" in lib.pbd_last_error(None)
    # too many grid cells
    big = pbd.default_params(grid_size=[2048, 1024, 1])
    rc = lib.pbd_build_grid_noalloc(ctypes.byref(big), ctypes.c_void_p(16), 10, ctypes.c_void_p(16),
                                    ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == PBD_ERR_INVALID_ARGUMENT
    assert b"grid cells exceed" in lib.pbd_last_error(None)
