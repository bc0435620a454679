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
    """Requests beyond the fixed scratch are refused with an error code.
    The buffers handed in are real device buffers large enough for what the
    request claims, so that the call could not fault even if the limit
    checks ran after a launch."""
    torch = pytest.importorskip("torch")
    lib = pbd.load_library()
    params = pbd.default_params()
    n_big = (1 << 18) + 1
    pos = torch.zeros((n_big, 4), dtype=torch.float32, device="cuda")
    idx = torch.zeros(n_big, dtype=torch.int32, device="cuda")
    cells = params.grid_size[0] * params.grid_size[1] * params.grid_size[2]
    cs = torch.zeros(cells, dtype=torch.int32, device="cuda")
    ce = torch.zeros(cells, dtype=torch.int32, device="cuda")
    # too many particles
    rc = lib.pbd_build_grid_noalloc(ctypes.byref(params), pos.data_ptr(), n_big, idx.data_ptr(), cs.data_ptr(),
                                    ce.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == PBD_ERR_INVALID_ARGUMENT
    assert b"exceed the limit" in lib.pbd_last_error(None)
    # too many grid cells
    big = pbd.default_params(grid_size=[2048, 1024, 1])
    cs2 = torch.zeros(2048 * 1024, dtype=torch.int32, device="cuda")
    ce2 = torch.zeros(2048 * 1024, dtype=torch.int32, device="cuda")
    rc = lib.pbd_build_grid_noalloc(ctypes.byref(big), pos.data_ptr(), 10, idx.data_ptr(), cs2.data_ptr(),
                                    ce2.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == PBD_ERR_INVALID_ARGUMENT
    assert b"grid cells exceed" in lib.pbd_last_error(None)
