"""pxf_cell_starts_noalloc: cell binning for callers that cannot allocate device memory.

A renderer that owns every device buffer (its own allocator, graphics interop) or a real-time
thread that must not allocate hands the library device buffers it already has; the library then
bins the particles with nothing but a fixed scratch array compiled into it. This test feeds the
entry point the particles of a simulation, twice in a row, and compares the per-cell counts with
what the simulation's own binning (pxf_read_grid PXF_GRID_CELL_COUNT) reports for the same
particles. Device buffers for the test's inputs and outputs come from torch.
"""
import ctypes as C

import numpy as np
import pytest

import pxlengine_gb300 as P
from gpu_util import dam

pytestmark = pytest.mark.gpu


def test_cell_starts_noalloc_matches_simulation_binning(lib):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    f = dam(res=40, ppc=6, iters=20)
    with P.FluidState(f, fps=24.0, seed=3) as s:
        dims = (C.c_uint32 * 3)(*s.dims)
        origin = (C.c_float * 3)(*[float(x) for x in f.bounds[0]])
        ncell = s.n_cells
        out = torch.zeros(ncell + 1, dtype=torch.int32, device="cuda")
        for call in range(2):
            parts = s.read_particles()
            s.step(1)   # the substep bins exactly these particles before its P2G
            want = s.read_grid("cell_count")
            d_parts = torch.from_numpy(parts).to("cuda")
            rc = lib.pxf_cell_starts_noalloc(C.c_void_p(d_parts.data_ptr()), parts.shape[0], dims, origin,
                                             C.c_float(s.cell), C.c_void_p(out.data_ptr()), None)
            assert rc == 0, lib.pxf_last_error(None).decode()
            torch.cuda.synchronize()
            start = out.cpu().numpy().view(np.uint32)
            assert start[0] == 0 and start[-1] == parts.shape[0]
            np.testing.assert_array_equal(np.diff(start.astype(np.int64)), want.astype(np.int64))
        # Sizes beyond the fixed scratch are refused with a message.
        big = (C.c_uint32 * 3)(4096, 4096, 2)
        rc = lib.pxf_cell_starts_noalloc(C.c_void_p(d_parts.data_ptr()), 1, big, origin, C.c_float(s.cell),
                                         C.c_void_p(out.data_ptr()), None)
        assert rc == -1 and "16777216" in lib.pxf_last_error(None).decode()


def _host_starts(parts, dims, origin, h):
    """Exclusive per-cell prefix sum on the host: cell = clamp(floor((x - o) * f32(1/h))) per axis,
    every step rounded to float32 as on the device."""
    inv_h = np.float32(1.0) / np.float32(h)
    idx = []
    for a in range(3):
        t = (parts[:, a].astype(np.float32) - np.float32(origin[a])) * inv_h
        idx.append(np.clip(np.floor(t).astype(np.int64), 0, dims[a] - 1))
    cell = idx[0] + dims[0] * (idx[1] + dims[1] * idx[2])
    counts = np.bincount(cell, minlength=int(np.prod(dims)))
    return np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)


def test_cell_starts_noalloc_large_grid_and_empty(lib):
    """A grid above 2^21 cells (more than 1024 scan chunks: the chunk scan carries between its
    passes), particles partly outside the grid (clamped into the boundary cells), and n = 0."""
    torch = pytest.importorskip("torch")
    dims = (256, 128, 128)
    h = 1.0 / 256
    origin = (0.0, 0.0, 0.0)
    rng = np.random.default_rng(5)
    n = 1_500_000
    parts = np.zeros((n, 8), dtype=np.float32)
    ext = np.array([dims[0] * h, dims[1] * h, dims[2] * h], dtype=np.float32)
    parts[:, :3] = rng.uniform(-0.1, 1.1, (n, 3)).astype(np.float32) * ext
    want = _host_starts(parts, dims, origin, h)
    cd = (C.c_uint32 * 3)(*dims)
    co = (C.c_float * 3)(*origin)
    out = torch.zeros(int(np.prod(dims)) + 1, dtype=torch.int32, device="cuda")
    d_parts = torch.from_numpy(parts).to("cuda")
    for _ in range(2):
        rc = lib.pxf_cell_starts_noalloc(C.c_void_p(d_parts.data_ptr()), n, cd, co, C.c_float(h),
                                         C.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.pxf_last_error(None).decode()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)
    # n = 0: every start is 0 (the buffer held the previous call's scan)
    rc = lib.pxf_cell_starts_noalloc(None, 0, cd, co, C.c_float(h), C.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.pxf_last_error(None).decode()
    torch.cuda.synchronize()
    assert not out.cpu().numpy().any()

