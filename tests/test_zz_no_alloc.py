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
