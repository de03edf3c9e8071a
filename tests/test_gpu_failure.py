"""Failure detection without a GPU fault: host waits that run out report PXF_ETIMEDOUT and leave
the work running; the persistent solve's grid barrier gives up after its bound when a block never
arrives (a block of the self-test kernel returns at once), sets its error flag and every block
returns, so the context stays usable."""
import ctypes as C

import numpy as np
import pytest

import pxlengine_gb300 as P
from pxlengine_gb300 import _lib as L
from gpu_util import dam

pytestmark = pytest.mark.gpu


def test_grid_barrier_selftest_completes(lib):
    t = C.c_uint32(7)
    assert lib.pxf_selftest_grid_barrier(304, -1, 100.0, 50, C.byref(t)) == 0
    assert t.value == 0


def test_grid_barrier_wait_runs_out_and_context_survives(lib):
    t = C.c_uint32(0)
    assert lib.pxf_selftest_grid_barrier(152, 0, 5.0, 3, C.byref(t)) == 0
    assert t.value == 1
    # the device is still usable: a normal simulation steps and matches a fresh run
    f = dam(res=24, ppc=4, iters=20)
    out = []
    for _ in range(2):
        with P.FluidState(f, fps=24.0) as s:
            s.step(3)
            out.append(s.read_particles())
    np.testing.assert_array_equal(out[0], out[1])


def test_host_wait_timeout_reports_and_recovers(lib):
    f = dam(res=96, ppc=8, iters=80)
    with P.FluidState(f, fps=15.0) as s:
        assert lib.pxf_set_wait_timeout(s.h, 1e-7) == 0
        with pytest.raises(P.FluidError) as ei:
            s.step(6)
            s.sync()
        assert ei.value.code == L.PXF_ETIMEDOUT
        assert lib.pxf_set_wait_timeout(s.h, 60.0) == 0
        s.sync()
        assert s.steps_done == 6
        s.step(1)
        s.sync()
        assert s.steps_done == 7


def test_iteration_cap_is_reported_not_hidden(lib):
    f = dam(res=32, ppc=4)
    opts = P.make_options(solver="pcg", rtol=1e-14, max_iter=3, restart=50)
    with P.FluidState(f, fps=15.0, options=opts) as s:
        s.step(2)
        it, rel, status = s.solver_stats()
        assert status == 1 and it == 3
