"""Serving form: continuous batching with HBM-footprint admission. Each request's result is the
same alone and in the mix (bit for bit), admission respects the budget, cancellation frees the
request, oversized requests are rejected, and the worker thread drains the queue."""
import time

import numpy as np
import pytest

import pxlengine_gb300 as P
from pxlengine_gb300 import _lib as L
from gpu_util import dam

pytestmark = pytest.mark.gpu


def _requests():
    return [
        (dam(res=32, ppc=4, iters=20), 0, 7),
        (P.Fluid("b", [[0, 0, 0], [0.8, 0.6, 0.5]], [P.FluidBlock([0.1, 0.0, 0.1], [0.5, 0.4, 0.4], [0.5, 0, 0])],
                 resolution=40, particles_per_cell=5, pressure_iterations=25), 3, 5),
        (P.Fluid("c", [[0, 0, 0], [0.3, 0.9, 0.3]], [P.FluidBlock([0.0, 0.3, 0.0], [0.3, 0.9, 0.15])],
                 resolution=36, particles_per_cell=6, pressure_iterations=15), 9, 9),
    ]


def _alone(fluid, seed, n):
    with P.FluidState(fluid, fps=24.0, seed=seed) as s:
        s.step(n)
        return s.read_particles()


def test_results_same_alone_and_in_mix(lib):
    reqs = _requests()
    alone = [_alone(f, seed, n) for f, seed, n in reqs]
    srv = P.Server()
    ids = [srv.submit(reqs[0][0], reqs[0][2], seed=reqs[0][1])]
    for _ in range(3):
        srv.tick()
    ids.append(srv.submit(reqs[1][0], reqs[1][2], seed=reqs[1][1]))   # arrives while request 0 runs
    srv.tick()
    ids.append(srv.submit(reqs[2][0], reqs[2][2], seed=reqs[2][1]))
    for _ in range(100):
        srv.tick()
        if all(srv.status(i).state == L.REQ_DONE for i in ids):
            break
    for i, ref in zip(ids, alone):
        st = srv.status(i)
        assert st.state == L.REQ_DONE and st.substeps_done == st.substeps_total
        np.testing.assert_array_equal(srv.take_result(i), ref)
    s = srv.stats()
    assert s["completed"] == 3 and s["active"] == 0 and s["reserved_bytes"] == 0
    assert s["p99_substep_ms"] >= s["p50_substep_ms"] > 0
    srv.close()


def test_admission_by_footprint(lib):
    f = dam(res=32, ppc=4, iters=10)
    need = f.to_desc()
    import ctypes as C
    b = C.c_uint64()
    assert lib.pxf_estimate_bytes(C.byref(need), None, C.byref(b)) == 0
    srv = P.Server(hbm_budget_bytes=int(b.value * 1.5))   # one request fits at a time
    a = srv.submit(f, 3)
    c = srv.submit(f, 3, seed=1)
    srv.tick()
    assert srv.status(a).state == L.REQ_RUNNING and srv.status(c).state == L.REQ_QUEUED
    for _ in range(20):
        srv.tick()
    assert srv.status(a).state == L.REQ_DONE and srv.status(c).state == L.REQ_DONE
    st = srv.stats()
    assert st["peak_reserved_bytes"] <= int(b.value * 1.5)
    np.testing.assert_array_equal(srv.take_result(c), _alone(f, 1, 3))
    srv.close()


def test_cancel_and_reject(lib):
    f = dam(res=32, ppc=4, iters=10)
    srv = P.Server(hbm_budget_bytes=300_000_000)   # ~10x a 32-grid request, < a 256-grid one
    a = srv.submit(f, 50)
    srv.tick()
    srv.cancel(a)
    srv.tick()
    assert srv.status(a).state == L.REQ_CANCELLED
    assert srv.stats()["reserved_bytes"] == 0
    big = dam(res=256, ppc=8)
    r = srv.submit(big, 10)
    st = srv.status(r)
    assert st.state == L.REQ_FAILED and st.error == L.PXF_ENOMEM
    with pytest.raises(P.FluidError):
        srv.take_result(r)
    srv.close()


def test_worker_thread_drains_queue(lib):
    reqs = _requests()
    srv = P.Server()
    srv.start()
    ids = []
    for f, seed, n in reqs:
        ids.append(srv.submit(f, n, seed=seed))
        time.sleep(0.01)
    t0 = time.time()
    while time.time() - t0 < 60:
        if all(srv.status(i).state == L.REQ_DONE for i in ids):
            break
        time.sleep(0.01)
    srv.stop()
    for i, (f, seed, n) in zip(ids, reqs):
        np.testing.assert_array_equal(srv.take_result(i), _alone(f, seed, n))
    srv.close()
