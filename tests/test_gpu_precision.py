"""Precision form: Jacobi PCG with FP32 vectors, FP64 dots, FP64 solution and FP64 restarts,
against the FP64 oracle solve of the same pressure system."""
import numpy as np
import pytest

import oracle
import pxlengine_gb300 as P
from gpu_util import DIV_VOLUME_TOL, PCG_RTOL, dam, divergence_after_projection, grids_equal, oracle_for

pytestmark = pytest.mark.gpu


def _pre_pressure(o):
    for st in ("clear", "p2g", "normalize", "forces", "divergence"):
        o.stage(st)


@pytest.mark.parametrize("res", [32, 64])
def test_pcg_against_fp64_oracle(lib, res):
    f = dam(res=res, ppc=8)
    opts = P.make_options(solver="pcg", rtol=PCG_RTOL, max_iter=4000, restart=50)
    with P.FluidState(f, fps=15.0, options=opts) as s:
        o64 = oracle_for(s, f)
        o64.set_pressure("pcg64", rtol=1e-12, max_iter=20000)
        for _ in range(3):
            # The oracle starts each substep from the GPU's particles, runs the same FP32
            # pre-pressure stages (bit-exact) and solves the identical system in FP64.
            o64.write(oracle.PARTICLES, s.read_particles())
            s.step(1)
            it, rel, status = s.solver_stats()
            assert status == 0 and rel <= PCG_RTOL, (it, rel, status)
            _pre_pressure(o64)
            grids_equal(s, o64, names=("cell_count", "cell_type", "vel_old", "divergence"))
            o64.stage("pressure")
            x64 = o64.read(oracle.PRESSURE64)
            xg = s.read_grid("pressure64")
            scale = max(1.0, float(np.max(np.abs(x64))))
            assert float(np.max(np.abs(xg - x64))) <= 1e-4 * scale
            vel = s.read_grid("vel")
            ct = s.read_grid("cell_type")
            div = divergence_after_projection(vel, ct, s.dims, s.cell)
            assert float(np.max(np.abs(div))) * s.dt <= DIV_VOLUME_TOL


@pytest.mark.parametrize("precond,mode", [("mg", "mgpcg"), ("jacobi", "pcg")])
def test_pcg_matches_mixed_oracle_iterations(lib, precond, mode):
    f = dam(res=32, ppc=4)
    opts = P.make_options(solver="pcg", rtol=PCG_RTOL, max_iter=4000, restart=50, precond=precond)
    with P.FluidState(f, fps=15.0, options=opts) as s:
        om = oracle_for(s, f)
        om.set_pressure(mode, rtol=PCG_RTOL, max_iter=4000, restart=50)
        s.step(1)
        om.step(1)
        it_g, rel_g, st_g = s.solver_stats()
        it_o, rel_o = om.pcg_stats()
        assert st_g == 0 and rel_g <= PCG_RTOL and rel_o <= PCG_RTOL
        assert abs(int(it_g) - int(it_o)) <= max(2, it_o // 10), (it_g, it_o)
        # Everything before the solve is bit-exact; the solution agrees to the solver tolerance.
        grids_equal(s, om, names=("cell_count", "cell_type", "vel_old", "divergence"))
        xg = s.read_grid("pressure64")
        xo = om.read(oracle.PRESSURE64)
        assert float(np.max(np.abs(xg - xo))) <= 1e-4 * max(1.0, float(np.max(np.abs(xo))))


def test_pcg_iteration_cap_reports_status(lib):
    f = dam(res=32, ppc=4)
    opts = P.make_options(solver="pcg", rtol=1e-12, max_iter=5, restart=50)
    with P.FluidState(f, fps=15.0, options=opts) as s:
        s.step(1)
        it, rel, status = s.solver_stats()
        assert status == 1 and it == 5 and rel > 1e-12


@pytest.mark.parametrize("precond", ["mg", "jacobi"])
def test_persistent_solve_matches_graph_loop(lib, monkeypatch, precond):
    """The persistent cooperative solve (one launch, grid barriers) and the cooperative smoothing
    kernels run the same phases over the same chunks as the graph of kernels, so all three give
    identical bits."""
    f = dam(res=48, ppc=4)
    opts = P.make_options(solver="pcg", rtol=PCG_RTOL, max_iter=4000, restart=50, precond=precond)
    out = {}
    for mode, env in (("graph", {}), ("persistent", {"PXF_PCG_PERSISTENT": "1"}), ("coop", {"PXF_MG_COOP": "1"})):
        for k in ("PXF_PCG_PERSISTENT", "PXF_MG_COOP"):
            monkeypatch.setenv(k, env.get(k, "0"))
        with P.FluidState(f, fps=15.0, options=opts) as s:
            s.step(3)
            out[mode] = (s.read_particles(), s.read_grid("pressure64"), s.solver_stats())
    for mode in ("persistent", "coop"):
        assert out[mode][2][2] == 0 and out[mode][2][0] == out["graph"][2][0]
        assert np.array_equal(out[mode][0], out["graph"][0])
        assert np.array_equal(out[mode][1], out["graph"][1])


def test_precision_solve_is_deterministic(lib):
    """Fixed-order reductions and overlapped (programmatic) launches: two runs give the same bits."""
    f = dam(res=96, ppc=4)
    opts = P.make_options(solver="pcg", rtol=PCG_RTOL, max_iter=4000, restart=50)
    out = []
    for _ in range(2):
        with P.FluidState(f, fps=15.0, options=opts) as s:
            s.step(6)
            out.append((s.read_particles(), s.read_grid("pressure64"), s.solver_stats()))
    assert out[0][2] == out[1][2]
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
