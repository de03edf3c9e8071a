"""The red-black GS pressure solve streamed through shared memory (two iterations per pass over
HBM, units of x-y tiles times z segments) against the oracle's plain sweep order, bit for bit
(shaders/fluid.slang:167-182, crates/pxl-render/src/fluid.rs:295-300).

The library streams only grids of 2^24 cells and more by default; these tests force the streamed
solve (PXF_GS_STREAM=1, read when a simulation's batch is built) on small grids: several tiles in
x and y and several z segments, odd grid sides, iteration counts whose last pass holds one
iteration and counts that leave the result in the second buffer, and a batch whose simulations
stop iterating after different passes."""
import numpy as np
import pytest

import pxlengine_gb300 as P
from gpu_util import dam, grids_equal, oracle_for, particles_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def streamed(monkeypatch):
    monkeypatch.setenv("PXF_GS_STREAM", "1")


def test_many_units_bit_exact(lib):
    # 130 x 65 x 97: three tiles in x, three in y, seven z segments of 16 planes (the last short)
    f = P.Fluid("units", [[0, 0, 0], [1.3, 0.65, 0.97]], [P.FluidBlock([0, 0, 0], [0.5, 0.45, 0.97])],
                resolution=130, particles_per_cell=2, pressure_iterations=80)
    with P.FluidState(f, fps=15.0, seed=2) as s:
        assert s.dims == (130, 65, 97)
        o = oracle_for(s, f)
        s.step(2)
        o.step(2)
        grids_equal(s, o)
        particles_equal(s, o)


def test_rows_of_four_cells_bit_exact(lib):
    # x side a multiple of 4 (counts travel as 4-cell words) and several units
    f = dam(res=128, ppc=2, iters=80, fill_max=(0.3, 0.4, 0.5))
    with P.FluidState(f, fps=15.0, seed=6) as s:
        assert s.dims[0] % 4 == 0
        o = oracle_for(s, f)
        s.step(2)
        o.step(2)
        grids_equal(s, o)
        particles_equal(s, o)


@pytest.mark.parametrize("iters", [1, 2, 5, 7])
def test_iteration_counts_bit_exact(lib, iters):
    f = dam(res=40, ppc=4, iters=iters)
    with P.FluidState(f, fps=24.0, seed=4) as s:
        o = oracle_for(s, f)
        s.step(3)
        o.step(3)
        grids_equal(s, o)
        particles_equal(s, o)


def test_batch_of_iteration_counts_bit_exact(lib):
    """One launch per pass serves simulations with 3, 12 and 80 iterations (and a precision-solver
    simulation beside them); each GS member equals its own oracle run."""
    fl = [dam(res=24, ppc=3, iters=3), dam(res=44, ppc=2, iters=12, fill_max=(0.4, 0.3, 0.5)),
          P.Fluid("odd", [[0, 0, 0], [1.17, 0.71, 0.53]], [P.FluidBlock([0.05, 0.02, 0.03], [0.6, 0.5, 0.5])],
                  resolution=37, particles_per_cell=3, pressure_iterations=80)]
    sims = [P.FluidState(f, fps=24.0, seed=i) for i, f in enumerate(fl)]
    pcg = P.FluidState(dam(res=32, ppc=2), fps=24.0, seed=9, options=P.make_options(solver="pcg", rtol=1e-6))
    oracles = [oracle_for(s, f) for s, f in zip(sims, fl)]
    b = P.Batch()
    try:
        for s in sims + [pcg]:
            b.add(s)
        b.step(3)
        b.sync()
        for s, o in zip(sims, oracles):
            o.step(3)
            grids_equal(s, o)
            particles_equal(s, o)
    finally:
        b.close()
        for s in sims + [pcg]:
            s.close()


def test_pressure_warm_start_kept_across_substeps(lib):
    """The solve starts from the previous substep's pressure: after substeps whose last pass wrote
    the second buffer (5 iterations: passes of 2, 2 and 1), the next substeps still match."""
    f = dam(res=32, ppc=4, iters=5)
    with P.FluidState(f, fps=24.0, seed=7) as s:
        o = oracle_for(s, f)
        for _ in range(4):
            s.step(1)
            o.step(1)
        grids_equal(s, o, names=("pressure", "vel"))
        p = s.read_grid("pressure")
        assert np.isfinite(p).all() and np.abs(p).max() > 0
