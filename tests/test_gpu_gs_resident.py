"""The red-black GS pressure solve as one cooperative launch whose blocks own fixed cell ranges
and wait only for the blocks within one z-plane of them, against the oracle's plain sweep order,
bit for bit (shaders/fluid.slang:167-182, crates/pxl-render/src/fluid.rs:295-300).

The library takes this path for red-black grids of 2^21 cells up to the streamed threshold when
the plan fits; these tests force it (PXF_GS_RESIDENT=1, read when a simulation's batch is built)
on smaller grids, and PXF_GS_RESIDENT=0 keeps one launch per colour. PXF_GS_RES_CELLS (read once
per process) sets the smallest range per block; these tests use the default, so small grids get
one or a few blocks and the larger ones up to one per SM, with two to four neighbours each. The failure path:
a block that returns at once (PXF_GS_RES_SKIP) leaves its neighbours' waits to run out
(PXF_GS_RES_LIMIT_MS); they set the error word, every block returns, the host reports
PXF_ETIMEDOUT and the context stays usable."""
import numpy as np
import pytest

import pxlengine_gb300 as P
from pxlengine_gb300 import _lib as L
from gpu_util import dam, grids_equal, oracle_for, particles_equal

pytestmark = pytest.mark.gpu


def kernels_of(s):
    return {name: launches for name, launches, _ in s.profile_substep()}


@pytest.fixture(autouse=True)
def resident(monkeypatch):
    monkeypatch.setenv("PXF_GS_RESIDENT", "1")
    monkeypatch.setenv("PXF_GS_STREAM", "0")


def test_path_is_taken(lib):
    f = dam(res=64, ppc=2, iters=80)
    with P.FluidState(f, fps=24.0, seed=1) as s:
        k = kernels_of(s)
        assert k.get("k_gs_resident") == 1
        assert "k_pressure_rb_list" not in k


@pytest.mark.parametrize("res,iters", [(16, 80), (40, 80), (37, 7), (96, 80)])
def test_bit_exact(lib, res, iters):
    f = dam(res=res, ppc=3, iters=iters)
    with P.FluidState(f, fps=24.0, seed=res) as s:
        o = oracle_for(s, f)
        s.step(3)
        o.step(3)
        grids_equal(s, o)
        particles_equal(s, o)


def test_many_blocks_odd_grid_bit_exact(lib):
    # 130 x 65 x 97 (819,650 cells): the whole GPU's blocks, ranges that end inside rows and planes
    f = P.Fluid("odd", [[0, 0, 0], [1.3, 0.65, 0.97]], [P.FluidBlock([0, 0, 0], [0.5, 0.45, 0.97])],
                resolution=130, particles_per_cell=2, pressure_iterations=80)
    with P.FluidState(f, fps=15.0, seed=2) as s:
        assert s.dims == (130, 65, 97)
        o = oracle_for(s, f)
        s.step(2)
        o.step(2)
        grids_equal(s, o)
        particles_equal(s, o)


def test_same_bits_as_one_launch_per_colour(lib, monkeypatch):
    f = dam(res=64, ppc=4, iters=80, fill_max=(0.4, 0.45, 0.5))
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("PXF_GS_RESIDENT", mode)
        with P.FluidState(f, fps=24.0, seed=5) as s:
            s.step(12)
            out[mode] = (s.read_grid("pressure"), s.read_particles())
    np.testing.assert_array_equal(out["1"][0].view(np.uint32), out["0"][0].view(np.uint32))
    np.testing.assert_array_equal(out["1"][1].view(np.uint32), out["0"][1].view(np.uint32))


def test_batch_shares_blocks_bit_exact(lib):
    """One launch serves red-black simulations of different sizes and iteration counts (and a
    precision-solver simulation beside them); each equals its own oracle run."""
    fl = [dam(res=24, ppc=3, iters=3), dam(res=64, ppc=2, iters=12, fill_max=(0.4, 0.3, 0.5)),
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


def test_neighbour_wait_runs_out_and_context_survives(lib, monkeypatch):
    monkeypatch.setenv("PXF_GS_RES_SKIP", "1")
    monkeypatch.setenv("PXF_GS_RES_LIMIT_MS", "5")
    f = dam(res=64, ppc=2, iters=80)
    with P.FluidState(f, fps=24.0, seed=3) as s:
        with pytest.raises(P.FluidError) as ei:
            s.step(1)
            s.sync()
        assert ei.value.code == L.PXF_ETIMEDOUT
        assert "timed out" in str(ei.value)
    monkeypatch.delenv("PXF_GS_RES_SKIP")
    monkeypatch.delenv("PXF_GS_RES_LIMIT_MS")
    with P.FluidState(f, fps=24.0, seed=3) as s:
        o = oracle_for(s, f)
        s.step(2)
        o.step(2)
        grids_equal(s, o)
