"""Parity with the oracle at the benchmark configurations' own sizes (shaders/fluid.slang:87-220,
schedule crates/pxl-render/src/fluid.rs:278-306), through the C ABI.

- 64 x 32 x 32 dam break (108,000 particles, red-black GS with 80 iterations): bit-exact after
  200 substeps;
- 256 x 128 x 128 dam break (8,001,504 particles) with the reference GS: bit-exact after 2
  substeps;
- 512 x 256 x 256 double dam break (95,134,176 particles): bit-exact after one substep, which runs
  the automatic P2G tile pick and the red-black GS streamed through shared memory on real data;
- 256 x 128 x 128 with the precision solver: pressure against the oracle's FP64 solve of the same
  system and the post-projection divergence;
- a batch whose members start from N(0, 0.5) velocities: each red-black member bit-exact with the
  oracle fed that member's seeded particles, the precision member within the solver tolerance.
"""
import numpy as np
import pytest

import oracle
import pxlengine_gb300 as P
from gpu_util import DIV_VOLUME_TOL, PCG_RTOL, dam, divergence_after_projection, grids_equal, oracle_for, \
    particles_equal

pytestmark = pytest.mark.gpu


def test_dam64_200_substeps_bit_exact(lib):
    f = dam(res=64, ppc=8, iters=80)
    with P.FluidState(f, fps=15.0, seed=0) as s:
        assert s.dims == (64, 32, 32) and s.particle_count() == 108000
        o = oracle_for(s, f)
        s.step(200)
        o.step(200)
        grids_equal(s, o)
        particles_equal(s, o)


def test_dam256_gs_two_substeps_bit_exact(lib):
    f = dam(res=256, ppc=8, iters=80)
    with P.FluidState(f, fps=15.0, seed=0) as s:
        assert s.dims == (256, 128, 128) and s.particle_count() == 8001504
        o = oracle_for(s, f)
        s.step(2)
        o.step(2)
        grids_equal(s, o)
        particles_equal(s, o)


def test_dam512_one_substep_bit_exact(lib):
    f = P.Fluid("dam512", [[0, 0, 0], [2, 1, 1]],
                [P.FluidBlock([0, 0, 0], [0.6, 0.6, 1.0]), P.FluidBlock([1.4, 0, 0], [2.0, 0.6, 1.0])],
                resolution=512, particles_per_cell=8, substeps=8, pressure_iterations=80)
    with P.FluidState(f, fps=15.0, seed=0, options=P.make_options(lift_grid_limits=True)) as s:
        assert s.dims == (512, 256, 256)
        o = oracle_for(s, f)
        s.step(1)
        o.step(1)
        grids_equal(s, o)
        particles_equal(s, o)


def test_dam256_precision_against_fp64(lib):
    f = dam(res=256, ppc=8)
    opts = P.make_options(solver="pcg", rtol=PCG_RTOL, max_iter=4000, restart=50)
    with P.FluidState(f, fps=15.0, seed=0, options=opts) as s:
        s.step(2)
        o64 = oracle_for(s, f)
        o64.set_pressure("pcg64", rtol=1e-10, max_iter=100000)
        s.step(1)
        it, rel, status = s.solver_stats()
        assert status == 0 and rel <= PCG_RTOL, (it, rel, status)
        for st in ("clear", "p2g", "normalize", "forces", "divergence"):
            o64.stage(st)
        grids_equal(s, o64, names=("cell_count", "cell_type", "vel_old", "divergence"))
        o64.stage("pressure")
        x64 = o64.read(oracle.PRESSURE64)
        xg = s.read_grid("pressure64")
        assert float(np.max(np.abs(xg - x64))) <= 1e-4 * max(1.0, float(np.max(np.abs(x64))))
        div = divergence_after_projection(s.read_grid("vel"), s.read_grid("cell_type"), s.dims, s.cell)
        assert float(np.max(np.abs(div))) * s.dt <= DIV_VOLUME_TOL


def test_batched_random_velocity_members_against_oracle(lib):
    specs = [(dam(res=32, ppc=4, iters=20), 0, "gs"),
             (P.Fluid("b", [[0, 0, 0], [0.8, 0.6, 0.5]], [P.FluidBlock([0.1, 0.0, 0.1], [0.5, 0.4, 0.4])],
                      resolution=48, particles_per_cell=5, pressure_iterations=35), 3, "gs"),
             (dam(res=40, ppc=6, iters=20), 2, "pcg")]
    sims = [P.FluidState(f, fps=24.0, seed=seed, options=P.make_options(
        solver=solver, rtol=PCG_RTOL, max_iter=4000, restart=50, velocity_sigma=0.5, velocity_seed=seed + 1))
        for f, seed, solver in specs]
    oracles = []
    for s, (f, _, solver) in zip(sims, specs):
        p0 = s.read_particles()
        assert np.abs(p0[:, 4:7]).max() > 0   # the seeded N(0, 0.5) velocities reach the oracle
        o = oracle_for(s, f, particles=p0)
        if solver == "pcg":
            o.set_pressure("mgpcg", rtol=PCG_RTOL, max_iter=4000, restart=50)
        oracles.append(o)
    b = P.Batch()
    try:
        for s in sims:
            b.add(s)
        b.step(1)
        b.sync()
        for s, o, (f, _, solver) in zip(sims, oracles, specs):
            o.step(1)
            if solver == "gs":
                grids_equal(s, o)
                particles_equal(s, o)
            else:
                grids_equal(s, o, names=("cell_count", "cell_type", "vel_old", "divergence"))
                xg, xo = s.read_grid("pressure64"), o.read(oracle.PRESSURE64)
                assert float(np.max(np.abs(xg - xo))) <= 1e-4 * max(1.0, float(np.max(np.abs(xo))))
        # two more substeps of the red-black members: still bit for bit
        b.step(2)
        b.sync()
        for s, o, (f, _, solver) in zip(sims, oracles, specs):
            if solver == "gs":
                o.step(2)
                grids_equal(s, o)
                particles_equal(s, o)
    finally:
        b.close()
        for s in sims:
            s.close()
