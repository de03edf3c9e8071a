"""Helpers shared by the GPU tests: build a GPU simulation and the oracle on identical inputs."""
import numpy as np

import oracle
import pxlengine_gb300 as P

# Tolerances. The FP32 substep is claimed bit-exact against the oracle (same operations in the
# same order, no contraction), so every comparison of the reference form uses tolerance 0.
EXACT = 0.0
# Precision solver: relative residual target and the bound on the post-projection divergence,
# expressed as the fraction of a cell's volume gained or lost in one substep (|div| * dt).
PCG_RTOL = 1e-6
DIV_VOLUME_TOL = 1e-5


def dam(res=32, ppc=4, fill_max=(0.25, 0.5, 0.5), bounds=((0, 0, 0), (1, 0.5, 0.5)), iters=80, flip=0.95,
        velocity=(0.0, 0.0, 0.0), substeps=8):
    return P.Fluid("dam", [list(bounds[0]), list(bounds[1])],
                   [P.FluidBlock([bounds[0][0], bounds[0][1], bounds[0][2]], list(fill_max), list(velocity))],
                   resolution=res, particles_per_cell=ppc, pressure_iterations=iters, flip=flip, substeps=substeps)


def oracle_for(sim: P.FluidState, fluid: P.Fluid, particles=None, dtype=np.float32):
    p = sim.read_particles() if particles is None else particles
    return oracle.OracleSim(sim.dims, sim.cell, sim.dt, fluid.flip, fluid.bounds[0], fluid.gravity,
                            fluid.pressure_iterations, p, dtype=dtype)


def grids_equal(sim: P.FluidState, o, names=("cell_count", "cell_type", "vel_old", "divergence", "pressure", "vel"),
                acc=False):
    table = {"vel": oracle.VEL, "vel_old": oracle.VEL_OLD, "acc": oracle.ACC, "wacc": oracle.WACC,
             "cell_count": oracle.CELL_COUNT, "cell_type": oracle.CELL_TYPE, "pressure": oracle.PRESSURE,
             "divergence": oracle.DIVERGENCE}
    names = list(names) + (["acc", "wacc"] if acc else [])
    for n in names:
        g = sim.read_grid(n)
        r = o.read(table[n])
        if g.dtype.kind == "f":
            bad = np.flatnonzero(g.view(np.uint32) != r.astype(g.dtype).view(np.uint32))
        else:
            bad = np.flatnonzero(g != r)
        assert bad.size == 0, f"{n}: {bad.size} mismatches, first at {bad[:5]}: gpu {g[bad[:5]]} oracle {r[bad[:5]]}"


def particles_equal(sim: P.FluidState, o):
    g = sim.read_particles()
    r = o.read(oracle.PARTICLES)
    bad = np.flatnonzero(np.any(g.view(np.uint32) != r.view(np.uint32), axis=1))
    assert bad.size == 0, f"particles: {bad.size} mismatches, first {bad[:3]}: gpu {g[bad[:3]]} oracle {r[bad[:3]]}"


def divergence_after_projection(vel: np.ndarray, ctype: np.ndarray, dims, h):
    """FP64 divergence of a face velocity field at the fluid cells (fluid.slang:153-165)."""
    nx, ny, nz = dims
    nu = (nx + 1) * ny * nz
    nv = nx * (ny + 1) * nz
    u = vel[:nu].astype(np.float64).reshape(nz, ny, nx + 1)
    v = vel[nu:nu + nv].astype(np.float64).reshape(nz, ny + 1, nx)
    w = vel[nu + nv:].astype(np.float64).reshape(nz + 1, ny, nx)
    d = (u[:, :, 1:] - u[:, :, :-1]) + (v[:, 1:, :] - v[:, :-1, :]) + (w[1:] - w[:-1])
    d = d.reshape(-1) / h
    return np.where(ctype == 1, d, 0.0)
