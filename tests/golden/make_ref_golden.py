"""Generates tests/golden/ref_golden.npz: states computed by pxlengine's own shader.

shaders/fluid.slang, compiled for the CPU by oracle/ref_build.py and driven with the host
schedule of crates/pxl-render/src/fluid.rs (oracle/ref.py), runs two seeded scenes; the file keeps
what the CUDA library must reproduce bit for bit on a GPU machine, where the reference checkout is
absent (tests/test_gpu_reference_golden.py):
  dam: bounds [[0,0,0],[1,0.5,0.5]], resolution 24, fill [0,0,0]..[0.3,0.4,0.5], 4 particles per
       cell, seed 0, fps 24, 8 substeps per frame, FLIP 0.95, 80 red-black iterations: the seeded
       particles, then after 8 substeps the particles, pressure, face velocities and cell types, and
       the surface pass of those particles with FluidState::new's surface grid (refine 2, particle
       radius 2, iso from fluid.rs:150-156; x*x*x for powi(3)).
  odd: bounds [[0,0,0],[1.17,0.71,0.53]], resolution 25, fill [0.05,0.02,0.03]..[0.6,0.5,0.5]
       moving at (1.5,-0.5,0.25), 2 particles per cell, seed 0, fps 24, 8 substeps per frame,
       FLIP 0.6, 7 iterations: particles and pressure after 5 substeps.
  grid: the agents' neighbour grid (shaders/sim.slang:28-104) of 3,000 agents uniform in
       [-2, 2]^3 (numpy seed 5), cell size 0.1, table 8,192: offsets, counts and the ids of each cell
       in ascending order (the shader's own order inside a cell follows its atomics).
Seeding is the oracle's restatement of fluid.rs:119-148 (itself checked against golden.json).

Run (needs the reference checkout): python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")


def run(bounds, res, fill, ppc, iters, substeps, flip, fps=24.0, per_frame=8):
    dims, h = oracle.grid(bounds, res)
    p0 = oracle.seed_particles(bounds, res, fill, ppc, 0)
    r = ref.RefSim(dims, h, oracle.dt_for(fps, per_frame), flip, bounds[0], [0.0, -9.81, 0.0], iters, p0)
    r.step(substeps)
    return r, p0, dims, h


def main():
    assert ref.available(), "the reference checkout is needed to generate these fixtures"
    out = {}
    r, p0, dims, h = run([[0, 0, 0], [1, 0.5, 0.5]], 24, [{"min": [0, 0, 0], "max": [0.3, 0.4, 0.5]}], 4, 80, 8, 0.95)
    out["dam_dims"] = np.array(dims, dtype=np.uint32)
    out["dam_initial"] = p0
    for k in ("particles", "pressure", "vel", "cell_type"):
        out["dam_" + k] = r.read(k)
    refine, radius_cells, ppc = 2, np.float32(2.0), 4
    sdims = np.array([d * refine for d in dims], dtype=np.uint32)
    sh = np.float32(np.float32(h) / np.float32(refine))
    radius = np.float32(radius_cells * sh)
    x = np.float32(radius / np.float32(h))
    iso = np.float32(np.float32(0.5) * np.float32(ppc) * np.float32(np.float32(0.638) * np.float32(x * x * x)))
    m = ref.surface_nets(out["dam_particles"], sdims, sh, radius, iso, [0, 0, 0], 2_000_000, 2_000_000)
    out["dam_surface_params"] = np.array([sh, radius, iso], dtype=np.float32)
    out["dam_surface_dims"] = sdims
    out["dam_vertices"] = m["vertices"]
    out["dam_indices"] = m["indices"]
    r, p0, dims, h = run([[0, 0, 0], [1.17, 0.71, 0.53]], 25,
                         [{"min": [0.05, 0.02, 0.03], "max": [0.6, 0.5, 0.5], "velocity": [1.5, -0.5, 0.25]}],
                         2, 7, 5, 0.6)
    out["odd_dims"] = np.array(dims, dtype=np.uint32)
    out["odd_particles"] = r.read("particles")
    out["odd_pressure"] = r.read("pressure")
    rng = np.random.default_rng(5)
    agents = np.zeros((3000, 16), dtype=np.float32)
    agents[:, :3] = rng.uniform(-2, 2, (3000, 3)).astype(np.float32)
    offs, cnts, srt = ref.grid_sort(agents, 0.1, 8192)
    for h in np.nonzero(cnts)[0]:
        srt[offs[h]:offs[h] + cnts[h]] = np.sort(srt[offs[h]:offs[h] + cnts[h]])
    out["grid_positions"] = agents[:, :3].copy()
    out["grid_offsets"] = offs
    out["grid_counts"] = cnts
    out["grid_sorted"] = srt
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
