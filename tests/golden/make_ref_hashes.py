"""Generates tests/golden/ref_hashes.json: SHA-256 digests of states that pxlengine's own shader
computes on the benchmark workloads, too large to store as arrays.

shaders/fluid.slang, compiled for the CPU by oracle/ref_build.py and driven with the host schedule
of crates/pxl-render/src/fluid.rs (oracle/ref.py), runs bench.py's reference-solver workloads from
their seeded state (seed 0; seeding by the oracle's restatement of fluid.rs:119-148):
  dam64     64 x 32 x 32, 108,000 particles, GS 80: 200 substeps;
  dam256_gs 256 x 128 x 128, 8,001,504 particles, GS 80: 2 substeps;
  dam512    512 x 256 x 256, 95,134,176 particles, GS 80: 1 substep;
  scene     the reference's example scene as bench.py's DAM_BREAK_SCENE states it (64 x 38 x 32,
            139,200 particles, render fps 24, 8 substeps per frame): 24 frames (192 substeps), and
            the surface mesh of the final particles (refine 2, particle radius 2, iso as
            fluid.rs:150-156 with x*x*x for powi(3)).
For each: the particle count and the digests of the particles ([N, 8] float32 bytes) and of the
pressure (float32 bytes, x-fastest), plus the first particle in clear for diagnosis; for the scene
also the digests of the mesh's vertex records ([V, 8] float32) and triangle indices ([T, 3] uint32).
tests/test_gpu_reference_hashes.py requires the CUDA library to produce the same digests.

Run (needs the reference checkout; a few minutes, about 8 GB of memory for dam512):
    python tests/golden/make_ref_hashes.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_hashes.json")

# the reference-solver workloads of bench.py (bounds, resolution, fill, particles per cell, fps,
# substeps per frame, iterations) and the substeps each digest is taken after
SCENES = {
    "dam64": (((0, 0, 0), (1, 0.5, 0.5)), 64, [((0, 0, 0), (0.25, 0.5, 0.5))], 8, 15.0, 8, 80, 200),
    "dam256_gs": (((0, 0, 0), (1, 0.5, 0.5)), 256, [((0, 0, 0), (0.25, 0.5, 0.5))], 8, 15.0, 8, 80, 2),
    "dam512": (((0, 0, 0), (2, 1, 1)), 512, [((0, 0, 0), (0.6, 0.6, 1.0)), ((1.4, 0, 0), (2.0, 0.6, 1.0))],
               8, 15.0, 8, 80, 1),
    "scene": (((-1, 0, -0.5), (1, 1.2, 0.5)), 64, [((-0.97, 0.03, -0.47), (-0.35, 0.95, 0.47))], 8, 24.0, 8, 80,
              192),
}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(names=None):
    assert ref.available(), "the reference checkout is needed to generate these digests"
    out = {}
    if os.path.exists(OUT):
        out = json.load(open(OUT))
    for name, (bounds, res, fill, ppc, fps, per_frame, iters, substeps) in SCENES.items():
        if names and name not in names:
            continue
        b = [list(bounds[0]), list(bounds[1])]
        dims, h = oracle.grid(b, res)
        p0 = oracle.seed_particles(b, res, [{"min": list(lo), "max": list(hi)} for lo, hi in fill], ppc, 0)
        r = ref.RefSim(dims, h, oracle.dt_for(fps, per_frame), 0.95, b[0], [0.0, -9.81, 0.0], iters, p0)
        del p0
        r.step(substeps)
        parts = r.read("particles")
        out[name] = {"dims": list(dims), "particles": int(parts.shape[0]), "substeps": substeps,
                     "sha256_particles": digest(parts), "sha256_pressure": digest(r.read("pressure")),
                     "first_particle": [float(v) for v in parts[0]]}
        if name == "scene":
            refine, ppc = 2, 8
            sh = np.float32(np.float32(h) / np.float32(refine))
            radius = np.float32(np.float32(2.0) * sh)
            x = np.float32(radius / np.float32(h))
            iso = np.float32(np.float32(0.5) * np.float32(ppc) * np.float32(np.float32(0.638) * np.float32(x * x * x)))
            m = ref.surface_nets(parts, [d * refine for d in dims], sh, radius, iso, b[0], 2_000_000, 2_000_000)
            out[name]["mesh_vertices"] = int(m["vertices"].shape[0])
            out[name]["mesh_triangles"] = int(m["indices"].shape[0])
            out[name]["sha256_vertices"] = digest(m["vertices"])
            out[name]["sha256_indices"] = digest(m["indices"])
        print(name, out[name]["particles"], out[name]["sha256_particles"][:16], flush=True)
        del r, parts
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
