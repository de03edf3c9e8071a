"""The CUDA library against digests of what pxlengine's own shader computes on the benchmark's
reference-solver workloads (tests/golden/ref_hashes.json, written by
tests/golden/make_ref_hashes.py from shaders/fluid.slang run on the CPU): 64 x 32 x 32 after 200
substeps, 256 x 128 x 128 after 2 and the 512 x 256 x 256 double dam break after 1 — particles and
pressure, bit for bit (SHA-256 of the float32 bytes) — and the reference's example scene after 24
frames, surface mesh included."""
import hashlib
import json
import os

import numpy as np
import pytest

import bench
import pxlengine_gb300 as P

pytestmark = pytest.mark.gpu

HASHES = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_hashes.json")))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["dam64", "dam256_gs", "dam512"])
def test_workload_matches_reference(lib, name):
    want = HASHES[name]
    cfg = bench.CONFIGS[name]
    opts = P.make_options(solver="gs", lift_grid_limits=cfg["lift"])
    with P.FluidState(bench.make_fluid(P, cfg), fps=cfg["fps"], seed=0, options=opts) as s:
        assert list(s.dims) == want["dims"] and s.particle_count() == want["particles"]
        s.step(want["substeps"])
        parts = s.read_particles()
        assert digest(parts) == want["sha256_particles"], f"first particle {parts[0]} vs {want['first_particle']}"
        assert digest(s.read_grid("pressure")) == want["sha256_pressure"]


def test_example_scene_24_frames_from_json(lib):
    """The reference's example scene through the scene-JSON front end (bench.py's
    DAM_BREAK_SCENE: render fps 24, seed 0): 24 frames of 8 substeps, then the surface mesh, the
    same bits as the reference's shader (particles, pressure, vertex records, triangles)."""
    want = HASHES["scene"]
    with P.FluidState.from_json(bench.DAM_BREAK_SCENE) as s:
        assert list(s.dims) == want["dims"] and s.particle_count() == want["particles"]
        s.step(want["substeps"])
        assert digest(s.read_particles()) == want["sha256_particles"]
        assert digest(s.read_grid("pressure")) == want["sha256_pressure"]
        m = s.surface_mesh()
        assert len(m["vertices"]) == want["mesh_vertices"] and len(m["indices"]) == want["mesh_triangles"]
        assert digest(m["vertices"]) == want["sha256_vertices"]
        assert digest(m["indices"].astype(np.uint32)) == want["sha256_indices"]
