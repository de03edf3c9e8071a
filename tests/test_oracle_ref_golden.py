"""The oracle against the fixtures that pxlengine's own shader produced (tests/golden/ref_golden.npz,
written by tests/golden/make_ref_golden.py from shaders/fluid.slang run on the CPU): the same
seeded scenes through the oracle give the same bits. Runs everywhere; the GPU library meets the
same fixtures in tests/test_gpu_reference_golden.py."""
import os

import numpy as np

import oracle

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz"))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_dam_scene():
    bounds = [[0, 0, 0], [1, 0.5, 0.5]]
    dims, h = oracle.grid(bounds, 24)
    assert dims == tuple(GOLD["dam_dims"])
    p0 = oracle.seed_particles(bounds, 24, [{"min": [0, 0, 0], "max": [0.3, 0.4, 0.5]}], 4, 0)
    assert np.array_equal(bits(p0), bits(GOLD["dam_initial"]))
    o = oracle.OracleSim(dims, h, oracle.dt_for(24.0, 8), 0.95, bounds[0], [0, -9.81, 0], 80, p0)
    o.step(8)
    assert np.array_equal(bits(o.read(oracle.PARTICLES)), bits(GOLD["dam_particles"]))
    assert np.array_equal(bits(o.read(oracle.PRESSURE)), bits(GOLD["dam_pressure"]))
    assert np.array_equal(bits(o.read(oracle.VEL)), bits(GOLD["dam_vel"]))
    assert np.array_equal(o.read(oracle.CELL_TYPE), GOLD["dam_cell_type"])
    sh, radius, iso = (np.float32(v) for v in GOLD["dam_surface_params"])
    m = oracle.surface_nets(GOLD["dam_particles"], GOLD["dam_surface_dims"], sh, radius, iso, [0, 0, 0],
                           2_000_000, 2_000_000)
    assert np.array_equal(bits(m["vertices"]), bits(GOLD["dam_vertices"]))
    assert np.array_equal(m["indices"], GOLD["dam_indices"])


def test_odd_scene():
    bounds = [[0, 0, 0], [1.17, 0.71, 0.53]]
    dims, h = oracle.grid(bounds, 25)
    assert dims == tuple(GOLD["odd_dims"])
    p0 = oracle.seed_particles(bounds, 25, [{"min": [0.05, 0.02, 0.03], "max": [0.6, 0.5, 0.5],
                                             "velocity": [1.5, -0.5, 0.25]}], 2, 0)
    o = oracle.OracleSim(dims, h, oracle.dt_for(24.0, 8), 0.6, bounds[0], [0, -9.81, 0], 7, p0)
    o.step(5)
    assert np.array_equal(bits(o.read(oracle.PARTICLES)), bits(GOLD["odd_particles"]))
    assert np.array_equal(bits(o.read(oracle.PRESSURE)), bits(GOLD["odd_pressure"]))


def test_neighbor_grid():
    from oracle import neighbor_grid as NG
    o, c, srt = NG.grid_sort(GOLD["grid_positions"], 0.1, 8192)
    assert np.array_equal(o, GOLD["grid_offsets"]) and np.array_equal(c, GOLD["grid_counts"])
    assert np.array_equal(srt, GOLD["grid_sorted"])


def test_digests_of_the_benchmark_workloads():
    """The oracle reproduces the reference shader's digests on 64 x 32 x 32 after 200 substeps and
    256 x 128 x 128 after 2 (tests/golden/ref_hashes.json)."""
    import hashlib
    import json
    hashes = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_hashes.json")))
    for name, res in (("dam64", 64), ("dam256_gs", 256)):
        want = hashes[name]
        b = [[0, 0, 0], [1, 0.5, 0.5]]
        dims, h = oracle.grid(b, res)
        p0 = oracle.seed_particles(b, res, [{"min": [0, 0, 0], "max": [0.25, 0.5, 0.5]}], 8, 0)
        o = oracle.OracleSim(dims, h, oracle.dt_for(15.0, 8), 0.95, b[0], [0, -9.81, 0], 80, p0)
        o.step(want["substeps"])
        dig = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
        assert dig(o.read(oracle.PARTICLES)) == want["sha256_particles"], name
        assert dig(o.read(oracle.PRESSURE)) == want["sha256_pressure"], name


def test_example_scene_digests():
    """The oracle reproduces the reference shader's example scene after 24 frames (192 substeps)
    and its surface mesh (tests/golden/ref_hashes.json)."""
    import hashlib
    import json
    want = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                       "ref_hashes.json")))["scene"]
    dig = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    b = [[-1, 0, -0.5], [1, 1.2, 0.5]]
    dims, h = oracle.grid(b, 64)
    p0 = oracle.seed_particles(b, 64, [{"min": [-0.97, 0.03, -0.47], "max": [-0.35, 0.95, 0.47]}], 8, 0)
    o = oracle.OracleSim(dims, h, oracle.dt_for(24.0, 8), 0.95, b[0], [0, -9.81, 0], 80, p0)
    o.step(want["substeps"])
    parts = o.read(oracle.PARTICLES)
    assert dig(parts) == want["sha256_particles"] and dig(o.read(oracle.PRESSURE)) == want["sha256_pressure"]
    sh = np.float32(np.float32(h) / np.float32(2))
    radius = np.float32(np.float32(2.0) * sh)
    x = np.float32(radius / np.float32(h))
    iso = np.float32(np.float32(0.5) * np.float32(8) * np.float32(np.float32(0.638) * np.float32(x * x * x)))
    m = oracle.surface_nets(parts, [d * 2 for d in dims], sh, radius, iso, b[0], 2_000_000, 2_000_000)
    assert dig(m["vertices"]) == want["sha256_vertices"] and dig(m["indices"]) == want["sha256_indices"]
