"""The oracle against pxlengine's own shader: shaders/fluid.slang compiled for the CPU
(oracle/ref_build.py + oracle/slang_shim.h; the host schedule of crates/pxl-render/src/fluid.rs:
278-318) runs the same seeded scenes, and every array the substep writes — particles, face
velocities before and after forces, the P2G fixed-point sums, cell counts and types, divergence,
pressure — must be the same bits after every stage of every substep; the surface pass (density,
phi, cell vertices, vertex records, triangles, counters with and without the overflow caps)
likewise. The shader's built-ins are bound to the semantics slang_shim.h states (lerp = FMix,
normalize = v / sqrt(dot), max / min / clamp, truncating int()).

Skipped where the reference checkout is absent (the GPU machine): the fixtures that
tests/golden/make_ref_golden.py wrote from the same runner stand in there."""
import numpy as np
import pytest

import oracle
from oracle import ref

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference checkout not available")

SEL = {"particles": oracle.PARTICLES, "vel": oracle.VEL, "vel_old": oracle.VEL_OLD, "acc": oracle.ACC,
       "wacc": oracle.WACC, "cell_count": oracle.CELL_COUNT, "cell_type": oracle.CELL_TYPE,
       "pressure": oracle.PRESSURE, "divergence": oracle.DIVERGENCE}


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype.itemsize == 4 else a


def same(a, b):
    return a.shape == b.shape and np.array_equal(bits(a), bits(b))


def pair(bounds, res, fill, ppc, iters, fps=24.0, substeps=8, flip=0.95, gravity=(0.0, -9.81, 0.0), seed=0):
    dims, h = oracle.grid(bounds, res)
    p = oracle.seed_particles(bounds, res, fill, ppc, seed)
    dt = oracle.dt_for(fps, substeps)
    o = oracle.OracleSim(dims, h, dt, flip, bounds[0], list(gravity), iters, p)
    r = ref.RefSim(dims, h, dt, flip, bounds[0], list(gravity), iters, p)
    return o, r, dims, h


def compare_stages(o, r, substeps):
    for step in range(substeps):
        for st in ref.STAGES:
            o.stage(st)
            r.stage(st)
            for name, sel in SEL.items():
                a, b = o.read(sel), r.read(name)
                assert same(a, b), (f"substep {step}, after {st}: {name} differs at "
                                    f"{np.flatnonzero(bits(a).reshape(-1) != bits(b).reshape(-1))[:5]}")


def test_dam_break_every_stage():
    o, r, _, _ = pair([[0, 0, 0], [1, 0.5, 0.5]], 24, [{"min": [0, 0, 0], "max": [0.3, 0.4, 0.5]}], 4, 80)
    compare_stages(o, r, 8)


def test_odd_grid_moving_fill_few_iterations():
    # odd sides, a fill block with an initial velocity, 7 red-black iterations, FLIP 0.6
    o, r, dims, _ = pair([[0, 0, 0], [1.17, 0.71, 0.53]], 37,
                         [{"min": [0.05, 0.02, 0.03], "max": [0.6, 0.5, 0.5], "velocity": [1.5, -0.5, 0.25]}],
                         3, 7, flip=0.6)
    assert dims[0] % 2 == 1
    compare_stages(o, r, 5)


def test_two_blocks_and_side_gravity_full_substeps():
    o, r, _, _ = pair([[-1, 0, -0.5], [1, 1.2, 0.5]], 32,
                      [{"min": [-0.97, 0.03, -0.47], "max": [-0.35, 0.95, 0.47]},
                       {"min": [0.5, 0.03, -0.2], "max": [0.9, 0.5, 0.2], "velocity": [-2.0, 0.0, 0.0]}],
                      4, 80, gravity=(0.5, -9.81, 0.25))
    for _ in range(6):
        o.step(1)
        r.step(1)
        for name, sel in SEL.items():
            assert same(o.read(sel), r.read(name)), name


def test_reference_cpu_case_64x32x32():
    # the reference's own CPU-runnable configuration: 64 x 32 x 32, 8 particles per cell, GS 80
    o, r, dims, _ = pair([[0, 0, 0], [1, 0.5, 0.5]], 64, [{"min": [0, 0, 0], "max": [0.25, 0.5, 0.5]}], 8, 80,
                         fps=15.0)
    assert dims == (64, 32, 32)
    for _ in range(3):
        o.step(1)
        r.step(1)
    for name, sel in SEL.items():
        assert same(o.read(sel), r.read(name)), name


@pytest.mark.parametrize("caps", [(200000, 400000), (60, 40), (3000, 7)])
def test_surface_nets(caps):
    o, _, dims, h = pair([[0, 0, 0], [1, 0.5, 0.5]], 24, [{"min": [0, 0, 0], "max": [0.3, 0.4, 0.5]}], 4, 80)
    o.step(4)
    parts = o.read(oracle.PARTICLES)
    refine, ppc = 2, 4
    sdims = [d * refine for d in dims]
    sh = np.float32(h / refine)
    radius = np.float32(2.0 * sh)
    iso = np.float32(0.5 * ppc * (0.638 * (radius / h) ** 3))
    a = oracle.surface_nets(parts, sdims, sh, radius, iso, [0, 0, 0], *caps)
    b = ref.surface_nets(parts, sdims, sh, radius, iso, [0, 0, 0], *caps)
    for k in ("density", "phi", "cell_vert", "vertices", "indices"):
        assert same(a[k], b[k]), k
    assert a["counts"] == b["counts"]
    assert b["counts"][0] > 0 and b["counts"][1] > 0


def test_committed_fixtures_come_from_the_runner(tmp_path, monkeypatch):
    """tests/golden/ref_golden.npz is what the reference runner writes today."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_ref_golden", os.path.join(here, "golden", "make_ref_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    monkeypatch.setattr(mod, "OUT", str(tmp_path / "fresh.npz"))
    mod.main()
    fresh = np.load(tmp_path / "fresh.npz")
    committed = np.load(os.path.join(here, "golden", "ref_golden.npz"))
    assert sorted(fresh.files) == sorted(committed.files)
    for k in fresh.files:
        assert np.array_equal(fresh[k], committed[k]), k


@pytest.mark.parametrize("n,cell_size,spread,table", [(0, 1.0, 1.0, 1024), (1, 0.5, 1.0, 1024), (5000, 0.01, 0.001, 16384),
                                                       (40000, 0.05, 4.0, 131072), (70000, 0.0, 1.0, 262144),
                                                       (200000, 0.5, 40.0, 1 << 19)])
def test_neighbor_grid(n, cell_size, spread, table):
    """The agents' neighbour grid of shaders/sim.slang:28-104 (grid_clear .. grid_scatter with the
    dispatches of crates/pxl-render/src/sim.rs:258-270, workgroups as teams of host threads)
    against oracle/neighbor_grid.py: offsets and counts equal, each cell's ids equal as a set
    (grid_scatter's atomics order them)."""
    from oracle import neighbor_grid as NG
    rng = np.random.default_rng(n + 7)
    a = np.zeros((n, 16), dtype=np.float32)
    a[:, :3] = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    a[:, 3:] = np.float32(7.0)
    ro, rc, rs = ref.grid_sort(a, cell_size, table)
    wo, wc, ws = NG.grid_sort(a[:, :3], cell_size, table)
    assert np.array_equal(ro, wo) and np.array_equal(rc, wc)
    h = NG.cells(a[:, :3], cell_size, table)
    assert np.array_equal(h[rs], np.repeat(np.arange(table, dtype=np.uint32), wc))
    key = lambda s: np.sort(h[s].astype(np.int64) * (n + 1) + s)
    assert np.array_equal(key(rs), key(ws))
