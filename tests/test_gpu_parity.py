"""Parity of the CUDA substep (through the C ABI) with the CPU oracle on identical inputs.

The reference form is compared bit for bit: integer arrays (cell counts, flags, P2G sums) and
every FP32 array (velocities, divergence, pressure, particles)."""
import hashlib

import numpy as np
import pytest

import oracle
import pxlengine_gb300 as P
from gpu_util import dam, grids_equal, oracle_for, particles_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", range(3))
def test_device_seeding_matches_golden(lib, golden, case):
    c = golden["seeding"][case]
    f = P.Fluid("s", c["bounds"], [P.FluidBlock(b["min"], b["max"], b.get("velocity", (0, 0, 0))) for b in c["fill"]],
                resolution=c["resolution"], particles_per_cell=c["ppc"])
    with P.FluidState(f, fps=24.0, seed=c["seed"]) as s:
        p = s.read_particles()
        assert p.shape == (c["count"], 8)
        assert hashlib.sha256(p[:c["hashed"]].tobytes()).hexdigest() == c["sha256_f32"]
        ref = oracle.seed_particles(c["bounds"], c["resolution"], c["fill"], c["ppc"], c["seed"])
        np.testing.assert_array_equal(p, ref)


def test_dam_break_scene_from_json(lib):
    scene = ('{"version":1,"nodes":[{"type":"camera"}],"fluids":[{"name":"water",'
             '"bounds":[[-1,0,-0.5],[1,1.2,0.5]],"resolution":64,'
             '"fill":[{"min":[-0.97,0.03,-0.47],"max":[-0.35,0.95,0.47]}],"substeps":8,"flip":0.95}]}')
    with P.FluidState.from_json(scene) as s:
        assert s.particle_count() == 139200
        assert s.dims == (64, 38, 32)
        assert abs(s.dt - np.float32(1.0 / (24.0 * 8))) == 0


@pytest.mark.parametrize("shape", ["dam32", "odd", "thin", "vel_blocks"])
def test_one_substep_bit_exact(lib, shape):
    if shape == "dam32":
        f = dam(res=32, ppc=4)
    elif shape == "odd":   # dims not multiples of any tile shape
        f = P.Fluid("odd", [[0, 0, 0], [1.17, 0.71, 0.53]],
                    [P.FluidBlock([0.05, 0.02, 0.03], [0.6, 0.5, 0.5], [0.3, -0.2, 0.1])],
                    resolution=37, particles_per_cell=3, pressure_iterations=30)
    elif shape == "thin":  # one axis at the 4-cell minimum
        f = P.Fluid("thin", [[0, 0, 0], [1, 0.25, 1]], [P.FluidBlock([0, 0, 0], [1, 0.25, 0.6])],
                    resolution=16, particles_per_cell=1, pressure_iterations=10)
    else:
        f = P.Fluid("two", [[-0.5, 0, 0], [0.5, 0.6, 0.4]],
                    [P.FluidBlock([-0.5, 0, 0], [-0.2, 0.4, 0.4], [2.0, 0, 0]),
                     P.FluidBlock([0.1, 0.0, 0.0], [0.5, 0.2, 0.4], [-1.0, 0.5, 0.25])],
                    resolution=40, particles_per_cell=6, pressure_iterations=40, flip=0.8)
    opts = P.make_options(keep_p2g_sums=True)
    with P.FluidState(f, fps=24.0, seed=5, options=opts) as s:
        o = oracle_for(s, f)
        s.step(1)
        o.step(1)
        grids_equal(s, o, acc=True)
        particles_equal(s, o)


def test_thirty_substeps_bit_exact(lib):
    f = dam(res=40, ppc=8, iters=80)
    with P.FluidState(f, fps=15.0, seed=0) as s:
        o = oracle_for(s, f)
        s.step(30)
        o.step(30)
        grids_equal(s, o)
        particles_equal(s, o)


def _random_state(s, pile):
    n = s.particle_count()
    nx, ny, nz = s.dims
    h = np.float32(s.cell)
    rng = np.random.default_rng(1234)
    p = np.zeros((n, 8), dtype=np.float32)
    lo = h * np.float32(1.001)
    hi = h * (np.array([nx, ny, nz], dtype=np.float32) - np.float32(1.001))
    p[:, :3] = (lo + rng.random((n, 3), dtype=np.float32) * (hi - lo)).astype(np.float32)
    k = n // 4
    p[:k, :3] = (rng.integers(1, [nx - 1, ny - 1, nz - 1], size=(k, 3)).astype(np.float32) * h)
    p[k:k + pile, :3] = np.float32(5.5) * h           # a pile of particles in one cell
    p[:, 4:7] = rng.normal(0, 2.0, (n, 3)).astype(np.float32)
    p[:50, 4:7] *= np.float32(50.0)
    s.write_particles(p)
    return p


@pytest.mark.parametrize("pile", [300, 5000])
def test_random_particles_and_edges(lib, pile):
    """Arbitrary particle states: jittered positions, exact cell-boundary positions, a pile of
    particles in one cell (5000 exceeds the packed P2G accumulation's per-cell bound and takes
    the two-atomic path), velocities of both signs and magnitudes."""
    f = dam(res=24, ppc=2) if pile < 1000 else dam(res=32, ppc=8)
    with P.FluidState(f, fps=24.0, seed=1, options=P.make_options(keep_p2g_sums=True)) as s:
        p = _random_state(s, pile)
        np.testing.assert_array_equal(s.read_particles(), p * np.array([1, 1, 1, 0, 1, 1, 1, 0], np.float32))
        o = oracle_for(s, f)
        s.step(1)
        o.step(1)
        grids_equal(s, o, acc=True)
        particles_equal(s, o)
        s.step(3)
        o.step(3)
        grids_equal(s, o)
        particles_equal(s, o)


@pytest.mark.parametrize("order", ["1", "0"])
def test_p2g_variants_on_a_pile(lib, monkeypatch, order):
    """Every P2G tile shape and lane mapping, with the heaviest-first tile order or in index
    order, gives the oracle's integer sums on a random state with a 5000-particle pile in one
    cell."""
    monkeypatch.setenv("PXF_P2G_ORDER", order)
    f = dam(res=32, ppc=8)
    ref = None
    for lanes in ("0", "1"):
        monkeypatch.setenv("PXF_P2G_STRIDED", lanes)
        for shape in range(5):
            opts = P.make_options(keep_p2g_sums=True, p2g_tile=shape)
            with P.FluidState(f, fps=24.0, seed=1, options=opts) as s:
                _random_state(s, 5000)
                if ref is None:
                    ref = oracle_for(s, f)
                    ref.step(1)
                s.step(1)
                grids_equal(s, ref, acc=True)
                particles_equal(s, ref)


@pytest.mark.parametrize("fair", ["0", "4294967295"])
def test_p2g_automatic_shape_branches(lib, monkeypatch, fair):
    """The automatic P2G tile shape is two IF nodes in the substep graph whose conditions a
    kernel sets from the 32x8x8 tile buckets (eager substeps read the buckets back). Forcing
    the small tiles (threshold 0) or the large ones (no threshold) gives the oracle's bits over
    graph and eager substeps of a random state with a pile."""
    monkeypatch.delenv("PXF_P2G_TILE", raising=False)
    monkeypatch.setenv("PXF_P2G_FAIR", fair)
    f = dam(res=32, ppc=8)
    with P.FluidState(f, fps=24.0, seed=1, options=P.make_options(keep_p2g_sums=True)) as s:
        _random_state(s, 5000)
        o = oracle_for(s, f)
        s.step(2)
        s.profile_substep()
        o.step(3)
        grids_equal(s, o, acc=True)
        particles_equal(s, o)


def test_run_to_run_determinism(lib):
    f = dam(res=48, ppc=8, iters=40)
    out = []
    for _ in range(2):
        with P.FluidState(f, fps=15.0) as s:
            s.step(10)
            out.append((s.read_particles(), s.read_grid("vel"), s.read_grid("pressure")))
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_advance_to_frame_and_rewind(lib):
    f = dam(res=24, ppc=4, iters=30, substeps=8)
    with P.FluidState(f, fps=24.0) as s:
        p0 = s.read_particles()
        o = oracle_for(s, f, particles=p0)
        s.fluid_advance(1.0)
        assert s.steps_done == 8
        o.step(8)
        particles_equal(s, o)
        s.fluid_advance(2.5)
        assert s.steps_done == 20
        o.step(12)
        particles_equal(s, o)
        # Backwards seek: particles re-seeded, pressure warm start kept (fluid.rs:271-275).
        warm = s.read_grid("pressure")
        s.fluid_advance(0.5)
        assert s.steps_done == 4
        o2 = oracle_for(s, f, particles=p0)
        o2.write(oracle.PRESSURE, warm)
        o2.step(4)
        particles_equal(s, o2)
        s.fluid_advance(0.5)   # same frame: no work
        assert s.steps_done == 4


def test_snapshot_restore(lib):
    f = dam(res=24, ppc=4, iters=20)
    with P.FluidState(f, fps=24.0) as s:
        s.step(3)
        snap = s.snapshot()
        s.step(2)
        a = s.read_particles()
        s.restore(snap)
        assert s.steps_done == 3
        s.step(2)
        np.testing.assert_array_equal(a, s.read_particles())


def test_large_grid_properties(lib):
    """256 x 128 x 128 dam break (8.0M particles): conservation and containment after substeps."""
    f = dam(res=256, ppc=8, iters=20)
    with P.FluidState(f, fps=15.0) as s:
        assert s.particle_count() == 8001504
        s.step(3)
        p = s.read_particles()
        counts = s.read_grid("cell_count")
        assert int(counts.sum(dtype=np.int64)) == 8001504
        nx, ny, nz = s.dims
        h = np.float32(s.cell)
        lo = h * np.float32(1.001)
        hi = h * (np.array([nx, ny, nz], dtype=np.float32) - np.float32(1.001))
        assert np.all(np.isfinite(p))
        assert np.all(p[:, :3] >= lo) and np.all(p[:, :3] <= hi)
        ct = s.read_grid("cell_type")
        assert np.array_equal(ct == 1, (counts > 0) & (ct != 2))


def test_stress_double_dam_break_512(lib):
    """512 x 256 x 256 with two boxes against opposite walls (about 95M particles, beyond the scene
    validator's limits): conservation, finiteness and containment after two substeps."""
    f = P.Fluid("stress", [[0, 0, 0], [2, 1, 1]],
                [P.FluidBlock([0, 0, 0], [0.6, 0.6, 1.0]), P.FluidBlock([1.4, 0, 0], [2.0, 0.6, 1.0])],
                resolution=512, particles_per_cell=8, substeps=8, pressure_iterations=80)
    with P.FluidState(f, fps=15.0, options=P.make_options(lift_grid_limits=True)) as s:
        n = s.particle_count()
        assert s.dims == (512, 256, 256) and 94_000_000 < n < 96_500_000
        s.step(2)
        counts = s.read_grid("cell_count")
        assert int(counts.sum(dtype=np.int64)) == n
        p = s.read_particles()
        assert np.all(np.isfinite(p))
        h = np.float32(s.cell)
        hi = h * (np.array([512, 256, 256], dtype=np.float32) - np.float32(1.001))
        assert np.all(p[:, :3] >= h * np.float32(1.001)) and np.all(p[:, :3] <= hi)
