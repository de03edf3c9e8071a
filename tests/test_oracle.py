"""The CPU oracle against the golden vectors and the reference's own stated values."""
import hashlib

import numpy as np
import pytest


def test_grid_known_answers(orc, golden):
    # crates/pxl-scene/src/lib.rs:886-899
    n, h = orc.grid([[0, 0, 0], [2, 1, 1]], 32)
    assert n == (32, 16, 16)
    assert abs(h - 0.0625) < 1e-6
    for g in golden["grid"]:
        n, h = orc.grid(g["bounds"], g["resolution"])
        assert list(n) == g["n"]
        assert np.float32(h) == np.float32(g["h"])


def test_lcg_stream(orc, golden):
    s = 0x9E3779B97F4A7C15
    for v in golden["lcg_seed0_first64"]:
        x, s = orc.lcg(s)
        assert np.float32(x) == np.float32(v)
    assert str(s) == golden["lcg_seed0_state_after64"]


@pytest.mark.parametrize("case", range(3))
def test_seeding_matches_golden(orc, golden, case):
    c = golden["seeding"][case]
    p = orc.seed_particles(c["bounds"], c["resolution"], c["fill"], c["ppc"], c["seed"])
    assert p.shape == (c["count"], 8)
    assert hashlib.sha256(p[:c["hashed"]].tobytes()).hexdigest() == c["sha256_f32"]
    np.testing.assert_array_equal(p[:len(c["first"])], np.asarray(c["first"], dtype=np.float32))


def test_dam_break_particle_count(orc, golden):
    # docs/ROADMAP.md:83 states 139k particles for the dam-break example.
    c = golden["seeding"][0]
    assert c["count"] == 139200
    assert abs(c["count"] - golden["reference_stated"]["dam_break_particles_approx"]) < 1000


def test_steps_for_frame(orc, golden):
    for c in golden["steps_for_frame"]:
        assert orc.steps_for_frame(c["warmup"], c["fps"], c["substeps"], c["frame"]) == c["steps"]


def _dam(orc, res=32, ppc=4, iters=20):
    b = [[0, 0, 0], [1, 0.5, 0.5]]
    dims, h = orc.grid(b, res)
    p = orc.seed_particles(b, res, [{"min": [0, 0, 0], "max": [0.25, 0.5, 0.5]}], ppc, 0)
    return dims, h, p


def test_oracle_thread_count_invariance(orc):
    dims, h, p = _dam(orc)
    dt = orc.dt_for(15, 8)
    res = []
    for t in (1, 4):
        orc.num_threads(t)
        s = orc.OracleSim(dims, h, dt, 0.95, [0, 0, 0], [0, -9.81, 0], 20, p)
        s.step(5)
        res.append((s.read(orc.PARTICLES), s.read(orc.VEL), s.read(orc.PRESSURE), s.read(orc.ACC)))
    orc.num_threads(0)
    for a, b in zip(res[0], res[1]):
        np.testing.assert_array_equal(a, b)


def test_oracle_invariants(orc):
    dims, h, p = _dam(orc)
    dt = orc.dt_for(15, 8)
    s = orc.OracleSim(dims, h, dt, 0.95, [0, 0, 0], [0, -9.81, 0], 20, p)
    s.step(10)
    q = s.read(orc.PARTICLES)
    n = np.array(dims, dtype=np.float32)
    lo = np.float32(0) + np.float32(h) * np.float32(1.001)
    hi = np.float32(0) + np.float32(h) * (n - np.float32(1.001))
    assert q.shape[0] == p.shape[0]
    assert np.all(q[:, :3] >= lo) and np.all(q[:, :3] <= hi)
    assert int(s.read(orc.CELL_COUNT).sum()) == p.shape[0]
    ct = s.read(orc.CELL_TYPE).reshape(dims[2], dims[1], dims[0])
    assert np.all(ct[0] == 2) and np.all(ct[-1] == 2) and np.all(ct[:, 0] == 2) and np.all(ct[:, :, -1] == 2)


def test_pcg_forms_converge_to_fp64(orc):
    dims, h, p = _dam(orc, res=32, ppc=4)
    dt = orc.dt_for(15, 8)
    sims = {}
    for mode, rtol in (("pcg", 1e-6), ("pcg64", 1e-12)):
        s = orc.OracleSim(dims, h, dt, 0.95, [0, 0, 0], [0, -9.81, 0], 20, p)
        s.set_pressure(mode, rtol=rtol, max_iter=5000)
        for _ in ("clear", "p2g", "normalize", "forces", "divergence", "pressure"):
            s.stage(_)
        it, rel = s.pcg_stats()
        assert rel <= rtol * 1.0001, (mode, it, rel)
        sims[mode] = s
    x32 = sims["pcg"].read(orc.PRESSURE64)
    x64 = sims["pcg64"].read(orc.PRESSURE64)
    assert np.max(np.abs(x32 - x64)) <= 1e-4 * max(1.0, np.max(np.abs(x64)))
