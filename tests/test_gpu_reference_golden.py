"""The CUDA library against states computed by pxlengine's own shader (shaders/fluid.slang run on
the CPU; tests/golden/ref_golden.npz, written by tests/golden/make_ref_golden.py): the same seeded
scenes through the C ABI give the same bits — seeding, 8 and 5 substeps of the reference solver
(particles, pressure, face velocities, cell types) and the surface mesh of the final particles."""
import os

import numpy as np
import pytest

import pxlengine_gb300 as P
from gpu_util import dam

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz"))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_dam_scene(lib):
    f = dam(res=24, ppc=4, fill_max=(0.3, 0.4, 0.5), iters=80)
    with P.FluidState(f, fps=24.0, seed=0) as s:
        assert s.dims == tuple(GOLD["dam_dims"])
        assert np.array_equal(bits(s.read_particles()), bits(GOLD["dam_initial"]))
        s.step(8)
        assert np.array_equal(bits(s.read_particles()), bits(GOLD["dam_particles"]))
        assert np.array_equal(bits(s.read_grid("pressure")), bits(GOLD["dam_pressure"]))
        assert np.array_equal(bits(s.read_grid("vel")), bits(GOLD["dam_vel"]))
        assert np.array_equal(s.read_grid("cell_type").astype(np.uint32), GOLD["dam_cell_type"])
        info = s.surface_info()
        assert tuple(info["dims"]) == tuple(GOLD["dam_surface_dims"])
        sh, radius, iso = (np.float32(v) for v in GOLD["dam_surface_params"])
        assert (np.float32(info["cell"]), np.float32(info["radius"]), np.float32(info["iso"])) == (sh, radius, iso)
        m = s.surface_mesh()
        assert not m["overflow"]
        assert np.array_equal(bits(m["vertices"]), bits(GOLD["dam_vertices"]))
        assert np.array_equal(m["indices"].astype(np.uint32), GOLD["dam_indices"])


def test_odd_scene(lib):
    f = P.Fluid("odd", [[0, 0, 0], [1.17, 0.71, 0.53]],
                [P.FluidBlock([0.05, 0.02, 0.03], [0.6, 0.5, 0.5], [1.5, -0.5, 0.25])],
                resolution=25, particles_per_cell=2, pressure_iterations=7, flip=0.6)
    with P.FluidState(f, fps=24.0, seed=0) as s:
        assert s.dims == tuple(GOLD["odd_dims"])
        s.step(5)
        assert np.array_equal(bits(s.read_particles()), bits(GOLD["odd_particles"]))
        assert np.array_equal(bits(s.read_grid("pressure")), bits(GOLD["odd_pressure"]))


def test_neighbor_grid(lib):
    torch = pytest.importorskip("torch")
    import ctypes as C
    pos = GOLD["grid_positions"]
    n, table = pos.shape[0], 8192
    rec = np.zeros((n, 16), dtype=np.float32)
    rec[:, :3] = pos
    d_rec = torch.from_numpy(rec).to("cuda")
    off = torch.zeros(table, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(table, dtype=torch.int32, device="cuda")
    srt = torch.zeros(n, dtype=torch.int32, device="cuda")
    sb = lib.pxf_grid_scratch_bytes(n, table)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    rc = lib.pxf_grid_sort(C.c_void_p(d_rec.data_ptr()), 16, n, C.c_float(0.1), table, C.c_void_p(off.data_ptr()),
                           C.c_void_p(cnt.data_ptr()), C.c_void_p(srt.data_ptr()), C.c_void_p(scratch.data_ptr()),
                           sb, None)
    assert rc == 0, lib.pxf_last_error(None).decode()
    torch.cuda.synchronize()
    o, c, s = (t.cpu().numpy().view(np.uint32) for t in (off, cnt, srt))
    assert np.array_equal(o, GOLD["grid_offsets"]) and np.array_equal(c, GOLD["grid_counts"])
    for h in np.nonzero(c)[0]:
        s[o[h]:o[h] + c[h]] = np.sort(s[o[h]:o[h] + c[h]])
    assert np.array_equal(s, GOLD["grid_sorted"])
