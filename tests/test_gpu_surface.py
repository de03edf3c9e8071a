"""Surface nets on the GPU (pxf_surface_mesh) against the oracle's restatement of
shaders/fluid.slang:222-355 on the same particles: density, phi, cell vertices, vertex records
and triangles bit for bit, including the reference's caps on overflow."""
import numpy as np
import pytest

import oracle
import pxlengine_gb300 as P
from gpu_util import dam

pytestmark = pytest.mark.gpu


def _oracle_mesh(s, f, max_tris):
    info = s.surface_info()
    return oracle.surface_nets(s.read_particles(), info["dims"], info["cell"], info["radius"], info["iso"],
                               f.bounds[0], max_tris, max_tris)


def _same(s, m, o):
    np.testing.assert_array_equal(s.read_grid("surf_density"), o["density"])
    np.testing.assert_array_equal(s.read_grid("surf_phi"), o["phi"])
    np.testing.assert_array_equal(s.read_grid("surf_cell_vert"), o["cell_vert"])
    np.testing.assert_array_equal(m["vertices"], o["vertices"])
    np.testing.assert_array_equal(m["indices"], o["indices"])


@pytest.mark.parametrize("refine,substeps", [(2, 0), (2, 6), (1, 4), (3, 2)])
def test_mesh_bit_exact(lib, refine, substeps):
    f = dam(res=32, ppc=8, iters=30)
    f.surface_refine = refine
    with P.FluidState(f, fps=15.0) as s:
        s.step(substeps)
        m = s.surface_mesh()
        assert not m["overflow"] and len(m["vertices"]) > 0 and len(m["indices"]) > 0
        _same(s, m, _oracle_mesh(s, f, f.max_triangles))


def test_mesh_overflow_caps(lib):
    f = dam(res=32, ppc=8, iters=30)
    f.max_triangles = 900
    with P.FluidState(f, fps=15.0) as s:
        s.step(3)
        m = s.surface_mesh()
        assert m["overflow"]
        o = _oracle_mesh(s, f, 900)
        _same(s, m, o)
        assert len(m["vertices"]) == 900 and len(m["indices"]) <= 900 and len(m["indices"]) % 2 == 0


def test_mesh_from_scene_json_matches_oracle(lib):
    """The dam-break scene (examples/dam-break.json's fluid block) with a non-default refinement,
    radius and triangle budget, meshed after a frame."""
    scene = ('{"version":1,"nodes":[{"type":"camera"}],"fluids":[{"name":"water",'
             '"bounds":[[-1,0,-0.5],[1,1.2,0.5]],"resolution":48,'
             '"fill":[{"min":[-0.97,0.03,-0.47],"max":[-0.35,0.95,0.47]}],"substeps":8,"flip":0.95,'
             '"surface_refine":2,"particle_radius":1.6,"max_triangles":400000}]}')
    f = P.Fluid("water", [[-1, 0, -0.5], [1, 1.2, 0.5]], [], max_triangles=400000)
    with P.FluidState.from_json(scene) as s:
        s.fluid_advance(1.0)
        m = s.surface_mesh()
        _same(s, m, _oracle_mesh(s, f, 400000))
        out = s.surface_mesh()
        np.testing.assert_array_equal(out["vertices"], m["vertices"])
        np.testing.assert_array_equal(out["indices"], m["indices"])


def test_mesh_into_caller_buffers(lib):
    """pxf_surface_mesh_into writes the same mesh into the caller's device buffers at vbase / ibase
    (fluid.slang:313-314, 343-351), indices counted from vbase, and touches nothing else."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    f = dam(res=32, ppc=8, iters=30)
    with P.FluidState(f, fps=15.0) as s:
        s.step(4)
        o = _oracle_mesh(s, f, f.max_triangles)
        nv, ni = len(o["vertices"]), len(o["indices"])
        vbase, ibase = 37, 3 * 11
        vb = torch.full(((vbase + nv + 5) * 8,), -7.0, dtype=torch.float32, device="cuda")
        ib = torch.full((ibase + 3 * ni + 9,), -1, dtype=torch.int32, device="cuda")
        for cap_v, cap_t in ((0, 0), (nv // 2, ni // 3)):
            vb.fill_(-7.0)
            ib.fill_(-1)
            cv, ct, ov = C.c_uint32(), C.c_uint32(), C.c_int32()
            rc = lib.pxf_surface_mesh_into(s.h, C.c_void_p(vb.data_ptr()), vbase, cap_v, C.c_void_p(ib.data_ptr()),
                                           ibase, cap_t, C.byref(cv), C.byref(ct), C.byref(ov), None)
            assert rc == 0, lib.pxf_last_error(s.h).decode()
            v = vb.cpu().numpy().reshape(-1, 8)
            i = ib.cpu().numpy().view(np.uint32)
            if cap_v == 0:
                assert (cv.value, ct.value, ov.value) == (nv, ni, 0)
                np.testing.assert_array_equal(v[vbase:vbase + nv], o["vertices"])
                np.testing.assert_array_equal(i[ibase:ibase + 3 * ni].reshape(-1, 3), o["indices"])
            else:
                o2 = oracle.surface_nets(s.read_particles(), s.surface_info()["dims"], s.surface_info()["cell"],
                                         s.surface_info()["radius"], s.surface_info()["iso"], f.bounds[0],
                                         cap_v, cap_t)
                assert ov.value == 1 and cv.value == len(o2["vertices"]) and ct.value == len(o2["indices"])
                np.testing.assert_array_equal(v[vbase:vbase + cv.value], o2["vertices"])
                np.testing.assert_array_equal(i[ibase:ibase + 3 * ct.value].reshape(-1, 3), o2["indices"])
            n_written = cv.value
            assert (v[:vbase] == -7.0).all() and (v[vbase + n_written:] == -7.0).all()
            assert (i[:ibase] == 0xFFFFFFFF).all()
