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
