"""Scene-JSON front end: defaults, strictness and validation messages of the reference
(crates/pxl-scene/src/lib.rs:49-129, 710-735), exercised through the C ABI without a GPU."""
import ctypes as C
import json

import pytest

import pxlengine_gb300 as P
from pxlengine_gb300 import _lib as L

# The scene of the reference's `fluids_validate` test (crates/pxl-scene/src/lib.rs:886-899).
OK = {"version": 1, "nodes": [{"type": "camera"}],
      "fluids": [{"name": "w", "bounds": [[0, 0, 0], [2, 1, 1]], "resolution": 32,
                  "fill": [{"min": [0.1, 0.1, 0.1], "max": [0.5, 0.5, 0.5]}]}]}


def count(lib, scene):
    text = scene if isinstance(scene, str) else json.dumps(scene)
    rc = lib.pxf_scene_fluid_count(text.encode())
    msg = lib.pxf_last_error(None).decode()
    return rc, msg


def with_fluid(**kw):
    s = json.loads(json.dumps(OK))
    s["fluids"][0].update(kw)
    return s


def test_fluids_validate_reference_case(lib):
    assert count(lib, OK) == (1, count(lib, OK)[1])
    f = P.Fluid("w", [[0, 0, 0], [2, 1, 1]], [P.FluidBlock([0.1] * 3, [0.5] * 3)], resolution=32)
    n, h = f.grid()
    assert n == (32, 16, 16) and abs(h - 0.0625) < 1e-6
    outside = with_fluid(fill=[{"min": [0.1, 0.1, 0.1], "max": [0.5, 0.5, 1.5]}])
    rc, msg = count(lib, outside)
    assert rc == L.PXF_EINVAL and "inside" in msg
    assert msg == "fluids[0] 'w': each fill block must have max > min and lie inside `bounds`"


@pytest.mark.parametrize("field,value", [("resolution", 15), ("resolution", 257), ("particles_per_cell", 0),
                                         ("particles_per_cell", 65), ("substeps", 0), ("substeps", 65),
                                         ("surface_refine", 0), ("surface_refine", 4), ("flip", 1.5),
                                         ("flip", -0.1), ("pressure_iterations", 0)])
def test_range_checks(lib, field, value):
    rc, msg = count(lib, with_fluid(**{field: value}))
    assert rc == L.PXF_EINVAL
    assert msg == ("fluids[0] 'w': resolution 16..256, particles_per_cell 1..64, substeps 1..64, "
                   "surface_refine 1..3, flip 0..1")


def test_bounds_and_fill_checks(lib):
    rc, msg = count(lib, with_fluid(bounds=[[0, 0, 0], [2, 0, 1]]))
    assert rc == L.PXF_EINVAL and msg.endswith("bounds must be [min, max] with max > min on every axis")
    rc, msg = count(lib, with_fluid(fill=[]))
    assert rc == L.PXF_EINVAL and msg.endswith("needs at least one `fill` block of liquid")
    rc, msg = count(lib, with_fluid(fill=[{"min": [0.5, 0.1, 0.1], "max": [0.5, 0.5, 0.5]}]))
    assert rc == L.PXF_EINVAL and "inside" in msg


def test_grid_too_large(lib):
    # 256 cells along x of a 2:2:1 box is 256 x 256 x 128 = 8.4M cells: accepted; a cube at 256 is 16.8M.
    rc, _ = count(lib, with_fluid(bounds=[[0, 0, 0], [2, 2, 1]], resolution=256))
    assert rc == 1
    rc, msg = count(lib, with_fluid(bounds=[[0, 0, 0], [1, 1, 1]], resolution=256))
    assert rc == L.PXF_EINVAL and msg.endswith("grid too large (lower resolution)")


def test_strict_fields(lib):
    rc, msg = count(lib, with_fluid(resolutoin=32))
    assert rc == L.PXF_EINVAL and "unknown field `resolutoin`" in msg and msg.startswith("invalid scene: ")
    s = json.loads(json.dumps(OK))
    s["fluids"][0]["fill"][0]["vel"] = [0, 0, 0]
    rc, msg = count(lib, s)
    assert rc == L.PXF_EINVAL and "unknown field `vel`" in msg
    s = json.loads(json.dumps(OK))
    del s["fluids"][0]["name"]
    rc, msg = count(lib, s)
    assert rc == L.PXF_EINVAL and "missing field `name`" in msg
    rc, msg = count(lib, with_fluid(resolution=32.0))
    assert rc == L.PXF_EINVAL and "expected u32" in msg
    rc, msg = count(lib, with_fluid(resolution=-1))
    assert rc == L.PXF_EINVAL and "expected u32" in msg
    rc, msg = count(lib, '{"version":1,"nodes":[{"type":"camera"}],"fluids":[')
    assert rc == L.PXF_EINVAL and msg.startswith("invalid scene: ")


def test_scene_level_checks(lib):
    s = json.loads(json.dumps(OK))
    s["version"] = 2
    assert count(lib, s) == (L.PXF_EINVAL, "scene version 2 is not supported (expected 1)")
    s = json.loads(json.dumps(OK))
    s["nodes"] = []
    rc, msg = count(lib, s)
    assert rc == L.PXF_EINVAL and msg.startswith("scene has no camera node")
    s = json.loads(json.dumps(OK))
    s["render"] = {"fps": 0}
    assert count(lib, s) == (L.PXF_EINVAL, "render.fps must be > 0")
    s = json.loads(json.dumps(OK))
    s["sims"] = []
    rc, msg = count(lib, s)
    assert rc == L.PXF_EINVAL and "unknown field `sims`" in msg


def test_defaults_and_dam_break_scene(lib):
    # The dam-break fluid block (fill and bounds of the reference's example scene) with every
    # optional field left to its default; materials are accepted and ignored.
    scene = {"version": 1, "nodes": [{"type": "camera", "translation": [1.2, 1.5, 2.9]}],
             "render": {"resolution": [1280, 720], "bounces": 12},
             "fluids": [{"name": "water", "bounds": [[-1, 0, -0.5], [1, 1.2, 0.5]], "resolution": 64,
                         "fill": [{"min": [-0.97, 0.03, -0.47], "max": [-0.35, 0.95, 0.47]}],
                         "substeps": 8, "flip": 0.95,
                         "materials": [{"inputs": {"transmission_weight": 1, "specular_ior": 1.33}}]}],
             "animation": {"frame_end": 119}}
    rc, msg = count(lib, scene)
    assert rc == 1, msg
    d = L.FluidDesc()
    lib.pxf_fluid_desc_init(C.byref(d))
    assert (d.resolution, d.particles_per_cell, d.substeps, d.pressure_iterations) == (64, 8, 8, 80)
    assert abs(d.flip - 0.95) < 1e-7 and list(d.gravity) == pytest.approx([0, -9.81, 0])
    assert (d.surface_refine, d.particle_radius, d.warmup, d.max_triangles) == (2, 2.0, 0.0, 2_000_000)


def test_python_mirror_validate():
    f = P.Fluid("w", [[0, 0, 0], [2, 1, 1]], [P.FluidBlock([0.1] * 3, [0.5] * 3)], resolution=300)
    with pytest.raises(P.FluidError) as e:
        f.validate(index=3)
    assert str(e.value).startswith("fluids[3] 'w': resolution 16..256")
    f.validate(lift_grid_limits=True)
