"""Oracle surface nets (shaders/fluid.slang:222-355) on CPU: a ball of particles gives a closed,
consistently wound mesh with unit normals pointing out of the liquid, vertices inside their cells,
and the reference's caps and counters on overflow."""
import numpy as np

import oracle


def _ball(n_side=24, center=(0.5, 0.5, 0.5), radius=0.25, spacing=1.0 / 48):
    g = (np.arange(n_side * 2) + 0.5) * spacing
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    pts = pts[np.linalg.norm(pts - np.asarray(center), axis=1) < radius]
    out = np.zeros((pts.shape[0], 8), dtype=np.float32)
    out[:, :3] = pts
    return out


def _mesh(max_tris=2_000_000):
    # a 24^3 grid of h = 1/24, refine 2 -> 48^3 surface cells, radius 2 surface cells
    p = _ball()
    sh = np.float32(1.0 / 48)
    radius = np.float32(2.0) * sh
    x = radius / np.float32(1.0 / 24)
    iso = np.float32(0.5) * np.float32(8) * (np.float32(0.638) * (x * x * x))
    return p, oracle.surface_nets(p, (48, 48, 48), sh, radius, iso, (0, 0, 0), max_tris, max_tris)


def test_ball_mesh_is_closed_and_outward():
    p, m = _mesh()
    v, t = m["vertices"], m["indices"]
    assert len(v) > 100 and len(t) > 200 and m["counts"] == (len(v), len(t))
    # every edge is shared by exactly two triangles, once in each direction
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    fwd = {tuple(x) for x in e}
    assert len(fwd) == len(e)
    assert all((b, a) in fwd for a, b in fwd)
    # unit normals pointing away from the ball's centre
    n = v[:, 4:7]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    assert np.all(np.sum(n * (v[:, :3] - 0.5), axis=1) > 0)
    # triangle winding agrees with the vertex normals
    a, b, c = v[t[:, 0], :3], v[t[:, 1], :3], v[t[:, 2], :3]
    fn = np.cross(b - a, c - a)
    assert np.mean(np.sum(fn * n[t[:, 0]], axis=1) > 0) > 0.99


def test_vertices_sit_in_their_cells():
    _, m = _mesh()
    cv = m["cell_vert"]
    cells = np.nonzero(cv != 0xffffffff)[0]
    assert len(cells) == len(m["vertices"])
    v = m["vertices"][cv[cells]]
    ijk = np.stack([cells % 48, (cells // 48) % 48, cells // (48 * 48)], 1)
    local = v[:, :3] * 48 - ijk
    assert np.all(local >= -1e-5) and np.all(local <= 1 + 1e-5)
    # vertex order is ascending cell order
    assert np.all(np.diff(cv[cells].astype(np.int64)) == 1)


def test_overflow_caps_follow_the_reference():
    _, full = _mesh()
    cap = len(full["vertices"]) // 2
    _, m = _mesh(max_tris=cap)
    assert m["counts"][0] == len(full["vertices"])           # the counter still counts every vertex
    assert len(m["vertices"]) == cap and len(m["indices"]) <= cap
    assert np.array_equal(m["vertices"], full["vertices"][:cap])
    assert int(m["indices"].max()) < cap                     # quads touching dropped vertices are gone
