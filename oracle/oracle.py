"""ctypes binding of the CPU oracle (test infrastructure only).

Mirrors oracle/flip_oracle.cpp, which restates shaders/fluid.slang:38-220 and
crates/pxl-render/src/fluid.rs:97-180,234-236 of the pxlengine project.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

# Array selectors shared with orc_sim_read / orc_sim_write.
PARTICLES, VEL, VEL_OLD, ACC, WACC, CELL_COUNT, CELL_TYPE, PRESSURE, DIVERGENCE, PRESSURE64 = range(10)
STAGES = ("clear", "p2g", "normalize", "forces", "divergence", "pressure", "project", "g2p")


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    lib = C.CDLL(path)
    u32p = C.POINTER(C.c_uint32)
    f32p = C.POINTER(C.c_float)
    lib.orc_num_threads.argtypes = [C.c_int]
    lib.orc_num_threads.restype = C.c_int
    lib.orc_grid.argtypes = [f32p, C.c_uint32, u32p, f32p]
    lib.orc_lcg.argtypes = [C.POINTER(C.c_uint64)]
    lib.orc_lcg.restype = C.c_float
    lib.orc_seed.argtypes = [f32p, C.c_uint32, f32p, C.c_uint32, C.c_uint32, C.c_uint32, f32p, C.c_int64]
    lib.orc_seed.restype = C.c_int64
    lib.orc_steps_for_frame.argtypes = [C.c_double, C.c_double, C.c_uint32, C.c_double]
    lib.orc_steps_for_frame.restype = C.c_uint64
    lib.orc_dt.argtypes = [C.c_double, C.c_uint32]
    lib.orc_dt.restype = C.c_float
    lib.orc_sim_new.argtypes = [C.c_int, u32p, C.c_float, C.c_float, C.c_float, f32p, f32p, C.c_uint32, f32p, C.c_uint32]
    lib.orc_sim_new.restype = C.c_void_p
    lib.orc_sim_free.argtypes = [C.c_void_p]
    lib.orc_sim_set_pressure.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_uint32, C.c_uint32]
    lib.orc_sim_set_mg.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
    lib.orc_sim_pcg_stats.argtypes = [C.c_void_p, u32p, C.POINTER(C.c_double)]
    lib.orc_sim_stage.argtypes = [C.c_void_p, C.c_int]
    lib.orc_sim_step.argtypes = [C.c_void_p, C.c_uint32]
    lib.orc_sim_read.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.orc_sim_write.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.orc_surface_nets.argtypes = [C.c_void_p, C.c_int64, u32p, C.c_float, C.c_float, C.c_float, f32p,
                                     C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, u32p]
    _lib = lib
    return lib


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def num_threads(n: int = 0) -> int:
    return load().orc_num_threads(n)


def grid(bounds, resolution):
    """Fluid::grid (crates/pxl-scene/src/lib.rs:123-128) -> ((nx, ny, nz), h)."""
    b, bp = _f32(np.asarray(bounds, dtype=np.float32).reshape(6))
    n = (C.c_uint32 * 3)()
    h = C.c_float()
    load().orc_grid(bp, resolution, n, C.byref(h))
    return (n[0], n[1], n[2]), h.value


def lcg(state: int):
    """One lcg() draw (crates/pxl-render/src/fluid.rs:97-100) -> (value, new_state)."""
    s = C.c_uint64(state)
    v = load().orc_lcg(C.byref(s))
    return v, s.value


def seed_particles(bounds, resolution, fill, ppc, seed):
    """FluidState::new seeding (fluid.rs:119-148) -> float32 array [N, 8] in the AoS layout."""
    b, bp = _f32(np.asarray(bounds, dtype=np.float32).reshape(6))
    rows = []
    for blk in fill:
        vel = blk.get("velocity", [0.0, 0.0, 0.0])
        rows.append(list(blk["min"]) + list(blk["max"]) + list(vel))
    f, fp = _f32(np.asarray(rows, dtype=np.float32).reshape(-1))
    lib = load()
    n = lib.orc_seed(bp, resolution, fp, len(rows), ppc, seed, None, 0)
    out = np.zeros((n, 8), dtype=np.float32)
    lib.orc_seed(bp, resolution, fp, len(rows), ppc, seed, out.ctypes.data_as(C.POINTER(C.c_float)), n)
    return out


def surface_nets(particles, sdims, sh, radius, iso, origin, max_verts, max_tris):
    """Surface nets of particles ([N, 8] float32) on a surface grid of sdims cells
    (shaders/fluid.slang:222-355); vertices in ascending cell order, triangles in ascending node
    and axis order. Returns density, phi, cell_vert, vertices [V, 8], indices [T, 3] and the
    uncapped counts."""
    lib = load()
    p = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 8)
    sx, sy, sz = (int(v) for v in sdims)
    nn, nc = (sx + 1) * (sy + 1) * (sz + 1), sx * sy * sz
    den = np.empty(nn, dtype=np.int32)
    phi = np.empty(nn, dtype=np.float32)
    cv = np.empty(nc, dtype=np.uint32)
    verts = np.zeros((max_verts, 8), dtype=np.float32)
    idx = np.zeros((max_tris, 3), dtype=np.uint32)
    cnt = (C.c_uint32 * 2)()
    d = (C.c_uint32 * 3)(sx, sy, sz)
    o = (C.c_float * 3)(*[float(v) for v in origin])
    lib.orc_surface_nets(p.ctypes.data, p.shape[0], d, float(sh), float(radius), float(iso), o, int(max_verts),
                         int(max_tris), den.ctypes.data, phi.ctypes.data, cv.ctypes.data, verts.ctypes.data,
                         idx.ctypes.data, cnt)
    nv, nt = min(cnt[0], max_verts), min(cnt[1], max_tris) // 2 * 2
    return {"density": den, "phi": phi, "cell_vert": cv, "vertices": verts[:nv], "indices": idx[:nt],
            "counts": (cnt[0], cnt[1])}


def steps_for_frame(warmup, fps, substeps, frame):
    return load().orc_steps_for_frame(float(warmup), float(fps), int(substeps), float(frame))


def dt_for(fps, substeps):
    return load().orc_dt(float(fps), int(substeps))


class OracleSim:
    """One simulation on the CPU oracle. dtype float32 (reference semantics) or float64."""

    def __init__(self, dims, h, dt, flip, origin, gravity, iterations, particles, dtype=np.float32):
        lib = load()
        self.lib = lib
        self.dims = tuple(int(x) for x in dims)
        self.dtype = np.dtype(dtype)
        nx, ny, nz = self.dims
        self.n_cells = nx * ny * nz
        self.n_faces = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
        parts, pp = _f32(np.asarray(particles, dtype=np.float32).reshape(-1, 8))
        self.n_particles = parts.shape[0]
        n = (C.c_uint32 * 3)(*self.dims)
        o, op = _f32(origin)
        g, gp = _f32(gravity)
        self.h = lib.orc_sim_new(1 if self.dtype == np.float64 else 0, n, h, dt, flip, op, gp,
                                 iterations, pp, self.n_particles)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_sim_free(self.h)
            self.h = None

    def set_pressure(self, mode, rtol=1e-6, max_iter=2000, restart=50):
        modes = {"gs": 0, "pcg": 1, "pcg64": 2, "mgpcg": 3}
        self.lib.orc_sim_set_pressure(self.h, modes.get(mode, mode), rtol, max_iter, restart)

    def set_mg(self, coarse_iters=2, pairs=2):
        self.lib.orc_sim_set_mg(self.h, coarse_iters, pairs)

    def pcg_stats(self):
        it = C.c_uint32()
        rr = C.c_double()
        self.lib.orc_sim_pcg_stats(self.h, C.byref(it), C.byref(rr))
        return it.value, rr.value

    def stage(self, name):
        rc = self.lib.orc_sim_stage(self.h, STAGES.index(name))
        assert rc == 0

    def step(self, n=1):
        self.lib.orc_sim_step(self.h, n)

    def _shape(self, which):
        fdt = self.dtype
        return {
            PARTICLES: ((self.n_particles, 8), fdt), VEL: ((self.n_faces,), fdt), VEL_OLD: ((self.n_faces,), fdt),
            ACC: ((self.n_faces,), np.int32), WACC: ((self.n_faces,), np.int32),
            CELL_COUNT: ((self.n_cells,), np.uint32), CELL_TYPE: ((self.n_cells,), np.uint32),
            PRESSURE: ((self.n_cells,), fdt), DIVERGENCE: ((self.n_cells,), fdt),
            PRESSURE64: ((self.n_cells,), np.float64),
        }[which]

    def read(self, which):
        shape, dt = self._shape(which)
        out = np.zeros(shape, dtype=dt)
        rc = self.lib.orc_sim_read(self.h, which, out.ctypes.data, out.nbytes)
        assert rc == 0, rc
        return out

    def write(self, which, arr):
        shape, dt = self._shape(which)
        a = np.ascontiguousarray(np.asarray(arr, dtype=dt).reshape(shape))
        rc = self.lib.orc_sim_write(self.h, which, a.ctypes.data, a.nbytes)
        assert rc == 0, rc
