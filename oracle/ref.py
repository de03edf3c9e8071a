"""ctypes binding of the reference runner (test infrastructure only): pxlengine's own
shaders/fluid.slang and shaders/sim.slang compiled for the CPU by oracle/ref_build.py
(oracle/_ref/libref_shaders.so).
Available where the reference checkout is, or where a build made from it was carried along
(`available()`); the GPU tests use the fixtures that tests/golden/make_ref_golden.py wrote from it.
The substep's dispatches run on all host threads (OpenMP; integer atomics for InterlockedAdd)."""
import ctypes as C

import numpy as np

from . import ref_build as _build

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    if path is None:
        return None
    lib = C.CDLL(path)
    u32p = C.POINTER(C.c_uint32)
    f32p = C.POINTER(C.c_float)
    lib.ref_sim_new.argtypes = [u32p, C.c_float, C.c_float, C.c_float, f32p, f32p, C.c_uint32, f32p, C.c_uint32]
    lib.ref_sim_new.restype = C.c_void_p
    lib.ref_sim_free.argtypes = [C.c_void_p]
    lib.ref_num_threads.argtypes = [C.c_int]
    lib.ref_num_threads.restype = C.c_int
    lib.ref_sim_stage.argtypes = [C.c_void_p, C.c_int]
    lib.ref_sim_stage.restype = C.c_int
    lib.ref_sim_step.argtypes = [C.c_void_p, C.c_uint32]
    lib.ref_sim_read.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
    lib.ref_sim_read.restype = C.c_int
    lib.ref_surface_nets.argtypes = [C.c_void_p, C.c_uint32, u32p, C.c_float, C.c_float, C.c_float, f32p,
                                     C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, u32p]
    lib.ref_surface_nets.restype = C.c_int
    lib.ref_grid_sort.argtypes = [f32p, C.c_uint32, C.c_float, C.c_uint32, u32p, u32p, u32p]
    lib.ref_grid_sort.restype = C.c_int
    _lib = lib
    return lib


def available() -> bool:
    return load() is not None


def num_threads(n: int = 0) -> int:
    return load().ref_num_threads(n)


STAGES = ("clear", "p2g", "normalize", "forces", "divergence", "pressure", "project", "g2p")
ARRAYS = ("particles", "vel", "vel_old", "acc", "wacc", "cell_count", "cell_type", "pressure", "divergence")


class RefSim:
    """One simulation run by the reference's own kernels (FP32) on the host cores."""

    def __init__(self, dims, h, dt, flip, origin, gravity, iterations, particles):
        lib = load()
        assert lib is not None, "the reference checkout is not available"
        self.lib = lib
        self.dims = tuple(int(x) for x in dims)
        nx, ny, nz = self.dims
        self.n_cells = nx * ny * nz
        self.n_faces = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
        parts = np.ascontiguousarray(np.asarray(particles, dtype=np.float32).reshape(-1, 8))
        self.n_particles = parts.shape[0]
        n = (C.c_uint32 * 3)(*self.dims)
        o = (C.c_float * 3)(*[float(v) for v in origin])
        g = (C.c_float * 3)(*[float(v) for v in gravity])
        self.h = lib.ref_sim_new(n, h, dt, flip, o, g, iterations, parts.ctypes.data_as(C.POINTER(C.c_float)),
                                 self.n_particles)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_sim_free(self.h)
            self.h = None

    def stage(self, name):
        assert self.lib.ref_sim_stage(self.h, STAGES.index(name)) == 0

    def step(self, n=1):
        self.lib.ref_sim_step(self.h, n)

    def read(self, name):
        shape, dt = {
            "particles": ((self.n_particles, 8), np.float32), "vel": ((self.n_faces,), np.float32),
            "vel_old": ((self.n_faces,), np.float32), "acc": ((self.n_faces,), np.int32),
            "wacc": ((self.n_faces,), np.int32), "cell_count": ((self.n_cells,), np.uint32),
            "cell_type": ((self.n_cells,), np.uint32), "pressure": ((self.n_cells,), np.float32),
            "divergence": ((self.n_cells,), np.float32),
        }[name]
        out = np.zeros(shape, dtype=dt)
        assert self.lib.ref_sim_read(self.h, ARRAYS.index(name), out.ctypes.data, out.nbytes) == 0
        return out


def surface_nets(particles, sdims, sh, radius, iso, origin, max_verts, max_tris):
    """The reference's surface pass (s_clear .. s_quads) of particles ([N, 8] float32): density,
    phi, cell_vert, vertices [V, 8] (position, 0, normal, 0), indices [T, 3] and the counters."""
    lib = load()
    assert lib is not None, "the reference checkout is not available"
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
    assert lib.ref_surface_nets(p.ctypes.data, p.shape[0], d, float(sh), float(radius), float(iso), o,
                                int(max_verts), int(max_tris), den.ctypes.data, phi.ctypes.data, cv.ctypes.data,
                                verts.ctypes.data, idx.ctypes.data, cnt) == 0
    nv, nt = min(cnt[0], max_verts), min(cnt[1], max_tris) // 2 * 2
    return {"density": den, "phi": phi, "cell_vert": cv, "vertices": verts[:nv], "indices": idx[:nt],
            "counts": (cnt[0], cnt[1])}


def grid_sort(agents, cell_size, table_size):
    """The reference's neighbour grid (sim.slang:32-104 with the dispatches of sim.rs:258-270) of
    agents ([N, 16] float32 records, position first): (offsets, counts, sorted). The order of the
    agents inside one cell follows the atomics of grid_scatter."""
    lib = load()
    assert lib is not None, "the reference checkout is not available"
    a = np.ascontiguousarray(agents, dtype=np.float32).reshape(-1, 16)
    n = a.shape[0]
    offsets = np.zeros(table_size, dtype=np.uint32)
    counts = np.zeros(table_size, dtype=np.uint32)
    srt = np.zeros(max(n, 1), dtype=np.uint32)
    u32p = C.POINTER(C.c_uint32)
    rc = lib.ref_grid_sort(a.ctypes.data_as(C.POINTER(C.c_float)), n, float(cell_size), int(table_size),
                           offsets.ctypes.data_as(u32p), counts.ctypes.data_as(u32p), srt.ctypes.data_as(u32p))
    assert rc == 0, rc
    return offsets, counts, srt[:n]
