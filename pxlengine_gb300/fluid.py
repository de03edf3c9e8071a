"""Host-side mirror of pxlengine's liquid interface over libpxlflip.so.

Names follow the reference:
  Fluid / FluidBlock      crates/pxl-scene/src/lib.rs:49-129 (fields, defaults, grid())
  FluidState              crates/pxl-render/src/fluid.rs:74-246 (new, particle_count, steps_for_frame)
  FluidState.fluid_advance  Renderer::fluid_advance, simulation part (fluid.rs:265-306)
Errors raise FluidError carrying the library's message (the reference's anyhow context strings).
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _lib as L


class FluidError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


@dataclass
class FluidBlock:
    min: Sequence[float]
    max: Sequence[float]
    velocity: Sequence[float] = (0.0, 0.0, 0.0)


@dataclass
class Fluid:
    name: str
    bounds: Sequence[Sequence[float]]
    fill: Sequence[FluidBlock]
    resolution: int = 64
    particles_per_cell: int = 8
    substeps: int = 8
    flip: float = 0.95
    gravity: Sequence[float] = (0.0, -9.81, 0.0)
    pressure_iterations: int = 80
    surface_refine: int = 2
    particle_radius: float = 2.0
    warmup: float = 0.0
    max_triangles: int = 2_000_000
    _keep: list = field(default_factory=list, repr=False, compare=False)

    def to_desc(self) -> L.FluidDesc:
        d = L.FluidDesc()
        L.load().pxf_fluid_desc_init(C.byref(d))
        name = self.name.encode()
        blocks = (L.FillBlock * max(1, len(self.fill)))()
        for i, b in enumerate(self.fill):
            if isinstance(b, dict):
                b = FluidBlock(b["min"], b["max"], b.get("velocity", (0.0, 0.0, 0.0)))
            blocks[i].min[:] = [float(x) for x in b.min]
            blocks[i].max[:] = [float(x) for x in b.max]
            blocks[i].velocity[:] = [float(x) for x in b.velocity]
        self._keep[:] = [name, blocks]
        d.name = name
        for a in range(2):
            d.bounds[a][:] = [float(x) for x in self.bounds[a]]
        d.resolution = int(self.resolution)
        d.fill = C.cast(blocks, C.POINTER(L.FillBlock))
        d.fill_count = len(self.fill)
        d.particles_per_cell = int(self.particles_per_cell)
        d.substeps = int(self.substeps)
        d.flip = float(self.flip)
        d.gravity[:] = [float(x) for x in self.gravity]
        d.pressure_iterations = int(self.pressure_iterations)
        d.surface_refine = int(self.surface_refine)
        d.particle_radius = float(self.particle_radius)
        d.warmup = float(self.warmup)
        d.max_triangles = int(self.max_triangles)
        return d

    def grid(self) -> Tuple[Tuple[int, int, int], float]:
        """Fluid::grid (crates/pxl-scene/src/lib.rs:123-128): (cells per axis, cell size)."""
        d = self.to_desc()
        n = (C.c_uint32 * 3)()
        h = C.c_float()
        L.load().pxf_fluid_grid(C.byref(d), n, C.byref(h))
        return (n[0], n[1], n[2]), h.value

    def validate(self, index: int = 0, lift_grid_limits: bool = False) -> None:
        """The fluid checks of Scene::validate (crates/pxl-scene/src/lib.rs:710-735)."""
        d = self.to_desc()
        buf = C.create_string_buffer(512)
        rc = L.load().pxf_validate(C.byref(d), index, 1 if lift_grid_limits else 0, buf, 512)
        if rc != 0:
            raise FluidError(rc, buf.value.decode())


def make_options(solver: str = "gs", rtol: float = 1e-6, max_iter: int = 2000, restart: int = 50,
                 lift_grid_limits: bool = False, keep_p2g_sums: bool = False, velocity_sigma: float = 0.0,
                 velocity_seed: int = 0, wait_timeout_s: float = 600.0, p2g_tile: int = -1,
                 precond: str = "mg", coarse_iters: int = 2, smooth_pairs: int = 2) -> L.Options:
    o = L.Options()
    L.load().pxf_options_init(C.byref(o))
    o.pressure_solver = {"gs": L.PXF_PRESSURE_RBGS, "pcg": L.PXF_PRESSURE_PCG}[solver]
    o.pcg_rtol = rtol
    o.pcg_max_iter = max_iter
    o.pcg_restart = restart
    o.lift_grid_limits = 1 if lift_grid_limits else 0
    o.keep_p2g_sums = 1 if keep_p2g_sums else 0
    o.velocity_sigma = velocity_sigma
    o.velocity_seed = velocity_seed
    o.wait_timeout_s = wait_timeout_s
    o.p2g_tile = p2g_tile
    o.pcg_precond = {"mg": 0, "jacobi": 1}[precond]
    o.mg_coarse_iters = coarse_iters
    o.mg_smooth_pairs = smooth_pairs
    return o


def steps_for_frame(warmup: float, fps: float, substeps: int, frame: float) -> int:
    """fluid.rs:234-236."""
    return int(L.load().pxf_steps_for_frame(float(warmup), float(fps), int(substeps), float(frame)))


def _check(rc: int, handle=None):
    if rc != 0:
        msg = L.load().pxf_last_error(handle)
        raise FluidError(rc, msg.decode() if msg else f"error {rc}")


_GRID_DTYPES = {"vel": np.float32, "vel_old": np.float32, "acc": np.int32, "wacc": np.int32,
                "cell_count": np.uint32, "cell_type": np.uint32, "pressure": np.float32,
                "divergence": np.float32, "pressure64": np.float64, "surf_density": np.int32,
                "surf_phi": np.float32, "surf_cell_vert": np.uint32}


class FluidState:
    """One liquid simulation on the GPU (crates/pxl-render/src/fluid.rs:74-94)."""

    def __init__(self, fluid: Optional[Fluid] = None, fps: float = 24.0, seed: int = 0,
                 options: Optional[L.Options] = None, _handle=None):
        self._lib = L.load()
        self.h = None
        if _handle is not None:
            self.h = _handle
        else:
            d = fluid.to_desc()
            out = C.c_void_p()
            rc = self._lib.pxf_create_ex(C.byref(d), seed, float(fps), C.byref(options) if options else None,
                                         C.byref(out))
            _check(rc)
            self.h = out
        self.fluid = fluid
        n = (C.c_uint32 * 3)()
        hh = C.c_float()
        dt = C.c_float()
        self._lib.pxf_grid_info(self.h, n, C.byref(hh), C.byref(dt))
        self.dims = (n[0], n[1], n[2])
        self.cell = hh.value
        self.dt = dt.value
        nx, ny, nz = self.dims
        self.n_cells = nx * ny * nz
        self.n_faces = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)

    @classmethod
    def from_json(cls, scene_json: str, index: int = 0, options: Optional[L.Options] = None) -> "FluidState":
        """Scene::from_json + FluidState::new for fluids[index]."""
        lib = L.load()
        out = C.c_void_p()
        rc = lib.pxf_create_from_json_ex(scene_json.encode(), index, C.byref(options) if options else None,
                                         C.byref(out))
        _check(rc)
        return cls(_handle=out)

    def close(self):
        if self.h is not None:
            self._lib.pxf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ reference interface
    def particle_count(self) -> int:
        return int(self._lib.pxf_particle_count(self.h))

    @property
    def steps_done(self) -> int:
        return int(self._lib.pxf_steps_done(self.h))

    def fluid_advance(self, frame: float) -> None:
        """Step to scene frame `frame` (fluid.rs:265-306, simulation part)."""
        _check(self._lib.pxf_advance_to_frame(self.h, float(frame)), self.h)

    # ------------------------------------------------------------------ direct control
    def step(self, n: int = 1) -> None:
        _check(self._lib.pxf_step(self.h, int(n)), self.h)

    def sync(self) -> None:
        _check(self._lib.pxf_sync(self.h), self.h)

    def step_timed(self, n: int = 1) -> float:
        """Device milliseconds of n substeps (CUDA events on the simulation's stream)."""
        ms = C.c_double()
        _check(self._lib.pxf_step_timed(self.h, int(n), C.byref(ms)), self.h)
        return ms.value

    def profile_substep(self):
        """One substep launched stage by stage: [(stage, launches, device ms)]."""
        recs = (L.StageTime * 32)()
        cnt = C.c_uint32()
        _check(self._lib.pxf_profile_substep(self.h, recs, 32, C.byref(cnt)), self.h)
        return [(recs[i].name.decode(), recs[i].launches, recs[i].ms) for i in range(min(cnt.value, 32))]

    def surface_info(self) -> dict:
        """Surface grid (pxf_surface_info): cells per axis, cell size, splat radius, iso level."""
        d = (C.c_uint32 * 3)()
        cell, rad, iso = C.c_float(), C.c_float(), C.c_float()
        _check(self._lib.pxf_surface_info(self.h, d, C.byref(cell), C.byref(rad), C.byref(iso)), self.h)
        return {"dims": (d[0], d[1], d[2]), "cell": cell.value, "radius": rad.value, "iso": iso.value}

    def surface_mesh(self) -> dict:
        """Surface nets of the current particles (pxf_surface_mesh): vertices [V, 8] float32
        ([x, y, z, 0, nx, ny, nz, 0]), indices [T, 3] uint32, overflow flag, device ms."""
        nv, nt = C.c_uint32(), C.c_uint32()
        ov = C.c_int32()
        ms = C.c_double()
        _check(self._lib.pxf_surface_mesh(self.h, C.byref(nv), C.byref(nt), C.byref(ov), C.byref(ms)), self.h)
        verts = np.empty((nv.value, 8), dtype=np.float32)
        idx = np.empty((nt.value, 3), dtype=np.uint32)
        _check(self._lib.pxf_read_mesh(self.h, verts.ctypes.data, nv.value, idx.ctypes.data, nt.value), self.h)
        return {"vertices": verts, "indices": idx, "overflow": bool(ov.value), "device_ms": ms.value}

    def mg_levels(self) -> dict:
        """Multigrid hierarchy of the last substep: cells and system cells per level, tail level."""
        cells = (C.c_uint32 * 16)()
        sysc = (C.c_uint32 * 16)()
        n = C.c_uint32()
        tail = C.c_int32()
        _check(self._lib.pxf_mg_level_info(self.h, cells, sysc, 16, C.byref(n), C.byref(tail)), self.h)
        k = min(n.value, 16)
        return {"cells": list(cells[:k]), "system_cells": list(sysc[:k]), "tail": tail.value}

    def autotune(self) -> dict:
        """One substep that also times every P2G variant and keeps the fastest (see pxf_autotune)."""
        r = L.TuneResult()
        _check(self._lib.pxf_autotune(self.h, C.byref(r)), self.h)
        return _tune_dict(r)

    def device_bytes(self) -> int:
        return int(self._lib.pxf_device_bytes(self.h))

    def read_particles(self) -> np.ndarray:
        """Particles as [N, 8] float32 [x, y, z, 0, vx, vy, vz, 0] in seeding order."""
        n = self.particle_count()
        out = np.empty((n, 8), dtype=np.float32)
        _check(self._lib.pxf_read_particles(self.h, out.ctypes.data, n), self.h)
        return out

    def write_particles(self, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(-1, 8)
        _check(self._lib.pxf_write_particles(self.h, a.ctypes.data, a.shape[0]), self.h)

    def read_grid(self, name: str) -> np.ndarray:
        dt = _GRID_DTYPES[name]
        n = self.n_faces if name in ("vel", "vel_old", "acc", "wacc") else self.n_cells
        if name.startswith("surf_"):
            sx, sy, sz = self.surface_info()["dims"]
            n = sx * sy * sz if name == "surf_cell_vert" else (sx + 1) * (sy + 1) * (sz + 1)
        out = np.empty(n, dtype=dt)
        _check(self._lib.pxf_read_grid(self.h, L.GRID[name], out.ctypes.data, out.nbytes), self.h)
        return out

    def write_pressure(self, p: np.ndarray) -> None:
        a = np.ascontiguousarray(p, dtype=np.float32).reshape(-1)
        _check(self._lib.pxf_write_grid(self.h, L.GRID["pressure"], a.ctypes.data, a.nbytes), self.h)

    def solver_stats(self):
        it = C.c_uint32()
        rr = C.c_double()
        st = C.c_uint32()
        _check(self._lib.pxf_solver_stats(self.h, C.byref(it), C.byref(rr), C.byref(st)), self.h)
        return it.value, rr.value, st.value

    def snapshot(self) -> "Snapshot":
        out = C.c_void_p()
        _check(self._lib.pxf_snapshot_take(self.h, C.byref(out)), self.h)
        return Snapshot(out)

    def restore(self, snap: "Snapshot") -> None:
        _check(self._lib.pxf_snapshot_restore(self.h, snap.h), self.h)


class HostBuffer:
    """Page-locked host memory (pxf_host_alloc) viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        self._lib = L.load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        ptr = C.c_void_p()
        _check(self._lib.pxf_host_alloc(self.nbytes, C.byref(ptr)))
        self.ptr = ptr
        buf = (C.c_char * self.nbytes).from_address(ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def close(self):
        if self.ptr is not None:
            self.array = None
            self._lib.pxf_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Snapshot:
    def __init__(self, h):
        self.h = h

    def __del__(self):
        if self.h is not None:
            L.load().pxf_snapshot_free(self.h)
            self.h = None


def _tune_dict(r) -> dict:
    return {"tile_shape": r.tile_shape, "lanes": r.lanes, "chosen": r.chosen.decode(),
            "variant_ms": [float(r.ms[i]) for i in range(min(r.variants, 16))]}


class Batch:
    """Many simulations advanced together: one launch per stage, one CUDA graph per substep."""

    def __init__(self):
        self._lib = L.load()
        out = C.c_void_p()
        _check(self._lib.pxf_batch_create(C.byref(out)))
        self.h = out
        self.members = []

    def _chk(self, rc):
        if rc != 0:
            msg = self._lib.pxf_batch_last_error(self.h)
            raise FluidError(rc, msg.decode() if msg else f"error {rc}")

    def add(self, sim: FluidState) -> None:
        self._chk(self._lib.pxf_batch_add(self.h, sim.h))
        self.members.append(sim)

    def remove(self, sim: FluidState) -> None:
        self._chk(self._lib.pxf_batch_remove(self.h, sim.h))
        self.members.remove(sim)

    def __len__(self):
        return int(self._lib.pxf_batch_size(self.h))

    def step(self, n: int = 1) -> None:
        self._chk(self._lib.pxf_batch_step(self.h, int(n)))

    def sync(self) -> None:
        self._chk(self._lib.pxf_batch_sync(self.h))

    def step_timed(self, n: int) -> float:
        """Device ms of n batched substeps (CUDA events on the batch's stream)."""
        ms = C.c_double()
        self._chk(self._lib.pxf_batch_step_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def autotune(self) -> dict:
        """One batched substep that also picks the fastest P2G variant (see pxf_batch_autotune)."""
        r = L.TuneResult()
        self._chk(self._lib.pxf_batch_autotune(self.h, C.byref(r)))
        return _tune_dict(r)

    def close(self):
        if self.h is not None:
            self._lib.pxf_batch_destroy(self.h)
            self.h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
