"""ctypes binding of libpxlflip.so (include/pxlflip.h).

The shared library is the product; this module only declares its C signatures. Loading fails
loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpxlflip.so")

PXF_OK, PXF_EINVAL, PXF_ECUDA, PXF_ENOMEM, PXF_ETIMEDOUT, PXF_ESTATE, PXF_ENOTFOUND = 0, -1, -2, -3, -4, -5, -6
PXF_PRESSURE_RBGS, PXF_PRESSURE_PCG = 0, 1
GRID = {"vel": 1, "vel_old": 2, "acc": 3, "wacc": 4, "cell_count": 5, "cell_type": 6, "pressure": 7,
        "divergence": 8, "pressure64": 9, "surf_density": 10, "surf_phi": 11, "surf_cell_vert": 12}

# Every exported function and its (restype, argtypes); the not-GPU tests check this list against
# the header and the library's dynamic symbol table.
EXPORTS = {}


class FillBlock(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("max", C.c_float * 3), ("velocity", C.c_float * 3)]


class FluidDesc(C.Structure):
    _fields_ = [("name", C.c_char_p), ("bounds", (C.c_float * 3) * 2), ("resolution", C.c_uint32),
                ("fill", C.POINTER(FillBlock)), ("fill_count", C.c_uint32),
                ("particles_per_cell", C.c_uint32), ("substeps", C.c_uint32), ("flip", C.c_float),
                ("gravity", C.c_float * 3), ("pressure_iterations", C.c_uint32), ("surface_refine", C.c_uint32),
                ("particle_radius", C.c_float), ("warmup", C.c_float), ("max_triangles", C.c_uint32)]


class Options(C.Structure):
    _fields_ = [("pressure_solver", C.c_uint32), ("pcg_rtol", C.c_double), ("pcg_max_iter", C.c_uint32),
                ("pcg_restart", C.c_uint32), ("lift_grid_limits", C.c_uint32), ("keep_p2g_sums", C.c_uint32),
                ("velocity_sigma", C.c_float), ("velocity_seed", C.c_uint32), ("wait_timeout_s", C.c_double),
                ("p2g_tile", C.c_int32), ("pcg_precond", C.c_uint32), ("mg_coarse_iters", C.c_uint32),
                ("mg_smooth_pairs", C.c_uint32)]


class StageTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint32), ("ms", C.c_double)]


class TuneResult(C.Structure):
    _fields_ = [("tile_shape", C.c_int32), ("lanes", C.c_int32), ("variants", C.c_uint32), ("ms", C.c_float * 16),
                ("chosen", C.c_char * 32)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_active", C.c_uint32), ("substeps_per_tick", C.c_uint32),
                ("wait_timeout_s", C.c_double)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("substeps_done", C.c_uint32),
                ("substeps_total", C.c_uint32), ("particles", C.c_uint32), ("device_bytes", C.c_uint64),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("ticks", C.c_uint64), ("submitted", C.c_uint64), ("admitted", C.c_uint64),
                ("completed", C.c_uint64), ("cancelled", C.c_uint64), ("rejected", C.c_uint64),
                ("active", C.c_uint32), ("queued", C.c_uint32), ("reserved_bytes", C.c_uint64),
                ("peak_reserved_bytes", C.c_uint64), ("particle_substeps", C.c_double),
                ("busy_device_ms", C.c_double), ("p50_substep_ms", C.c_double), ("p99_substep_ms", C.c_double),
                ("p50_tick_wall_ms", C.c_double), ("p99_tick_wall_ms", C.c_double), ("uptime_s", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)


def _sig():
    vp = C.c_void_p
    pp = C.POINTER(C.c_void_p)
    u32p = C.POINTER(C.c_uint32)
    dp = C.POINTER(FluidDesc)
    op = C.POINTER(Options)
    return {
        "pxf_fluid_desc_init": (None, [dp]),
        "pxf_options_init": (None, [op]),
        "pxf_validate": (C.c_int, [dp, C.c_uint32, C.c_uint32, C.c_char_p, C.c_size_t]),
        "pxf_fluid_grid": (C.c_int, [dp, u32p, C.POINTER(C.c_float)]),
        "pxf_steps_for_frame": (C.c_uint64, [C.c_double, C.c_double, C.c_uint32, C.c_double]),
        "pxf_create": (C.c_int, [dp, C.c_uint32, C.c_double, pp]),
        "pxf_create_ex": (C.c_int, [dp, C.c_uint32, C.c_double, op, pp]),
        "pxf_create_from_json": (C.c_int, [C.c_char_p, C.c_uint32, pp]),
        "pxf_create_from_json_ex": (C.c_int, [C.c_char_p, C.c_uint32, op, pp]),
        "pxf_scene_fluid_count": (C.c_int, [C.c_char_p]),
        "pxf_advance_to_frame": (C.c_int, [vp, C.c_double]),
        "pxf_step": (C.c_int, [vp, C.c_uint32]),
        "pxf_sync": (C.c_int, [vp]),
        "pxf_particle_count": (C.c_uint32, [vp]),
        "pxf_steps_done": (C.c_uint64, [vp]),
        "pxf_grid_info": (C.c_int, [vp, u32p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "pxf_device_bytes": (C.c_size_t, [vp]),
        "pxf_estimate_bytes": (C.c_int, [dp, op, C.POINTER(C.c_uint64)]),
        "pxf_read_particles": (C.c_int, [vp, vp, C.c_size_t]),
        "pxf_write_particles": (C.c_int, [vp, vp, C.c_size_t]),
        "pxf_read_grid": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "pxf_write_grid": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "pxf_solver_stats": (C.c_int, [vp, u32p, C.POINTER(C.c_double), u32p]),
        "pxf_snapshot_take": (C.c_int, [vp, pp]),
        "pxf_snapshot_restore": (C.c_int, [vp, vp]),
        "pxf_snapshot_free": (None, [vp]),
        "pxf_step_timed": (C.c_int, [vp, C.c_uint32, C.POINTER(C.c_double)]),
        "pxf_profile_substep": (C.c_int, [vp, C.POINTER(StageTime), C.c_uint32, u32p]),
        "pxf_autotune": (C.c_int, [vp, C.POINTER(TuneResult)]),
        "pxf_mg_level_info": (C.c_int, [vp, u32p, u32p, C.c_uint32, u32p, C.POINTER(C.c_int32)]),
        "pxf_set_wait_timeout": (C.c_int, [vp, C.c_double]),
        "pxf_surface_mesh": (C.c_int, [vp, u32p, u32p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
        "pxf_read_mesh": (C.c_int, [vp, vp, C.c_size_t, vp, C.c_size_t]),
        "pxf_surface_mesh_into": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, vp, C.c_uint32, C.c_uint32, u32p, u32p,
                                            C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
        "pxf_surface_info": (C.c_int, [vp, u32p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "pxf_mesh_device_buffers": (C.c_int, [vp, pp, pp]),
        "pxf_selftest_grid_barrier": (C.c_int, [C.c_uint32, C.c_int32, C.c_double, C.c_uint32, u32p]),
        "pxf_set_device": (C.c_int, [C.c_int]),
        "pxf_host_alloc": (C.c_int, [C.c_size_t, pp]),
        "pxf_host_free": (None, [vp]),
        "pxf_cell_starts_noalloc": (C.c_int, [vp, C.c_uint32, u32p, C.POINTER(C.c_float), C.c_float, vp, vp]),
        "pxf_grid_table_size": (C.c_uint32, [C.c_uint32]),
        "pxf_grid_scratch_bytes": (C.c_size_t, [C.c_uint32, C.c_uint32]),
        "pxf_grid_sort": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, vp, vp, vp, vp, C.c_size_t,
                                    vp]),
        "pxf_destroy": (None, [vp]),
        "pxf_last_error": (C.c_char_p, [vp]),
        "pxf_batch_create": (C.c_int, [pp]),
        "pxf_batch_add": (C.c_int, [vp, vp]),
        "pxf_batch_remove": (C.c_int, [vp, vp]),
        "pxf_batch_size": (C.c_uint32, [vp]),
        "pxf_batch_step": (C.c_int, [vp, C.c_uint32]),
        "pxf_batch_sync": (C.c_int, [vp]),
        "pxf_batch_destroy": (None, [vp]),
        "pxf_batch_last_error": (C.c_char_p, [vp]),
        "pxf_batch_step_timed": (C.c_int, [vp, C.c_uint32, C.POINTER(C.c_double)]),
        "pxf_batch_autotune": (C.c_int, [vp, C.POINTER(TuneResult)]),
        "pxf_server_config_init": (None, [C.POINTER(ServerConfig)]),
        "pxf_server_create": (C.c_int, [C.POINTER(ServerConfig), pp]),
        "pxf_server_submit": (C.c_int, [vp, dp, C.c_uint32, C.c_double, op, C.c_uint32, C.POINTER(C.c_uint64)]),
        "pxf_server_cancel": (C.c_int, [vp, C.c_uint64]),
        "pxf_server_tick": (C.c_int, [vp, u32p]),
        "pxf_server_status": (C.c_int, [vp, C.c_uint64, C.POINTER(RequestStatus)]),
        "pxf_server_take_result": (C.c_int, [vp, C.c_uint64, vp, C.c_size_t]),
        "pxf_server_stats_get": (C.c_int, [vp, C.POINTER(ServerStats)]),
        "pxf_server_start": (C.c_int, [vp]),
        "pxf_server_stop": (C.c_int, [vp]),
        "pxf_server_destroy": (None, [vp]),
        "pxf_server_last_error": (C.c_char_p, [vp]),
    }


EXPORTS.update(_sig())
_lib = None


def load(path: str = LIB_PATH):
    """Load libpxlflip.so and declare its signatures. Raises if the library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libpxlflip.so not built ({path}); run pxlengine_gb300.build.build() first")
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
