/* pxlflip — GB300 (sm_103a) FLIP liquid substep behind a plain C ABI.
 *
 * Drop-in for pxlengine's liquid path:
 *   scene JSON `fluids[]` block        crates/pxl-scene/src/lib.rs:49-129 (types, defaults, grid())
 *                                      crates/pxl-scene/src/lib.rs:710-735 (validation)
 *   FluidState::new                    crates/pxl-render/src/fluid.rs:109-228
 *   Renderer::fluid_advance (sim part) crates/pxl-render/src/fluid.rs:265-306
 *   the substep kernels                shaders/fluid.slang:87-220
 *
 * Conventions: functions return 0 (PXF_OK) or a negative PXF_E* code; the message of the last
 * failure is available from pxf_last_error(handle) (or pxf_last_error(NULL) for failures that
 * produced no handle). A handle is used by one host thread at a time and owns one CUDA stream.
 * The library owns all device memory; callers own every host buffer they pass. Host waits are
 * bounded (pxf_options.wait_timeout_s) and end in PXF_ETIMEDOUT instead of blocking forever.
 * No entry point falls back to the CPU: without a usable CUDA device creation fails.
 */
#ifndef PXLFLIP_H
#define PXLFLIP_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PXF_API __attribute__((visibility("default")))
#else
#define PXF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PXF_OK 0
#define PXF_EINVAL (-1)     /* invalid argument or scene validation failure */
#define PXF_ECUDA (-2)      /* CUDA runtime error */
#define PXF_ENOMEM (-3)     /* device memory could not be allocated / admission refused */
#define PXF_ETIMEDOUT (-4)  /* a bounded host wait expired */
#define PXF_ESTATE (-5)     /* call not valid in the handle's current state */
#define PXF_ENOTFOUND (-6)  /* unknown request id / fluid index out of range */

typedef struct pxf_sim pxf_sim;
typedef struct pxf_batch pxf_batch;
typedef struct pxf_server pxf_server;
typedef struct pxf_snapshot pxf_snapshot;

/* FluidBlock (crates/pxl-scene/src/lib.rs:87-94). */
typedef struct {
    float min[3];
    float max[3];
    float velocity[3];
} pxf_fill_block;

/* Fluid (crates/pxl-scene/src/lib.rs:49-85), every simulation field; `materials` is a renderer
 * concern and is not represented. */
typedef struct {
    const char* name;
    float bounds[2][3];
    uint32_t resolution;              /* default 64 */
    const pxf_fill_block* fill;
    uint32_t fill_count;
    uint32_t particles_per_cell;      /* default 8 */
    uint32_t substeps;                /* default 8 */
    float flip;                       /* default 0.95 */
    float gravity[3];                 /* default (0, -9.81, 0) */
    uint32_t pressure_iterations;     /* default 80 */
    uint32_t surface_refine;          /* default 2 */
    float particle_radius;            /* default 2 */
    float warmup;                     /* default 0 */
    uint32_t max_triangles;           /* default 2,000,000 */
} pxf_fluid_desc;

#define PXF_PRESSURE_RBGS 0u   /* red-black Gauss-Seidel, pressure_iterations sweeps (reference) */
#define PXF_PRESSURE_PCG 1u    /* PCG (multigrid or Jacobi preconditioner): FP32 vectors, double-float
                                  solution, FP64 reductions and FP64 restart residuals */

/* Options beyond the reference's Fluid block. pxf_options_init gives the reference behaviour. */
typedef struct {
    uint32_t pressure_solver;      /* PXF_PRESSURE_RBGS (default) or PXF_PRESSURE_PCG */
    double pcg_rtol;               /* relative residual |b - A x| / |b| target, default 1e-6 */
    uint32_t pcg_max_iter;         /* default 2000 */
    uint32_t pcg_restart;          /* FP64 residual recomputation period, default 50 */
    uint32_t lift_grid_limits;     /* 1: accept resolution > 256 and > 16M cells (benchmark entry) */
    uint32_t keep_p2g_sums;        /* 1: also store the int32 P2G sums (acc, wacc) for inspection */
    float velocity_sigma;          /* > 0: add N(0, sigma) per velocity component at seeding */
    uint32_t velocity_seed;        /* seed of that jitter */
    double wait_timeout_s;         /* bound on every host wait, default 600 s */
    int32_t p2g_tile;              /* P2G tile shape index (pxf_tune_result.tile_shape); -1: the
                                      autotuner's choice, else 32x4x4, or on very large grids a
                                      per-substep pick between 32x8x8 and 32x4x4 */
    uint32_t pcg_precond;          /* 0: multigrid V-cycle (default), 1: Jacobi */
    uint32_t mg_coarse_iters;      /* red-black iterations on the coarsest multigrid level, default 2 */
    uint32_t mg_smooth_pairs;      /* red-black pairs of pre- and of post-smoothing per level, default 2 */
} pxf_options;

PXF_API void pxf_fluid_desc_init(pxf_fluid_desc* desc);
PXF_API void pxf_options_init(pxf_options* opts);

/* Scene-JSON validation of one fluid (crates/pxl-scene/src/lib.rs:710-735, same messages).
 * Writes the message to msg (if cap > 0) and returns PXF_EINVAL on failure. */
PXF_API int pxf_validate(const pxf_fluid_desc* desc, uint32_t index, uint32_t lift_grid_limits, char* msg, size_t cap);

/* Fluid::grid (crates/pxl-scene/src/lib.rs:123-128). */
PXF_API int pxf_fluid_grid(const pxf_fluid_desc* desc, uint32_t dims[3], float* h);

/* steps_for_frame (crates/pxl-render/src/fluid.rs:234-236). */
PXF_API uint64_t pxf_steps_for_frame(double warmup, double fps, uint32_t substeps, double frame);

/* FluidState::new (crates/pxl-render/src/fluid.rs:109-228): validates, seeds particles with
 * the reference LCG (fluid.rs:97-100,121-148) and allocates the simulation on the current
 * CUDA device. `seed` is render.seed, `fps` is render.fps. */
PXF_API int pxf_create(const pxf_fluid_desc* desc, uint32_t seed, double fps, pxf_sim** out);
PXF_API int pxf_create_ex(const pxf_fluid_desc* desc, uint32_t seed, double fps, const pxf_options* opts, pxf_sim** out);

/* Scene::from_json + FluidState::new for fluids[fluid_index] (crates/pxl-scene/src/lib.rs:634-648,
 * crates/pxl-render/src/lib.rs:204-229): seed and fps come from the scene's `render` block. */
PXF_API int pxf_create_from_json(const char* scene_json, uint32_t fluid_index, pxf_sim** out);
PXF_API int pxf_create_from_json_ex(const char* scene_json, uint32_t fluid_index, const pxf_options* opts, pxf_sim** out);
/* Number of fluids in a scene (after validation), or a negative error code. */
PXF_API int pxf_scene_fluid_count(const char* scene_json);

/* Renderer::fluid_advance, simulation part (crates/pxl-render/src/fluid.rs:265-306): steps to
 * the substep count of `frame`, re-seeding from the initial particles on the first call and on
 * a backwards seek. Returns when the work is complete (bounded wait). */
PXF_API int pxf_advance_to_frame(pxf_sim* sim, double frame);

/* Enqueue n substeps (fluid.rs:289-303) without waiting; pxf_sync waits (bounded). */
PXF_API int pxf_step(pxf_sim* sim, uint32_t n_substeps);
PXF_API int pxf_sync(pxf_sim* sim);

/* FluidState::particle_count (fluid.rs:230-232). */
PXF_API uint32_t pxf_particle_count(const pxf_sim* sim);
PXF_API uint64_t pxf_steps_done(const pxf_sim* sim);
/* Grid dims, cell size and substep dt (FluidPush nx, ny, nz, h, dt; fluid.rs:158-166). */
PXF_API int pxf_grid_info(const pxf_sim* sim, uint32_t dims[3], float* h, float* dt);
PXF_API size_t pxf_device_bytes(const pxf_sim* sim);
/* Device bytes a simulation of this description would allocate (admission control). */
PXF_API int pxf_estimate_bytes(const pxf_fluid_desc* desc, const pxf_options* opts, uint64_t* bytes);

/* Particles in the reference buffer layout (fluid.slang:9, fluid.rs:143): n records of 8 floats
 * [x, y, z, 0, vx, vy, vz, 0] in seeding order. n must equal pxf_particle_count. */
PXF_API int pxf_read_particles(pxf_sim* sim, float* out, size_t n);
PXF_API int pxf_write_particles(pxf_sim* sim, const float* in, size_t n);

/* Grid buffers of the last completed substep (fluid.slang:23-30). */
#define PXF_GRID_VEL 1          /* float[F]  velocities after project, faces u, v, w */
#define PXF_GRID_VEL_OLD 2      /* float[F]  velocities after normalize */
#define PXF_GRID_ACC 3          /* int32[F]  P2G fixed-point sum of w*v*65536 (keep_p2g_sums) */
#define PXF_GRID_WACC 4         /* int32[F]  P2G fixed-point sum of w*65536 (keep_p2g_sums) */
#define PXF_GRID_CELL_COUNT 5   /* uint32[C] particles per cell at the last P2G */
#define PXF_GRID_CELL_TYPE 6    /* uint32[C] 0 air, 1 fluid, 2 solid */
#define PXF_GRID_PRESSURE 7     /* float[C] */
#define PXF_GRID_DIVERGENCE 8   /* float[C]  divergence before projection */
#define PXF_GRID_PRESSURE64 9   /* double[C] FP64 pressure (precision solver only) */
/* Surface grid of the last pxf_surface_mesh (S nodes = (sx+1)(sy+1)(sz+1), S cells = sx sy sz,
 * s* = n* x surface_refine; fluid.slang bindings 39-41). */
#define PXF_GRID_SURF_DENSITY 10  /* int32[S nodes]  fixed-point density x 4096 */
#define PXF_GRID_SURF_PHI 11      /* float[S nodes]  smoothed density - iso, -1 on the boundary */
#define PXF_GRID_SURF_CELL_VERT 12 /* uint32[S cells] vertex index or 0xffffffff */
PXF_API int pxf_read_grid(pxf_sim* sim, int which, void* out, size_t bytes);
/* Only PXF_GRID_PRESSURE (the warm start of the next solve) is writable. */
PXF_API int pxf_write_grid(pxf_sim* sim, int which, const void* in, size_t bytes);

/* Precision-solver statistics of the last substep: PCG steps, final FP64 relative residual and
 * status (0 converged, 1 iteration cap, 2 breakdown, 3 zero right-hand side). */
PXF_API int pxf_solver_stats(pxf_sim* sim, uint32_t* iterations, double* relres, uint32_t* status);

/* Multigrid hierarchy of the precision solver as of the last substep: per level its cells and
 * its system cells (fluid cells with a non-solid neighbour); *levels receives the level count,
 * *tail the first level solved inside one block. No reference counterpart. */
PXF_API int pxf_mg_level_info(pxf_sim* sim, uint32_t* cells, uint32_t* system_cells, uint32_t cap,
                              uint32_t* levels, int32_t* tail);

/* Device state snapshot (particles, pressure warm start, step counter). */
PXF_API int pxf_snapshot_take(pxf_sim* sim, pxf_snapshot** out);
PXF_API int pxf_snapshot_restore(pxf_sim* sim, const pxf_snapshot* snap);
PXF_API void pxf_snapshot_free(pxf_snapshot* snap);

/* ------------------------------------------------------------------ measurement
 * Device time of n substeps: CUDA events recorded on the simulation's own stream around the
 * substep graphs, bounded wait. No reference counterpart (the reference times whole frames on
 * the host, crates/pxl-render/src/lib.rs:234-250). */
PXF_API int pxf_step_timed(pxf_sim* sim, uint32_t n_substeps, double* device_ms);

/* One substep launched stage by stage (no graph) with CUDA events between the launches on the
 * simulation's stream. Fills up to cap records; *count receives the number of stages. */
typedef struct {
    char name[32];
    uint32_t launches;
    double ms;          /* summed device time of those launches */
} pxf_stage_time;
PXF_API int pxf_profile_substep(pxf_sim* sim, pxf_stage_time* out, uint32_t cap, uint32_t* count);

/* P2G autotuner. No reference counterpart (the reference has one fixed 256-thread dispatch per
 * kernel, shaders/fluid.slang:93-115). Runs one substep eagerly and, after its counting sort,
 * times every P2G variant (tile shape x lane mapping) three times on the simulation's own
 * particles; the fastest of the last two runs is used by every later substep. Every variant
 * writes the same bits, so the substep's result equals a normal substep's; it counts as one. */
typedef struct {
    int32_t tile_shape;   /* 0: 32x8x8, 1: 32x4x4, 2: 16x8x8, 3: 64x4x4, 4: 16x4x4 cells */
    int32_t lanes;        /* 1: strided lane mapping over a tile's particles, 0: blocked */
    uint32_t variants;    /* variants timed, in the order shape-major, lanes-minor */
    float ms[16];         /* device time of each variant, ms */
    char chosen[32];
} pxf_tune_result;
PXF_API int pxf_autotune(pxf_sim* sim, pxf_tune_result* out);

/* Changes the bound of the simulation's host waits (pxf_options.wait_timeout_s), e.g. a frame
 * deadline; a wait that runs out returns PXF_ETIMEDOUT and leaves the device work running. */
PXF_API int pxf_set_wait_timeout(pxf_sim* sim, double seconds);

/* Surface nets of the current particles (the meshing half of Renderer::fluid_advance,
 * crates/pxl-render/src/fluid.rs:308-330; kernels shaders/fluid.slang:222-355): density splat,
 * smoothing, vertices and quads into device buffers the library owns (allocated on the first
 * call: about 12 bytes per surface node and cell plus max_triangles x 44 bytes). Returns the
 * counts the reference reads back, capped like the reference (vertices <= max_triangles,
 * triangles <= max_triangles, even), and the overflow flag (fluid.rs:324-327). Vertices are
 * numbered by ascending surface cell and triangles by ascending node and axis (the reference's
 * order follows its atomic counters and varies from run to run). device_ms (optional) receives
 * the meshing's device time. */
PXF_API int pxf_surface_mesh(pxf_sim* sim, uint32_t* vertices, uint32_t* triangles, int32_t* overflow,
                             double* device_ms);
/* pxf_surface_mesh into the caller's device buffers, as the reference's s_verts / s_quads write
 * the renderer's global buffers (fluid.slang:313-314, 343-351; fluid.rs:308-330): vertex idx goes
 * to d_vertices[(vbase + idx) * 8 .. + 8] as (x, y, z, 0, nx, ny, nz, 0) floats, triangle t to
 * d_indices[ibase + 3 t .. + 3] as vertex indices counted from vbase. max_vertices /
 * max_triangles cap the writes (0: the fluid's max_triangles for both, like the reference); the
 * returned counts and overflow flag follow the reference's capping. The library's own mesh
 * buffers (pxf_read_mesh, pxf_mesh_device_buffers) are left as they were. */
PXF_API int pxf_surface_mesh_into(pxf_sim* sim, float* d_vertices, uint32_t vbase, uint32_t max_vertices,
                                  uint32_t* d_indices, uint32_t ibase, uint32_t max_triangles, uint32_t* vertices,
                                  uint32_t* triangles, int32_t* overflow, double* device_ms);
/* Surface grid of the simulation as FluidState::new sets it (fluid.rs:150-156): surface cells per
 * axis (grid cells x surface_refine), surface cell size, splat radius and iso level. */
PXF_API int pxf_surface_info(const pxf_sim* sim, uint32_t dims[3], float* cell, float* radius, float* iso);
/* Copies the mesh of the last pxf_surface_mesh: vertices as [x, y, z, 0, nx, ny, nz, 0] records
 * (the renderer's vertex layout), triangles as three vertex indices; n_vertices / n_triangles must
 * equal the counts pxf_surface_mesh returned. */
PXF_API int pxf_read_mesh(pxf_sim* sim, float* vertices, size_t n_vertices, uint32_t* indices, size_t n_triangles);
/* Device addresses of the mesh buffers (valid until the next pxf_surface_mesh or pxf_destroy),
 * for consumers that build acceleration structures or render from device memory directly. */
PXF_API int pxf_mesh_device_buffers(pxf_sim* sim, const void** vertices, const void** indices);

/* Self-test of the bounded grid barrier that the persistent precision solve uses (no reference
 * counterpart): `rounds` barriers over `blocks` co-resident blocks of 32 threads. With skip_block
 * >= 0 that block never arrives, so every other block's wait runs out after limit_ms (SM-clock
 * cycles at 2.07 GHz), sets the error flag and returns; the kernel then ends normally and the
 * context stays usable. *timed_out receives the flag (0 when every barrier completed). */
PXF_API int pxf_selftest_grid_barrier(uint32_t blocks, int32_t skip_block, double limit_ms, uint32_t rounds,
                                      uint32_t* timed_out);

/* Selects the CUDA device of the calling host thread for the simulations it creates (the
 * library links its own CUDA runtime, so a caller's runtime setting does not carry over). */
PXF_API int pxf_set_device(int device);

/* Page-locked host memory for fast particle transfers (cudaMallocHost / cudaFreeHost). */
PXF_API int pxf_host_alloc(size_t bytes, void** out);
PXF_API void pxf_host_free(void* p);

/* Cell binning that allocates nothing. No counterpart in the reference.
 * For callers that cannot call cudaMalloc: a renderer whose device memory all comes from its own
 * allocator or graphics interop, a real-time thread that must not allocate. The caller passes
 * n particle records on the device (d_particles: the [x,y,z,w,vx,vy,vz,w] layout of
 * pxf_read_particles) and an output buffer of C + 1 uint32 on the device (C = dims[0]*dims[1]*dims[2]);
 * d_cell_start receives the exclusive prefix sum of the particles per cell, with the cell of a
 * particle computed as in the substep: clamp(floor((x - origin) * inv_h)) per axis, where
 * inv_h = 1.0f / h is rounded to float once and each product is rounded to float; positions
 * outside the grid land in the nearest boundary cell. d_cell_start[C] = n.
 * The only scratch is a fixed 32 KiB array inside the library on each device that loads it (held
 * until the process exits), so grids are limited to 16,777,216 cells; larger grids return
 * PXF_EINVAL with a message in pxf_last_error(NULL). The first call in each CUDA context (the
 * context current on the calling thread, else the current device's primary context) looks up
 * that array's device address in that context: make it before any stream capture. The work is queued on `stream`
 * (a cudaStream_t; NULL = the default stream) and the call returns without waiting. Every call
 * shares the one scratch array, so calls whose work overlaps on the GPU race. */
PXF_API int pxf_cell_starts_noalloc(const float* d_particles, uint32_t n, const uint32_t dims[3], const float origin[3],
                                    float h, uint32_t* d_cell_start, void* stream);

/* ------------------------------------------------------------------ agent neighbour grid
 * Counting sort of agents by hashed cell, the neighbour grid an agent simulation rebuilds every
 * step (replaces grid_clear, grid_count, scan_local, scan_blocks, scan_add and grid_scatter,
 * shaders/sim.slang:5-7, 28-104, driven by crates/pxl-render/src/sim.rs:230-260).
 * d_agents: count records of stride_floats floats on the device, the position in the first three
 * (the reference's Agent record is 16 floats). A cell is (floor(x / cs), floor(y / cs),
 * floor(z / cs)) with cs = max(cell_size, 1e-6) and IEEE division, its hash
 * ((cx * 73856093) ^ (cy * 19349663) ^ (cz * 83492791)) & (table_size - 1) in 32-bit unsigned
 * arithmetic; table_size must be a power of two (pxf_grid_table_size gives the reference's choice).
 * Outputs on the device: d_counts[table_size] agents per cell, d_offsets[table_size] their
 * exclusive prefix sum (first slot of each cell) and d_sorted[count] the agent ids grouped by cell;
 * inside one cell the ids' order is unspecified, as in the reference. d_scratch (device) holds at
 * least pxf_grid_scratch_bytes(count, table_size) bytes; the call allocates nothing, queues its
 * work on `stream` (a cudaStream_t; NULL = the default stream) and returns without waiting. */
PXF_API uint32_t pxf_grid_table_size(uint32_t count);   /* (2 count).next_power_of_two() in [1024, 2^23], sim.rs:129 */
PXF_API size_t pxf_grid_scratch_bytes(uint32_t count, uint32_t table_size);
PXF_API int pxf_grid_sort(const float* d_agents, uint32_t stride_floats, uint32_t count, float cell_size,
                          uint32_t table_size, uint32_t* d_offsets, uint32_t* d_counts, uint32_t* d_sorted,
                          void* d_scratch, size_t scratch_bytes, void* stream);

PXF_API void pxf_destroy(pxf_sim* sim);
PXF_API const char* pxf_last_error(const pxf_sim* sim);

/* ------------------------------------------------------------------ batched form
 * Many simulations with uneven grids advance together: every stage is one launch over a packed
 * multi-grid work index and a whole substep is one CUDA graph launch. No reference counterpart
 * (the reference steps each FluidState alone, crates/pxl-render/src/lib.rs:238-247). A
 * simulation belongs to at most one batch; while it does, step it only through the batch. */
PXF_API int pxf_batch_create(pxf_batch** out);
PXF_API int pxf_batch_add(pxf_batch* b, pxf_sim* sim);
PXF_API int pxf_batch_remove(pxf_batch* b, pxf_sim* sim);
PXF_API uint32_t pxf_batch_size(const pxf_batch* b);
PXF_API int pxf_batch_step(pxf_batch* b, uint32_t n_substeps);
PXF_API int pxf_batch_sync(pxf_batch* b);
PXF_API void pxf_batch_destroy(pxf_batch* b);
PXF_API const char* pxf_batch_last_error(const pxf_batch* b);
/* n substeps of the whole batch with their device time (CUDA events on the batch's stream). */
PXF_API int pxf_batch_step_timed(pxf_batch* b, uint32_t n_substeps, double* device_ms);
/* pxf_autotune for the whole batch: one substep of every member, variants timed on all of them. */
PXF_API int pxf_batch_autotune(pxf_batch* b, pxf_tune_result* out);

/* ------------------------------------------------------------------ serving form
 * A continuous-batching request loop. Requests (a fluid description + a number of substeps) queue
 * on submit; every tick retires finished requests (their final particles move to host memory and
 * their device memory is freed), admits queued requests in arrival order while their estimated
 * device footprint fits the HBM budget, and advances every active request by one batched substep
 * (one CUDA graph launch). No reference counterpart: pxlengine runs one scene per process.
 * Thread safety: submit / cancel / status / take_result / stats may be called from any thread;
 * tick must be called from one thread at a time (or use pxf_server_start for a worker thread). */
typedef struct {
    uint64_t hbm_budget_bytes;     /* default 150e9 */
    uint32_t max_active;           /* default 256 */
    uint32_t substeps_per_tick;    /* default 1 */
    double wait_timeout_s;         /* bound on each tick's device wait, default 600 s */
} pxf_server_config;

#define PXF_REQ_QUEUED 0
#define PXF_REQ_RUNNING 1
#define PXF_REQ_DONE 2
#define PXF_REQ_CANCELLED 3
#define PXF_REQ_FAILED 4

typedef struct {
    int32_t state;                 /* PXF_REQ_* */
    int32_t error;                 /* PXF_E* when failed */
    uint32_t substeps_done;
    uint32_t substeps_total;
    uint32_t particles;
    uint64_t device_bytes;
    double submit_s, admit_s, finish_s;   /* server clock (seconds since creation) */
} pxf_request_status;

typedef struct {
    uint64_t ticks;
    uint64_t submitted, admitted, completed, cancelled, rejected;
    uint32_t active, queued;
    uint64_t reserved_bytes, peak_reserved_bytes;
    double particle_substeps;      /* total particle-substeps advanced */
    double busy_device_ms;         /* summed device time of the batched substeps */
    double p50_substep_ms, p99_substep_ms;   /* per-tick device time of one batched substep */
    double p50_tick_wall_ms, p99_tick_wall_ms;
    double uptime_s;
} pxf_server_stats;

PXF_API void pxf_server_config_init(pxf_server_config* cfg);
PXF_API int pxf_server_create(const pxf_server_config* cfg, pxf_server** out);
PXF_API int pxf_server_submit(pxf_server* s, const pxf_fluid_desc* desc, uint32_t seed, double fps,
                              const pxf_options* opts, uint32_t substeps, uint64_t* request_id);
PXF_API int pxf_server_cancel(pxf_server* s, uint64_t request_id);
PXF_API int pxf_server_tick(pxf_server* s, uint32_t* active);
PXF_API int pxf_server_status(pxf_server* s, uint64_t request_id, pxf_request_status* out);
/* Final particles of a finished request ([x,y,z,0,vx,vy,vz,0] records); releases the request. */
PXF_API int pxf_server_take_result(pxf_server* s, uint64_t request_id, float* out, size_t n);
PXF_API int pxf_server_stats_get(pxf_server* s, pxf_server_stats* out);
/* Worker thread that ticks while requests are queued or active (idle wait is bounded). */
PXF_API int pxf_server_start(pxf_server* s);
PXF_API int pxf_server_stop(pxf_server* s);
PXF_API void pxf_server_destroy(pxf_server* s);
PXF_API const char* pxf_server_last_error(const pxf_server* s);

#ifdef __cplusplus
}
#endif

#endif /* PXLFLIP_H */
