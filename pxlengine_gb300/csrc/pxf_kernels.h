// Host-visible launchers of the FLIP substep kernels (substep.cu, pcg.cu).
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "pxf_device.cuh"

namespace pxf {

// Device-resident work index of one stage.
using StageWork = Work;

constexpr uint32_t kScanChunk = 2048;     // cells per work item of the counting-sort scan
constexpr uint32_t kElemItem = 256;       // elements per item of the per-element kernels
constexpr int kMaxLevelsK = 12;           // multigrid levels (kMaxLevels in pxf_device.cuh)

int sm_count();

// Kernel launches issued by the calling host thread (eager or into a stream capture), and an
// optional per-thread log that the substep profiler installs to time every kernel separately.
struct LaunchLog {
    virtual void launched(const char* kernel, cudaStream_t st) = 0;
};
extern thread_local uint64_t g_kernel_launches;
extern thread_local LaunchLog* g_launch_log;
inline void note_launch(const char* kernel, cudaStream_t st) {
    ++g_kernel_launches;
    if (g_launch_log) g_launch_log->launched(kernel, st);
}
// A one-warp kernel that busy-waits `cycles` SM clocks (bounded by construction). The profiler
// puts one ahead of each eagerly launched segment so the host has queued the segment before
// the GPU reaches it, and the gaps between events are device time, not host launch time.
cudaError_t launch_hold(long long cycles, cudaStream_t st);
int grid_cap_per_sm();
void p2g_shape(int shape, int out[3]);
extern const int kNumP2GShapes;
constexpr int kMaxP2GShapes = 8;   // capacity of per-shape tables (kNumP2GShapes <= this)

cudaError_t launch_scan(const StageWork& chunks, const SimDev* sims, int n_sims, cudaStream_t st);
cudaError_t launch_scatter(const StageWork& parts, cudaStream_t st);
cudaError_t launch_bin(const StageWork& parts, cudaStream_t st);
// Heaviest-first processing order of a stage's P2G tiles, rebuilt every substep from the
// counting sort's cell starts: tiles go into log2 buckets of the particle count of their own
// cells (bucket = count leading zeros, 0 = heaviest, 32 = empty), so the blocks of the densest
// tiles start first and the light ones fill in behind them.
constexpr int kOrderBuckets = 33;
struct TileOrder {
    uint32_t* order = nullptr;    // [tiles] k-th tile to process
    uint32_t* bucket = nullptr;   // [tiles] bucket of every tile
    uint32_t* hist = nullptr;     // [2 * kOrderBuckets] bucket sizes, then placement cursors (zeroed first)
};
cudaError_t launch_tile_order(const StageWork& tiles, int shape, const TileOrder& o, cudaStream_t st);
cudaError_t launch_tile_weigh(const StageWork& tiles, int shape, const TileOrder& o, cudaStream_t st);   // buckets only
cudaError_t launch_tile_place(const StageWork& tiles, const TileOrder& o, cudaStream_t st);            // order from buckets
// Buckets of the 32x8x8 tiles (big) and of the 32x4x4 tiles (small) in one pass (the automatic pick).
cudaError_t launch_tile_weigh_pair(const StageWork& big, const StageWork& small, const TileOrder& ob,
                                  const TileOrder& os, cudaStream_t st);

// Automatic P2G tile shape: the large 32x8x8 tiles (least halo work) unless the heaviest one
// holds more particles than a fair share of the GPU's P2G block slots (FLIP packs cells with
// thousands of particles as a splash settles: that tile would outlast the others), then 32x4x4.
// The heaviest tile is taken at the lower end of its bucket (2^(31 - bucket) particles).
constexpr int kP2GAutoBig = 0, kP2GAutoSmall = 1;
__host__ __device__ inline bool p2g_small_for_bucket(int heaviest_bucket, uint32_t fair) {
    const uint32_t heaviest = heaviest_bucket >= 32 ? 0u : (1u << (31 - heaviest_bucket));
    return heaviest > fair;
}
inline bool p2g_pick_small(const uint32_t* hist, uint32_t fair) {
    int b = 0;
    while (b < kOrderBuckets - 1 && hist[b] == 0) b++;
    return p2g_small_for_bucket(b, fair);
}
uint32_t p2g_slots(int shape);   // resident P2G blocks of a tile shape on the whole GPU
// Sets the IF/ELSE condition of the P2G branches from the 32x8x8 buckets (graph capture only):
// 1 = large tiles, 0 = small.
cudaError_t launch_p2g_pick(const uint32_t* hist, uint32_t fair, cudaGraphConditionalHandle h, cudaStream_t st);
// lanes: bit 0 = strided lane mapping over a tile's particles (else blocked), bit 1 = whole x-rows
// per warp (else equal slices of the tile's particle list); order: null = item order.
cudaError_t launch_p2g(const StageWork& tiles, int shape, int lanes, const uint32_t* order, cudaStream_t st);

cudaError_t launch_divergence(const StageWork& cells, cudaStream_t st);
cudaError_t launch_pressure_rb(const StageWork& half_cells, uint32_t parity, uint32_t it, cudaStream_t st);
cudaError_t launch_project(const StageWork& cells, cudaStream_t st);   // one thread per cell
cudaError_t launch_g2p(const StageWork& parts, cudaStream_t st);

cudaError_t launch_gather_aos(const SimDev& s, float4* out, cudaStream_t st);
cudaError_t launch_scatter_aos(const SimDev& s, const float4* in, cudaStream_t st);
cudaError_t launch_counts_from_start(const SimDev& s, uint32_t* out, cudaStream_t st);

// Work indexes of the precision solver for one batch.
// The CG loop's stages visit only chunks that hold system cells: after the cell lists are built,
// one kernel compacts each stage's items into act[] / act_n (counters zeroed before it).
struct PcgWork {
    const SimDev* sims = nullptr;
    int n_sims = 0;
    StageWork chunks;                 // level-0 chunks of kScanChunk cells (precision simulations), compacted
    StageWork chunks_all;             // the same items, every chunk (list building, final copy)
    StageWork level[kMaxLevelsK];     // level-l chunks of multigrid simulations with a level below l, compacted
    StageWork coarse[kMaxLevelsK];    // level-(l+1) chunks of those simulations, compacted
    StageWork setup[kMaxLevelsK];     // level-(l+1) chunks of every multigrid simulation with level l+1
    uint32_t* act_n = nullptr;        // counters: [0] chunks, [1 + l] level[l], [1 + kMaxLevelsK + l] coarse[l]
    struct GridBar* sweep_bar = nullptr;  // grid barrier of the cooperative smoothing kernels
    uint32_t* tickets = nullptr;          // [2] last-block tickets of the control kernels that set conditions
    int setup_levels = 0;
    int max_levels = 0;                 // global-memory levels (below the shared-memory tail)
    int max_pairs = 1;                  // largest smoothing pair count of the batch's multigrid simulations
    bool any_mg = false, any_jacobi = false;
    size_t tail_smem = 0;               // dynamic shared memory of the tail kernel
};

constexpr uint32_t kTailCells = 8192;   // the shared-memory tail starts at the first level this small
static_assert(kTailCells <= 65536, "tail lists hold cell indices as 16-bit values");
// Shared-memory floats a tail level of nc cells takes: r, z (float), neighbour record and list (u16).
__host__ __device__ constexpr uint32_t tail_level_floats(uint32_t nc) { return 3 * nc; }
// List chunks (cells) of the system-cell lists: level 0 (PXF_L0_CHUNK; PXF_GS_CHUNK for the
// red-black GS) and the levels below it
// (PXF_COARSE_CHUNK); multiples of 256 up to 8192, read once per process.
uint32_t coarse_chunk();
uint32_t level0_chunk();      // level-0 list chunk of the precision solver
uint32_t level0_chunk_gs(uint64_t nc);   // level-0 list chunk of the red-black GS on nc cells
cudaError_t mg_tail_attr(size_t smem);

// Grid barrier of the persistent solve (device memory, zeroed at every launch).
struct GridBar {
    unsigned count;    // arrival word: top bit = barrier phase, low bits = arrivals
    unsigned gen;      // unused
    unsigned err;      // set when a wait exceeded kBarrierCycles
    unsigned pad;
};
constexpr long long kBarrierCycles = 4000000000LL;   // about 2 s at the GB300's clock

// One cooperative launch that runs the whole precision solve of a substep.
int pcg_solve_grid(size_t smem);
constexpr int kActCounters = 1 + 2 * kMaxLevelsK;
// Reference red-black GS streamed through shared memory, kGsIters iterations per pass over HBM:
// units of a kGsTileX x kGsTileY x-y tile (loaded with a halo of kGsHalo cells) and a z segment.
constexpr int kGsIters = 2;
constexpr int kGsHalo = 2 * kGsIters;
constexpr int kGsLoadX = 64, kGsLoadY = 32;
constexpr int kGsTileX = kGsLoadX - 2 * kGsHalo, kGsTileY = kGsLoadY - 2 * kGsHalo;
uint32_t gs_segment_planes(uint32_t nz);   // z planes of a unit
bool gs_stream_for(uint64_t cells);        // the streamed solve for a batch whose largest GS grid has `cells`
bool gs_resident_for(uint64_t cells);      // the one-launch red-black solve (largest GS grid of a batch)
void gs_res_knobs(long long& limit_cycles, int& skip);
cudaError_t gs_stream_attr();
// set-up (p_alt, right-hand side, counts, unit flags), ceil(max_iters / kGsIters) passes, copy-back
cudaError_t launch_gs_stream(const StageWork& units, uint32_t max_iters, cudaStream_t st);
// Reference red-black GS as one cooperative launch whose blocks own fixed cell ranges and wait
// only for the blocks within one z-plane of them (pressure_resident.cu).
constexpr uint32_t kGsResFlagStride = 32;   // flag words between two blocks' flags (a 128-byte line each)
struct GsResBlock {
    uint32_t sim;          // simulation of the batch
    uint32_t lo, hi;       // its cells [lo, hi)
    uint32_t dep0, dep1;   // blocks [dep0, dep1) within one z-plane of those cells, this one included
};
bool plan_gs_resident(const std::vector<SimDev>& sims, std::vector<GsResBlock>& plan, size_t& smem);
// Zeroes the flags, then the launch (2 x iterations half sweeps of every GS simulation).
cudaError_t launch_gs_resident(const SimDev* sims, const GsResBlock* plan, int blocks, uint32_t* flags,
                               uint32_t* err, size_t smem, long long limit_cycles, int skip, cudaStream_t st);
// Reference red-black GS over level-0 system-cell lists (lists first, then one launch per colour).
cudaError_t launch_gs_lists(const StageWork& chunks, cudaStream_t st);
cudaError_t launch_pressure_rb_list(const StageWork& chunks, uint32_t parity, uint32_t it, cudaStream_t st);
cudaError_t launch_barrier_selftest(GridBar* bar, int blocks, int skip, long long limit_cycles, int rounds,
                                    cudaStream_t st);
cudaError_t launch_pcg_solve(const PcgWork& pw, GridBar* bar, int grid, uint32_t guard, cudaStream_t st);

// Precision solver: multigrid setup + |b|^2 + state reset + first restart + first z = M^-1 r;
// then the loop body (direction + SpMV, update, conditional FP64 restart, preconditioner) while
// any simulation runs; finish writes the FP64 solution and the FP32 pressure copy.
cudaError_t launch_pcg_init(const PcgWork& pw, cudaStream_t st);
cudaError_t launch_pcg_body(const PcgWork& pw, cudaStream_t st);
cudaError_t launch_pcg_dir(const PcgWork& pw, cudaStream_t st);
// With a handle and a ticket the control kernel after the update also sets the restart IF node's
// condition (launch_pcg_update) or the loop's WHILE condition (launch_precond).
cudaError_t launch_pcg_update(const PcgWork& pw, cudaStream_t st, cudaGraphConditionalHandle h = 0,
                              uint32_t* ticket = nullptr);
cudaError_t launch_pcg_restart(const PcgWork& pw, cudaStream_t st);
cudaError_t launch_precond(const PcgWork& pw, cudaStream_t st, cudaGraphConditionalHandle h = 0,
                           uint32_t* ticket = nullptr);
cudaError_t launch_pcg_finish(const PcgWork& pw, cudaStream_t st);
cudaError_t launch_pcg_cond(const SimDev* sims, int n_sims, cudaGraphConditionalHandle h, cudaStream_t st);
// Sets an IF condition: does any simulation need an FP64 restart residual now?
// Host-driven fallback: a flag telling whether any simulation still runs.
cudaError_t launch_pcg_any(const SimDev* sims, int n_sims, uint32_t* flag, cudaStream_t st);

}  // namespace pxf
