// Host engine behind the C ABI (include/pxlflip.h): simulation state (FluidState,
// crates/pxl-render/src/fluid.rs:74-94), the per-frame advance (fluid.rs:265-306) and batches.
//
// Execution model: every simulation belongs to a batch (its own private batch of one, or a
// shared pxf_batch). A batch owns a CUDA stream, the device array of SimDev descriptors and the
// work index of each stage, and one instantiated CUDA graph that performs a whole substep for
// all its simulations:
//   scan+classify (3) -> scatter -> P2G -> divergence -> pressure -> project -> G2P
// The red-black pressure loop is unrolled into the graph (2 x iterations launches); the
// precision solver's loop is a conditional while-node whose body runs until every simulation
// has converged, so no host round trip happens inside a substep.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pxlflip.h"
#include "engine.h"
#include "pxf_device.cuh"
#include "surface.h"
#include "pxf_kernels.h"
#include "scene.h"
#include "seed.h"

using namespace pxf;

namespace {

thread_local std::string g_last_error;

int set_global_error(int code, const std::string& m) {
    g_last_error = m;
    return code;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

// --------------------------------------------------------------------------------- batch
namespace pxf {

struct KernelTimer;

struct BatchImpl {
    std::vector<pxf_sim*> sims;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;         // body capture of the conditional node
    cudaStream_t side2 = nullptr;        // body capture of the nested restart IF node
    bool if_ok = true;                   // nested IF node usable inside the while body
    bool persistent = false;             // the captured substep uses the persistent solve
    bool retried_plain_if = false;
    SimDev* d_sims = nullptr;
    uint32_t* d_base = nullptr;
    size_t cap_sims = 0;
    StageWork w_parts, w_tiles, w_cells, w_half, w_faces, w_chunks;
    StageWork w_lchunks;                 // level-0 system-cell list chunks (PCG and the list GS)
    StageWork w_gsu;                     // units of the streamed red-black GS
    bool gs_stream = false;              // the red-black GS of this batch is streamed (largest grid)
    bool gs_res = false;                 // the red-black GS as one cooperative launch (pressure_resident.cu)
    std::vector<GsResBlock> res_plan;    // its blocks
    size_t res_smem = 0;
    void* d_res = nullptr;               // plan, flags and error word of that launch
    size_t cap_res = 0;
    GsResBlock* d_res_plan = nullptr;
    uint32_t* d_res_flags = nullptr;
    uint32_t* d_res_err = nullptr;
    long long res_limit = kBarrierCycles;
    int res_skip = -1;
    PcgWork pw;                          // precision-solver work indexes
    uint32_t max_gs_iters = 0;
    bool any_gs = false, any_pcg = false;
    int tile_shape = 0;
    int p2g_lanes = 1;                   // 1: strided lane mapping in P2G, 0: blocked
    bool tuned = false;                  // tile_shape / p2g_lanes chosen by autotune()
    StageWork w_tiles_s[kMaxP2GShapes];  // P2G tile index of every tile shape
    uint32_t* d_tile_base = nullptr;
    size_t cap_tile = 0;
    TileOrder ord;                       // heaviest-first P2G tile order (rebuilt every substep)
    size_t cap_order = 0;
    bool auto_shape = false;             // tile shape picked every substep (p2g_pick_small)
    bool p2g_if_ok = true;               // the automatic pick as an IF/ELSE node in captured graphs
    TileOrder ord_big;                   // buckets and order of the 32x8x8 tiles (the pick's input)
    size_t cap_order_big = 0;
    uint32_t fair = 0;                   // particles per P2G block slot (the pick's threshold)
    bool pick_dynamic = false;           // fair share large enough for the 32x8x8 tiles to win
    uint16_t* d_sim_of = nullptr;        // item -> simulation tables of every stage
    size_t cap_sim_of = 0;
    uint32_t* d_act = nullptr;           // compacted item lists of the CG loop's stages
    uint32_t* d_act_n = nullptr;
    size_t cap_act = 0;
    uint32_t* d_tickets = nullptr;       // last-block tickets of the condition-setting control kernels
    cudaGraphExec_t exec = nullptr;
    bool dirty = true;
    bool cond_ok = true;                 // conditional while-node usable
    // host-driven fallback for the precision loop
    cudaGraphExec_t exec_pre = nullptr, exec_body = nullptr, exec_post = nullptr;
    uint32_t* d_flag = nullptr;
    uint32_t* h_flag = nullptr;
    // persistent precision solve (one cooperative launch per substep)
    GridBar* d_bar = nullptr;
    bool persist_ok = true;
    int persist_grid = 0;
    uint32_t persist_guard = 0;
    double timeout_s = 600.0;
    std::string err;
    bool owned_by_sim = false;

    ~BatchImpl();
    int fail(int code, const std::string& m) { err = m; return code; }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(PXF_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
    int rebuild();
    int capture();
    int record_pre(cudaStream_t st);
    int record_post(cudaStream_t st);
    int record_gs_part(cudaStream_t st);     // scan .. divergence and the red-black sweeps
    int record_post_solve(cudaStream_t st);  // project, g2p
    cudaError_t record_gs(cudaStream_t st);  // the red-black sweeps
    cudaError_t p2g(int shape, int lanes, cudaStream_t st);   // tile order + P2G of a tile shape
    int record_p2g(cudaStream_t st);                          // P2G of the substep (automatic shape)
    cudaError_t p2g_branch(int shape, cudaStream_t st);
    cudaError_t capture_if(cudaStream_t st, cudaGraphConditionalHandle h);
    int step(uint32_t n);
    int wait();
    void drop_graphs();
    int profile(pxf_stage_time* out, uint32_t cap, uint32_t* count);
    int run_eager(KernelTimer* timer, pxf_tune_result* tune);
    cudaError_t capture_restart(cudaStream_t st, cudaGraphConditionalHandle h);
};

}  // namespace pxf

// --------------------------------------------------------------------------------- simulation
struct pxf_sim {
    FluidCfg cfg;
    pxf_options opts;
    uint32_t seed = 0;
    double fps = 24.0;
    uint32_t dims[3] = {0, 0, 0};
    float h = 0, dt = 0;
    SimDev dev{};                 // host copy of the device descriptor
    SeedPlan plan;
    void* mem = nullptr;          // one device allocation for every buffer
    size_t mem_bytes = 0;
    float4* pos0 = nullptr;       // initial particles (re-seed on rewind, fluid.rs:271-275)
    float4* vel0 = nullptr;
    uint64_t steps_done = 0;
    bool initialized = false;
    pxf::BatchImpl* batch = nullptr;      // batch that steps this simulation
    pxf::BatchImpl* own = nullptr;        // private batch of one
    void* surf_mem = nullptr;             // surface grid + mesh buffers (first pxf_surface_mesh)
    pxf::SurfDev surf{};
    uint32_t mesh_verts = 0, mesh_tris = 0;   // capped counts of the last mesh
    std::string err;

    int fail(int code, const std::string& m) { err = m; return code; }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(PXF_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
};

struct pxf_snapshot {
    std::vector<float4> pos, vel;
    std::vector<float> pressure;
    std::vector<double> x64;
    std::vector<float2> x2;
    uint64_t steps_done = 0;
    bool initialized = false;
    uint32_t np = 0, nc = 0;
};

struct pxf_batch {
    pxf::BatchImpl impl;
};

namespace pxf {

// Byte layout of one simulation's allocation.
struct Layout {
    size_t posA, velA, posB, velB, pos0, vel0, vel, vel_old, pressure, div, type, count, start, chunk, info, acc, wacc,
        x2, x64, r, z, p0, p1, Ap, partial, pcg, p_alt, rhs, gs_cnt, gs_flag, total;
    int nlev = 0;
    int dims[kMaxLevels][3];
    size_t ltype[kMaxLevels], linfo[kMaxLevels], lr[kMaxLevels], lz[kMaxLevels], llist[kMaxLevels], llcnt[kMaxLevels];
};

// Multigrid hierarchy: halve (rounding up) while the level has more than 512 cells and every
// axis has at least 2 cells.
static int mg_levels(const uint32_t n[3], int dims[kMaxLevels][3]) {
    int L = 0;
    dims[0][0] = int(n[0]); dims[0][1] = int(n[1]); dims[0][2] = int(n[2]);
    L = 1;
    while (L < kMaxLevels) {
        const int* d = dims[L - 1];
        if (int64_t(d[0]) * d[1] * d[2] <= 512 || d[0] < 2 || d[1] < 2 || d[2] < 2) break;
        for (int a = 0; a < 3; a++) dims[L][a] = (d[a] + 1) / 2;
        L++;
    }
    return L;
}

// Units of the streamed red-black GS: x-y tiles times z segments.
static void gs_unit_grid(const uint32_t n[3], uint32_t g[4]) {
    g[0] = (n[0] + kGsTileX - 1) / kGsTileX;
    g[1] = (n[1] + kGsTileY - 1) / kGsTileY;
    g[3] = gs_segment_planes(n[2]);
    g[2] = (n[2] + g[3] - 1) / g[3];
}

static uint32_t gs_units(const uint32_t n[3]) {
    uint32_t g[4];
    gs_unit_grid(n, g);
    return g[0] * g[1] * g[2];
}

static Layout layout_for(uint32_t np, const uint32_t n[3], const pxf_options& o) {
    const uint64_t nc = uint64_t(n[0]) * n[1] * n[2];
    const uint64_t nf = uint64_t(n[0] + 1) * n[1] * n[2] + uint64_t(n[0]) * (n[1] + 1) * n[2] + uint64_t(n[0]) * n[1] * (n[2] + 1);
    const uint64_t nchunks = (nc + kScanChunk - 1) / kScanChunk;
    const bool pcg = o.pressure_solver == PXF_PRESSURE_PCG;
    const uint64_t cs0 = pcg ? level0_chunk() : level0_chunk_gs(nc);
    const uint64_t lchunks = (nc + cs0 - 1) / cs0;
    Layout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t at = off; off += align256(bytes); return at; };
    L.posA = take(16ull * np);
    L.velA = take(16ull * np);
    // posB and velB are adjacent: together they double as the AoS staging buffer (32 B per particle).
    L.posB = take(16ull * np);
    L.velB = L.posB + 16ull * np;
    off = L.posB + align256(32ull * np);
    L.pos0 = take(16ull * np);
    L.vel0 = take(16ull * np);
    L.vel = take(4 * nf);
    L.vel_old = take(4 * nf);
    L.pressure = take(4 * nc);
    L.div = take(4 * nc);
    L.type = take(nc);
    L.count = take(4 * nc);
    L.start = take(4 * (nc + 1));
    L.chunk = take(4 * (nchunks + 1));   // + the dense-cell flag of the last binning
    L.info = take(2 * nc);
    L.acc = o.keep_p2g_sums ? take(4 * nf) : 0;
    L.wacc = o.keep_p2g_sums ? take(4 * nf) : 0;
    // level-0 system-cell lists (red then black per chunk): both pressure solvers walk them
    L.llist[0] = take(4 * lchunks * cs0);
    L.llcnt[0] = take(8 * lchunks);
    if (!pcg) {
        L.p_alt = take(4 * nc);
        L.rhs = take(4 * nc);
        L.gs_cnt = take(nc);
        L.gs_flag = take(4 * uint64_t(gs_units(n)));
    }
    if (pcg) {
        L.x2 = take(8 * nc);
        L.x64 = take(8 * nc);
        L.r = take(4 * nc);
        L.z = take(4 * nc);
        L.p0 = take(4 * nc);
        L.p1 = take(4 * nc);
        L.Ap = take(4 * nc);
        L.partial = take(8 * lchunks);
        L.pcg = take(sizeof(PcgState));
        if (o.pcg_precond == 0) {
            L.nlev = mg_levels(n, L.dims);
            for (int l = 1; l < L.nlev; l++) {
                const uint64_t c = uint64_t(L.dims[l][0]) * L.dims[l][1] * L.dims[l][2];
                const uint64_t ch = (c + coarse_chunk() - 1) / coarse_chunk();
                L.ltype[l] = take(c);
                L.linfo[l] = take(2 * c);
                L.lr[l] = take(4 * c);
                L.lz[l] = take(4 * c);
                L.llist[l] = take(4 * ch * coarse_chunk());
                L.llcnt[l] = take(8 * ch);
            }
        }
    }
    L.total = off;
    return L;
}

BatchImpl::~BatchImpl() {
    drop_graphs();
    if (d_sims) cudaFree(d_sims);
    if (d_base) cudaFree(d_base);
    if (d_flag) cudaFree(d_flag);
    if (h_flag) cudaFreeHost(h_flag);
    if (d_bar) cudaFree(d_bar);
    if (d_res) cudaFree(d_res);
    if (d_tile_base) cudaFree(d_tile_base);
    if (ord.order) cudaFree(ord.order);
    if (ord.bucket) cudaFree(ord.bucket);
    if (ord.hist) cudaFree(ord.hist);
    if (ord_big.order) cudaFree(ord_big.order);
    if (ord_big.bucket) cudaFree(ord_big.bucket);
    if (ord_big.hist) cudaFree(ord_big.hist);
    if (d_sim_of) cudaFree(d_sim_of);
    if (d_act) cudaFree(d_act);
    if (d_act_n) cudaFree(d_act_n);
    if (d_tickets) cudaFree(d_tickets);
    if (side) cudaStreamDestroy(side);
    if (side2) cudaStreamDestroy(side2);
    if (stream) cudaStreamDestroy(stream);
}

void BatchImpl::drop_graphs() {
    if (exec) cudaGraphExecDestroy(exec);
    if (exec_pre) cudaGraphExecDestroy(exec_pre);
    if (exec_body) cudaGraphExecDestroy(exec_body);
    if (exec_post) cudaGraphExecDestroy(exec_post);
    exec = exec_pre = exec_body = exec_post = nullptr;
}

static inline uint32_t cdiv(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

// Work-index stages: particles, P2G tiles, cells, half cells, faces, 2048-cell chunks, then the
// multigrid smoothing chunks of each level and the restriction chunks of each level.
constexpr int kStages = 8 + 3 * kMaxLevels;   // then streamed-GS units, and last the level-0 list chunks

int BatchImpl::rebuild() {
    cudaError_t e;
    if (!stream) {
        if ((e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
        if ((e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
        if ((e = cudaStreamCreateWithFlags(&side2, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(e, "stream");
    }
    drop_graphs();
    const int n = int(sims.size());
    trace("rebuild: %d simulations", n);
    if (n == 0) { dirty = false; return PXF_OK; }
    if (n > 65535) return fail(PXF_EINVAL, "a batch holds at most 65535 simulations");
    if (size_t(n) > cap_sims) {
        if (d_sims) cudaFree(d_sims);
        if (d_base) cudaFree(d_base);
        d_sims = nullptr;
        d_base = nullptr;
        cap_sims = std::max<size_t>(size_t(n), cap_sims * 2);
        if ((e = cudaMalloc(&d_sims, cap_sims * sizeof(SimDev))) != cudaSuccess) return cuda_fail(e, "batch table");
        if ((e = cudaMalloc(&d_base, kStages * (cap_sims + 1) * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "batch index");
    }
    if (!tuned) {
        tile_shape = p2g_shape_index();
        p2g_lanes = p2g_lanes_default();
        auto_shape = tile_shape < 0;
        if (auto_shape) tile_shape = kP2GAutoSmall;
        for (pxf_sim* sm : sims)
            if (sm->opts.p2g_tile >= 0 && sm->opts.p2g_tile < kNumP2GShapes) {
                tile_shape = sm->opts.p2g_tile;
                auto_shape = false;
            }
    } else {
        auto_shape = false;
    }
    int shape[3];
    p2g_shape(tile_shape, shape);
    // P2G tile indexes of every shape (the autotuner times them all)
    if (size_t(n) + 1 > cap_tile) {
        if (d_tile_base) cudaFree(d_tile_base);
        d_tile_base = nullptr;
        cap_tile = std::max<size_t>(size_t(n) + 1, 2 * cap_tile);
        if ((e = cudaMalloc(&d_tile_base, kNumP2GShapes * cap_tile * sizeof(uint32_t))) != cudaSuccess)
            return cuda_fail(e, "tile index");
    }
    std::vector<uint32_t> tbase(size_t(kNumP2GShapes) * (n + 1), 0);
    for (int v = 0; v < kNumP2GShapes; v++) {
        int sh[3];
        p2g_shape(v, sh);
        for (int i = 0; i < n; i++) {
            const SimDev& d = sims[i]->dev;
            tbase[v * (n + 1) + i + 1] = tbase[v * (n + 1) + i] + cdiv(d.nx, sh[0]) * cdiv(d.ny, sh[1]) * cdiv(d.nz, sh[2]);
        }
    }
    if ((e = cudaMemcpyAsync(d_tile_base, tbase.data(), tbase.size() * 4, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return cuda_fail(e, "tile index upload");
    std::vector<SimDev> host(n);
    std::vector<uint32_t> base(kStages * (n + 1), 0);
    max_gs_iters = 0;
    uint64_t max_gs_cells = 0;
    any_gs = any_pcg = false;
    pw = PcgWork();
    timeout_s = 0;
    for (int i = 0; i < n; i++) {
        pxf_sim* s = sims[i];
        host[i] = s->dev;
        const SimDev& d = s->dev;
        uint32_t items[kStages] = {
            cdiv(d.np, kElemItem),
            cdiv(d.nx, shape[0]) * cdiv(d.ny, shape[1]) * cdiv(d.nz, shape[2]),
            cdiv(d.nc, kElemItem),
            cdiv(uint64_t((d.nx + 1) / 2) * d.ny * d.nz, kElemItem),
            cdiv(d.nf, kElemItem),
            cdiv(d.nc, kScanChunk)};
        items[kStages - 1] = cdiv(d.nc, d.lev[0].cs);
        items[kStages - 2] = d.solver == 0 ? d.gs_ntx * d.gs_nty * d.gs_nzs : 0u;
        const bool mg = d.solver == 1 && d.precond == 0;
        for (int l = 0; l < kMaxLevels; l++) {
            // global-memory smoothing of level l and restriction to l + 1 exist below the tail
            const bool has = mg && l < d.tail;
            items[6 + l] = has ? cdiv(d.lev[l].nc, d.lev[l].cs) : 0;
            items[6 + kMaxLevels + l] = has ? cdiv(d.lev[l + 1].nc, d.lev[l + 1].cs) : 0;
            items[6 + 2 * kMaxLevels + l] = (mg && l + 1 < d.nlev) ? cdiv(d.lev[l + 1].nc, d.lev[l + 1].cs) : 0;
        }
        for (int k = 0; k < kStages; k++) base[k * (n + 1) + i + 1] = base[k * (n + 1) + i] + items[k];
        if (d.solver == 0) {
            any_gs = true;
            max_gs_iters = std::max(max_gs_iters, d.iterations);
            max_gs_cells = std::max<uint64_t>(max_gs_cells, d.nc);
        } else {
            any_pcg = true;
            if (mg) {
                pw.any_mg = true;
                pw.max_levels = std::max(pw.max_levels, d.tail + 1);
                pw.max_pairs = std::max(pw.max_pairs, int(d.mg_pairs));
                pw.setup_levels = std::max(pw.setup_levels, d.nlev);
                size_t bytes = 0;
                for (int l = d.tail; l < d.nlev; l++) bytes += 4 * size_t(tail_level_floats(d.lev[l].nc));
                pw.tail_smem = std::max(pw.tail_smem, bytes);
            }
            else pw.any_jacobi = true;
        }
        timeout_s = std::max(timeout_s, s->opts.wait_timeout_s);
        if (d.solver == 1) persist_guard = std::max(persist_guard, d.max_iter + 2);
    }
    if (timeout_s <= 0) timeout_s = 600.0;
    if ((e = cudaMemcpyAsync(d_sims, host.data(), n * sizeof(SimDev), cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return cuda_fail(e, "batch table upload");
    if ((e = cudaMemcpyAsync(d_base, base.data(), base.size() * 4, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
        return cuda_fail(e, "batch index upload");
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_fail(e, "batch upload");
    StageWork* ws[kStages];
    ws[0] = &w_parts; ws[1] = &w_tiles; ws[2] = &w_cells; ws[3] = &w_half; ws[4] = &w_faces; ws[5] = &w_chunks;
    ws[kStages - 1] = &w_lchunks;
    ws[kStages - 2] = &w_gsu;
    for (int l = 0; l < kMaxLevels; l++) {
        ws[6 + l] = &pw.level[l];
        ws[6 + kMaxLevels + l] = &pw.coarse[l];
        ws[6 + 2 * kMaxLevels + l] = &pw.setup[l];
    }
    for (int k = 0; k < kStages; k++) {
        ws[k]->sims = d_sims;
        ws[k]->base = d_base + k * (n + 1);
        ws[k]->n_sims = n;
        ws[k]->total = base[k * (n + 1) + n];
    }
    size_t max_tiles = 1;
    for (int v = 0; v < kNumP2GShapes; v++) {
        w_tiles_s[v].sims = d_sims;
        w_tiles_s[v].base = d_tile_base + v * (n + 1);
        w_tiles_s[v].n_sims = n;
        w_tiles_s[v].total = tbase[v * (n + 1) + n];
        max_tiles = std::max<size_t>(max_tiles, w_tiles_s[v].total);
    }
    if (max_tiles > cap_order) {
        if (ord.order) cudaFree(ord.order);
        if (ord.bucket) cudaFree(ord.bucket);
        ord.order = ord.bucket = nullptr;
        cap_order = std::max(max_tiles, 2 * cap_order);
        if ((e = cudaMalloc(&ord.order, cap_order * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tile order");
        if ((e = cudaMalloc(&ord.bucket, cap_order * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tile order");
    }
    if (!ord.hist && (e = cudaMalloc(&ord.hist, 2 * kOrderBuckets * sizeof(uint32_t))) != cudaSuccess)
        return cuda_fail(e, "tile order");
    if (w_tiles_s[kP2GAutoBig].total > cap_order_big) {
        if (ord_big.order) cudaFree(ord_big.order);
        if (ord_big.bucket) cudaFree(ord_big.bucket);
        ord_big.order = ord_big.bucket = nullptr;
        cap_order_big = std::max<size_t>(w_tiles_s[kP2GAutoBig].total, 2 * cap_order_big);
        if ((e = cudaMalloc(&ord_big.order, cap_order_big * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tile order");
        if ((e = cudaMalloc(&ord_big.bucket, cap_order_big * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tile order");
    }
    if (!ord_big.hist && (e = cudaMalloc(&ord_big.hist, 2 * kOrderBuckets * sizeof(uint32_t))) != cudaSuccess)
        return cuda_fail(e, "tile order");
    {
        uint64_t np_all = 0;
        for (pxf_sim* sm : sims) np_all += sm->dev.np;
        const char* fv = std::getenv("PXF_P2G_FAIR");   // threshold override (tests)
        const uint64_t f = fv ? std::strtoull(fv, nullptr, 10) : np_all / std::max<uint32_t>(p2g_slots(kP2GAutoBig), 1u);
        fair = uint32_t(std::min<uint64_t>(f, 0xffffffffull));
        // Below 65536 particles per slot the pick chooses the small tiles as soon as FLIP packs a
        // tile to 32 particles per cell, and both shapes run about equally before that: the
        // small tiles are used without a per-substep pick.
        pick_dynamic = fv != nullptr || fair >= 65536u;
    }
    pw.sims = d_sims;
    pw.n_sims = n;
    pw.chunks = w_lchunks;
    pw.chunks_all = w_lchunks;
    // simulation of every item of every stage (one load instead of a search), for several simulations
    {
        size_t total = 0;
        std::vector<StageWork*> all(ws, ws + kStages);
        for (int v = 0; v < kNumP2GShapes; v++) all.push_back(&w_tiles_s[v]);
        for (StageWork* w : all) total += w->total;
        std::vector<uint16_t> sim_of;
        if (n > 1) {
            sim_of.resize(total);
            size_t off = 0;
            for (StageWork* w : all) {
                const uint32_t* b = (w >= &w_tiles_s[0] && w < &w_tiles_s[0] + kMaxP2GShapes)
                                        ? tbase.data() + (w - &w_tiles_s[0]) * (n + 1)
                                        : base.data() + (std::find(ws, ws + kStages, w) - ws) * (n + 1);
                for (int i = 0; i < n; i++)
                    for (uint32_t it = b[i]; it < b[i + 1]; it++) sim_of[off + it] = uint16_t(i);
                off += w->total;
            }
        }
        if (sim_of.size() > cap_sim_of) {
            if (d_sim_of) cudaFree(d_sim_of);
            d_sim_of = nullptr;
            cap_sim_of = std::max(sim_of.size(), 2 * cap_sim_of);
            if ((e = cudaMalloc(&d_sim_of, cap_sim_of * sizeof(uint16_t))) != cudaSuccess) return cuda_fail(e, "item table");
        }
        if (!sim_of.empty() &&
            (e = cudaMemcpyAsync(d_sim_of, sim_of.data(), sim_of.size() * 2, cudaMemcpyHostToDevice, stream)) != cudaSuccess)
            return cuda_fail(e, "item table upload");
        size_t off = 0;
        for (StageWork* w : all) {
            w->sim_of = n > 1 ? d_sim_of + off : nullptr;
            off += w->total;
        }
        pw.chunks.sim_of = pw.chunks_all.sim_of = w_lchunks.sim_of;
        if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_fail(e, "item table upload");
    }
    // compacted item lists of the CG loop's stages (batches; PXF_CG_COMPACT=1 / 0 forces them on / off)
    static const int compact_env = [] {
        const char* v = std::getenv("PXF_CG_COMPACT");
        return v ? (v[0] == '1' ? 1 : 0) : -1;
    }();
    const bool compact = compact_env < 0 ? n > 1 : compact_env == 1;
    pw.act_n = nullptr;
    if (any_pcg && compact) {
        size_t need = pw.chunks.total;
        for (int l = 0; l < kMaxLevels; l++) need += pw.level[l].total + pw.coarse[l].total;
        if (need > cap_act) {
            if (d_act) cudaFree(d_act);
            d_act = nullptr;
            cap_act = std::max(need, 2 * cap_act);
            if ((e = cudaMalloc(&d_act, cap_act * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "work lists");
        }
        if (!d_act_n && (e = cudaMalloc(&d_act_n, kActCounters * sizeof(uint32_t))) != cudaSuccess)
            return cuda_fail(e, "work lists");
        size_t off = 0;
        pw.act_n = d_act_n;
        pw.chunks.act = d_act + off;
        pw.chunks.act_n = d_act_n;
        off += pw.chunks.total;
        for (int l = 0; l < kMaxLevels; l++) {
            pw.level[l].act = d_act + off;
            pw.level[l].act_n = d_act_n + 1 + l;
            off += pw.level[l].total;
            pw.coarse[l].act = d_act + off;
            pw.coarse[l].act_n = d_act_n + 1 + kMaxLevels + l;
            off += pw.coarse[l].total;
        }
    }
    if (pw.any_mg && (e = mg_tail_attr(pw.tail_smem)) != cudaSuccess) return cuda_fail(e, "tail kernel attribute");
    gs_stream = any_gs && gs_stream_for(max_gs_cells);
    if (gs_stream && (e = gs_stream_attr()) != cudaSuccess) return cuda_fail(e, "streamed GS attribute");
    gs_res = false;
    if (any_gs && !gs_stream && gs_resident_for(max_gs_cells) && plan_gs_resident(host, res_plan, res_smem)) {
        const size_t nb = res_plan.size();
        const size_t plan_bytes = align256(nb * sizeof(GsResBlock));
        const size_t flag_bytes = align256(nb * kGsResFlagStride * sizeof(uint32_t));
        const size_t need = plan_bytes + flag_bytes + 256;
        if (need > cap_res) {
            if (d_res) cudaFree(d_res);
            d_res = nullptr;
            cap_res = need;
            if ((e = cudaMalloc(&d_res, cap_res)) != cudaSuccess) return cuda_fail(e, "red-black solve plan");
        }
        d_res_plan = static_cast<GsResBlock*>(d_res);
        d_res_flags = reinterpret_cast<uint32_t*>(static_cast<char*>(d_res) + plan_bytes);
        d_res_err = reinterpret_cast<uint32_t*>(static_cast<char*>(d_res) + plan_bytes + flag_bytes);
        if ((e = cudaMemcpy(d_res_plan, res_plan.data(), nb * sizeof(GsResBlock), cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemset(d_res_err, 0, sizeof(uint32_t))) != cudaSuccess)
            return cuda_fail(e, "red-black solve plan");
        gs_res_knobs(res_limit, res_skip);
        gs_res = true;
    }
    if (any_pcg && !d_bar) {
        // [0]: the persistent solve's barrier, [1]: the cooperative smoothing kernels'
        if ((e = cudaMalloc(&d_bar, 2 * sizeof(GridBar))) != cudaSuccess) return cuda_fail(e, "grid barrier");
        if ((e = cudaMemset(d_bar, 0, 2 * sizeof(GridBar))) != cudaSuccess) return cuda_fail(e, "grid barrier");
    }
    pw.sweep_bar = (pw.any_mg && d_bar) ? d_bar + 1 : nullptr;
    if (any_pcg && !d_tickets) {
        if ((e = cudaMalloc(&d_tickets, 2 * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tickets");
        if ((e = cudaMemset(d_tickets, 0, 2 * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(e, "tickets");
    }
    pw.tickets = any_pcg ? d_tickets : nullptr;
    if (any_pcg) persist_grid = pcg_solve_grid(pw.tail_smem);
    trace("rebuild: indexes uploaded, capturing");
    int rc = capture();
    trace("rebuild: capture rc=%d", rc);
    if (rc) return rc;
    dirty = false;
    return PXF_OK;
}

int BatchImpl::record_gs_part(cudaStream_t st) {
    const int n = int(sims.size());
    cudaError_t e;
    if ((e = launch_scan(w_chunks, d_sims, n, st)) != cudaSuccess) return cuda_fail(e, "scan");
    if ((e = launch_scatter(w_parts, st)) != cudaSuccess) return cuda_fail(e, "scatter");
    if (int rc = record_p2g(st)) return rc;
    if ((e = launch_divergence(w_cells, st)) != cudaSuccess) return cuda_fail(e, "divergence");
    if (any_gs && (e = record_gs(st)) != cudaSuccess) return cuda_fail(e, "pressure");
    return PXF_OK;
}

// The reference red-black GS: on large grids streamed through shared memory, kGsIters
// iterations per pass (pressure_stream.cu); otherwise 2 x iterations launches over the level-0
// system-cell lists (built once per substep), or, with PXF_GS_DENSE=1, over every cell of one colour.
cudaError_t BatchImpl::record_gs(cudaStream_t st) {
    static const bool dense = [] { const char* v = std::getenv("PXF_GS_DENSE"); return v && v[0] == '1'; }();
    cudaError_t e = cudaSuccess;
    if (gs_stream && !dense) return launch_gs_stream(w_gsu, max_gs_iters, st);
    if (gs_res && !dense)
        return launch_gs_resident(d_sims, d_res_plan, int(res_plan.size()), d_res_flags, d_res_err, res_smem, res_limit,
                                  res_skip, st);
    if (!dense && (e = launch_gs_lists(w_lchunks, st)) != cudaSuccess) return e;
    for (uint32_t it = 0; it < max_gs_iters; it++)
        for (uint32_t parity = 0; parity < 2; parity++) {
            e = dense ? launch_pressure_rb(w_half, parity, it, st) : launch_pressure_rb_list(w_lchunks, parity, it, st);
            if (e != cudaSuccess) return e;
        }
    return e;
}

int BatchImpl::record_post_solve(cudaStream_t st) {
    cudaError_t e;
    if ((e = launch_project(w_cells, st)) != cudaSuccess) return cuda_fail(e, "project");
    if ((e = launch_g2p(w_parts, st)) != cudaSuccess) return cuda_fail(e, "g2p");
    return PXF_OK;
}

// Work split inside a P2G block (lane-mapping bit 1): whole x-rows per warp (the picked large
// tiles: uniformly dense states) or equal slices of the tile's concatenated rows (default);
// PXF_P2G_ROWS=0/1 (read per recording) forces one.
static int p2g_rows(bool dflt) {
    const char* v = std::getenv("PXF_P2G_ROWS");
    const bool rows = v ? v[0] == '1' : dflt;
    return rows ? 2 : 0;
}

// PXF_P2G_ORDER=0 (read per recording) processes the tiles in index order.
cudaError_t BatchImpl::p2g(int shape, int lanes, cudaStream_t st) {
    const char* v = std::getenv("PXF_P2G_ORDER");
    const bool ordered = !(v && v[0] == '0');
    cudaError_t e;
    if (ordered && (e = launch_tile_order(w_tiles_s[shape], shape, ord, st)) != cudaSuccess) return e;
    return launch_p2g(w_tiles_s[shape], shape, lanes | p2g_rows(false), ordered ? ord.order : nullptr, st);
}

// The automatic pick as one IF/ELSE node (condition set by k_p2g_pick): the 32x8x8 P2G, else
// the 32x4x4 P2G; both bodies captured on the side stream.
cudaError_t BatchImpl::capture_if(cudaStream_t st, cudaGraphConditionalHandle h) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
    alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)];
    std::memset(np_raw, 0, sizeof(np_raw));
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_raw);
    cudaGraphNode_t node;
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 2;   // [0]: condition set, [1]: else
        e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    for (int branch = 0; branch < 2 && e == cudaSuccess; branch++) {
        cudaGraph_t body = np.conditional.phGraph_out[branch];
        e = cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e1 = p2g_branch(branch == 0 ? kP2GAutoBig : kP2GAutoSmall, side);
            cudaGraph_t out = body;
            cudaError_t e2 = cudaStreamEndCapture(side, &out);
            e = e1 != cudaSuccess ? e1 : e2;
        }
    }
    return e;
}

// P2G of one shape of the automatic pick: placement of its tiles (buckets from the pair pass),
// then the P2G in that heaviest-first order.
cudaError_t BatchImpl::p2g_branch(int shape, cudaStream_t st) {
    const TileOrder& o = shape == kP2GAutoBig ? ord_big : ord;
    cudaError_t e = launch_tile_place(w_tiles_s[shape], o, st);
    return e != cudaSuccess ? e : launch_p2g(w_tiles_s[shape], shape, p2g_lanes | p2g_rows(shape == kP2GAutoBig), o.order, st);
}

// P2G of one substep. With the automatic shape: the buckets of both shapes, then the pick —
// inside a capture an IF/ELSE node whose condition k_p2g_pick sets, eagerly a read-back of the
// buckets (captures without conditional nodes use the small tiles).
int BatchImpl::record_p2g(cudaStream_t st) {
    cudaError_t e;
    if (!auto_shape || !pick_dynamic) {
        if ((e = p2g(tile_shape, p2g_lanes, st)) != cudaSuccess) return cuda_fail(e, "p2g");
        return PXF_OK;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(st, &cs)) != cudaSuccess) return cuda_fail(e, "p2g");
    const bool capturing = cs == cudaStreamCaptureStatusActive;
    static const bool no_cond = [] { const char* v = std::getenv("PXF_NO_COND_GRAPH"); return v && v[0] == '1'; }();
    if ((e = launch_tile_weigh_pair(w_tiles_s[kP2GAutoBig], w_tiles_s[kP2GAutoSmall], ord_big, ord, st)) != cudaSuccess)
        return cuda_fail(e, "tile weigh");
    if (capturing && (!p2g_if_ok || no_cond || !cond_ok)) {
        if ((e = p2g_branch(kP2GAutoSmall, st)) != cudaSuccess) return cuda_fail(e, "p2g");
        return PXF_OK;
    }
    if (capturing) {
        cudaGraph_t cg = nullptr;
        cudaGraphConditionalHandle h = 0;
        e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 0, 0);
        if (e == cudaSuccess) e = launch_p2g_pick(ord_big.hist, fair, h, st);
        if (e == cudaSuccess) e = capture_if(st, h);
        if (e != cudaSuccess) {
            p2g_if_ok = false;    // the capture fails; the next one uses the small tiles throughout
            return cuda_fail(e, "p2g pick");
        }
        return PXF_OK;
    }
    uint32_t hist[2 * kOrderBuckets];
    if ((e = cudaMemcpyAsync(hist, ord_big.hist, sizeof(hist), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(e, "tile weigh");
    if (int rc = wait()) return rc;
    if ((e = p2g_branch(p2g_pick_small(hist, fair) ? kP2GAutoSmall : kP2GAutoBig, st)) != cudaSuccess)
        return cuda_fail(e, "p2g");
    return PXF_OK;
}

int BatchImpl::record_pre(cudaStream_t st) {
    const int n = int(sims.size());
    cudaError_t e;
    if ((e = launch_scan(w_chunks, d_sims, n, st)) != cudaSuccess) return cuda_fail(e, "scan");
    if ((e = launch_scatter(w_parts, st)) != cudaSuccess) return cuda_fail(e, "scatter");
    if (int rc = record_p2g(st)) return rc;
    if ((e = launch_divergence(w_cells, st)) != cudaSuccess) return cuda_fail(e, "divergence");
    if (any_gs && (e = record_gs(st)) != cudaSuccess) return cuda_fail(e, "pressure");
    if (any_pcg && (e = launch_pcg_init(pw, st)) != cudaSuccess) return cuda_fail(e, "pcg init");
    return PXF_OK;
}

int BatchImpl::record_post(cudaStream_t st) {
    cudaError_t e;
    if (any_pcg && (e = launch_pcg_finish(pw, st)) != cudaSuccess) return cuda_fail(e, "pcg finish");
    if ((e = launch_project(w_cells, st)) != cudaSuccess) return cuda_fail(e, "project");
    if ((e = launch_g2p(w_parts, st)) != cudaSuccess) return cuda_fail(e, "g2p");
    return PXF_OK;
}

// Inside the captured while body: `if (any simulation needs an FP64 restart) { restart kernels }`
// as a nested IF node; plain (self-skipping) launches when nesting is unavailable.
// The restart kernels as an IF node whose condition the control kernel after the update set
// (handle h, created on the body graph before that kernel).
cudaError_t BatchImpl::capture_restart(cudaStream_t st, cudaGraphConditionalHandle h) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
    alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)];
    std::memset(np_raw, 0, sizeof(np_raw));
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_raw);
    cudaGraphNode_t node;
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(side2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e1 = launch_pcg_restart(pw, side2);
            cudaGraph_t out = body;
            cudaError_t e2 = cudaStreamEndCapture(side2, &out);
            e = e1 != cudaSuccess ? e1 : e2;
        }
    }
    if (e != cudaSuccess) if_ok = false;
    return e;
}

static cudaError_t end_capture_to_exec(cudaStream_t st, cudaGraphExec_t* exec) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return e;
}

int BatchImpl::capture() {
    const int n = int(sims.size());
    cudaError_t e;
    // The precision loop is a graph of kernels (a conditional WHILE node around one CG iteration);
    // PXF_PCG_PERSISTENT=1, read at each capture, selects the persistent cooperative solve instead
    // (one launch, grid barriers between phases; slower on one large simulation).
    const char* persist_env = std::getenv("PXF_PCG_PERSISTENT");
    const bool want_persist = persist_env && persist_env[0] == '1';
    const bool had_p2g_if = p2g_if_ok;
    if (any_pcg && persist_ok && want_persist && persist_grid > 0) {
        if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cuda_fail(e, "begin capture");
        int rc = record_gs_part(stream);
        cudaError_t el = rc ? cudaSuccess : launch_pcg_solve(pw, d_bar, persist_grid, persist_guard, stream);
        if (!rc && el == cudaSuccess) rc = record_post_solve(stream);
        cudaGraphExec_t ex = nullptr;
        e = end_capture_to_exec(stream, &ex);
        if (!rc && el == cudaSuccess && e == cudaSuccess) {
            exec = ex;
            persistent = true;
            return PXF_OK;
        }
        if (ex) cudaGraphExecDestroy(ex);
        cudaGetLastError();
        if (rc && had_p2g_if && !p2g_if_ok) return capture();   // once more without the P2G IF/ELSE node
        if (rc) return rc;
        persist_ok = false;   // fall back to the graph-of-kernels loop
    }
    persistent = false;
    // PXF_NO_COND_GRAPH=1 selects the host-driven precision loop (its graphs have no conditional
    // node, which is what kernel profilers need to attribute the loop's kernels).
    static const bool no_cond = [] { const char* v = std::getenv("PXF_NO_COND_GRAPH"); return v && v[0] == '1'; }();
    if (no_cond) cond_ok = false;
    if (!any_pcg || cond_ok) {
        if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return cuda_fail(e, "begin capture");
        int rc = record_pre(stream);
        bool cond_failed = false;
        if (!rc && any_pcg) {
            // while (any simulation still solving) { body }
            cudaStreamCaptureStatus cs;
            cudaGraph_t cg = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            cudaGraphConditionalHandle h;
            // cudaGraphNodeParams holds a union without a default constructor: zeroed raw storage.
            alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)];
            std::memset(np_raw, 0, sizeof(np_raw));
            cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_raw);
            cudaGraphNode_t cn;
            e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, &cg, &deps, nullptr, &nd);
            if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault);
            if (e == cudaSuccess) e = launch_pcg_cond(d_sims, n, h, stream);
            if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, &cg, &deps, nullptr, &nd);
            if (e == cudaSuccess) {
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = h;
                np.conditional.type = cudaGraphCondTypeWhile;
                np.conditional.size = 1;
                e = cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &np);
            }
            if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(stream, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
            if (e == cudaSuccess) {
                cudaGraph_t body = np.conditional.phGraph_out[0];
                e = cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) {
                    // body: direction, update (its control kernel sets the restart IF), the restart
                    // IF node, the preconditioner (its control kernel sets the loop condition)
                    cudaError_t e1 = launch_pcg_dir(pw, side);
                    cudaGraphConditionalHandle hif = 0;
                    if (e1 == cudaSuccess && if_ok) {
                        cudaStreamCaptureStatus bs;
                        cudaGraph_t bg = nullptr;
                        e1 = cudaStreamGetCaptureInfo(side, &bs, nullptr, &bg, nullptr, nullptr, nullptr);
                        if (e1 == cudaSuccess) e1 = cudaGraphConditionalHandleCreate(&hif, bg, 0, cudaGraphCondAssignDefault);
                        if (e1 != cudaSuccess) if_ok = false;
                    }
                    if (e1 == cudaSuccess) e1 = if_ok ? launch_pcg_update(pw, side, hif, d_tickets) : launch_pcg_update(pw, side);
                    if (e1 == cudaSuccess) e1 = if_ok ? capture_restart(side, hif) : launch_pcg_restart(pw, side);
                    if (e1 == cudaSuccess) e1 = launch_precond(pw, side, h, d_tickets + 1);
                    cudaGraph_t out = body;
                    cudaError_t e3 = cudaStreamEndCapture(side, &out);
                    e = e1 != cudaSuccess ? e1 : e3;
                }
            }
            if (e != cudaSuccess) cond_failed = true;
        }
        if (!rc && !cond_failed) rc = record_post(stream);
        cudaGraphExec_t ex = nullptr;
        e = end_capture_to_exec(stream, &ex);
        if (!rc && !cond_failed && e == cudaSuccess) {
            exec = ex;
            return PXF_OK;
        }
        if (ex) cudaGraphExecDestroy(ex);
        cudaGetLastError();
        if (rc && had_p2g_if && !p2g_if_ok) return capture();   // once more without the P2G IF/ELSE node
        if (rc) return rc;
        if (!if_ok && !retried_plain_if) {
            retried_plain_if = true;
            return capture();   // once more with the restart kernels as plain launches
        }
        if (!cond_failed && e != cudaSuccess) return cuda_fail(e, "graph instantiate");
        cond_ok = false;   // fall through to the host-driven precision loop
    }
    // Host-driven precision loop: pre graph, body graph (8 steps + flag), post graph.
    if (!d_flag) {
        if ((e = cudaMalloc(&d_flag, 4)) != cudaSuccess) return cuda_fail(e, "flag");
        if ((e = cudaMallocHost(&h_flag, 4)) != cudaSuccess) return cuda_fail(e, "flag");
    }
    if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_fail(e, "capture");
    int rc = record_pre(stream);
    if ((e = end_capture_to_exec(stream, &exec_pre)) != cudaSuccess && !rc) return cuda_fail(e, "graph pre");
    if (rc) return rc;
    if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_fail(e, "capture");
    for (int k = 0; k < 8; k++) launch_pcg_body(pw, stream);
    launch_pcg_any(d_sims, n, d_flag, stream);
    cudaMemcpyAsync(h_flag, d_flag, 4, cudaMemcpyDeviceToHost, stream);
    if ((e = end_capture_to_exec(stream, &exec_body)) != cudaSuccess) return cuda_fail(e, "graph body");
    if ((e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_fail(e, "capture");
    rc = record_post(stream);
    if ((e = end_capture_to_exec(stream, &exec_post)) != cudaSuccess && !rc) return cuda_fail(e, "graph post");
    return rc;
}

// Bounded wait on the batch stream.
int BatchImpl::wait() {
    if (!stream) return PXF_OK;
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "event");
    e = cudaEventRecord(ev, stream);
    if (e != cudaSuccess) { cudaEventDestroy(ev); return cuda_fail(e, "event record"); }
    const auto t0 = std::chrono::steady_clock::now();
    int spins = 0;
    while (true) {
        e = cudaEventQuery(ev);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) { cudaEventDestroy(ev); return cuda_fail(e, "device work failed"); }
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s) {
            cudaEventDestroy(ev);
            return fail(PXF_ETIMEDOUT, "device work did not finish within " + std::to_string(timeout_s) + " s");
        }
        if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(spins > 4096 ? 500 : 20));
    }
    cudaEventDestroy(ev);
    if (d_bar && (persistent || pw.sweep_bar)) {
        GridBar hb[2];
        e = cudaMemcpy(hb, d_bar, sizeof(hb), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "grid barrier state");
        if ((persistent && hb[0].err) || (pw.sweep_bar && hb[1].err))
            return fail(PXF_ETIMEDOUT, "the pressure solve stopped: a grid barrier wait timed out");
    }
    if (gs_res && d_res_err) {
        uint32_t he = 0;
        e = cudaMemcpy(&he, d_res_err, sizeof(he), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "red-black solve state");
        if (he) {
            cudaMemset(d_res_err, 0, sizeof(uint32_t));
            return fail(PXF_ETIMEDOUT, "the red-black pressure solve stopped: a wait for a neighbouring block timed out");
        }
    }
    return PXF_OK;
}

int BatchImpl::step(uint32_t nsteps) {
    if (sims.empty() || nsteps == 0) return PXF_OK;
    if (dirty) {
        int rc = rebuild();
        if (rc) return rc;
    }
    cudaError_t e;
    for (uint32_t k = 0; k < nsteps; k++) {
        if (exec) {
            if ((e = cudaGraphLaunch(exec, stream)) != cudaSuccess) return cuda_fail(e, "substep launch");
        } else {
            if ((e = cudaGraphLaunch(exec_pre, stream)) != cudaSuccess) return cuda_fail(e, "substep launch");
            for (uint32_t guard = 0; guard < 1u << 20; guard++) {
                if ((e = cudaGraphLaunch(exec_body, stream)) != cudaSuccess) return cuda_fail(e, "pcg launch");
                int rc = wait();
                if (rc) return rc;
                if (*h_flag == 0) break;
            }
            if ((e = cudaGraphLaunch(exec_post, stream)) != cudaSuccess) return cuda_fail(e, "substep launch");
        }
    }
    for (pxf_sim* s : sims) s->steps_done += nsteps;
    return PXF_OK;
}

// Records an event after every kernel the library launches on the simulation's stream, so each
// kernel's device time is the gap to the event before it.
struct KernelTimer : LaunchLog {
    cudaStream_t stream;
    std::vector<cudaEvent_t> evs;
    std::vector<std::pair<size_t, const char*>> spans;     // (index of the event ending the kernel, name)
    std::vector<std::pair<size_t, size_t>> segments;       // (first span of a segment, its start event)
    bool ok = true;
    explicit KernelTimer(cudaStream_t s) : stream(s) {}
    ~KernelTimer() {
        for (auto& e : evs) cudaEventDestroy(e);
    }
    size_t record() {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess || cudaEventRecord(e, stream) != cudaSuccess) ok = false;
        evs.push_back(e);
        return evs.size() - 1;
    }
    // Starts a segment: a hold kernel long enough for the host to queue the segment behind it.
    void segment(double hold_us) {
        launch_hold((long long)(hold_us * 2.1e3), stream);
        segments.push_back({spans.size(), record()});
    }
    void launched(const char* kernel, cudaStream_t st) override {
        if (st != stream) return;
        const size_t e = record();
        spans.push_back({e, kernel});
    }
    // Event that starts span i: the segment start for a segment's first kernel, else the end of
    // the kernel before it.
    size_t start_of(size_t i) const {
        size_t from = 0;
        for (const auto& sg : segments)
            if (sg.first <= i) from = sg.first == i ? sg.second : spans[i - 1].first;
        return from;
    }
};

// One substep launched eagerly (no graph). With a timer: a hold kernel starts each segment the
// host queues in one go. With `tune`: after the counting sort every P2G variant (tile shape x
// lane mapping) runs three times with events around it; the fastest of the last two runs becomes
// the batch's choice. Every variant writes the same bits, so the substep's result is unchanged.
int BatchImpl::run_eager(KernelTimer* timer, pxf_tune_result* tune) {
    if (dirty) {
        int rc = rebuild();
        if (rc) return rc;
    }
    const int n = int(sims.size());
    cudaError_t e;
    if (timer) timer->segment(1000.0 + 40.0 * (any_gs ? max_gs_iters : 0));
    if ((e = launch_scan(w_chunks, d_sims, n, stream)) != cudaSuccess) return cuda_fail(e, "scan");
    if ((e = launch_scatter(w_parts, stream)) != cudaSuccess) return cuda_fail(e, "scatter");
    if (tune) {
        const int nv = kNumP2GShapes * 2;
        std::vector<cudaEvent_t> evs(2 * nv * 3, nullptr);
        for (auto& x : evs)
            if ((e = cudaEventCreate(&x)) != cudaSuccess) return cuda_fail(e, "tune events");
        for (int rep = 0; rep < 3; rep++)
            for (int v = 0; v < nv; v++) {
                const int shape = v >> 1, lanes = v & 1;
                cudaEventRecord(evs[2 * (rep * nv + v)], stream);
                if ((e = p2g(shape, lanes, stream)) != cudaSuccess) return cuda_fail(e, "p2g");
                cudaEventRecord(evs[2 * (rep * nv + v) + 1], stream);
            }
        int rc = wait();
        if (rc) return rc;
        int best = 0;
        float best_ms = 0;
        std::memset(tune, 0, sizeof(*tune));
        tune->variants = uint32_t(nv);
        for (int v = 0; v < nv; v++) {
            float m = 1e30f;
            for (int rep = 1; rep < 3; rep++) {
                float t = 0;
                cudaEventElapsedTime(&t, evs[2 * (rep * nv + v)], evs[2 * (rep * nv + v) + 1]);
                m = std::min(m, t);
            }
            if (v < 16) tune->ms[v] = m;
            if (v == 0 || m < best_ms) { best = v; best_ms = m; }
        }
        for (auto& x : evs) cudaEventDestroy(x);
        tile_shape = best >> 1;
        p2g_lanes = best & 1;
        tuned = true;
        w_tiles = w_tiles_s[tile_shape];
        tune->tile_shape = tile_shape;
        tune->lanes = p2g_lanes;
        int sh[3];
        p2g_shape(tile_shape, sh);
        std::snprintf(tune->chosen, sizeof(tune->chosen), "p2g %dx%dx%d %s", sh[0], sh[1], sh[2],
                      p2g_lanes ? "strided" : "blocked");
        dirty = true;    // recapture: later substeps use the chosen variant
    } else if (int rc = record_p2g(stream)) {
        return rc;
    }
    if ((e = launch_divergence(w_cells, stream)) != cudaSuccess) return cuda_fail(e, "divergence");
    if (any_gs && (e = record_gs(stream)) != cudaSuccess) return cuda_fail(e, "pressure");
    if (any_pcg && persistent) {
        if ((e = launch_pcg_solve(pw, d_bar, persist_grid, persist_guard, stream)) != cudaSuccess)
            return cuda_fail(e, "pcg solve");
    } else if (any_pcg) {
        if (!d_flag) {
            if ((e = cudaMalloc(&d_flag, 4)) != cudaSuccess) return cuda_fail(e, "flag");
            if ((e = cudaMallocHost(&h_flag, 4)) != cudaSuccess) return cuda_fail(e, "flag");
        }
        if ((e = launch_pcg_init(pw, stream)) != cudaSuccess) return cuda_fail(e, "pcg init");
        for (uint32_t guard = 0; guard < 100000; guard++) {
            if ((e = launch_pcg_any(d_sims, n, d_flag, stream)) != cudaSuccess) return cuda_fail(e, "pcg");
            cudaMemcpyAsync(h_flag, d_flag, 4, cudaMemcpyDeviceToHost, stream);
            int rc = wait();
            if (rc) return rc;
            if (*h_flag == 0) break;
            if (timer) timer->segment(1000.0);
            if ((e = launch_pcg_body(pw, stream)) != cudaSuccess) return cuda_fail(e, "pcg");
        }
        if (timer) timer->segment(200.0);
        if ((e = launch_pcg_finish(pw, stream)) != cudaSuccess) return cuda_fail(e, "pcg finish");
    }
    if ((e = launch_project(w_cells, stream)) != cudaSuccess) return cuda_fail(e, "project");
    if ((e = launch_g2p(w_parts, stream)) != cudaSuccess) return cuda_fail(e, "g2p");
    int rc = wait();
    if (rc) return rc;
    for (pxf_sim* sm : sims) sm->steps_done += 1;
    return PXF_OK;
}

// One substep launched kernel by kernel (eager, no graph) with an event after each kernel.
// Records are per kernel name, in order of first launch: launches and summed device time.
int BatchImpl::profile(pxf_stage_time* out, uint32_t cap, uint32_t* count) {
    KernelTimer timer(stream);
    struct Guard {
        LaunchLog* old;
        explicit Guard(LaunchLog* l) : old(g_launch_log) { g_launch_log = l; }
        ~Guard() { g_launch_log = old; }
    };
    {
        Guard g(&timer);
        int rc = run_eager(&timer, nullptr);
        if (rc) return rc;
    }
    if (!timer.ok) return fail(PXF_ECUDA, "profiler events");
    struct Rec { const char* name; uint32_t launches; double ms; };
    std::vector<Rec> recs;
    for (size_t i = 0; i < timer.spans.size(); i++) {
        float ms = 0;
        cudaEventElapsedTime(&ms, timer.evs[timer.start_of(i)], timer.evs[timer.spans[i].first]);
        const char* name = timer.spans[i].second;
        int k = -1;
        for (size_t j = 0; j < recs.size(); j++) if (std::strcmp(recs[j].name, name) == 0) k = int(j);
        if (k < 0) { recs.push_back({name, 0, 0.0}); k = int(recs.size() - 1); }
        recs[k].launches++;
        recs[k].ms += ms;
    }
    *count = uint32_t(recs.size());
    for (uint32_t i = 0; i < cap && i < recs.size(); i++) {
        std::snprintf(out[i].name, sizeof(out[i].name), "%s", recs[i].name);
        out[i].launches = recs[i].launches;
        out[i].ms = recs[i].ms;
    }
    return PXF_OK;
}

void set_global_error_message(const std::string& m) { g_last_error = m; }

static uint32_t chunk_env(const char* name, uint32_t dflt) {
    const char* v = std::getenv(name);
    const long k = v ? std::atol(v) : long(dflt);
    return (k >= 256 && k <= 8192 && k % 256 == 0) ? uint32_t(k) : dflt;
}

uint32_t coarse_chunk() {
    static const uint32_t cs = chunk_env("PXF_COARSE_CHUNK", 1024);
    return cs;
}

// z planes of a streamed-GS unit (PXF_GS_ZS overrides: 8 .. 4096): 40, 16 on grids of at most 128
// planes. On the 512 x 256 x 256 dam break (one block per SM, units of 56 x 24 cells times a
// segment) 40 planes measured 14.9 ms per substep over the first 20 timed substeps and 16.0 over
// 100, against 15.3 / 16.1 for 48, 16.8 for 64 and 14.8 / 16.7 for 80.
uint32_t gs_segment_planes(uint32_t nz) {
    static const uint32_t fixed = [] {
        const char* v = std::getenv("PXF_GS_ZS");
        const long k = v ? std::atol(v) : 0;
        return (k >= 8 && k <= 4096) ? uint32_t(k) : 0u;
    }();
    if (fixed) return fixed;
    return nz <= 128 ? 16u : 40u;
}

// The streamed red-black GS for batches whose largest red-black grid has at least 2^24 cells;
// below that the list sweeps, whose working set stays in L2, are faster. PXF_GS_STREAM=0/1
// (read at every batch rebuild) forces either.
bool gs_stream_for(uint64_t cells) {
    const char* v = std::getenv("PXF_GS_STREAM");
    if (v && (v[0] == '0' || v[0] == '1')) return v[0] == '1';
    return cells >= (uint64_t(1) << 24);
}

// The red-black GS below the streamed threshold as one cooperative launch (pressure_resident.cu)
// for batches whose largest red-black grid has at least 2^21 cells, where it fits: 1.66 against
// 1.81 ms per substep at 256x128x128, but 0.41 against 0.35 ms at 64x32x32, where one launch per
// colour costs less than the block-to-block waits. PXF_GS_RESIDENT=0/1 (read at every batch
// rebuild) forces either.
bool gs_resident_for(uint64_t cells) {
    const char* v = std::getenv("PXF_GS_RESIDENT");
    if (v && (v[0] == '0' || v[0] == '1')) return v[0] == '1';
    return cells >= (uint64_t(1) << 21);
}

// Failure-path test knobs of that launch, read at every batch rebuild: PXF_GS_RES_LIMIT_MS bounds
// each wait (default about 2 s), PXF_GS_RES_SKIP names a block that returns at once, so the blocks
// that wait for it run out of time, set the error word and return.
void gs_res_knobs(long long& limit_cycles, int& skip) {
    const char* l = std::getenv("PXF_GS_RES_LIMIT_MS");
    const double ms = l ? std::atof(l) : 0.0;
    limit_cycles = (ms > 0.0 && ms <= 10000.0) ? (long long)(ms * 2.1e6) : kBarrierCycles;
    const char* k = std::getenv("PXF_GS_RES_SKIP");
    skip = k ? std::atoi(k) : -1;
}

uint32_t level0_chunk() {
    static const uint32_t cs = chunk_env("PXF_L0_CHUNK", 5120);
    return cs;
}

// The red-black GS sweeps one colour per launch with one cell per thread: on grids up to 2^23
// cells smaller chunks (more blocks) pay (2.00 vs 2.08 ms per substep at 256x128x128 with 2048
// against 4096 cells), on larger ones larger chunks keep the sweeps' block count down (17.0, 17.5
// and 18.8 ms at 512x256x256 with 6144, 4096 and 2048 cells).
uint32_t level0_chunk_gs(uint64_t nc) {
    static const uint32_t fixed = chunk_env("PXF_GS_CHUNK", 0);
    if (fixed) return fixed;
    return nc <= (uint64_t(1) << 23) ? 2048u : 6144u;
}

bool trace_on() {
    static const bool on = [] { const char* v = std::getenv("PXF_TRACE"); return v && v[0] == '1'; }();
    return on;
}

void trace(const char* fmt, ...) {
    if (!trace_on()) return;
    va_list ap;
    va_start(ap, fmt);
    std::fprintf(stderr, "[pxf] ");
    std::vfprintf(stderr, fmt, ap);
    std::fprintf(stderr, "\n");
    std::fflush(stderr);
    va_end(ap);
}

int p2g_lanes_default() {
    const char* v = std::getenv("PXF_P2G_STRIDED");
    return v ? (std::atoi(v) ? 1 : 0) : 1;
}

// P2G tile shape: -1 (default) picks 32x8x8 or 32x4x4 every substep from the particle
// distribution (p2g_pick_small); PXF_P2G_TILE=<index> fixes one shape (read per recording).
int p2g_shape_index() {
    const char* env = std::getenv("PXF_P2G_TILE");
    if (!env) return -1;
    const int shape = std::atoi(env);
    return shape >= 0 && shape < kNumP2GShapes ? shape : -1;
}

}  // namespace pxf

// --------------------------------------------------------------------------------- helpers
namespace {

int ensure_device(std::string& err) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        err = std::string("no CUDA device available: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        cudaGetLastError();
        return PXF_ECUDA;
    }
    return PXF_OK;
}

int sim_bin(pxf_sim* s, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(s->dev.count, 0, size_t(s->dev.nc) * 4, st);
    if (e != cudaSuccess) return s->cuda_fail(e, "clear counts");
    // A private one-simulation work index for the binning launch.
    StageWork w;
    w.sims = s->own->d_sims;
    w.base = s->own->d_base;   // stage 0 (particles) of the private batch
    w.n_sims = 1;
    w.total = cdiv(s->dev.np, kElemItem);
    if ((e = launch_bin(w, st)) != cudaSuccess) return s->cuda_fail(e, "bin");
    return PXF_OK;
}

// Restores the initial particles (fluid.rs:271-275).
int sim_reset_particles(pxf_sim* s, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(s->dev.posA, s->pos0, 16ull * s->dev.np, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->dev.velA, s->vel0, 16ull * s->dev.np, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return s->cuda_fail(e, "reset particles");
    return sim_bin(s, st);
}

cudaStream_t sim_stream(pxf_sim* s) { return s->batch ? s->batch->stream : s->own->stream; }

// Waits for all work queued on the simulation's batch.
int sim_wait(pxf_sim* s) {
    BatchImpl* b = s->batch ? s->batch : s->own;
    int rc = b->wait();
    if (rc) return s->fail(rc, b->err);
    return PXF_OK;
}

int create_impl(const FluidCfg& cfg, uint32_t seed, double fps, const pxf_options* optsp, pxf_sim** out) {
    if (!out) return set_global_error(PXF_EINVAL, "out is NULL");
    *out = nullptr;
    pxf_options opts;
    if (optsp) opts = *optsp; else pxf_options_init(&opts);
    std::string msg;
    if (!validate_fluid(cfg, 0, opts.lift_grid_limits != 0, msg)) return set_global_error(PXF_EINVAL, msg);
    if (!(fps > 0.0)) return set_global_error(PXF_EINVAL, "render.fps must be > 0");
    if (opts.pressure_solver > PXF_PRESSURE_PCG) return set_global_error(PXF_EINVAL, "unknown pressure_solver");
    if (opts.pcg_precond > 1) return set_global_error(PXF_EINVAL, "unknown pcg_precond");
    if (ensure_device(msg)) return set_global_error(PXF_ECUDA, msg);

    std::unique_ptr<pxf_sim> s(new pxf_sim());
    s->cfg = cfg;
    s->opts = opts;
    s->seed = seed;
    s->fps = fps;
    fluid_grid(cfg.bounds, cfg.resolution, s->dims, s->h);
    const float origin[3] = {cfg.bounds[0][0], cfg.bounds[0][1], cfg.bounds[0][2]};
    if (!seed_plan(origin, s->h, s->dims, cfg.fill.data(), uint32_t(cfg.fill.size()), cfg.particles_per_cell, seed, s->plan))
        return set_global_error(PXF_EINVAL, "fluid '" + cfg.name + "': fill blocks are not representable");
    s->plan.sigma = opts.velocity_sigma;
    s->plan.vseed = opts.velocity_seed;
    if (s->plan.total == 0)   // fluid.rs:149
        return set_global_error(PXF_EINVAL, "fluid '" + cfg.name + "': fill blocks contain no grid cells");
    if (s->plan.total >= 0xffffffffull)
        return set_global_error(PXF_EINVAL, "fluid '" + cfg.name + "': too many particles");
    const uint32_t np = uint32_t(s->plan.total);
    const Layout L = layout_for(np, s->dims, opts);

    SimDev& d = s->dev;
    d.nx = int(s->dims[0]); d.ny = int(s->dims[1]); d.nz = int(s->dims[2]);
    d.np = np;
    d.h = s->h;
    s->dt = float(1.0 / (fps * double(cfg.substeps)));   // fluid.rs:164
    d.dt = s->dt;
    d.flip = cfg.flip;
    d.inv_h = 1.0f / s->h;                               // fluid.rs:166
    for (int a = 0; a < 3; a++) { d.o[a] = origin[a]; d.g[a] = cfg.gravity[a]; }
    d.nu = (s->dims[0] + 1) * s->dims[1] * s->dims[2];
    d.nv = s->dims[0] * (s->dims[1] + 1) * s->dims[2];
    d.nw = s->dims[0] * s->dims[1] * (s->dims[2] + 1);
    d.nf = d.nu + d.nv + d.nw;
    d.nc = s->dims[0] * s->dims[1] * s->dims[2];
    d.iterations = cfg.pressure_iterations;
    d.solver = opts.pressure_solver;
    d.rtol = opts.pcg_rtol;
    d.max_iter = opts.pcg_max_iter;
    d.restart = opts.pcg_restart ? opts.pcg_restart : 50;
    d.precond = opts.pcg_precond;
    d.coarse_iters = opts.mg_coarse_iters ? opts.mg_coarse_iters : 2;
    d.mg_pairs = opts.mg_smooth_pairs ? opts.mg_smooth_pairs : 2;

    cudaError_t e = cudaMalloc(&s->mem, L.total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_global_error(PXF_ENOMEM, "fluid '" + cfg.name + "': cannot allocate " + std::to_string(L.total) +
                                                " bytes of device memory: " + cudaGetErrorString(e));
    }
    s->mem_bytes = L.total;
    char* m = static_cast<char*>(s->mem);
    d.posA = reinterpret_cast<float4*>(m + L.posA);
    d.velA = reinterpret_cast<float4*>(m + L.velA);
    d.posB = reinterpret_cast<float4*>(m + L.posB);
    d.velB = reinterpret_cast<float4*>(m + L.velB);
    s->pos0 = reinterpret_cast<float4*>(m + L.pos0);
    s->vel0 = reinterpret_cast<float4*>(m + L.vel0);
    d.vel = reinterpret_cast<float*>(m + L.vel);
    d.vel_old = reinterpret_cast<float*>(m + L.vel_old);
    d.pressure = reinterpret_cast<float*>(m + L.pressure);
    d.div = reinterpret_cast<float*>(m + L.div);
    d.type = reinterpret_cast<uint8_t*>(m + L.type);
    d.count = reinterpret_cast<uint32_t*>(m + L.count);
    d.start = reinterpret_cast<uint32_t*>(m + L.start);
    d.chunk = reinterpret_cast<uint32_t*>(m + L.chunk);
    d.info = reinterpret_cast<uint16_t*>(m + L.info);
    d.acc = opts.keep_p2g_sums ? reinterpret_cast<int32_t*>(m + L.acc) : nullptr;
    d.wacc = opts.keep_p2g_sums ? reinterpret_cast<int32_t*>(m + L.wacc) : nullptr;
    d.lev[0].nx = d.nx; d.lev[0].ny = d.ny; d.lev[0].nz = d.nz;
    d.lev[0].nc = d.nc;
    d.lev[0].type = d.type;
    d.lev[0].info = d.info;
    d.lev[0].cs = opts.pressure_solver == PXF_PRESSURE_PCG ? level0_chunk() : level0_chunk_gs(d.nc);
    d.lev[0].list = reinterpret_cast<uint32_t*>(m + L.llist[0]);
    d.lev[0].lcnt = reinterpret_cast<uint32_t*>(m + L.llcnt[0]);
    if (opts.pressure_solver != PXF_PRESSURE_PCG) {
        uint32_t g[4];
        gs_unit_grid(s->dims, g);
        d.p_alt = reinterpret_cast<float*>(m + L.p_alt);
        d.rhs = reinterpret_cast<float*>(m + L.rhs);
        d.gs_cnt = reinterpret_cast<uint8_t*>(m + L.gs_cnt);
        d.gs_flag = reinterpret_cast<uint32_t*>(m + L.gs_flag);
        d.gs_ntx = g[0];
        d.gs_nty = g[1];
        d.gs_nzs = g[2];
        d.gs_zs = g[3];
    }
    if (opts.pressure_solver == PXF_PRESSURE_PCG) {
        d.x2 = reinterpret_cast<float2*>(m + L.x2);
        d.x64 = reinterpret_cast<double*>(m + L.x64);
        d.r = reinterpret_cast<float*>(m + L.r);
        d.z = reinterpret_cast<float*>(m + L.z);
        d.p0 = reinterpret_cast<float*>(m + L.p0);
        d.p1 = reinterpret_cast<float*>(m + L.p1);
        d.Ap = reinterpret_cast<float*>(m + L.Ap);
        d.partial = reinterpret_cast<double*>(m + L.partial);
        d.pcg = reinterpret_cast<PcgState*>(m + L.pcg);
        d.nlev = L.nlev > 0 ? L.nlev : 1;
        d.tail = 0;
        while (d.tail + 1 < d.nlev && uint64_t(L.dims[d.tail][0]) * L.dims[d.tail][1] * L.dims[d.tail][2] > kTailCells) d.tail++;
        d.lev[0].r = d.r;
        d.lev[0].z = d.z;
        for (int l = 1; l < L.nlev; l++) {
            MgLevel& v = d.lev[l];
            v.nx = L.dims[l][0]; v.ny = L.dims[l][1]; v.nz = L.dims[l][2];
            v.nc = uint32_t(v.nx) * uint32_t(v.ny) * uint32_t(v.nz);
            v.type = reinterpret_cast<uint8_t*>(m + L.ltype[l]);
            v.info = reinterpret_cast<uint16_t*>(m + L.linfo[l]);
            v.r = reinterpret_cast<float*>(m + L.lr[l]);
            v.z = reinterpret_cast<float*>(m + L.lz[l]);
            v.cs = coarse_chunk();
            v.list = reinterpret_cast<uint32_t*>(m + L.llist[l]);
            v.lcnt = reinterpret_cast<uint32_t*>(m + L.llcnt[l]);
        }
    }

    s->own = new BatchImpl();
    s->own->owned_by_sim = true;
    s->own->sims.push_back(s.get());
    int rc = s->own->rebuild();
    if (rc) {
        std::string m2 = s->own->err;
        delete s->own;
        cudaFree(s->mem);
        return set_global_error(rc, m2);
    }
    cudaStream_t st = s->own->stream;
    // Grid buffers start at zero (the reference leaves them uninitialised, fluid.rs:204).
    e = cudaMemsetAsync(s->mem, 0, L.total, st);
    if (e == cudaSuccess) e = launch_seed(s->plan, d.posA, d.velA, s->pos0, s->vel0, st);
    if (e != cudaSuccess) {
        delete s->own;
        cudaFree(s->mem);
        return set_global_error(PXF_ECUDA, std::string("seeding: ") + cudaGetErrorString(e));
    }
    rc = sim_bin(s.get(), st);
    if (!rc) rc = sim_wait(s.get());
    if (rc) {
        std::string m2 = s->err;
        delete s->own;
        cudaFree(s->mem);
        return set_global_error(rc, m2);
    }
    *out = s.release();
    return PXF_OK;
}

}  // namespace

// --------------------------------------------------------------------------------- C ABI
extern "C" {

void pxf_fluid_desc_init(pxf_fluid_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    FluidCfg def;
    d->name = "";
    d->resolution = def.resolution;
    d->particles_per_cell = def.particles_per_cell;
    d->substeps = def.substeps;
    d->flip = def.flip;
    std::memcpy(d->gravity, def.gravity, sizeof(d->gravity));
    d->pressure_iterations = def.pressure_iterations;
    d->surface_refine = def.surface_refine;
    d->particle_radius = def.particle_radius;
    d->warmup = def.warmup;
    d->max_triangles = def.max_triangles;
}

void pxf_options_init(pxf_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->pressure_solver = PXF_PRESSURE_RBGS;
    o->pcg_rtol = 1e-6;
    o->pcg_max_iter = 2000;
    o->pcg_restart = 50;
    o->wait_timeout_s = 600.0;
    o->p2g_tile = -1;
    o->pcg_precond = 0;
    o->mg_coarse_iters = 2;
    o->mg_smooth_pairs = 2;
}

int pxf_validate(const pxf_fluid_desc* desc, uint32_t index, uint32_t lift, char* msg, size_t cap) {
    if (!desc) return PXF_EINVAL;
    FluidCfg f;
    f.from_desc(*desc);
    std::string m;
    const bool ok = validate_fluid(f, index, lift != 0, m);
    if (msg && cap) {
        std::snprintf(msg, cap, "%s", m.c_str());
    }
    return ok ? PXF_OK : PXF_EINVAL;
}

int pxf_fluid_grid(const pxf_fluid_desc* desc, uint32_t dims[3], float* h) {
    if (!desc || !dims || !h) return PXF_EINVAL;
    fluid_grid(desc->bounds, desc->resolution, dims, *h);
    return PXF_OK;
}

uint64_t pxf_steps_for_frame(double warmup, double fps, uint32_t substeps, double frame) {
    double v = std::round((warmup + frame / fps) * fps * double(substeps));
    if (!(v > 0.0)) return 0;   // .max(0.0); NaN saturates to 0 in `as u64`
    return v >= 18446744073709551615.0 ? UINT64_MAX : uint64_t(v);
}

int pxf_create(const pxf_fluid_desc* desc, uint32_t seed, double fps, pxf_sim** out) {
    return pxf_create_ex(desc, seed, fps, nullptr, out);
}

int pxf_create_ex(const pxf_fluid_desc* desc, uint32_t seed, double fps, const pxf_options* opts, pxf_sim** out) {
    if (!desc) return set_global_error(PXF_EINVAL, "desc is NULL");
    FluidCfg f;
    f.from_desc(*desc);
    return create_impl(f, seed, fps, opts, out);
}

int pxf_create_from_json(const char* json, uint32_t index, pxf_sim** out) {
    return pxf_create_from_json_ex(json, index, nullptr, out);
}

int pxf_create_from_json_ex(const char* json, uint32_t index, const pxf_options* opts, pxf_sim** out) {
    SceneFluids sc;
    std::string msg;
    if (!parse_scene(json, sc, msg)) return set_global_error(PXF_EINVAL, msg);
    if (index >= sc.fluids.size())
        return set_global_error(PXF_ENOTFOUND, "scene has " + std::to_string(sc.fluids.size()) + " fluids, no index " +
                                                   std::to_string(index));
    // fps: render.fps as f32 widened to f64 (crates/pxl-render/src/lib.rs:223).
    return create_impl(sc.fluids[index], sc.seed, double(sc.fps), opts, out);
}

int pxf_scene_fluid_count(const char* json) {
    SceneFluids sc;
    std::string msg;
    if (!parse_scene(json, sc, msg)) return set_global_error(PXF_EINVAL, msg);
    return int(sc.fluids.size());
}

int pxf_advance_to_frame(pxf_sim* s, double frame) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (s->batch && s->batch != s->own) return s->fail(PXF_ESTATE, "simulation is stepped by a batch");
    const uint64_t target = pxf_steps_for_frame(double(s->cfg.warmup), s->fps, s->cfg.substeps, frame);
    if (!s->initialized || target < s->steps_done) {
        int rc = sim_reset_particles(s, s->own->stream);
        if (rc) return rc;
        s->steps_done = 0;
        s->initialized = true;
    }
    if (target > s->steps_done) {
        const uint64_t n = target - s->steps_done;
        for (uint64_t k = 0; k < n; k += 0x40000000ull) {
            int rc = s->own->step(uint32_t(std::min<uint64_t>(n - k, 0x40000000ull)));
            if (rc) return s->fail(rc, s->own->err);
        }
    }
    return sim_wait(s);
}

int pxf_step(pxf_sim* s, uint32_t n) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (s->batch && s->batch != s->own) return s->fail(PXF_ESTATE, "simulation is stepped by a batch");
    s->initialized = true;
    int rc = s->own->step(n);
    if (rc) return s->fail(rc, s->own->err);
    return PXF_OK;
}

int pxf_sync(pxf_sim* s) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    return sim_wait(s);
}

uint32_t pxf_particle_count(const pxf_sim* s) { return s ? s->dev.np : 0; }
uint64_t pxf_steps_done(const pxf_sim* s) { return s ? s->steps_done : 0; }
size_t pxf_device_bytes(const pxf_sim* s) { return s ? s->mem_bytes : 0; }

int pxf_grid_info(const pxf_sim* s, uint32_t dims[3], float* h, float* dt) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (dims) std::memcpy(dims, s->dims, sizeof(s->dims));
    if (h) *h = s->h;
    if (dt) *dt = s->dt;
    return PXF_OK;
}

int pxf_estimate_bytes(const pxf_fluid_desc* desc, const pxf_options* optsp, uint64_t* bytes) {
    if (!desc || !bytes) return set_global_error(PXF_EINVAL, "NULL argument");
    pxf_options opts;
    if (optsp) opts = *optsp; else pxf_options_init(&opts);
    FluidCfg f;
    f.from_desc(*desc);
    uint32_t n[3];
    float h;
    fluid_grid(f.bounds, f.resolution, n, h);
    SeedPlan plan;
    const float origin[3] = {f.bounds[0][0], f.bounds[0][1], f.bounds[0][2]};
    if (!seed_plan(origin, h, n, f.fill.data(), uint32_t(f.fill.size()), f.particles_per_cell, 0, plan))
        return set_global_error(PXF_EINVAL, "fill blocks are not representable");
    *bytes = layout_for(uint32_t(std::min<uint64_t>(plan.total, 0xffffffffull)), n, opts).total;
    return PXF_OK;
}

int pxf_read_particles(pxf_sim* s, float* out, size_t n) {
    if (!s || !out) return set_global_error(PXF_EINVAL, "NULL argument");
    if (n != s->dev.np) return s->fail(PXF_EINVAL, "particle count mismatch");
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaStream_t st = sim_stream(s);
    float4* staging = s->dev.posB;   // posB|velB: 32 B per particle, free between substeps
    cudaError_t e = launch_gather_aos(s->dev, staging, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, staging, 32ull * n, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return s->cuda_fail(e, "read particles");
    return sim_wait(s);
}

int pxf_write_particles(pxf_sim* s, const float* in, size_t n) {
    if (!s || !in) return set_global_error(PXF_EINVAL, "NULL argument");
    if (n != s->dev.np) return s->fail(PXF_EINVAL, "particle count mismatch");
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaStream_t st = sim_stream(s);
    float4* staging = s->dev.posB;
    cudaError_t e = cudaMemcpyAsync(staging, in, 32ull * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_scatter_aos(s->dev, staging, st);
    if (e != cudaSuccess) return s->cuda_fail(e, "write particles");
    rc = sim_bin(s, st);
    if (rc) return rc;
    s->initialized = true;
    return sim_wait(s);
}

int pxf_read_grid(pxf_sim* s, int which, void* out, size_t bytes) {
    if (!s || !out) return set_global_error(PXF_EINVAL, "NULL argument");
    const SimDev& d = s->dev;
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaStream_t st = sim_stream(s);
    cudaError_t e = cudaSuccess;
    auto need = [&](size_t b) { return bytes == b; };
    switch (which) {
        case PXF_GRID_VEL:
        case PXF_GRID_VEL_OLD:
            if (!need(4ull * d.nf)) return s->fail(PXF_EINVAL, "size mismatch");
            e = cudaMemcpyAsync(out, which == PXF_GRID_VEL ? d.vel : d.vel_old, bytes, cudaMemcpyDeviceToHost, st);
            break;
        case PXF_GRID_ACC:
        case PXF_GRID_WACC:
            if (!d.acc) return s->fail(PXF_ESTATE, "P2G sums are kept only with keep_p2g_sums");
            if (!need(4ull * d.nf)) return s->fail(PXF_EINVAL, "size mismatch");
            e = cudaMemcpyAsync(out, which == PXF_GRID_ACC ? d.acc : d.wacc, bytes, cudaMemcpyDeviceToHost, st);
            break;
        case PXF_GRID_CELL_COUNT: {
            if (!need(4ull * d.nc)) return s->fail(PXF_EINVAL, "size mismatch");
            uint32_t* tmp = nullptr;
            e = cudaMalloc(&tmp, bytes);
            if (e == cudaSuccess) e = launch_counts_from_start(d, tmp, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, bytes, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (tmp) cudaFree(tmp);
            break;
        }
        case PXF_GRID_CELL_TYPE: {
            if (!need(4ull * d.nc)) return s->fail(PXF_EINVAL, "size mismatch");
            std::vector<uint8_t> t(d.nc);
            e = cudaMemcpyAsync(t.data(), d.type, d.nc, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaSuccess) {
                uint32_t* o = static_cast<uint32_t*>(out);
                for (uint32_t i = 0; i < d.nc; i++) o[i] = t[i];
            }
            break;
        }
        case PXF_GRID_PRESSURE:
        case PXF_GRID_DIVERGENCE:
            if (!need(4ull * d.nc)) return s->fail(PXF_EINVAL, "size mismatch");
            e = cudaMemcpyAsync(out, which == PXF_GRID_PRESSURE ? d.pressure : d.div, bytes, cudaMemcpyDeviceToHost, st);
            break;
        case PXF_GRID_PRESSURE64:
            if (!d.x64) return s->fail(PXF_ESTATE, "FP64 pressure exists only with the precision solver");
            if (!need(8ull * d.nc)) return s->fail(PXF_EINVAL, "size mismatch");
            e = cudaMemcpyAsync(out, d.x64, bytes, cudaMemcpyDeviceToHost, st);
            break;
        case PXF_GRID_SURF_DENSITY:
        case PXF_GRID_SURF_PHI:
        case PXF_GRID_SURF_CELL_VERT: {
            if (!s->surf_mem) return s->fail(PXF_ESTATE, "no surface mesh has been made yet");
            const SurfDev& S = s->surf;
            const size_t nn = size_t(S.sx + 1) * (S.sy + 1) * (S.sz + 1), sc = size_t(S.sx) * S.sy * S.sz;
            const size_t want = 4 * (which == PXF_GRID_SURF_CELL_VERT ? sc : nn);
            if (!need(want)) return s->fail(PXF_EINVAL, "size mismatch");
            const void* src = which == PXF_GRID_SURF_DENSITY ? static_cast<const void*>(S.density)
                              : which == PXF_GRID_SURF_PHI  ? static_cast<const void*>(S.phi)
                                                            : static_cast<const void*>(S.cell_vert);
            e = cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToHost, st);
            break;
        }
        default:
            return s->fail(PXF_EINVAL, "unknown grid buffer");
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "read grid");
    return sim_wait(s);
}

// Surface grid and iso level as FluidState::new sets them (fluid.rs:150-156); powi(3) is x*x*x.
static SurfDev surface_params(const pxf_sim* s) {
    const FluidCfg& f = s->cfg;
    SurfDev S{};
    const uint32_t r = f.surface_refine;
    S.sx = s->dims[0] * r;
    S.sy = s->dims[1] * r;
    S.sz = s->dims[2] * r;
    S.sh = s->h / float(r);
    S.radius = f.particle_radius * S.sh;
    const float x = S.radius / s->h;
    const float kernel_volume = 0.638f * (x * x * x);
    S.iso = 0.5f * float(f.particles_per_cell) * kernel_volume;
    S.ox = s->dev.o[0];
    S.oy = s->dev.o[1];
    S.oz = s->dev.o[2];
    S.max_verts = f.max_triangles;
    S.max_tris = f.max_triangles;
    return S;
}

int pxf_surface_info(const pxf_sim* s, uint32_t dims[3], float* cell, float* radius, float* iso) {
    if (!s || !dims) return set_global_error(PXF_EINVAL, "NULL argument");
    const SurfDev S = surface_params(s);
    dims[0] = S.sx;
    dims[1] = S.sy;
    dims[2] = S.sz;
    if (cell) *cell = S.sh;
    if (radius) *radius = S.radius;
    if (iso) *iso = S.iso;
    return PXF_OK;
}

// The surface grid's working buffers and the library-owned mesh buffers (first meshing call).
static int surface_buffers(pxf_sim* s) {
    if (s->surf_mem) return PXF_OK;
    const FluidCfg& f = s->cfg;
    if (f.surface_refine == 0) return s->fail(PXF_EINVAL, "surface_refine must be at least 1");
    SurfDev S = surface_params(s);
    const uint64_t nn = uint64_t(S.sx + 1) * (S.sy + 1) * (S.sz + 1), sc = uint64_t(S.sx) * S.sy * S.sz;
    if (nn >= (1ull << 32)) return s->fail(PXF_EINVAL, "surface grid too large (2^32 nodes)");
    size_t off = 0;
    auto take = [&](size_t b) { const size_t o = off; off += align256(b); return o; };
    const size_t o_den = take(4 * nn), o_phi = take(4 * nn), o_cv = take(4 * sc);
    const size_t o_v = take(size_t(S.max_verts) * 32), o_i = take(size_t(S.max_tris) * 12);
    const size_t o_vc = take(4 * size_t(surface_chunks(sc))), o_qc = take(4 * size_t(surface_chunks(nn)));
    const size_t o_ct = take(16);
    void* mem = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&mem, off)) != cudaSuccess) {
        cudaGetLastError();
        return s->fail(PXF_ENOMEM, "surface buffers: " + std::to_string(off) + " bytes");
    }
    char* b = static_cast<char*>(mem);
    S.density = reinterpret_cast<int32_t*>(b + o_den);
    S.phi = reinterpret_cast<float*>(b + o_phi);
    S.cell_vert = reinterpret_cast<uint32_t*>(b + o_cv);
    S.verts = reinterpret_cast<float4*>(b + o_v);
    S.indices = reinterpret_cast<uint32_t*>(b + o_i);
    S.vchunk = reinterpret_cast<uint32_t*>(b + o_vc);
    S.qchunk = reinterpret_cast<uint32_t*>(b + o_qc);
    S.counters = reinterpret_cast<uint32_t*>(b + o_ct);
    s->surf_mem = mem;
    s->surf = S;
    return PXF_OK;
}

// Meshing with the given output view; the capped counts and the overflow flag as the reference
// reads them back (fluid.rs:321-327).
static int surface_run(pxf_sim* s, const SurfDev& S, uint32_t* vertices, uint32_t* triangles, int32_t* overflow,
                       double* device_ms) {
    cudaStream_t st = sim_stream(s);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    cudaError_t e = launch_surface(S, s->dev.posA, s->dev.np, st);
    cudaEventRecord(e1, st);
    if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return s->cuda_fail(e, "surface launch");
    }
    int rc = sim_wait(s);
    float ms = 0;
    if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    uint32_t cnt[2] = {0, 0};
    if ((e = cudaMemcpy(cnt, S.counters, 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return s->cuda_fail(e, "surface counters");
    const uint32_t mv = S.max_verts, mt = S.max_tris;
    if (vertices) *vertices = std::min(cnt[0], mv);
    if (triangles) *triangles = std::min(cnt[1], mt) / 2 * 2;
    if (overflow) *overflow = (cnt[0] > mv || cnt[1] > mt) ? 1 : 0;
    if (device_ms) *device_ms = ms;
    return PXF_OK;
}

int pxf_surface_mesh(pxf_sim* s, uint32_t* vertices, uint32_t* triangles, int32_t* overflow, double* device_ms) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    int rc = sim_wait(s);
    if (!rc) rc = surface_buffers(s);
    if (rc) return rc;
    uint32_t v = 0, t = 0;
    if ((rc = surface_run(s, s->surf, &v, &t, overflow, device_ms))) return rc;
    s->mesh_verts = v;
    s->mesh_tris = t;
    if (vertices) *vertices = v;
    if (triangles) *triangles = t;
    return PXF_OK;
}

int pxf_surface_mesh_into(pxf_sim* s, float* d_vertices, uint32_t vbase, uint32_t max_vertices, uint32_t* d_indices,
                          uint32_t ibase, uint32_t max_triangles, uint32_t* vertices, uint32_t* triangles,
                          int32_t* overflow, double* device_ms) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (!d_vertices || !d_indices) return s->fail(PXF_EINVAL, "NULL vertex or index buffer");
    int rc = sim_wait(s);
    if (!rc) rc = surface_buffers(s);
    if (rc) return rc;
    SurfDev S = s->surf;
    S.verts = reinterpret_cast<float4*>(d_vertices) + 2 * size_t(vbase);   // out_verts[(vbase + idx) * 2 + k]
    S.indices = d_indices + size_t(ibase);                                   // out_indices[ibase + t * 3 + k]
    if (max_vertices) S.max_verts = max_vertices;
    if (max_triangles) S.max_tris = max_triangles;
    return surface_run(s, S, vertices, triangles, overflow, device_ms);
}

int pxf_read_mesh(pxf_sim* s, float* vertices, size_t n_vertices, uint32_t* indices, size_t n_triangles) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (!s->surf_mem) return s->fail(PXF_ESTATE, "no surface mesh has been made yet");
    if (n_vertices != s->mesh_verts || n_triangles != s->mesh_tris)
        return s->fail(PXF_EINVAL, "counts differ from the last pxf_surface_mesh");
    if ((n_vertices && !vertices) || (n_triangles && !indices)) return s->fail(PXF_EINVAL, "NULL buffer");
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    if (n_vertices) e = cudaMemcpy(vertices, s->surf.verts, n_vertices * 32, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n_triangles) e = cudaMemcpy(indices, s->surf.indices, n_triangles * 12, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return s->cuda_fail(e, "read mesh");
    return PXF_OK;
}

int pxf_mesh_device_buffers(pxf_sim* s, const void** vertices, const void** indices) {
    if (!s || !vertices || !indices) return set_global_error(PXF_EINVAL, "NULL argument");
    if (!s->surf_mem) return s->fail(PXF_ESTATE, "no surface mesh has been made yet");
    *vertices = s->surf.verts;
    *indices = s->surf.indices;
    return PXF_OK;
}

int pxf_write_grid(pxf_sim* s, int which, const void* in, size_t bytes) {
    if (!s || !in) return set_global_error(PXF_EINVAL, "NULL argument");
    if (which != PXF_GRID_PRESSURE) return s->fail(PXF_EINVAL, "only the pressure warm start is writable");
    const SimDev& d = s->dev;
    if (bytes != 4ull * d.nc) return s->fail(PXF_EINVAL, "size mismatch");
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaStream_t st = sim_stream(s);
    cudaError_t e = cudaMemcpyAsync(d.pressure, in, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d.x64) {
        const float* p = static_cast<const float*>(in);
        std::vector<double> x(d.nc);
        std::vector<float2> x2(d.nc);
        for (uint32_t i = 0; i < d.nc; i++) {
            x[i] = double(p[i]);
            x2[i] = make_float2(p[i], 0.0f);
        }
        e = cudaMemcpyAsync(d.x64, x.data(), 8ull * d.nc, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d.x2, x2.data(), 8ull * d.nc, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "write grid");
    return sim_wait(s);
}

int pxf_solver_stats(pxf_sim* s, uint32_t* iters, double* relres, uint32_t* status) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (!s->dev.pcg) return s->fail(PXF_ESTATE, "the red-black solver keeps no statistics");
    int rc = sim_wait(s);
    if (rc) return rc;
    PcgState st;
    cudaError_t e = cudaMemcpy(&st, s->dev.pcg, sizeof(st), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return s->cuda_fail(e, "solver stats");
    if (iters) *iters = st.iters;
    if (relres) *relres = st.relres;
    if (status) *status = st.status;
    return PXF_OK;
}

int pxf_mg_level_info(pxf_sim* s, uint32_t* cells, uint32_t* system_cells, uint32_t cap, uint32_t* levels,
                      int32_t* tail) {
    if (!s || !levels || !tail) return set_global_error(PXF_EINVAL, "NULL argument");
    if (s->dev.solver != 1 || s->dev.precond != 0) return s->fail(PXF_ESTATE, "the simulation has no multigrid");
    int rc = sim_wait(s);
    if (rc) return rc;
    *levels = uint32_t(s->dev.nlev);
    *tail = s->dev.tail;
    for (int l = 0; l < s->dev.nlev && uint32_t(l) < cap; l++) {
        const MgLevel& L = s->dev.lev[l];
        if (cells) cells[l] = L.nc;
        if (system_cells) {
            const uint32_t nch = (L.nc + L.cs - 1) / L.cs;
            std::vector<uint32_t> cnt(2 * size_t(nch));
            cudaError_t e = cudaMemcpy(cnt.data(), L.lcnt, cnt.size() * 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return s->cuda_fail(e, "level lists");
            uint64_t t = 0;
            for (uint32_t v : cnt) t += v;
            system_cells[l] = uint32_t(t);
        }
    }
    return PXF_OK;
}

int pxf_snapshot_take(pxf_sim* s, pxf_snapshot** out) {
    if (!s || !out) return set_global_error(PXF_EINVAL, "NULL argument");
    int rc = sim_wait(s);
    if (rc) return rc;
    std::unique_ptr<pxf_snapshot> snap(new pxf_snapshot());
    const SimDev& d = s->dev;
    snap->np = d.np;
    snap->nc = d.nc;
    snap->pos.resize(d.np);
    snap->vel.resize(d.np);
    snap->pressure.resize(d.nc);
    cudaError_t e = cudaMemcpy(snap->pos.data(), d.posA, 16ull * d.np, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(snap->vel.data(), d.velA, 16ull * d.np, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(snap->pressure.data(), d.pressure, 4ull * d.nc, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && d.x64) {
        snap->x64.resize(d.nc);
        snap->x2.resize(d.nc);
        e = cudaMemcpy(snap->x64.data(), d.x64, 8ull * d.nc, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(snap->x2.data(), d.x2, 8ull * d.nc, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return s->cuda_fail(e, "snapshot");
    snap->steps_done = s->steps_done;
    snap->initialized = s->initialized;
    *out = snap.release();
    return PXF_OK;
}

int pxf_snapshot_restore(pxf_sim* s, const pxf_snapshot* snap) {
    if (!s || !snap) return set_global_error(PXF_EINVAL, "NULL argument");
    const SimDev& d = s->dev;
    if (snap->np != d.np || snap->nc != d.nc) return s->fail(PXF_EINVAL, "snapshot belongs to another simulation shape");
    int rc = sim_wait(s);
    if (rc) return rc;
    cudaStream_t st = sim_stream(s);
    cudaError_t e = cudaMemcpyAsync(d.posA, snap->pos.data(), 16ull * d.np, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.velA, snap->vel.data(), 16ull * d.np, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.pressure, snap->pressure.data(), 4ull * d.nc, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d.x64 && snap->x64.size() == d.nc)
        e = cudaMemcpyAsync(d.x64, snap->x64.data(), 8ull * d.nc, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d.x2 && snap->x2.size() == d.nc)
        e = cudaMemcpyAsync(d.x2, snap->x2.data(), 8ull * d.nc, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return s->cuda_fail(e, "restore");
    rc = sim_bin(s, st);
    if (rc) return rc;
    s->steps_done = snap->steps_done;
    s->initialized = snap->initialized;
    return sim_wait(s);
}

void pxf_snapshot_free(pxf_snapshot* snap) { delete snap; }

int pxf_step_timed(pxf_sim* s, uint32_t n, double* ms) {
    if (!s || !ms) return set_global_error(PXF_EINVAL, "NULL argument");
    if (s->batch && s->batch != s->own) return s->fail(PXF_ESTATE, "simulation is stepped by a batch");
    BatchImpl* b = s->own;
    if (b->dirty) {
        int rc = b->rebuild();
        if (rc) return s->fail(rc, b->err);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, b->stream);
    s->initialized = true;
    int rc = b->step(n);
    cudaEventRecord(e1, b->stream);
    if (!rc) rc = b->wait();
    float t = 0;
    if (!rc) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return s->fail(rc, b->err);
    *ms = double(t);
    return PXF_OK;
}

int pxf_profile_substep(pxf_sim* s, pxf_stage_time* out, uint32_t cap, uint32_t* count) {
    if (!s || !count) return set_global_error(PXF_EINVAL, "NULL argument");
    if (s->batch && s->batch != s->own) return s->fail(PXF_ESTATE, "simulation is stepped by a batch");
    s->initialized = true;
    int rc = s->own->profile(out, cap, count);
    if (rc) return s->fail(rc, s->own->err);
    return PXF_OK;
}

int pxf_set_wait_timeout(pxf_sim* s, double seconds) {
    if (!s) return set_global_error(PXF_EINVAL, "sim is NULL");
    if (!(seconds > 0.0)) return s->fail(PXF_EINVAL, "the wait timeout must be positive");
    s->opts.wait_timeout_s = seconds;
    BatchImpl* b = s->batch ? s->batch : s->own;
    b->timeout_s = 0;
    for (pxf_sim* m : b->sims) b->timeout_s = std::max(b->timeout_s, m->opts.wait_timeout_s);
    if (b->sims.empty()) b->timeout_s = seconds;
    return PXF_OK;
}

int pxf_selftest_grid_barrier(uint32_t blocks, int32_t skip_block, double limit_ms, uint32_t rounds,
                              uint32_t* timed_out) {
    if (!timed_out || blocks == 0 || rounds == 0 || !(limit_ms > 0.0) || limit_ms > 10000.0)
        return set_global_error(PXF_EINVAL, "selftest: blocks, rounds > 0, 0 < limit_ms <= 10000 and an output");
    GridBar* bar = nullptr;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaMalloc(&bar, sizeof(GridBar));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = launch_barrier_selftest(bar, int(std::min<uint32_t>(blocks, 1u << 20)), skip_block,
                                    (long long)(limit_ms * 2.07e6), int(std::min<uint32_t>(rounds, 1000u)), st);
    cudaEvent_t ev = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) {
        // bounded host wait: the kernel's own waits end within rounds x limit
        const double budget = 10.0 + 2.0 * double(std::min<uint32_t>(rounds, 1000u)) * limit_ms / 1e3;
        const auto t0 = std::chrono::steady_clock::now();
        while ((e = cudaEventQuery(ev)) == cudaErrorNotReady) {
            if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > budget) break;
            std::this_thread::sleep_for(std::chrono::microseconds(100));
        }
    }
    int rc = PXF_OK;
    if (e == cudaErrorNotReady) {
        rc = set_global_error(PXF_ETIMEDOUT, "selftest kernel did not finish");
    } else if (e != cudaSuccess) {
        rc = set_global_error(PXF_ECUDA, std::string("selftest: ") + cudaGetErrorString(e));
    } else {
        GridBar hb;
        e = cudaMemcpy(&hb, bar, sizeof(hb), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = set_global_error(PXF_ECUDA, std::string("selftest: ") + cudaGetErrorString(e));
        else *timed_out = hb.err;
    }
    if (ev) cudaEventDestroy(ev);
    if (rc != PXF_ETIMEDOUT) {
        if (st) cudaStreamDestroy(st);
        if (bar) cudaFree(bar);
    }
    return rc;
}

int pxf_set_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_global_error(PXF_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    return PXF_OK;
}

int pxf_host_alloc(size_t bytes, void** out) {
    if (!out) return set_global_error(PXF_EINVAL, "out is NULL");
    cudaError_t e = cudaMallocHost(out, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return set_global_error(PXF_ENOMEM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    return PXF_OK;
}

void pxf_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

void pxf_destroy(pxf_sim* s) {
    if (!s) return;
    if (s->batch && s->batch != s->own) {
        BatchImpl* b = s->batch;
        b->wait();
        b->sims.erase(std::remove(b->sims.begin(), b->sims.end(), s), b->sims.end());
        b->dirty = true;
    }
    if (s->own) {
        s->own->wait();
        delete s->own;
    }
    if (s->mem) cudaFree(s->mem);
    if (s->surf_mem) cudaFree(s->surf_mem);
    delete s;
}

const char* pxf_last_error(const pxf_sim* s) { return s ? s->err.c_str() : g_last_error.c_str(); }

// ---------------------------------------------------------------------------- batches
int pxf_batch_create(pxf_batch** out) {
    if (!out) return set_global_error(PXF_EINVAL, "out is NULL");
    std::string msg;
    if (ensure_device(msg)) return set_global_error(PXF_ECUDA, msg);
    *out = new pxf_batch();
    return PXF_OK;
}

int pxf_batch_add(pxf_batch* b, pxf_sim* s) {
    if (!b || !s) return set_global_error(PXF_EINVAL, "NULL argument");
    if (s->batch && s->batch != s->own) return b->impl.fail(PXF_ESTATE, "simulation already belongs to a batch");
    int rc = s->own->wait();
    if (rc) return b->impl.fail(rc, s->own->err);
    rc = b->impl.wait();
    if (rc) return rc;
    s->batch = &b->impl;
    s->initialized = true;
    b->impl.sims.push_back(s);
    b->impl.dirty = true;
    return PXF_OK;
}

int pxf_batch_remove(pxf_batch* b, pxf_sim* s) {
    if (!b || !s) return set_global_error(PXF_EINVAL, "NULL argument");
    auto it = std::find(b->impl.sims.begin(), b->impl.sims.end(), s);
    if (it == b->impl.sims.end()) return b->impl.fail(PXF_ENOTFOUND, "simulation is not in this batch");
    int rc = b->impl.wait();
    if (rc) return rc;
    b->impl.sims.erase(it);
    s->batch = nullptr;
    b->impl.dirty = true;
    return PXF_OK;
}

uint32_t pxf_batch_size(const pxf_batch* b) { return b ? uint32_t(b->impl.sims.size()) : 0; }

int pxf_batch_step(pxf_batch* b, uint32_t n) {
    if (!b) return set_global_error(PXF_EINVAL, "batch is NULL");
    return b->impl.step(n);
}

int pxf_batch_sync(pxf_batch* b) {
    if (!b) return set_global_error(PXF_EINVAL, "batch is NULL");
    return b->impl.wait();
}

void pxf_batch_destroy(pxf_batch* b) {
    if (!b) return;
    b->impl.wait();
    for (pxf_sim* s : b->impl.sims) s->batch = nullptr;
    delete b;
}

const char* pxf_batch_last_error(const pxf_batch* b) { return b ? b->impl.err.c_str() : g_last_error.c_str(); }

int pxf_autotune(pxf_sim* s, pxf_tune_result* out) {
    if (!s || !out) return set_global_error(PXF_EINVAL, "NULL argument");
    if (s->batch && s->batch != s->own) return s->fail(PXF_ESTATE, "simulation is stepped by a batch");
    s->initialized = true;
    int rc = s->own->run_eager(nullptr, out);
    if (rc) return s->fail(rc, s->own->err);
    return PXF_OK;
}

int pxf_batch_autotune(pxf_batch* b, pxf_tune_result* out) {
    if (!b || !out) return set_global_error(PXF_EINVAL, "NULL argument");
    BatchImpl& B = b->impl;
    if (B.sims.empty()) return B.fail(PXF_ESTATE, "empty batch");
    for (pxf_sim* s : B.sims) s->initialized = true;
    return B.run_eager(nullptr, out);
}

int pxf_batch_step_timed(pxf_batch* b, uint32_t n, double* ms) {
    if (!b || !ms) return set_global_error(PXF_EINVAL, "NULL argument");
    BatchImpl& B = b->impl;
    *ms = 0;
    if (B.sims.empty() || n == 0) return PXF_OK;
    if (B.dirty) {
        int rc = B.rebuild();
        if (rc) return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, B.stream);
    int rc = B.step(n);
    cudaEventRecord(e1, B.stream);
    if (!rc) rc = B.wait();
    float t = 0;
    if (!rc) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *ms = double(t);
    return PXF_OK;
}

}  // extern "C"
