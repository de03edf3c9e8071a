// Red-black Gauss-Seidel pressure solve (shaders/fluid.slang:167-182, host loop
// crates/pxl-render/src/fluid.rs:295-300) as one cooperative launch per substep whose blocks
// synchronise only with the blocks they neighbour.
//
// The reference runs 2 x iterations dependent passes; launched one per colour, every pass pays a
// kernel's start and drain plus its cells' chain of L2 round trips (list entry, then flags, then
// neighbours). Here each block owns a fixed range of cells [lo, hi) of one simulation for the
// whole solve. Its system cells (fluid, at least one non-solid neighbour: the cells the reference
// updates) are compacted once into shared memory as packed entries (cell, fluid-neighbour mask,
// non-solid count), red then black, and evaluates their right-hand sides div * h * h / dt once
// (the reference's expression and order), so a half sweep is one round of neighbour loads from L2
// per cell; the division by the count is the exact one for a divisor known in advance. Shared memory stays at 4 bytes per cell of the range: the rest of the SM's 256 KB is L1,
// which stages the in-flight loads (caching the right-hand side beside the entries left it too
// small and was slower).
//
// Between half sweeps a block publishes how many it has finished (one flag word per block,
// release) and waits (acquire) only for the blocks whose ranges lie within one z-plane of its own
// (cells c - nx*ny .. c + nx*ny): those are the only ones whose cells its cells read or whose
// reads its writes could overtake. Half sweep k (colour k & 1) starts once every such block has
// finished half sweep k - 1:
//   - the other colour's values it reads were written in half sweep k - 1 (read after write);
//   - its neighbours have finished reading this colour's old values, which they read in half
//     sweep k - 1 (write after read).
// A cell's update reads only the other colour, so every update sees exactly the values of the
// reference's order and the result is the reference's bits.
//
// Waits are bounded (clock64 limit): a block that gives up sets the error word and returns, and
// the others return at their next wait that does not complete. Every block of the launch is
// co-resident (cooperative launch of at most one block per SM).
#include <algorithm>
#include <cstdlib>
#include <cuda/atomic>
#include <vector>

#include "pxf_device.cuh"
#include "pxf_kernels.h"

namespace pxf {

namespace {

constexpr int kThreads = 1024;
constexpr int kGroup = 4;              // entries per thread whose loads are issued together
constexpr uint32_t kRelBits = 20;      // packed entry: cell - lo (20 bits), neighbour mask (6), count (3)

struct ResArgs {
    const SimDev* sims;
    const GsResBlock* plan;
    uint32_t* flags;    // [blocks * kGsResFlagStride]: half sweeps finished by each block
    uint32_t* err;      // set when a wait ran out
    long long limit;    // clock64 cycles a wait may take
    int skip;           // block that returns at once (failure-path test), -1: none
};

// Waits until every block of [dep0, dep1) but this one has finished `k` half sweeps (one lane of
// warp 0 per block). False when a wait ran out or another block gave up.
__device__ __forceinline__ bool wait_deps(const ResArgs& a, const GsResBlock& B, uint32_t k) {
    __shared__ int bad;
    if (threadIdx.x < 32) {
        const uint32_t d = B.dep0 + threadIdx.x;
        bool ok = true;
        if (d < B.dep1 && d != blockIdx.x) {
            cuda::atomic_ref<uint32_t, cuda::thread_scope_device> f(a.flags[size_t(d) * kGsResFlagStride]);
            cuda::atomic_ref<uint32_t, cuda::thread_scope_device> err(*a.err);
            const long long t0 = clock64();
            uint32_t spins = 0;
            while (f.load(cuda::memory_order_acquire) < k) {
                if ((++spins & 63u) == 0u &&
                    (err.load(cuda::memory_order_relaxed) || clock64() - t0 > a.limit)) {
                    err.store(1u, cuda::memory_order_relaxed);
                    ok = false;
                    break;
                }
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (threadIdx.x == 0) bad = ok ? 0 : 1;
    }
    __syncthreads();
    return !bad;
}

// Exclusive block scan of two counts; totals in tr, tb.
__device__ __forceinline__ void scan2(uint32_t nr, uint32_t nb, uint32_t& pr, uint32_t& pb, uint32_t& tr,
                                      uint32_t& tb) {
    __shared__ uint32_t wr[32], wb[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t xr = nr, xb = nb;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t yr = __shfl_up_sync(0xffffffffu, xr, d), yb = __shfl_up_sync(0xffffffffu, xb, d);
        if (lane >= d) { xr += yr; xb += yb; }
    }
    if (lane == 31) { wr[wid] = xr; wb[wid] = xb; }
    __syncthreads();
    uint32_t br = 0, bb = 0;
    tr = tb = 0;
    for (int k = 0; k < kThreads / 32; k++) {
        const uint32_t r = wr[k], b = wb[k];
        if (k < wid) { br += r; bb += b; }
        tr += r;
        tb += b;
    }
    pr = br + xr - nr;
    pb = bb + xb - nb;
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 1) k_gs_resident(ResArgs a) {
    extern __shared__ uint32_t ent[];   // red entries from the front of ent[0, cap), black ones from its back
    __shared__ float rcp[8];            // RN(1 / cnt)
    const GsResBlock B = a.plan[blockIdx.x];
    if (int(blockIdx.x) == a.skip) return;
    const SimDev& s = a.sims[B.sim];
    const uint32_t lo = B.lo, hi = B.hi, cap = hi - lo;
    const uint32_t nx = uint32_t(s.nx), ny = uint32_t(s.ny), nxy = nx * ny;
    const uint16_t* __restrict__ info = s.info;
    const float* __restrict__ dv = s.div;
    const float rh = s.h, rdt = s.dt;
    float* rhs = s.rhs;                 // div * h * h / dt of the block's system cells, this launch
    if (threadIdx.x < 8) rcp[threadIdx.x] = threadIdx.x ? 1.0f / float(threadIdx.x) : 0.0f;

    // ---- the block's system cells, once: eight consecutive cells per thread per round
    uint32_t nred = 0, nblk = 0;
    for (uint32_t r0 = lo; r0 < hi; r0 += 8 * kThreads) {
        const uint32_t c0 = r0 + 8 * threadIdx.x;
        uint32_t inf[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t redm = 0, blkm = 0;
        if (c0 < hi) {
            if (c0 + 8 <= hi) {
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(info + c0));   // c0 % 8 == 0
                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    inf[2 * q] = w[q] & 0xffffu;
                    inf[2 * q + 1] = w[q] >> 16;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; q++) inf[q] = c0 + q < hi ? uint32_t(__ldg(info + c0 + q)) : 0u;
            }
            uint32_t x = c0 % nx, y = (c0 / nx) % ny, z = c0 / nxy;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const uint32_t f = inf[q];
                if ((f & 0x8000u) && ((f >> 8) & 7u)) {
                    if ((x + y + z) & 1u) blkm |= 1u << q; else redm |= 1u << q;
                }
                if (++x == nx) {
                    x = 0;
                    if (++y == ny) { y = 0; ++z; }
                }
            }
        }
        uint32_t pr, pb, tr, tb;
        scan2(__popc(redm), __popc(blkm), pr, pb, tr, tb);
        pr += nred;
        pb += nblk;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (!((redm | blkm) & (1u << q))) continue;
            const uint32_t c = c0 + q;
            ent[(redm & (1u << q)) ? pr++ : cap - 1 - pb++] =
                (c - lo) | ((inf[q] & 63u) << kRelBits) | (((inf[q] >> 8) & 7u) << (kRelBits + 6));
            rhs[c] = __ldg(dv + c) * rh * rh / rdt;   // fluid.slang:181
        }
        nred += tr;
        nblk += tb;
    }
    __syncthreads();

    // ---- 2 x iterations half sweeps
    float* __restrict__ p = s.pressure;
    const uint32_t half_sweeps = 2u * s.iterations;
    for (uint32_t k = 0; k < half_sweeps; k++) {
        if (k && !wait_deps(a, B, k)) return;
        const bool black = k & 1u;
        const uint32_t n = black ? nblk : nred;
        // kGroup entries per thread at a time, every neighbour load issued before the first store
        // (the cells of one colour never neighbour each other)
        for (uint32_t i0 = threadIdx.x; i0 < n; i0 += kGroup * kThreads) {
            uint32_t c[kGroup], m[kGroup];
            float v[kGroup][6], d[kGroup];
#pragma unroll
            for (int j = 0; j < kGroup; j++) {
                const uint32_t i = i0 + j * kThreads;
                const uint32_t e = i < n ? ent[black ? cap - 1 - i : i] : 0u;
                c[j] = lo + (e & ((1u << kRelBits) - 1u));
                m[j] = e >> kRelBits;   // fluid-neighbour mask in bits 0-5, non-solid count in bits 6-8; 0: none
            }
#pragma unroll
            for (int j = 0; j < kGroup; j++) {
                const uint32_t cc = c[j], mm = m[j];
                v[j][0] = (mm & 1u) ? __ldcg(p + cc - 1) : 0.0f;
                v[j][1] = (mm & 2u) ? __ldcg(p + cc + 1) : 0.0f;
                v[j][2] = (mm & 4u) ? __ldcg(p + cc - nx) : 0.0f;
                v[j][3] = (mm & 8u) ? __ldcg(p + cc + nx) : 0.0f;
                v[j][4] = (mm & 16u) ? __ldcg(p + cc - nxy) : 0.0f;
                v[j][5] = (mm & 32u) ? __ldcg(p + cc + nxy) : 0.0f;
                d[j] = mm ? rhs[cc] : 0.0f;   // written by this block before the first barrier
            }
#pragma unroll
            for (int j = 0; j < kGroup; j++) {
                const uint32_t mm = m[j];
                if (!mm) continue;
                float sum = 0.0f;   // fluid neighbours in the reference's order -x +x -y +y -z +z
                if (mm & 1u) sum += v[j][0];
                if (mm & 2u) sum += v[j][1];
                if (mm & 4u) sum += v[j][2];
                if (mm & 8u) sum += v[j][3];
                if (mm & 16u) sum += v[j][4];
                if (mm & 32u) sum += v[j][5];
                p[c[j]] = div_count(sum - d[j], (mm >> 6) & 7u, rcp);   // fluid.slang:181-182
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            cuda::atomic_ref<uint32_t, cuda::thread_scope_device> f(a.flags[size_t(blockIdx.x) * kGsResFlagStride]);
            __threadfence();
            f.store(k + 1u, cuda::memory_order_release);
        }
    }
}

size_t res_smem(uint32_t cells) { return size_t(cells) * sizeof(uint32_t); }

size_t max_dyn_smem() {
    static const size_t v = [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 0;
        return size_t(optin > 4096 ? optin - 4096 : 0);   // room for the kernel's static shared memory
    }();
    return v;
}

}  // namespace

// Blocks and their cell ranges, for the GS simulations of a batch. A simulation's cells are split
// into equal ranges (multiples of 8 cells) of at least `min_cells`; the batch gets at most one block
// per SM, shared between the simulations by their cell counts. False when it does not fit: more
// simulations than SMs, a range whose entries exceed shared memory, or a block with more than 31
// other blocks within one z-plane.
bool plan_gs_resident(const std::vector<SimDev>& sims, std::vector<GsResBlock>& plan, size_t& smem) {
    plan.clear();
    smem = 0;
    const uint32_t cap = uint32_t(sm_count());
    static const uint32_t min_cells = [] {
        const char* v = std::getenv("PXF_GS_RES_CELLS");
        const unsigned long x = v ? std::strtoul(v, nullptr, 10) : 4096ul;
        return uint32_t(std::clamp<unsigned long>(x, 8ul, 1ul << 20));
    }();
    std::vector<int> gs;
    uint64_t total = 0;
    for (int i = 0; i < int(sims.size()); i++)
        if (sims[i].solver == 0 && sims[i].iterations > 0) {
            gs.push_back(i);
            total += sims[i].nc;
        }
    if (gs.empty() || gs.size() > cap || total == 0) return false;
    std::vector<uint32_t> g(gs.size());
    uint32_t used = 0;
    for (size_t k = 0; k < gs.size(); k++) {
        const uint64_t nc = sims[gs[k]].nc;
        uint64_t share = std::max<uint64_t>(1, cap * nc / total);
        share = std::min<uint64_t>(share, std::max<uint64_t>(1, nc / min_cells));
        g[k] = uint32_t(share);
        used += g[k];
    }
    while (used > cap) {
        const size_t big = size_t(std::max_element(g.begin(), g.end()) - g.begin());
        if (g[big] <= 1) return false;
        g[big]--;
        used--;
    }
    const size_t limit = max_dyn_smem();
    for (size_t k = 0; k < gs.size(); k++) {
        const SimDev& s = sims[gs[k]];
        const uint64_t nc = s.nc, nxy = uint64_t(s.nx) * s.ny;
        const uint64_t R = ((nc + g[k] - 1) / g[k] + 7) / 8 * 8;
        if (R >= (uint64_t(1) << kRelBits) || res_smem(uint32_t(R)) > limit) return false;
        smem = std::max(smem, res_smem(uint32_t(R)));
        const uint32_t nb = uint32_t((nc + R - 1) / R), off = uint32_t(plan.size());
        for (uint32_t j = 0; j < nb; j++) {
            const uint64_t lo = j * R, hi = std::min<uint64_t>(nc, lo + R);
            const uint64_t a = lo > nxy ? lo - nxy : 0, b = std::min<uint64_t>(nc, hi + nxy);
            const uint32_t d0 = uint32_t(a / R), d1 = uint32_t((b - 1) / R + 1);
            if (d1 - d0 > 32) return false;   // one lane of a warp per block of the range
            plan.push_back(GsResBlock{uint32_t(gs[k]), uint32_t(lo), uint32_t(hi), off + d0, off + d1});
        }
    }
    if (plan.size() > cap) return false;
    int per_sm = 0;
    if (cudaFuncSetAttribute(k_gs_resident, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gs_resident, kThreads, smem) != cudaSuccess ||
        uint64_t(per_sm) * cap < plan.size())
        return false;
    return true;
}

cudaError_t launch_gs_resident(const SimDev* sims, const GsResBlock* plan, int blocks, uint32_t* flags,
                               uint32_t* err, size_t smem, long long limit, int skip, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(flags, 0, size_t(blocks) * kGsResFlagStride * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    ResArgs a{sims, plan, flags, err, limit, skip};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(blocks));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_gs_resident, a);
    note_launch("k_gs_resident", st);
    return e;
}

}  // namespace pxf
