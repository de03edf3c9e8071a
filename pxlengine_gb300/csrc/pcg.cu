// Precision pressure solve: preconditioned CG on the system that shaders/fluid.slang:167-182
// relaxes, for each fluid cell i
//     cnt_i p_i - sum_{fluid j} p_j = -(div_i h h / dt),     cnt_i = non-solid neighbours,
// with a geometric multigrid V-cycle (or Jacobi) preconditioner.
//
// Precision: vectors r, z, p, Ap and the whole V-cycle are FP32. The solution x is kept as a
// double-float pair (hi + lo, 48-bit significand) so the true residual can fall below FP32's
// cond(A)·eps floor. The FP64 steps are the reductions and the restart residual:
//   * dot products: each product is formed exactly (FP32 two-product), a warp sums its products
//     in double-float, and warp / block / chunk sums are FP64 in a fixed order;
//   * restart: x is widened to FP64 and r = b - A x is evaluated in FP64 (every `restart` steps,
//     when the recurrence residual reaches the target, and at the iteration cap); convergence is
//     declared on that FP64 residual, |r| <= rtol |b|.
// (GB300's FP64 pipe runs at about 1 TFLOP/s, 1/60 of FP32, so FP64 is kept out of per-cell work.)
//
// Work: every kernel iterates compacted, colour-split lists of the system cells of each chunk
// (built once per substep with a block scan, so the order of every reduction is fixed). Partial
// sums are per level-0 chunk; a control step per simulation sums them in chunk order and advances
// that simulation's state. No atomics, no fences in the arithmetic: results do not depend on
// scheduling or on the other simulations of a batch.
//
// Multigrid (level l+1 halves each axis, rounding up): a coarse cell is AIR if any child is AIR,
// else FLUID if any child is FLUID, else SOLID (children outside the fine grid are SOLID); each
// level's operator is the 7-point system above built from its own types. V-cycle: red-black
// Gauss-Seidel pre-smoothing (red from zero, black), restriction r_c = 1/2 * sum of the children's
// residuals, recursion, prolongation (each child += its parent's correction, fused into the first
// post-smoothing sweep), post-smoothing (black, red). Levels with at most kTailCells cells run
// inside one block in shared memory; the coarsest level (<= 512 cells) runs `coarse_iters`
// red-black then as many black-red iterations from zero. Restriction is prolongation^T / 2 and the
// sweeps mirror each other, so the cycle is symmetric.
//
// Execution: each step is a device "phase" function. The phases run either as separate kernels
// (graph-captured, the loop as a conditional while-node) or all inside one persistent cooperative
// kernel per substep with grid barriers between phases. Barrier waits are bounded: a wait that
// exceeds its limit raises an error flag that the host reports, and every block returns.
#include <cstdlib>
#include <cuda/atomic>
#include "pxf_device.cuh"
#include "pxf_kernels.h"

namespace pxf {

namespace {

constexpr int THREADS = 256;

// ---------------------------------------------------------------- double-float arithmetic
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = a.hi + b.hi;
    const float bv = s - a.hi;
    float e = (a.hi - (s - bv)) + (b.hi - bv);
    e += a.lo + b.lo;
    const float hi = s + e;
    return {hi, e - (hi - s)};
}

// Block sum of a double-float accumulator in a fixed order; valid in thread 0.
__device__ __forceinline__ double block_sum(DF a, double* sh) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const DF t{__shfl_down_sync(0xffffffffu, a.hi, d), __shfl_down_sync(0xffffffffu, a.lo, d)};
        a = df_add(a, t);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = double(a.hi) + double(a.lo);
    __syncthreads();
    double out = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < int(blockDim.x >> 5); k++) out += sh[k];
    __syncthreads();
    return out;
}

__device__ __forceinline__ bool in_system(uint32_t inf) { return (inf & 0x8000u) && ((inf >> 8) & 7u); }
__device__ __forceinline__ float cnt_of(uint32_t inf) { return float((inf >> 8) & 7u); }

__device__ __forceinline__ int64_t nbr(int q, int64_t nx, int64_t nxy) {
    switch (q) {
        case 0: return -1;
        case 1: return 1;
        case 2: return -nx;
        case 3: return nx;
        case 4: return -nxy;
        default: return nxy;
    }
}

__device__ __forceinline__ float rhs_of(const SimDev& s, uint32_t c) {
    return s.div[c] * s.h * s.h / s.dt;   // fluid.slang:181
}

// Per-simulation scalars, written by the previous step's control: read through L2.
__device__ __forceinline__ uint32_t ldu(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ double ldd(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ldf(const float* p) { return __ldcg(p); }

__device__ __forceinline__ bool active(const SimDev& s) { return s.solver == 1 && !ldu(&s.pcg->done); }

__device__ __forceinline__ uint32_t nchunks0(const SimDev& s) { return (s.nc + s.lev[0].cs - 1) / s.lev[0].cs; }

// Fixed-order sum of a simulation's chunk partials (one block per simulation).
__device__ __forceinline__ double sum_partials(const SimDev& s, double* sh) {
    const uint32_t n = nchunks0(s);
    double p = 0;
    // eight loads in flight per thread, added in the same order as a plain strided loop
    uint32_t k = threadIdx.x;
    for (; k + 7 * blockDim.x < n; k += 8 * blockDim.x) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = __ldcg(s.partial + k + u * blockDim.x);
#pragma unroll
        for (int u = 0; u < 8; u++) p += v[u];
    }
    for (; k < n; k += blockDim.x) p += __ldcg(s.partial + k);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) p += __shfl_down_sync(0xffffffffu, p, d);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = p;
    __syncthreads();
    double out = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < int(blockDim.x >> 5); k++) out += sh[k];
    __syncthreads();
    return out;
}

// Entries [lo, hi) of chunk `chunk` of a level's system-cell list for colour 0 (red), 1 (black)
// or 2 (both).
__device__ __forceinline__ void seg(const MgLevel& L, uint32_t chunk, int color, uint32_t& lo, uint32_t& hi) {
    const uint32_t nr = __ldcg(L.lcnt + 2 * chunk), nb = __ldcg(L.lcnt + 2 * chunk + 1);
    lo = color == 1 ? nr : 0u;
    hi = color == 0 ? nr : nr + nb;
}

__device__ __forceinline__ const uint32_t* list_of(const MgLevel& L, uint32_t chunk) {
    return L.list + size_t(chunk) * L.cs;
}

// Programmatic dependent launch. The kernels of the CG loop are launched so that each may start
// while the one before it drains. Until dep_wait() returns (the previous kernel has completed and
// its writes are visible) a kernel reads only what stays fixed during the solve: the simulation
// descriptors and the cell lists and their counts. Every block waits before it exits, so a
// kernel completes only after the one before it, and dependents are released only after the
// wait. Outside such a launch both instructions return at once.
__device__ __forceinline__ void dep_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace

// ============================================================================ phases
// Every phase walks its work index with a block-strided loop, so it serves both the standalone
// kernels and the persistent kernel.

// Compacts each chunk of level l into its red then black system cells, in ascending cell order.
__device__ void ph_cell_lists(const Work& w, int l, uint32_t solver = 1) {
    __shared__ uint32_t wr[32], wb[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != solver) continue;
        const MgLevel L = sp->lev[l];
        const uint32_t chunk = item - w.base[si];
        const uint32_t nx = uint32_t(L.nx), ny = uint32_t(L.ny), nxy = nx * ny;
        const uint32_t per = L.cs / blockDim.x;   // 8 on level 0, 1 below
        const uint32_t c0 = chunk * L.cs + threadIdx.x * per;
        uint32_t redm = 0, blkm = 0;
        for (uint32_t k = 0; k < per; k++) {
            const uint32_t c = c0 + k;
            if (c >= L.nc || !in_system(L.info[c])) continue;
            const uint32_t par = (c % nx + (c / nx) % ny + c / nxy) & 1u;
            if (par) blkm |= 1u << k; else redm |= 1u << k;
        }
        const uint32_t nr = __popc(redm), nb = __popc(blkm);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = int(blockDim.x >> 5);
        uint32_t xr = nr, xb = nb;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t yr = __shfl_up_sync(0xffffffffu, xr, d), yb = __shfl_up_sync(0xffffffffu, xb, d);
            if (lane >= d) { xr += yr; xb += yb; }
        }
        if (lane == 31) { wr[wid] = xr; wb[wid] = xb; }
        __syncthreads();
        uint32_t br = 0, bb = 0, tr = 0, tb = 0;
        for (int k = 0; k < nw; k++) {
            if (k < wid) { br += wr[k]; bb += wb[k]; }
            tr += wr[k];
            tb += wb[k];
        }
        uint32_t pr = br + xr - nr, pb = tr + bb + xb - nb;
        uint32_t* out = L.list + size_t(chunk) * L.cs;
        for (uint32_t k = 0; k < per; k++) {
            if (redm & (1u << k)) out[pr++] = c0 + k;
            if (blkm & (1u << k)) out[pb++] = c0 + k;
        }
        if (threadIdx.x == 0) {
            L.lcnt[2 * chunk] = tr;
            L.lcnt[2 * chunk + 1] = tb;
        }
        __syncthreads();
    }
}

// Appends the items of stage w whose chunk of level `lev` holds system cells to the stage's act
// list (one thread per item; the order of the list does not matter: items are independent and
// every reduction keeps one partial per chunk). With zero_partial, empty level-0 chunks get a
// zero partial, which no later step overwrites.
__device__ void compact_stage(const Work& w, int lev, uint32_t* count, bool zero_partial) {
    uint32_t* out = const_cast<uint32_t*>(w.act);
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < w.total; item += gridDim.x * blockDim.x) {
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 1) continue;
        const uint32_t chunk = item - __ldg(w.base + si);
        const MgLevel& L = sp->lev[lev];
        const uint32_t n = __ldcg(L.lcnt + 2 * chunk) + __ldcg(L.lcnt + 2 * chunk + 1);
        if (n) out[atomicAdd(count, 1u)] = item;
        else if (zero_partial) sp->partial[chunk] = 0.0;
    }
}

__device__ void ph_compact(const PcgWork& pw) {
    Work c = pw.chunks_all;
    c.act = pw.chunks.act;
    compact_stage(c, 0, pw.act_n, true);
    for (int l = 0; l + 1 < pw.max_levels; l++) {
        if (pw.level[l].total) {
            Work a = pw.level[l];
            compact_stage(a, l, pw.act_n + 1 + l, false);
        }
        if (pw.coarse[l].total) {
            Work b = pw.coarse[l];
            compact_stage(b, l + 1, pw.act_n + 1 + kMaxLevelsK + l, false);
        }
    }
}

// Type of level l+1 from its children on level l (work: level-(l+1) chunks).
__device__ void ph_coarsen(const Work& w, int l) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 1) continue;
        const MgLevel F = sp->lev[l], Cc = sp->lev[l + 1];
        const uint32_t per = Cc.cs / blockDim.x;
        for (uint32_t k = 0; k < per; k++) {
            const uint32_t P = (item - w.base[si]) * Cc.cs + k * blockDim.x + threadIdx.x;
            if (P >= Cc.nc) continue;
            const int I = int(P % uint32_t(Cc.nx)), J = int((P / uint32_t(Cc.nx)) % uint32_t(Cc.ny));
            const int K = int(P / (uint32_t(Cc.nx) * uint32_t(Cc.ny)));
            bool air = false, fluid = false;
#pragma unroll
            for (int ch = 0; ch < 8; ch++) {
                const int i = 2 * I + (ch & 1), j = 2 * J + ((ch >> 1) & 1), kk = 2 * K + (ch >> 2);
                if (i >= F.nx || j >= F.ny || kk >= F.nz) continue;
                const uint8_t t = F.type[uint32_t(i) + uint32_t(F.nx) * (uint32_t(j) + uint32_t(F.ny) * uint32_t(kk))];
                air |= (t == AIR);
                fluid |= (t == FLUID);
            }
            Cc.type[P] = air ? AIR : (fluid ? FLUID : SOLID);
        }
    }
}

// Neighbour record of level l+1 (as k_divergence builds it for level 0).
__device__ void ph_info(const Work& w, int l) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 1) continue;
        const MgLevel L = sp->lev[l + 1];
        const uint32_t per = L.cs / blockDim.x;
        for (uint32_t k = 0; k < per; k++) {
            const uint32_t c = (item - w.base[si]) * L.cs + k * blockDim.x + threadIdx.x;
            if (c >= L.nc) continue;
            uint16_t info = 0;
            if (L.type[c] == FLUID) {
                const int i = int(c % uint32_t(L.nx)), j = int((c / uint32_t(L.nx)) % uint32_t(L.ny));
                const int kk = int(c / (uint32_t(L.nx) * uint32_t(L.ny)));
                const int q3[6][3] = {{i - 1, j, kk}, {i + 1, j, kk}, {i, j - 1, kk},
                                      {i, j + 1, kk}, {i, j, kk - 1}, {i, j, kk + 1}};
                uint32_t mask = 0, cnt = 0;
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    const int a = q3[q][0], b = q3[q][1], d = q3[q][2];
                    uint8_t t = SOLID;
                    if (a >= 0 && b >= 0 && d >= 0 && a < L.nx && b < L.ny && d < L.nz)
                        t = L.type[uint32_t(a) + uint32_t(L.nx) * (uint32_t(b) + uint32_t(L.ny) * uint32_t(d))];
                    if (t != SOLID) cnt++;
                    if (t == FLUID) mask |= 1u << q;
                }
                info = uint16_t(mask | (cnt << 8) | 0x8000u);
            }
            L.info[c] = info;
        }
    }
}

// One red-black half sweep of A z = r on level l over the system cells of one colour.
// Pass p of a simulation's smoothing pairs runs only if p < its mg_pairs.
// mode 0: z = (r + sum z_n) / cnt; mode 1: the other colour is zero (z = r / cnt);
// mode 2: as 0 with the coarse correction of level l+1 added to every neighbour on the fly
// (fused prolongation); mode 3: as 0, then the chunk's partial r.z over all system cells.
__device__ void ph_smooth(const Work& w, int l, int color, int mode_in, int pass) {
    __shared__ double sh[32];
    constexpr int SE = 1;   // entries per thread whose operands are in flight together
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 1 || sp->precond != 0 || uint32_t(pass) >= sp->mg_pairs) continue;
        // the r.z partial comes with the last red sweep of the simulation's post-smoothing
        const int mode = (mode_in == 3 && uint32_t(pass) + 1 != sp->mg_pairs) ? 0 : mode_in;
        const MgLevel L = sp->lev[l];
        const uint32_t nx = uint32_t(L.nx), ny = uint32_t(L.ny), nxy = nx * ny;
        const uint32_t chunk = item - w.base[si];
        const MgLevel Cc = (mode == 2) ? sp->lev[l + 1] : L;
        const uint32_t cnx = uint32_t(Cc.nx), cnxy = uint32_t(Cc.nx) * uint32_t(Cc.ny);
        uint32_t lo, hi;
        seg(L, chunk, color, lo, hi);
        const uint32_t* __restrict__ lst = list_of(L, chunk);
        const uint16_t* __restrict__ info = L.info;
        const float* __restrict__ r = L.r;
        float* __restrict__ z = L.z;
        bool waited = false;
        bool stop = false;
        for (uint32_t e0 = lo + threadIdx.x; !stop && (e0 < hi || !waited); e0 += SE * blockDim.x) {
            // fixed during the solve: list entries, records and, for mode 2, the coarse cells above
            // the neighbours and whether they are in the coarse system
            uint32_t cc[SE], ii[SE], pin[SE], P[SE][6];
            bool hh[SE];
#pragma unroll
            for (int u = 0; u < SE; u++) {
                const uint32_t e = e0 + u * blockDim.x;
                hh[u] = e < hi;
                cc[u] = hh[u] ? __ldcg(lst + e) : 0u;
                ii[u] = hh[u] ? uint32_t(info[cc[u]]) : 0u;
                pin[u] = 0;
#pragma unroll
                for (int q = 0; q < 6; q++) P[u][q] = 0;
                if (hh[u] && mode == 2) {
                    const uint32_t c = cc[u], i = c % nx, j = (c / nx) % ny, kk = c / nxy;
#pragma unroll
                    for (int q = 0; q < 6; q++) {
                        if (!(ii[u] & (1u << q))) continue;
                        const int dx = q == 0 ? -1 : (q == 1 ? 1 : 0);
                        const int dy = q == 2 ? -1 : (q == 3 ? 1 : 0);
                        const int dz = q == 4 ? -1 : (q == 5 ? 1 : 0);
                        P[u][q] = (uint32_t(int(i) + dx) >> 1) + cnx * (uint32_t(int(j) + dy) >> 1) +
                                  cnxy * (uint32_t(int(kk) + dz) >> 1);
                        if (in_system(Cc.info[P[u][q]])) pin[u] |= 1u << q;
                    }
                }
            }
            if (!waited) {
                dep_wait();
                waited = true;
                if (ldu(&sp->pcg->done)) { stop = true; break; }
            }
            // every operand of the entries, issued before any store
            float rv[SE], zn[SE][6], zc[SE][6];
#pragma unroll
            for (int u = 0; u < SE; u++) {
                rv[u] = 0.0f;
#pragma unroll
                for (int q = 0; q < 6; q++) { zn[u][q] = 0.0f; zc[u][q] = 0.0f; }
                if (!hh[u]) continue;
                rv[u] = r[cc[u]];
                if (mode != 1) {
#pragma unroll
                    for (int q = 0; q < 6; q++)
                        if (ii[u] & (1u << q)) zn[u][q] = z[uint32_t(int64_t(cc[u]) + nbr(q, nx, nxy))];
                }
                if (mode == 2) {
#pragma unroll
                    for (int q = 0; q < 6; q++)
                        if (pin[u] & (1u << q)) zc[u][q] = Cc.z[P[u][q]];
                }
            }
#pragma unroll
            for (int u = 0; u < SE; u++) {
                if (!hh[u]) continue;
                // the reference's sums: r, then each system neighbour's z (plus its parent's
                // correction in mode 2), in neighbour order
                float sum = rv[u];
                if (mode == 2) {
#pragma unroll
                    for (int q = 0; q < 6; q++) {
                        if (!(ii[u] & (1u << q))) continue;
                        float t = zn[u][q];
                        if (pin[u] & (1u << q)) t += zc[u][q];
                        sum += t;
                    }
                } else if (mode != 1) {
#pragma unroll
                    for (int q = 0; q < 6; q++)
                        if (ii[u] & (1u << q)) sum += zn[u][q];
                }
                z[cc[u]] = sum / cnt_of(ii[u]);
            }
        }
        if (stop) continue;
        if (mode == 3) {
            // r.z over every system cell of the chunk (the other colour was final before this sweep).
            __syncthreads();
            DF acc{0.f, 0.f};
            uint32_t a0, a1;
            seg(L, chunk, 2, a0, a1);
            for (uint32_t e = a0 + threadIdx.x; e < a1; e += blockDim.x) {
                const uint32_t c = lst[e];
                acc = df_add(acc, two_prod(r[c], z[c]));
            }
            const double t = block_sum(acc, sh);
            if (threadIdx.x == 0) sp->partial[chunk] = t;
        }
    }
}

// r_{l+1} = 1/2 * sum over the children of their residual r - A z (level l); 8 lanes per coarse
// cell, children summed by a fixed shuffle tree. Work: level-(l+1) chunks.
__device__ void ph_restrict(const Work& w, int l) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 1 || sp->precond != 0) continue;
        const MgLevel F = sp->lev[l], Cc = sp->lev[l + 1];
        const uint32_t nx = uint32_t(F.nx), nxy = uint32_t(F.nx) * uint32_t(F.ny);
        const uint32_t chunk = item - w.base[si];
        uint32_t lo, hi;
        seg(Cc, chunk, 2, lo, hi);
        const uint32_t* lst = list_of(Cc, chunk);
        // Below the tail, level l+1's first half sweep (red from zero: z = r / cnt) is done here.
        const bool first_sweep = l + 1 < sp->tail;
        // One coarse cell per thread. Its first pass reads the children's records (fixed during
        // the solve) before dep_wait().
        bool waited = false;
        for (uint32_t e = lo + threadIdx.x; e < hi || (!waited && e == lo + threadIdx.x); e += blockDim.x) {
            const bool h = e < hi;
            uint32_t P = 0, cc[8], inf[8];
            bool red = false;
            if (h) {
                P = __ldcg(lst + e);
                const int I = int(P % uint32_t(Cc.nx)), J = int((P / uint32_t(Cc.nx)) % uint32_t(Cc.ny));
                const int K = int(P / (uint32_t(Cc.nx) * uint32_t(Cc.ny)));
                red = ((I + J + K) & 1) == 0;
#pragma unroll
                for (int chd = 0; chd < 8; chd++) {
                    const int i = 2 * I + (chd & 1), j = 2 * J + ((chd >> 1) & 1), kk = 2 * K + (chd >> 2);
                    const bool in = i < F.nx && j < F.ny && kk < F.nz;
                    cc[chd] = in ? uint32_t(i) + nx * uint32_t(j) + nxy * uint32_t(kk) : 0u;
                    inf[chd] = in ? uint32_t(F.info[cc[chd]]) : 0u;
                }
            }
            if (!waited) {
                dep_wait();
                waited = true;
                if (ldu(&sp->pcg->done)) break;
            }
            if (!h) continue;
            float res[8];
#pragma unroll
            for (int chd = 0; chd < 8; chd++) {
                res[chd] = 0.0f;
                if (!in_system(inf[chd])) continue;
                const uint32_t c = cc[chd];
                float az = cnt_of(inf[chd]) * F.z[c];
#pragma unroll
                for (int q = 0; q < 6; q++)
                    if (inf[chd] & (1u << q)) az -= F.z[uint32_t(int64_t(c) + nbr(q, nx, nxy))];
                res[chd] = F.r[c] - az;
            }
            // ((c0 + c1) + (c2 + c3)) + ((c4 + c5) + (c6 + c7))
            const float sum = ((res[0] + res[1]) + (res[2] + res[3])) + ((res[4] + res[5]) + (res[6] + res[7]));
            const float rc = 0.5f * sum;
            Cc.r[P] = rc;
            if (first_sweep && red) Cc.z[P] = rc / cnt_of(Cc.info[P]);
        }
        if (!waited) dep_wait();
    }
}

// ------------------------------------------------------------------ shared-memory tail
// Levels tail..nlev-1 (the tail level holds at most kTailCells cells) run as one V-cycle inside
// one block per simulation, in shared memory. Input r of the tail level, output z of the tail
// level; when the tail is level 0 the block also writes the level-0 chunk partials of r.z.
// Each level keeps in shared memory its r and z, a copy of the neighbour record (zero outside
// the system) and its system cells as one list, red cells first, gathered from the level's
// global per-chunk lists. A cell's update reads only the other colour, so the order in which a
// sweep visits its cells changes no result.
struct TailLevel {
    int nx, ny, nz;
    uint32_t nc;
    float* r;
    float* z;
    uint16_t* info;
    uint16_t* list;      // system cells: red [0, nred), black [nred, nsys)
    uint32_t nred, nsys;
};

constexpr uint32_t kTailMaxChunks = 32;   // list chunks per tail level (kTailCells / 256 at most)
constexpr int kTailMaxLevels = 6;         // tail levels: kTailCells down to the coarsest (<= 512 cells)

__device__ void tail_smooth(const TailLevel& L, uint32_t color, int mode, const TailLevel* C) {
    const int nx = L.nx, ny = L.ny, nxy = L.nx * L.ny;
    const int off[6] = {-1, 1, -nx, nx, -nxy, nxy};
    const uint16_t* lst = color ? L.list + L.nred : L.list;
    const uint32_t n = color ? L.nsys - L.nred : L.nred;
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int c = int(lst[e]);
        const uint32_t inf = L.info[c];
        float sum = L.r[c];
        if (mode == 2) {
            const int i = c % nx, j = (c / nx) % ny, kk = c / nxy;
#pragma unroll
            for (int q = 0; q < 6; q++) {
                if (!(inf & (1u << q))) continue;
                const int dx = q == 0 ? -1 : (q == 1 ? 1 : 0);
                const int dy = q == 2 ? -1 : (q == 3 ? 1 : 0);
                const int dz = q == 4 ? -1 : (q == 5 ? 1 : 0);
                float zn = L.z[c + off[q]];
                const uint32_t P = uint32_t((i + dx) >> 1) + uint32_t(C->nx) * (uint32_t((j + dy) >> 1) +
                                   uint32_t(C->ny) * uint32_t((kk + dz) >> 1));
                if (C->info[P]) zn += C->z[P];
                sum += zn;
            }
        } else if (mode != 1) {
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (inf & (1u << q)) sum += L.z[c + off[q]];
        }
        L.z[c] = sum / cnt_of(inf);
    }
    __syncthreads();
}

__device__ void tail_restrict(const TailLevel& F, const TailLevel& Cc) {
    const int nx = F.nx, nxy = F.nx * F.ny;
    const int off[6] = {-1, 1, -nx, nx, -nxy, nxy};
    const uint32_t cnx = uint32_t(Cc.nx), cnxy = uint32_t(Cc.nx) * uint32_t(Cc.ny);
    for (uint32_t e = threadIdx.x; e < Cc.nsys; e += blockDim.x) {
        const uint32_t P = Cc.list[e];
        const int I = int(P % cnx), J = int((P / cnx) % uint32_t(Cc.ny)), K = int(P / cnxy);
        float sum = 0.0f;
#pragma unroll
        for (int chd = 0; chd < 8; chd++) {
            const int i = 2 * I + (chd & 1), j = 2 * J + ((chd >> 1) & 1), kk = 2 * K + (chd >> 2);
            if (i >= F.nx || j >= F.ny || kk >= F.nz) continue;
            const int c = i + nx * j + nxy * kk;
            const uint32_t inf = F.info[c];
            if (!inf) continue;
            float az = cnt_of(inf) * F.z[c];
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (inf & (1u << q)) az -= F.z[c + off[q]];
            sum += F.r[c] - az;
        }
        Cc.r[P] = 0.5f * sum;
    }
    __syncthreads();
}

__device__ void ph_tail(const SimDev* sims, int n_sims, float* tsm) {
    __shared__ double sh[32];
    // per tail level: list counts of its chunks and their offsets in the gathered list
    __shared__ uint32_t cr[kTailMaxLevels][kTailMaxChunks], cb[kTailMaxLevels][kTailMaxChunks];
    __shared__ uint32_t orr[kTailMaxLevels][kTailMaxChunks], obb[kTailMaxLevels][kTailMaxChunks];
    __shared__ uint32_t tot[kTailMaxLevels][2];
    for (int si = blockIdx.x; si < n_sims; si += gridDim.x) {
        const SimDev* sp = sims + si;
        if (sp->solver != 1 || sp->precond != 0) continue;
        const int T = sp->tail, NL = sp->nlev;
        TailLevel lv[kMaxLevels];
        float* base = tsm;
        // all levels at once, in three steps: records and list counts, offsets, list entries
        for (int l = T; l < NL; l++) {
            const MgLevel& g = sp->lev[l];
            TailLevel& t = lv[l];
            t.nx = g.nx; t.ny = g.ny; t.nz = g.nz; t.nc = g.nc;
            t.r = base;
            t.z = base + g.nc;
            t.info = reinterpret_cast<uint16_t*>(base + 2 * g.nc);
            t.list = t.info + g.nc;
            base += tail_level_floats(g.nc);
            for (uint32_t c = threadIdx.x; c < g.nc; c += blockDim.x) {
                const uint32_t inf = __ldcg(g.info + c);
                t.info[c] = in_system(inf) ? uint16_t(inf) : uint16_t(0);
            }
            const uint32_t nch = (g.nc + g.cs - 1) / g.cs;
            for (uint32_t k = threadIdx.x; k < nch; k += blockDim.x) {
                cr[l - T][k] = __ldcg(g.lcnt + 2 * k);
                cb[l - T][k] = __ldcg(g.lcnt + 2 * k + 1);
            }
        }
        __syncthreads();
        if (int(threadIdx.x) < NL - T) {
            const int lt = int(threadIdx.x);
            const MgLevel& g = sp->lev[T + lt];
            const uint32_t nch = (g.nc + g.cs - 1) / g.cs;
            uint32_t a = 0, b = 0;
            for (uint32_t k = 0; k < nch; k++) { orr[lt][k] = a; a += cr[lt][k]; }
            for (uint32_t k = 0; k < nch; k++) { obb[lt][k] = a + b; b += cb[lt][k]; }
            tot[lt][0] = a;
            tot[lt][1] = a + b;
        }
        __syncthreads();
        for (int l = T; l < NL; l++) {
            const MgLevel& g = sp->lev[l];
            TailLevel& t = lv[l];
            const int lt = l - T;
            t.nred = tot[lt][0];
            t.nsys = tot[lt][1];
            const uint32_t nch = (g.nc + g.cs - 1) / g.cs;
            for (uint32_t e = threadIdx.x; e < nch * g.cs; e += blockDim.x) {
                const uint32_t k = e / g.cs, m = e - k * g.cs;
                if (m < cr[lt][k]) t.list[orr[lt][k] + m] = uint16_t(__ldcg(g.list + e));
                else if (m < cr[lt][k] + cb[lt][k]) t.list[obb[lt][k] + m - cr[lt][k]] = uint16_t(__ldcg(g.list + e));
            }
        }
        __syncthreads();
        // everything above is fixed during the solve; r is the previous kernel's output
        dep_wait();
        if (__ldcg(&sp->pcg->done)) {
            __syncthreads();
            continue;
        }
        for (uint32_t c = threadIdx.x; c < lv[T].nc; c += blockDim.x) lv[T].r[c] = __ldcg(sp->lev[T].r + c);
        __syncthreads();
        const uint32_t pairs = sp->mg_pairs;
        for (int l = T; l + 1 < NL; l++) {
            tail_smooth(lv[l], 0, 1, nullptr);
            tail_smooth(lv[l], 1, 0, nullptr);
            for (uint32_t x = 1; x < pairs; x++) {
                tail_smooth(lv[l], 0, 0, nullptr);
                tail_smooth(lv[l], 1, 0, nullptr);
            }
            tail_restrict(lv[l], lv[l + 1]);
        }
        {
            const TailLevel& Lc = lv[NL - 1];
            for (uint32_t c = threadIdx.x; c < Lc.nc; c += blockDim.x) Lc.z[c] = 0.0f;
            __syncthreads();
            const uint32_t it = sp->coarse_iters;
            for (uint32_t h = 0; h < it; h++) { tail_smooth(Lc, 0, 0, nullptr); tail_smooth(Lc, 1, 0, nullptr); }
            for (uint32_t h = 0; h < it; h++) { tail_smooth(Lc, 1, 0, nullptr); tail_smooth(Lc, 0, 0, nullptr); }
        }
        for (int l = NL - 2; l >= T; l--) {
            tail_smooth(lv[l], 1, 2, &lv[l + 1]);
            tail_smooth(lv[l], 0, 0, nullptr);
            for (uint32_t x = 1; x < pairs; x++) {
                tail_smooth(lv[l], 1, 0, nullptr);
                tail_smooth(lv[l], 0, 0, nullptr);
            }
        }
        {
            const MgLevel g = sp->lev[T];
            for (uint32_t c = threadIdx.x; c < g.nc; c += blockDim.x) g.z[c] = lv[T].z[c];
        }
        if (T == 0) {
            // level-0 chunk partials of r.z (the tail holds the whole level)
            const uint32_t nch = nchunks0(*sp);
            for (uint32_t ch = 0; ch < nch; ch++) {
                DF acc{0.f, 0.f};
                const uint32_t cs0 = sp->lev[0].cs;
                const uint32_t end = min((ch + 1) * cs0, sp->nc);
                for (uint32_t c = ch * cs0 + threadIdx.x; c < end; c += blockDim.x)
                    if (lv[0].info[c]) acc = df_add(acc, two_prod(lv[0].r[c], lv[0].z[c]));
                const double t = block_sum(acc, sh);
                if (threadIdx.x == 0) sp->partial[ch] = t;
            }
        }
        __syncthreads();
    }
}

// Jacobi preconditioner: z = r / cnt, partial r.z.
__device__ void ph_jacobi(const Work& w) {
    __shared__ double sh[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1 || s.precond != 1) continue;
        const uint32_t chunk = item - w.base[si];
        DF acc{0.f, 0.f};
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t* lst = list_of(s.lev[0], chunk);
        dep_wait();
        if (ldu(&s.pcg->done)) continue;
        for (uint32_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            const uint32_t inf = s.info[c];
            const float r = s.r[c];
            const float z = r / cnt_of(inf);
            s.z[c] = z;
            acc = df_add(acc, two_prod(r, z));
        }
        const double t = block_sum(acc, sh);
        if (threadIdx.x == 0) s.partial[chunk] = t;
    }
}

// Partial |b|^2.
__device__ void ph_init(const Work& w) {
    __shared__ double sh[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        DF acc{0.f, 0.f};
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t* lst = list_of(s.lev[0], chunk);
        for (uint32_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            const float b = rhs_of(s, lst[e]);
            acc = df_add(acc, two_prod(b, b));
        }
        const double t = block_sum(acc, sh);
        if (threadIdx.x == 0) s.partial[chunk] = t;
    }
}

// x64 = hi + lo for simulations about to restart (or x = 0 for a zero right-hand side).
__device__ void ph_widen(const Work& w) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t* lst = list_of(s.lev[0], chunk);
        dep_wait();
        if (ldu(&s.pcg->done) || !ldu(&s.pcg->restart_now)) continue;
        const bool zero = ldu(&s.pcg->zero_x) != 0;
        for (uint32_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            if (zero) {
                s.x2[c] = make_float2(0.f, 0.f);
                s.x64[c] = 0.0;
            } else {
                const float2 x = s.x2[c];
                s.x64[c] = double(x.x) + double(x.y);
            }
        }
    }
}

// FP64 restart residual r = b - A x and its partial |r|^2.
__device__ void ph_resid(const Work& w) {
    __shared__ double sh[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        const int64_t nx = s.nx, nxy = int64_t(s.nx) * s.ny;
        double rr = 0;
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t* lst = list_of(s.lev[0], chunk);
        dep_wait();
        if (ldu(&s.pcg->done) || !ldu(&s.pcg->restart_now) || ldu(&s.pcg->zero_x)) continue;
        // as in ph_update: the level-0 red half sweep from zero
        const uint32_t nred = (s.precond == 0 && s.tail > 0) ? __ldcg(s.lev[0].lcnt + 2 * chunk) : 0u;
        for (uint32_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            const uint32_t inf = s.info[c];
            double ax = double(cnt_of(inf)) * s.x64[c];
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (inf & (1u << q)) ax -= s.x64[int64_t(c) + nbr(q, nx, nxy)];
            const double rd = -double(rhs_of(s, c)) - ax;
            const float rf = float(rd);
            s.r[c] = rf;
            if (e < nred) s.lev[0].z[c] = rf / cnt_of(inf);
            rr += rd * rd;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) rr += __shfl_down_sync(0xffffffffu, rr, d);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = rr;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int k2 = 0; k2 < int(blockDim.x >> 5); k2++) t += sh[k2];
            s.partial[chunk] = t;
        }
        __syncthreads();
    }
}

// The level-0 kernels of the CG loop read each thread's first two list entries and their
// neighbour records before dep_wait() (the lists are fixed during the solve), then issue the
// loads of both cells together; entries beyond the first two (chunks with more than
// 2 x 256 system cells) follow in a plain loop. The per-thread order of the reductions is the
// list order either way.
struct Two {
    uint32_t e0, e1, c0, c1, i0, i1;
    bool h0, h1;
};

__device__ __forceinline__ Two first_two(const uint32_t* lst, const uint16_t* info, uint32_t lo, uint32_t hi) {
    Two t;
    t.e0 = lo + threadIdx.x;
    t.e1 = t.e0 + blockDim.x;
    t.h0 = t.e0 < hi;
    t.h1 = t.e1 < hi;
    t.c0 = t.h0 ? __ldcg(lst + t.e0) : 0u;
    t.c1 = t.h1 ? __ldcg(lst + t.e1) : 0u;
    t.i0 = t.h0 ? uint32_t(info[t.c0]) : 0u;
    t.i1 = t.h1 ? uint32_t(info[t.c1]) : 0u;
    return t;
}

// p' = z + beta p (p' = z after a restart) at cell c and its six neighbours; Ap' = A p'.
struct DirCell {
    float pn, ap;
};

__device__ __forceinline__ DirCell dir_cell(uint32_t c, uint32_t inf, const float* __restrict__ z,
                                            const float* __restrict__ pold, bool fresh, float beta,
                                            int64_t nx, int64_t nxy) {
    const float pn = fresh ? z[c] : z[c] + beta * pold[c];
    float ap = cnt_of(inf) * pn;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        if (inf & (1u << q)) {
            const int64_t n = int64_t(c) + nbr(q, nx, nxy);
            ap -= fresh ? z[n] : z[n] + beta * pold[n];
        }
    }
    return {pn, ap};
}

// p' = z + beta p (p' = z after a restart); Ap = A p' (neighbours' p' formed on the fly);
// partial p'.Ap.
__device__ void ph_dir(const Work& w) {
    __shared__ double sh[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t* __restrict__ lst = list_of(s.lev[0], chunk);
        const uint16_t* __restrict__ info = s.info;
        const Two t = first_two(lst, info, lo, hi);
        dep_wait();
        const PcgState* st = s.pcg;
        const uint32_t done = ldu(&st->done);
        const uint32_t pbuf = ldu(&st->pbuf);
        const bool fresh = ldu(&st->fresh) != 0;
        const double betad = ldd(&st->beta);
        const float* __restrict__ z = s.z;
        const int64_t nx = s.nx, nxy = int64_t(s.nx) * s.ny;
        // the first two cells' z and p of both direction buffers, issued with the scalars (which
        // buffer holds the old direction is one of them)
        float za[2][7], pa[2][7], pb[2][7];
        const uint32_t cc[2] = {t.c0, t.c1}, ii[2] = {t.i0, t.i1};
        const bool hh[2] = {t.h0, t.h1};
#pragma unroll
        for (int u = 0; u < 2; u++) {
#pragma unroll
            for (int q = 0; q < 7; q++) {
                za[u][q] = 0.f;
                pa[u][q] = 0.f;
                pb[u][q] = 0.f;
            }
            if (!hh[u]) continue;
            za[u][6] = z[cc[u]];
            pa[u][6] = s.p0[cc[u]];
            pb[u][6] = s.p1[cc[u]];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                if (!(ii[u] & (1u << q))) continue;
                const int64_t n = int64_t(cc[u]) + nbr(q, nx, nxy);
                za[u][q] = z[n];
                pa[u][q] = s.p0[n];
                pb[u][q] = s.p1[n];
            }
        }
        if (done) continue;
        const float beta = fresh ? 0.0f : float(betad);
        const float* __restrict__ pold = pbuf ? s.p1 : s.p0;
        float* __restrict__ pnew = pbuf ? s.p0 : s.p1;
        float* __restrict__ Ap = s.Ap;
        DF acc{0.f, 0.f};
        DirCell dd[2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (!hh[u]) continue;
            // dir_cell's arithmetic on the values loaded above
            const float* po = pbuf ? pb[u] : pa[u];
            const float pn = fresh ? za[u][6] : za[u][6] + beta * po[6];
            float ap = cnt_of(ii[u]) * pn;
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (ii[u] & (1u << q)) ap -= fresh ? za[u][q] : za[u][q] + beta * po[q];
            dd[u] = {pn, ap};
        }
        const DirCell d0 = dd[0], d1 = dd[1];
        if (t.h0) {
            pnew[t.c0] = d0.pn;
            Ap[t.c0] = d0.ap;
            acc = df_add(acc, two_prod(d0.pn, d0.ap));
        }
        if (t.h1) {
            pnew[t.c1] = d1.pn;
            Ap[t.c1] = d1.ap;
            acc = df_add(acc, two_prod(d1.pn, d1.ap));
        }
        for (uint32_t e = t.e1 + blockDim.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            const DirCell d = dir_cell(c, info[c], z, pold, fresh, beta, nx, nxy);
            pnew[c] = d.pn;
            Ap[c] = d.ap;
            acc = df_add(acc, two_prod(d.pn, d.ap));
        }
        const double tt = block_sum(acc, sh);
        if (threadIdx.x == 0) s.partial[chunk] = tt;
    }
}

// x += alpha p (double-float), r -= alpha Ap (FP32), partial |r|^2; on multigrid simulations
// also the V-cycle's first half sweep on level 0 (red from zero: z = r / cnt).
__device__ void ph_update(const Work& w) {
    __shared__ double sh[32];
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        uint32_t lo, hi;
        seg(s.lev[0], chunk, 2, lo, hi);
        const uint32_t nred = (s.precond == 0 && s.tail > 0) ? __ldcg(s.lev[0].lcnt + 2 * chunk) : 0u;
        const uint32_t* __restrict__ lst = list_of(s.lev[0], chunk);
        const Two t = first_two(lst, s.info, lo, hi);
        dep_wait();
        const PcgState* st = s.pcg;
        float2* __restrict__ x2 = s.x2;
        float* __restrict__ r = s.r;
        const float* __restrict__ Ap = s.Ap;
        float* __restrict__ z = s.lev[0].z;
        const uint32_t done = ldu(&st->done);
        const uint32_t pbuf = ldu(&st->pbuf);
        const float ah = ldf(&st->alpha_hi), al = ldf(&st->alpha_lo);
        const float af = float(ldd(&st->alpha));
        // the first two cells' vectors, issued with the scalars (none depends on them)
        float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
        float r0 = 0.f, r1 = 0.f, a0 = 0.f, a1 = 0.f;
        if (t.h0) { x0 = x2[t.c0]; r0 = r[t.c0]; a0 = Ap[t.c0]; }
        if (t.h1) { x1 = x2[t.c1]; r1 = r[t.c1]; a1 = Ap[t.c1]; }
        // p of both direction buffers (which one is current is among the scalars above)
        const float q00 = t.h0 ? s.p0[t.c0] : 0.f, q01 = t.h0 ? s.p1[t.c0] : 0.f;
        const float q10 = t.h1 ? s.p0[t.c1] : 0.f, q11 = t.h1 ? s.p1[t.c1] : 0.f;
        if (done) continue;
        const float* __restrict__ p = pbuf ? s.p1 : s.p0;
        const float p0v = pbuf ? q01 : q00, p1v = pbuf ? q11 : q10;
        DF acc{0.f, 0.f};
        auto one = [&](uint32_t e, uint32_t c, uint32_t inf, float pc, float2 x, float rc, float apc) {
            DF d = two_prod(ah, pc);
            d.lo += al * pc;
            const DF xn = df_add(DF{x.x, x.y}, d);
            x2[c] = make_float2(xn.hi, xn.lo);
            const float rn = rc - af * apc;
            r[c] = rn;
            if (e < nred) z[c] = rn / cnt_of(inf);
            acc = df_add(acc, two_prod(rn, rn));
        };
        if (t.h0) one(t.e0, t.c0, t.i0, p0v, x0, r0, a0);
        if (t.h1) one(t.e1, t.c1, t.i1, p1v, x1, r1, a1);
        for (uint32_t e = t.e1 + blockDim.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            one(e, c, s.info[c], p[c], x2[c], r[c], Ap[c]);
        }
        const double tt = block_sum(acc, sh);
        if (threadIdx.x == 0) s.partial[chunk] = tt;
    }
}

// FP32 pressure copy and the FP64 solution at the end of the solve (all cells).
__device__ void ph_finish(const Work& w) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t cs0 = s.lev[0].cs;
        for (uint32_t k = 0; k < cs0 / blockDim.x; k++) {
            const uint32_t c = (item - w.base[si]) * cs0 + k * blockDim.x + threadIdx.x;
            if (c >= s.nc) continue;
            double x = 0.0;
            if (in_system(s.info[c])) {
                const float2 v = s.x2[c];
                x = double(v.x) + double(v.y);
            }
            s.x64[c] = x;
            s.pressure[c] = float(x);
        }
    }
}

// Control: one block per simulation sums the partials of the step before it and advances the
// state. phase 0: after |b|^2   1: after the restart residual   2: after r.z   3: after p.Ap
// 4: after |r|^2
__device__ void ph_ctl(const SimDev* sims, int n_sims, int phase) {
    __shared__ double sh[32];
    dep_wait();
    for (int si = blockIdx.x; si < n_sims; si += gridDim.x) {
        const SimDev& s = sims[si];
        if (s.solver != 1) continue;
        PcgState* st = s.pcg;
        if (phase != 0 && __ldcg(&st->done)) continue;
        if (phase == 1 && !__ldcg(&st->restart_now)) continue;
        const bool zero = phase == 1 && __ldcg(&st->zero_x);
        const double a = zero ? 0.0 : sum_partials(s, sh);
        if (threadIdx.x == 0) switch (phase) {
            case 0:
                st->bb = a;
                st->iters = 0;
                st->since = 0;
                st->done = 0;
                st->fresh = 1;
                st->status = 0;
                st->relres = 0;
                st->beta = 0;
                st->restart_now = 1;
                st->zero_x = a == 0.0 ? 1u : 0u;
                break;
            case 1:
                if (zero) {
                    st->done = 1;
                    st->status = 3;
                    st->relres = 0;
                } else {
                    const double tol2 = s.rtol * s.rtol * st->bb;
                    st->relres = sqrt(a / st->bb);
                    if (a <= tol2 || st->iters >= s.max_iter) {
                        st->done = 1;
                        st->status = a <= tol2 ? 0u : 1u;
                    }
                }
                break;
            case 2:
                if (st->restart_now) {
                    st->rz = a;
                    st->fresh = 1;
                    st->since = 0;
                    st->restart_now = 0;
                } else {
                    st->beta = a / st->rz;
                    st->rz = a;
                    st->fresh = 0;
                }
                break;
            case 3:
                st->pAp = a;
                st->pbuf ^= 1u;   // p' is now the current direction
                if (!(a > 0.0)) {
                    st->done = 1;
                    st->status = 2;
                } else {
                    const double alpha = st->rz / a;
                    st->alpha = alpha;
                    st->alpha_hi = float(alpha);
                    st->alpha_lo = float(alpha - double(float(alpha)));
                }
                break;
            default: {
                const double tol2 = s.rtol * s.rtol * st->bb;
                st->rr = a;
                st->iters += 1;
                st->since += 1;
                if (a <= tol2 || st->since >= s.restart || st->iters >= s.max_iter) st->restart_now = 1;
                break;
            }
        }
    }
}

__device__ __forceinline__ bool any_active(const SimDev* sims, int n_sims) {
    for (int i = 0; i < n_sims; i++)
        if (sims[i].solver == 1 && !__ldcg(&sims[i].pcg->done)) return true;
    return false;
}

__device__ __forceinline__ bool any_restart(const SimDev* sims, int n_sims) {
    for (int i = 0; i < n_sims; i++)
        if (sims[i].solver == 1 && !__ldcg(&sims[i].pcg->done) && __ldcg(&sims[i].pcg->restart_now)) return true;
    return false;
}

// ============================================================================ standalone kernels
__global__ void __launch_bounds__(THREADS) k_cell_lists(Work w, int l) { ph_cell_lists(w, l); }
__global__ void __launch_bounds__(THREADS) k_mg_coarsen(Work w, int l) { ph_coarsen(w, l); }
__global__ void __launch_bounds__(THREADS) k_mg_info(Work w, int l) { ph_info(w, l); }
__global__ void __launch_bounds__(THREADS) k_mg_smooth(Work w, int l, int color, int mode, int pass) {
    ph_smooth(w, l, color, mode, pass);
    dep_wait();
}
__global__ void __launch_bounds__(THREADS) k_mg_restrict(Work w, int l) { ph_restrict(w, l); dep_wait(); }
__global__ void __launch_bounds__(1024, 1) k_mg_tail(const SimDev* sims, int n_sims) {
    extern __shared__ float tsm[];
    ph_tail(sims, n_sims, tsm);
    dep_wait();
}
__global__ void __launch_bounds__(THREADS) k_compact(PcgWork pw) { ph_compact(pw); }

// ---------------------------------------------------------------- reference red-black GS
// Level-0 lists of the simulations that use the reference red-black Gauss-Seidel solve.
__global__ void __launch_bounds__(THREADS) k_gs_lists(Work w) { ph_cell_lists(w, 0, 0); }

// One colour of one red-black iteration (shaders/fluid.slang:167-182) over the colour's system
// cells of each chunk, the cells the reference updates (fluid, at least one non-solid
// neighbour): p = (sum of fluid neighbours' p in the order -x +x -y +y -z +z - div h h / dt) / cnt.
// A cell reads only the other colour, so visiting the list instead of the grid changes no bit.
// Before dep_wait() only what stays fixed during the solve is read (lists, records, divergence).
__global__ void __launch_bounds__(THREADS) k_pressure_rb_list(Work w, uint32_t parity, uint32_t it) {
    for (uint32_t w_k = blockIdx.x, w_n = work_count(w); w_k < w_n; w_k += gridDim.x) {
        const uint32_t item = work_item(w, w_k);
        const int si = find_sim(w, item);
        const SimDev* sp = w.sims + si;
        if (sp->solver != 0 || it >= sp->iterations) continue;
        const uint32_t chunk = item - w.base[si];
        const MgLevel& L = sp->lev[0];
        uint32_t lo, hi;
        seg(L, chunk, int(parity), lo, hi);
        const uint32_t* __restrict__ lst = list_of(L, chunk);
        const uint32_t e0 = lo + threadIdx.x;
        const bool h0 = e0 < hi;
        const uint32_t c0 = h0 ? __ldcg(lst + e0) : 0u;
        const uint32_t i0 = h0 ? uint32_t(sp->info[c0]) : 0u;
        const float rhs_h = sp->h, rhs_dt = sp->dt;
        const float d0 = h0 ? sp->div[c0] : 0.0f;
        const uint32_t nx = uint32_t(sp->nx), nxy = nx * uint32_t(sp->ny);
        float* __restrict__ p = sp->pressure;
        dep_wait();
        auto cell = [&](uint32_t c, uint32_t inf, float dv) {
            float sum = 0.0f;
            if (inf & 1u) sum += p[c - 1];
            if (inf & 2u) sum += p[c + 1];
            if (inf & 4u) sum += p[c - nx];
            if (inf & 8u) sum += p[c + nx];
            if (inf & 16u) sum += p[c - nxy];
            if (inf & 32u) sum += p[c + nxy];
            p[c] = (sum - dv * rhs_h * rhs_h / rhs_dt) / float((inf >> 8) & 7u);
        };
        if (h0) cell(c0, i0, d0);
        for (uint32_t e = e0 + blockDim.x; e < hi; e += blockDim.x) {
            const uint32_t c = lst[e];
            cell(c, sp->info[c], sp->div[c]);
        }
    }
    dep_wait();
}
__global__ void __launch_bounds__(THREADS) k_jacobi(Work w) { ph_jacobi(w); dep_wait(); }
__global__ void __launch_bounds__(THREADS) k_pcg_init(Work w) { ph_init(w); }
__global__ void __launch_bounds__(THREADS) k_pcg_widen(Work w) { ph_widen(w); dep_wait(); }
__global__ void __launch_bounds__(THREADS) k_pcg_resid(Work w) { ph_resid(w); dep_wait(); }
__global__ void __launch_bounds__(THREADS) k_pcg_dir(Work w) { ph_dir(w); dep_wait(); }
__global__ void __launch_bounds__(THREADS) k_pcg_update(Work w) { ph_update(w); dep_wait(); }
__global__ void __launch_bounds__(THREADS) k_pcg_finish(Work w) { ph_finish(w); }
// With a ticket, the block that finishes last also sets the loop's conditional handle: after a
// restart decision (phase 4) whether any simulation restarts, after r.z (phase 2) whether any is
// still solving. Each block publishes its state (fence) before taking its ticket, and the last one
// resets the ticket for the next use.
__global__ void __launch_bounds__(THREADS) k_pcg_ctl(const SimDev* sims, int n_sims, int phase,
                                                     cudaGraphConditionalHandle h, uint32_t* ticket) {
    ph_ctl(sims, n_sims, phase);
    if (!ticket) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            const bool any = phase == 4 ? any_restart(sims, n_sims) : any_active(sims, n_sims);
            cudaGraphSetConditional(h, any ? 1u : 0u);
            *ticket = 0;
        }
    }
}

// The same control step without a conditional handle (host-driven loop): no handle-setting
// code in the graph, which kernel profilers require.
__global__ void __launch_bounds__(THREADS) k_pcg_ctl_plain(const SimDev* sims, int n_sims, int phase) {
    ph_ctl(sims, n_sims, phase);
}

__global__ void k_pcg_cond(const SimDev* sims, int n_sims, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    cudaGraphSetConditional(h, any_active(sims, n_sims) ? 1u : 0u);
}

__global__ void k_pcg_any(const SimDev* sims, int n_sims, uint32_t* flag) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    *flag = any_active(sims, n_sims) ? 1u : 0u;
}

// ============================================================================ persistent solve
// Sense-reversing grid barrier on one word: block 0 adds 2^31 - (blocks - 1), every other block
// adds 1, so the word's top bit flips exactly when the last block arrives and its low 31 bits
// return to zero. Each block waits for the flip, at most kBarrierCycles; a block that gives up
// sets `err` and every block leaves the solve at its next barrier. The launch zeroes the whole
// GridBar, so a barrier left half-passed by an abandoned launch never reaches the next one.
__device__ __forceinline__ bool grid_sync(GridBar* b, long long limit = kBarrierCycles) {
    __shared__ int bad;
    __syncthreads();
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> word(b->count), err(b->err);
        const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
        __threadfence();
        const unsigned old = word.fetch_add(inc, cuda::memory_order_relaxed);
        const long long t0 = clock64();
        while (((word.load(cuda::memory_order_acquire) ^ old) & 0x80000000u) == 0u) {
            if (err.load(cuda::memory_order_relaxed) || clock64() - t0 > limit) {
                err.store(1u, cuda::memory_order_relaxed);
                break;
            }
        }
        __threadfence();
        bad = err.load(cuda::memory_order_relaxed) != 0u;
    }
    __syncthreads();
    return !bad;
}

struct SolveArgs {
    PcgWork pw;
    GridBar* bar;
    uint32_t guard;   // bound on the CG loop (largest iteration cap of the batch + 2)
};

#define SYNC_OR_RETURN() \
    if (!grid_sync(a.bar)) return

__device__ bool solve_precond(const SolveArgs& a, float* tsm) {
    const PcgWork& pw = a.pw;
    if (pw.any_jacobi) {
        ph_jacobi(pw.chunks);
        if (!grid_sync(a.bar)) return false;
    }
    if (pw.any_mg) {
        for (int l = 0; l + 1 < pw.max_levels; l++) {
            if (!pw.level[l].total) continue;
            ph_smooth(pw.level[l], l, 1, 0, 0);
            if (!grid_sync(a.bar)) return false;
            for (int x = 1; x < pw.max_pairs; x++) {
                ph_smooth(pw.level[l], l, 0, 0, x);
                if (!grid_sync(a.bar)) return false;
                ph_smooth(pw.level[l], l, 1, 0, x);
                if (!grid_sync(a.bar)) return false;
            }
            ph_restrict(pw.coarse[l], l);
            if (!grid_sync(a.bar)) return false;
        }
        ph_tail(pw.sims, pw.n_sims, tsm);
        if (!grid_sync(a.bar)) return false;
        for (int l = pw.max_levels - 2; l >= 0; l--) {
            if (!pw.level[l].total) continue;
            for (int x = 0; x < pw.max_pairs; x++) {
                ph_smooth(pw.level[l], l, 1, x == 0 ? 2 : 0, x);
                if (!grid_sync(a.bar)) return false;
                ph_smooth(pw.level[l], l, 0, l == 0 ? 3 : 0, x);
                if (!grid_sync(a.bar)) return false;
            }
        }
    }
    ph_ctl(pw.sims, pw.n_sims, 2);
    return grid_sync(a.bar);
}

__device__ bool solve_restart(const SolveArgs& a) {
    const PcgWork& pw = a.pw;
    ph_widen(pw.chunks);
    if (!grid_sync(a.bar)) return false;
    ph_resid(pw.chunks);
    if (!grid_sync(a.bar)) return false;
    ph_ctl(pw.sims, pw.n_sims, 1);
    return grid_sync(a.bar);
}

__global__ void __launch_bounds__(THREADS) k_pcg_solve(SolveArgs a) {
    extern __shared__ float tsm[];
    const PcgWork& pw = a.pw;
    // multigrid setup: system-cell lists and the coarse levels
    ph_cell_lists(pw.chunks_all, 0);
    SYNC_OR_RETURN();
    for (int l = 0; l + 1 < pw.setup_levels; l++) {
        if (!pw.setup[l].total) continue;
        ph_coarsen(pw.setup[l], l);
        SYNC_OR_RETURN();
        ph_info(pw.setup[l], l);
        SYNC_OR_RETURN();
        ph_cell_lists(pw.setup[l], l + 1);
        SYNC_OR_RETURN();
    }
    if (pw.act_n) {
        ph_compact(pw);
        SYNC_OR_RETURN();
    }
    ph_init(pw.chunks);
    SYNC_OR_RETURN();
    ph_ctl(pw.sims, pw.n_sims, 0);
    SYNC_OR_RETURN();
    if (!solve_restart(a)) return;
    if (!solve_precond(a, tsm)) return;
    for (uint32_t guard = 0; guard < a.guard; guard++) {
        if (!any_active(pw.sims, pw.n_sims)) break;
        ph_dir(pw.chunks);
        SYNC_OR_RETURN();
        ph_ctl(pw.sims, pw.n_sims, 3);
        SYNC_OR_RETURN();
        ph_update(pw.chunks);
        SYNC_OR_RETURN();
        ph_ctl(pw.sims, pw.n_sims, 4);
        SYNC_OR_RETURN();
        if (any_restart(pw.sims, pw.n_sims) && !solve_restart(a)) return;
        if (!solve_precond(a, tsm)) return;
    }
    ph_finish(pw.chunks_all);
}

// ---------------------------------------------------------------- cooperative smoothing
// One level's pre-smoothing (with the restriction below it) or post-smoothing as one cooperative
// launch: its half sweeps run as phases separated by the bounded grid barrier instead of one
// dependent launch each. Block b owns the level's chunks b, b + grid, ... (at most kCoopCPB);
// their cell lists and neighbour records, fixed during the solve, are read into shared memory once
// and every sweep then reads only r and z. In each round a thread takes one list entry of each of
// its block's chunks and issues all their loads before any store. Every block reaches every
// barrier (phases skip work, never return early); a barrier that times out sets the error flag and
// the blocks return.
constexpr int kCoopCPB = 4;

struct CoopChunk {
    uint32_t si, chunk, nred, nsys;   // nsys = 0: nothing to smooth (no chunk, other solver, done)
};

__device__ __forceinline__ void coop_sweep(const Work& lw, int l, int color, int mode_in, int pass, const CoopChunk* ch,
                                           const uint32_t* cells, const uint16_t* infos, uint32_t cs, double* sh) {
    constexpr int J = kCoopCPB;
    // per chunk: effective mode (-1: skip) and colour segment
    int mode[J];
    uint32_t lo[J], hi[J];
    uint32_t rounds = 0;
#pragma unroll
    for (int j = 0; j < J; j++) {
        mode[j] = -1;
        lo[j] = hi[j] = 0;
        if (!ch[j].nsys) continue;
        const SimDev* sp = lw.sims + ch[j].si;
        if (uint32_t(pass) >= sp->mg_pairs) continue;
        mode[j] = (mode_in == 3 && uint32_t(pass) + 1 != sp->mg_pairs) ? 0 : mode_in;
        lo[j] = color == 1 ? ch[j].nred : 0u;
        hi[j] = color == 0 ? ch[j].nred : ch[j].nsys;
        rounds = max(rounds, (hi[j] - lo[j] + blockDim.x - 1) / blockDim.x);
    }
    for (uint32_t rr = 0; rr < rounds; rr++) {
        float rv[J], zn[J][6], zc[J][6];
        uint32_t cc[J], ii[J], pin[J];
        uint32_t P[J][6];
#pragma unroll
        for (int j = 0; j < J; j++) {
            const uint32_t e = lo[j] + threadIdx.x + rr * blockDim.x;
            const bool h = mode[j] >= 0 && e < hi[j];
            cc[j] = h ? cells[j * cs + e] : 0u;
            ii[j] = h ? uint32_t(infos[j * cs + e]) : 0u;   // zero record: nothing to do
            pin[j] = 0;
            rv[j] = 0.0f;
#pragma unroll
            for (int q = 0; q < 6; q++) { zn[j][q] = 0.0f; zc[j][q] = 0.0f; P[j][q] = 0u; }
            if (!h) continue;
            const SimDev* sp = lw.sims + ch[j].si;
            const MgLevel& L = sp->lev[l];
            const uint32_t nx = uint32_t(L.nx), ny = uint32_t(L.ny), nxy = nx * ny;
            rv[j] = L.r[cc[j]];
            if (mode[j] != 1) {
#pragma unroll
                for (int q = 0; q < 6; q++)
                    if (ii[j] & (1u << q)) zn[j][q] = L.z[uint32_t(int64_t(cc[j]) + nbr(q, nx, nxy))];
            }
            if (mode[j] == 2) {
                const MgLevel& Cc = sp->lev[l + 1];
                const uint32_t cnx = uint32_t(Cc.nx), cnxy = uint32_t(Cc.nx) * uint32_t(Cc.ny);
                const uint32_t c = cc[j], i = c % nx, jj = (c / nx) % ny, kk = c / nxy;
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    if (!(ii[j] & (1u << q))) continue;
                    const int dx = q == 0 ? -1 : (q == 1 ? 1 : 0);
                    const int dy = q == 2 ? -1 : (q == 3 ? 1 : 0);
                    const int dz = q == 4 ? -1 : (q == 5 ? 1 : 0);
                    P[j][q] = (uint32_t(int(i) + dx) >> 1) + cnx * (uint32_t(int(jj) + dy) >> 1) +
                              cnxy * (uint32_t(int(kk) + dz) >> 1);
                    if (in_system(Cc.info[P[j][q]])) {
                        pin[j] |= 1u << q;
                        zc[j][q] = Cc.z[P[j][q]];
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
            if (!ii[j]) continue;
            // the same sums, in the same order, as ph_smooth
            float sum = rv[j];
            if (mode[j] == 2) {
#pragma unroll
                for (int q = 0; q < 6; q++) {
                    if (!(ii[j] & (1u << q))) continue;
                    float t = zn[j][q];
                    if (pin[j] & (1u << q)) t += zc[j][q];
                    sum += t;
                }
            } else if (mode[j] != 1) {
#pragma unroll
                for (int q = 0; q < 6; q++)
                    if (ii[j] & (1u << q)) sum += zn[j][q];
            }
            lw.sims[ch[j].si].lev[l].z[cc[j]] = sum / cnt_of(ii[j]);
        }
    }
    // r.z partials of the chunks whose last post-smoothing sweep this was (block-uniform)
    bool any3 = false;
#pragma unroll
    for (int j = 0; j < J; j++) any3 |= mode[j] == 3;
    if (any3) {
        __syncthreads();
#pragma unroll
        for (int j = 0; j < J; j++) {
            if (mode[j] != 3) continue;
            const SimDev* sp = lw.sims + ch[j].si;
            const MgLevel& L = sp->lev[l];
            DF acc{0.f, 0.f};
            for (uint32_t e = threadIdx.x; e < ch[j].nsys; e += blockDim.x) {
                const uint32_t c = cells[j * cs + e];
                acc = df_add(acc, two_prod(L.r[c], L.z[c]));
            }
            const double t = block_sum(acc, sh);
            if (threadIdx.x == 0) sp->partial[ch[j].chunk] = t;
        }
    }
}

// side 0: pre-smoothing and the restriction to level l+1; side 1: post-smoothing.
__global__ void __launch_bounds__(THREADS, 4) k_mg_level(Work lw, Work cw, int l, int side, int pairs, uint32_t cs,
                                                      GridBar* bar) {
    extern __shared__ uint32_t coop_mem[];
    __shared__ CoopChunk ch[kCoopCPB];
    __shared__ double sh[32];
    uint32_t* cells = coop_mem;
    uint16_t* infos = reinterpret_cast<uint16_t*>(coop_mem + kCoopCPB * cs);
    if (threadIdx.x < kCoopCPB) {
        CoopChunk c{0u, 0u, 0u, 0u};
        const uint32_t k = blockIdx.x + threadIdx.x * gridDim.x;
        if (k < lw.total) {
            const int si = find_sim(lw, k);
            const SimDev* sp = lw.sims + si;
            if (sp->solver == 1 && sp->precond == 0 && !ldu(&sp->pcg->done)) {
                const MgLevel& L = sp->lev[l];
                c.si = uint32_t(si);
                c.chunk = k - lw.base[si];
                c.nred = __ldcg(L.lcnt + 2 * c.chunk);
                c.nsys = c.nred + __ldcg(L.lcnt + 2 * c.chunk + 1);
            }
        }
        ch[threadIdx.x] = c;
    }
    __syncthreads();
    for (int j = 0; j < kCoopCPB; j++) {
        if (!ch[j].nsys) continue;
        const MgLevel& L = lw.sims[ch[j].si].lev[l];
        const uint32_t* lst = list_of(L, ch[j].chunk);
        for (uint32_t e = threadIdx.x; e < ch[j].nsys; e += blockDim.x) {
            const uint32_t c = __ldcg(lst + e);
            cells[j * cs + e] = c;
            infos[j * cs + e] = L.info[c];
        }
    }
    __syncthreads();
    if (side == 0) {
        coop_sweep(lw, l, 1, 0, 0, ch, cells, infos, cs, sh);
        for (int x = 1; x < pairs; x++) {
            if (!grid_sync(bar)) return;
            coop_sweep(lw, l, 0, 0, x, ch, cells, infos, cs, sh);
            if (!grid_sync(bar)) return;
            coop_sweep(lw, l, 1, 0, x, ch, cells, infos, cs, sh);
        }
        if (!grid_sync(bar)) return;
        ph_restrict(cw, l);
    } else {
        for (int x = 0; x < pairs; x++) {
            if (x && !grid_sync(bar)) return;
            coop_sweep(lw, l, 1, x == 0 ? 2 : 0, x, ch, cells, infos, cs, sh);
            if (!grid_sync(bar)) return;
            coop_sweep(lw, l, 0, l == 0 ? 3 : 0, x, ch, cells, infos, cs, sh);
        }
    }
}

// ============================================================================ launchers
// One block per work item (chunk): chunks of the air exit at once, and the block scheduler hands
// the rest to whichever SM frees first.
static unsigned grid_of(uint32_t total) { return total ? total : 1u; }

static inline Work mkw(const StageWork& sw) { return sw; }

// Grid of a stage: one block per item for a full stage; for a compacted stage (its length is
// known only on the device) at most 8 blocks per SM, block-strided over the list.
static unsigned grid_w(const StageWork& w) {
    if (!w.act) return grid_of(w.total);
    // PXF_CG_BLOCKS_PER_SM: blocks per SM of a compacted stage (default 8); a stage with at most
    // that many items gets one block per item.
    static const uint32_t per_sm = [] {
        const char* v = std::getenv("PXF_CG_BLOCKS_PER_SM");
        const int k = v ? std::atoi(v) : 8;
        return uint32_t(k > 0 ? k : 8);
    }();
    const uint32_t cap = uint32_t(sm_count()) * per_sm;
    return w.total < cap ? (w.total ? w.total : 1u) : cap;
}

// Launch of a CG-loop kernel with programmatic stream serialization (it may start while the
// kernel before it drains; see dep_wait). PXF_PDL=0 launches them in plain stream order.
template <typename... KArgs, typename... Args>
static void launch_dep(const char* name, void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem,
                       cudaStream_t st, Args... args) {
    static const bool pdl = [] { const char* v = std::getenv("PXF_PDL"); return !(v && v[0] == '0'); }();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, KArgs(args)...);
    note_launch(name, st);
}

static cudaError_t ctl(const PcgWork& pw, int phase, cudaStream_t st, cudaGraphConditionalHandle h = 0,
                       uint32_t* ticket = nullptr) {
    if (ticket) launch_dep("k_pcg_ctl", k_pcg_ctl, pw.n_sims, THREADS, 0, st, pw.sims, pw.n_sims, phase, h, ticket);
    else launch_dep("k_pcg_ctl", k_pcg_ctl_plain, pw.n_sims, THREADS, 0, st, pw.sims, pw.n_sims, phase);
    return cudaGetLastError();
}

cudaError_t mg_tail_attr(size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pcg_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    return e;
}

cudaError_t launch_mg_setup(const PcgWork& pw, cudaStream_t st) {
    if (pw.sweep_bar) {
        cudaError_t e = cudaMemsetAsync(pw.sweep_bar, 0, sizeof(GridBar), st);
        if (e != cudaSuccess) return e;
    }
    k_cell_lists<<<grid_of(pw.chunks_all.total), THREADS, 0, st>>>(mkw(pw.chunks_all), 0); note_launch("k_cell_lists", st);
    for (int l = 0; l + 1 < pw.setup_levels; l++) {
        if (!pw.setup[l].total) continue;
        k_mg_coarsen<<<grid_of(pw.setup[l].total), THREADS, 0, st>>>(mkw(pw.setup[l]), l); note_launch("k_mg_coarsen", st);
        k_mg_info<<<grid_of(pw.setup[l].total), THREADS, 0, st>>>(mkw(pw.setup[l]), l); note_launch("k_mg_info", st);
        k_cell_lists<<<grid_of(pw.setup[l].total), THREADS, 0, st>>>(mkw(pw.setup[l]), l + 1); note_launch("k_cell_lists", st);
    }
    if (pw.act_n) {
        cudaError_t e = cudaMemsetAsync(pw.act_n, 0, kActCounters * sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        const unsigned gc = std::min<unsigned>((pw.chunks_all.total + THREADS - 1) / THREADS, unsigned(sm_count()) * 4u);
        k_compact<<<gc ? gc : 1u, THREADS, 0, st>>>(pw); note_launch("k_compact", st);
    }
    return cudaGetLastError();
}

// Cooperative launch of k_mg_level over `grid` blocks with `smem` bytes of cached lists.
static cudaError_t launch_coop(unsigned grid, size_t smem, cudaStream_t st, const Work& lw, const Work& cw, int l,
                               int side, int pairs, uint32_t cs, GridBar* bar) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_mg_level, lw, cw, l, side, pairs, cs, bar);
    note_launch(side == 0 ? "k_mg_pre" : "k_mg_post", st);
    return e;
}

// Grid of the cooperative smoothing of a level: enough blocks that each caches at most kCoopCPB
// chunks, all co-resident; 0 when the level does not fit (it then runs one launch per sweep).
static unsigned coop_grid(const StageWork& lw, uint32_t cs, size_t* smem) {
    if (lw.act) return 0;
    *smem = size_t(kCoopCPB) * cs * 6;
    if (*smem > 200 * 1024) return 0;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_mg_level, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_level, THREADS, *smem) != cudaSuccess) return 0;
    const uint32_t cap = uint32_t(per_sm) * uint32_t(sm_count());
    const uint32_t need = (lw.total + kCoopCPB - 1) / kCoopCPB;
    if (need > cap || cap == 0) return 0;
    return std::min<uint32_t>(cap, std::max<uint32_t>(need, std::min<uint32_t>(lw.total, cap)));
}

static bool coop_smoothing() {
    const char* v = std::getenv("PXF_MG_COOP");
    return v && v[0] == '1';
}

cudaError_t launch_precond(const PcgWork& pw, cudaStream_t st, cudaGraphConditionalHandle h, uint32_t* ticket) {
    if (pw.any_jacobi) {
        launch_dep("k_jacobi", k_jacobi, grid_w(pw.chunks), THREADS, 0, st, mkw(pw.chunks));
    }
    if (pw.any_mg && coop_smoothing() && pw.sweep_bar) {
        // one cooperative launch per level and side where the level fits, else one launch per sweep
        cudaError_t e;
        for (int l = 0; l + 1 < pw.max_levels; l++) {
            if (!pw.level[l].total) continue;
            const uint32_t cs = l == 0 ? level0_chunk() : coarse_chunk();
            size_t smem = 0;
            const unsigned g = coop_grid(pw.level[l], cs, &smem);
            if (g) {
                if ((e = launch_coop(g, smem, st, mkw(pw.level[l]), mkw(pw.coarse[l]), l, 0, pw.max_pairs, cs,
                                     pw.sweep_bar)) != cudaSuccess)
                    return e;
                continue;
            }
            launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1, 0, 0);
            for (int x = 1; x < pw.max_pairs; x++) {
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 0, 0, x);
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1, 0, x);
            }
            launch_dep("k_mg_restrict", k_mg_restrict, grid_w(pw.coarse[l]), THREADS, 0, st, mkw(pw.coarse[l]), l);
        }
        launch_dep("k_mg_tail", k_mg_tail, pw.n_sims, 1024, pw.tail_smem, st, pw.sims, pw.n_sims);
        for (int l = pw.max_levels - 2; l >= 0; l--) {
            if (!pw.level[l].total) continue;
            const uint32_t cs = l == 0 ? level0_chunk() : coarse_chunk();
            size_t smem = 0;
            const unsigned g = coop_grid(pw.level[l], cs, &smem);
            if (g) {
                if ((e = launch_coop(g, smem, st, mkw(pw.level[l]), mkw(pw.level[l]), l, 1, pw.max_pairs, cs,
                                     pw.sweep_bar)) != cudaSuccess)
                    return e;
                continue;
            }
            for (int x = 0; x < pw.max_pairs; x++) {
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1,
                           x == 0 ? 2 : 0, x);
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 0,
                           l == 0 ? 3 : 0, x);
            }
        }
    } else if (pw.any_mg) {
        for (int l = 0; l + 1 < pw.max_levels; l++) {
            if (!pw.level[l].total) continue;
            // (the red half sweep from zero ran in the kernel that produced this level's r)
            launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1, 0, 0);
            for (int x = 1; x < pw.max_pairs; x++) {
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 0, 0, x);
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1, 0, x);
            }
            launch_dep("k_mg_restrict", k_mg_restrict, grid_w(pw.coarse[l]), THREADS, 0, st, mkw(pw.coarse[l]), l);
        }
        launch_dep("k_mg_tail", k_mg_tail, pw.n_sims, 1024, pw.tail_smem, st, pw.sims, pw.n_sims);
        for (int l = pw.max_levels - 2; l >= 0; l--) {
            if (!pw.level[l].total) continue;
            for (int x = 0; x < pw.max_pairs; x++) {
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 1,
                           x == 0 ? 2 : 0, x);
                launch_dep("k_mg_smooth", k_mg_smooth, grid_w(pw.level[l]), THREADS, 0, st, mkw(pw.level[l]), l, 0,
                           l == 0 ? 3 : 0, x);
            }
        }
    }
    return ctl(pw, 2, st, h, ticket);
}

cudaError_t launch_pcg_restart(const PcgWork& pw, cudaStream_t st) {
    launch_dep("k_pcg_widen", k_pcg_widen, grid_w(pw.chunks), THREADS, 0, st, mkw(pw.chunks));
    launch_dep("k_pcg_resid", k_pcg_resid, grid_w(pw.chunks), THREADS, 0, st, mkw(pw.chunks));
    return ctl(pw, 1, st);
}

cudaError_t launch_pcg_init(const PcgWork& pw, cudaStream_t st) {
    if (pw.tickets) {
        cudaError_t e = cudaMemsetAsync(pw.tickets, 0, 2 * sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
    }
    launch_mg_setup(pw, st);
    k_pcg_init<<<grid_w(pw.chunks), THREADS, 0, st>>>(mkw(pw.chunks)); note_launch("k_pcg_init", st);
    ctl(pw, 0, st);
    launch_pcg_restart(pw, st);
    return launch_precond(pw, st);
}

cudaError_t launch_pcg_dir(const PcgWork& pw, cudaStream_t st) {
    launch_dep("k_pcg_dir", k_pcg_dir, grid_w(pw.chunks), THREADS, 0, st, mkw(pw.chunks));
    return ctl(pw, 3, st);
}

cudaError_t launch_pcg_update(const PcgWork& pw, cudaStream_t st, cudaGraphConditionalHandle h, uint32_t* ticket) {
    launch_dep("k_pcg_update", k_pcg_update, grid_w(pw.chunks), THREADS, 0, st, mkw(pw.chunks));
    return ctl(pw, 4, st, h, ticket);
}

cudaError_t launch_pcg_body(const PcgWork& pw, cudaStream_t st) {
    launch_pcg_dir(pw, st);
    launch_pcg_update(pw, st);
    launch_pcg_restart(pw, st);
    return launch_precond(pw, st);
}

cudaError_t launch_pcg_cond(const SimDev* sims, int n_sims, cudaGraphConditionalHandle h, cudaStream_t st) {
    k_pcg_cond<<<1, 32, 0, st>>>(sims, n_sims, h); note_launch("k_pcg_cond", st);
    return cudaGetLastError();
}

cudaError_t launch_pcg_any(const SimDev* sims, int n_sims, uint32_t* flag, cudaStream_t st) {
    k_pcg_any<<<1, 32, 0, st>>>(sims, n_sims, flag); note_launch("k_pcg_any", st);
    return cudaGetLastError();
}

cudaError_t launch_pcg_finish(const PcgWork& pw, cudaStream_t st) {
    k_pcg_finish<<<grid_of(pw.chunks_all.total), THREADS, 0, st>>>(mkw(pw.chunks_all)); note_launch("k_pcg_finish", st);
    return cudaGetLastError();
}

// Self-test of the grid barrier's failure path: `rounds` barriers over a cooperative grid; block
// `skip` (if any) returns at once, so the others' waits run out after `limit` cycles, set the
// error flag and return. Every wait is bounded, so the kernel ends either way.
__global__ void k_barrier_selftest(GridBar* b, int skip, long long limit, int rounds) {
    if (int(blockIdx.x) == skip) return;
    for (int i = 0; i < rounds; i++)
        if (!grid_sync(b, limit)) return;
}

cudaError_t launch_barrier_selftest(GridBar* bar, int blocks, int skip, long long limit, int rounds, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_barrier_selftest, 32, 0);
    if (e != cudaSuccess) return e;
    const int cap = per_sm * sm_count();
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if ((e = cudaMemsetAsync(bar, 0, sizeof(GridBar), st)) != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(blocks));
    cfg.blockDim = dim3(32);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_barrier_selftest, bar, skip, limit, rounds);
    note_launch("k_barrier_selftest", st);
    return e;
}

cudaError_t launch_gs_lists(const StageWork& chunks, cudaStream_t st) {
    k_gs_lists<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks)); note_launch("k_gs_lists", st);
    return cudaGetLastError();
}

cudaError_t launch_pressure_rb_list(const StageWork& chunks, uint32_t parity, uint32_t it, cudaStream_t st) {
    launch_dep("k_pressure_rb_list", k_pressure_rb_list, grid_of(chunks.total), THREADS, 0, st, mkw(chunks), parity, it);
    return cudaGetLastError();
}

// Blocks of the persistent solve that are guaranteed co-resident on this device.
int pcg_solve_grid(size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_solve, THREADS, smem) != cudaSuccess) return 0;
    if (per_sm > 4) per_sm = 4;
    return per_sm * sm_count();
}

cudaError_t launch_pcg_solve(const PcgWork& pw, GridBar* bar, int grid, uint32_t guard, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), st);
    if (e != cudaSuccess) return e;
    if (pw.act_n && (e = cudaMemsetAsync(pw.act_n, 0, kActCounters * sizeof(uint32_t), st)) != cudaSuccess) return e;
    SolveArgs a;
    a.pw = pw;
    a.bar = bar;
    a.guard = guard;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = pw.tail_smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_pcg_solve, a);
    note_launch("k_pcg_solve", st);
    return e;
}

}  // namespace pxf
