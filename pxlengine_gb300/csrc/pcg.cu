// Precision pressure solve: Jacobi-preconditioned CG with FP32 vectors (r, p, Ap), an FP64
// solution x and FP64 dot products / restart residuals. It solves the system that
// shaders/fluid.slang:167-182 relaxes: for each fluid cell i,
//     cnt_i p_i - sum_{fluid j} p_j = -(div_i h h / dt),     cnt_i = non-solid neighbours.
//
// Per step, two passes over the cells plus a conditional third:
//   k_pcg_dir_spmv  p' = z + beta p (z = r / cnt, recomputed for the 6 neighbours on the fly),
//                   Ap = A p', partial p'.Ap                 -> alpha
//   k_pcg_update    x += alpha p', r -= alpha Ap, partial r.r and r.z
//                                                              -> beta, or a restart request
//   k_pcg_restart   r = b - A x in FP64 for simulations that asked for it -> converged / fresh
// Every reduction is per simulation: fixed-order block reductions into per-chunk partials, and
// the last block of a simulation sums those partials in chunk order. Results therefore do not
// depend on scheduling or on which other simulations share the launch.
#include "pxf_device.cuh"
#include "pxf_kernels.h"

namespace pxf {

namespace {

constexpr int THREADS = 256;
constexpr int PER_THREAD = kScanChunk / THREADS;   // 8 cells per thread

// Block-wide sums of two doubles in a fixed order. Result valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, d);
        b += __shfl_down_sync(0xffffffffu, b, d);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sh[2 * wid] = a; sh[2 * wid + 1] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = 0; b = 0;
        for (int k = 0; k < THREADS / 32; k++) { a += sh[2 * k]; b += sh[2 * k + 1]; }
    }
    __syncthreads();
}

// Writes this chunk's partials; returns true (in every thread) for the last chunk of the
// simulation to arrive, after which that block may read all partials of the simulation.
__device__ __forceinline__ bool arrive_last(const SimDev& s, uint32_t chunk, uint32_t nchunks, double a, double b,
                                            uint32_t* counter, bool* flag) {
    if (threadIdx.x == 0) {
        s.partial[2 * chunk] = a;
        s.partial[2 * chunk + 1] = b;
        __threadfence();
        const uint32_t prev = atomicAdd(counter, 1u);
        *flag = (prev == nchunks - 1);
    }
    __syncthreads();
    const bool last = *flag;
    if (last) __threadfence();
    return last;
}

// Fixed-order sum of the per-chunk partials (last block only). Result valid in thread 0.
__device__ __forceinline__ void sum_partials(const SimDev& s, uint32_t nchunks, double& a, double& b, double* sh) {
    a = 0; b = 0;
    for (uint32_t k = threadIdx.x; k < nchunks; k += THREADS) {
        a += __ldcg(s.partial + 2 * k);
        b += __ldcg(s.partial + 2 * k + 1);
    }
    block_sum2(a, b, sh);
}

__device__ __forceinline__ float rhs_of(const SimDev& s, uint32_t c) {
    return s.div[c] * s.h * s.h / s.dt;   // fluid.slang:181
}

__device__ __forceinline__ bool in_system(uint32_t inf) { return (inf & 0x8000u) && ((inf >> 8) & 7u); }

__device__ __forceinline__ int64_t nbr_off(const SimDev& s, int q) {
    const int64_t nx = s.nx, nxy = int64_t(s.nx) * s.ny;
    switch (q) {
        case 0: return -1;
        case 1: return 1;
        case 2: return -nx;
        case 3: return nx;
        case 4: return -nxy;
        default: return nxy;
    }
}

// Scalars of the precision solver live in device memory written by the previous launch's last
// block; read them through L2.
__device__ __forceinline__ uint32_t ld_u32(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ double ld_f64(const double* p) { return __ldcg(p); }

}  // namespace

// -------------------------------------------------------------------------- init
__global__ void __launch_bounds__(THREADS) k_pcg_init(Work w) {
    __shared__ double sh[16];
    __shared__ bool last;
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        const uint32_t chunk = item - w.base[si];
        const uint32_t nchunks = (s.nc + kScanChunk - 1) / kScanChunk;
        double bb = 0, unused = 0;
#pragma unroll
        for (int k = 0; k < PER_THREAD; k++) {
            const uint32_t c = chunk * kScanChunk + k * THREADS + threadIdx.x;
            if (c < s.nc && in_system(s.info[c])) {
                const double b = -double(rhs_of(s, c));
                bb += b * b;
            }
        }
        block_sum2(bb, unused, sh);
        PcgState* st = s.pcg;
        if (arrive_last(s, chunk, nchunks, bb, 0.0, &st->arrive, &last)) {
            sum_partials(s, nchunks, bb, unused, sh);
            if (threadIdx.x == 0) {
                st->bb = bb;
                st->iters = 0;
                st->since = 0;
                st->fresh = 1;
                st->status = 0;
                st->relres = 0;
                st->beta = 0;
                st->restart_now = 1;
                st->done = 0;
                st->zero_x = bb == 0.0 ? 1u : 0u;
                st->arrive = 0;
            }
        }
    }
}

// -------------------------------------------------------------------------- restart
// r = b - A x in FP64 for simulations that requested a restart (and the zero-rhs case).
__global__ void __launch_bounds__(THREADS) k_pcg_restart(Work w) {
    __shared__ double sh[16];
    __shared__ bool last;
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        PcgState* st = s.pcg;
        if (ld_u32(&st->done) || !ld_u32(&st->restart_now)) continue;
        const bool zero_x = ld_u32(&st->zero_x) != 0;
        const uint32_t chunk = item - w.base[si];
        const uint32_t nchunks = (s.nc + kScanChunk - 1) / kScanChunk;
        double rr = 0, rz = 0;
#pragma unroll
        for (int k = 0; k < PER_THREAD; k++) {
            const uint32_t c = chunk * kScanChunk + k * THREADS + threadIdx.x;
            if (c >= s.nc) continue;
            const uint32_t inf = s.info[c];
            if (!in_system(inf)) continue;
            if (zero_x) { s.x64[c] = 0.0; continue; }
            const float cnt = float((inf >> 8) & 7u);
            double ax = double(cnt) * s.x64[c];
#pragma unroll
            for (int q = 0; q < 6; q++)
                if (inf & (1u << q)) ax -= s.x64[int64_t(c) + nbr_off(s, q)];
            const double rd = -double(rhs_of(s, c)) - ax;
            const float rf = float(rd);
            s.r[c] = rf;
            rr += rd * rd;
            const float z = rf / cnt;
            rz += double(rf) * double(z);
        }
        block_sum2(rr, rz, sh);
        if (arrive_last(s, chunk, nchunks, rr, rz, &st->arrive, &last)) {
            sum_partials(s, nchunks, rr, rz, sh);
            if (threadIdx.x == 0) {
                st->arrive = 0;
                st->restart_now = 0;
                if (zero_x) {
                    st->done = 1;
                    st->status = 3;
                    st->relres = 0;
                } else {
                    const double tol2 = s.rtol * s.rtol * st->bb;
                    st->relres = sqrt(rr / st->bb);
                    if (rr <= tol2 || st->iters >= s.max_iter) {
                        st->done = 1;
                        st->status = rr <= tol2 ? 0u : 1u;
                    } else {
                        st->rz = rz;
                        st->fresh = 1;
                        st->since = 0;
                    }
                }
            }
        }
    }
}

// -------------------------------------------------------------------------- direction + SpMV
__device__ __forceinline__ float dir_of(const SimDev& s, const float* __restrict__ pold, int64_t c, uint32_t inf,
                                        bool fresh, float beta) {
    const float z = s.r[c] / float((inf >> 8) & 7u);
    return fresh ? z : z + beta * pold[c];
}

__global__ void __launch_bounds__(THREADS) k_pcg_dir_spmv(Work w) {
    __shared__ double sh[16];
    __shared__ bool last;
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        PcgState* st = s.pcg;
        if (ld_u32(&st->done)) continue;
        const uint32_t chunk = item - w.base[si];
        const uint32_t nchunks = (s.nc + kScanChunk - 1) / kScanChunk;
        const uint32_t pbuf = ld_u32(&st->pbuf);
        const float* pold = pbuf ? s.p1 : s.p0;
        float* pnew = pbuf ? s.p0 : s.p1;
        const bool fresh = ld_u32(&st->fresh) != 0;
        const float beta = float(ld_f64(&st->beta));
        double pap = 0, unused = 0;
#pragma unroll
        for (int k = 0; k < PER_THREAD; k++) {
            const uint32_t c = chunk * kScanChunk + k * THREADS + threadIdx.x;
            if (c >= s.nc) continue;
            const uint32_t inf = s.info[c];
            if (!in_system(inf)) continue;
            const float pn = dir_of(s, pold, c, inf, fresh, beta);
            float ap = float((inf >> 8) & 7u) * pn;
#pragma unroll
            for (int q = 0; q < 6; q++) {
                if (inf & (1u << q)) {
                    const int64_t nb = int64_t(c) + nbr_off(s, q);
                    ap -= dir_of(s, pold, nb, s.info[nb], fresh, beta);
                }
            }
            pnew[c] = pn;
            s.Ap[c] = ap;
            pap += double(pn) * double(ap);
        }
        block_sum2(pap, unused, sh);
        if (arrive_last(s, chunk, nchunks, pap, 0.0, &st->arrive, &last)) {
            sum_partials(s, nchunks, pap, unused, sh);
            if (threadIdx.x == 0) {
                st->arrive = 0;
                st->pbuf ^= 1u;   // p' is now the current direction
                st->pAp = pap;
                if (!(pap > 0.0)) {
                    st->done = 1;
                    st->status = 2;
                } else {
                    st->alpha = st->rz / pap;
                }
            }
        }
    }
}

// -------------------------------------------------------------------------- update
__global__ void __launch_bounds__(THREADS) k_pcg_update(Work w) {
    __shared__ double sh[16];
    __shared__ bool last;
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
        PcgState* st = s.pcg;
        if (ld_u32(&st->done)) continue;
        const uint32_t chunk = item - w.base[si];
        const uint32_t nchunks = (s.nc + kScanChunk - 1) / kScanChunk;
        const uint32_t pbuf = ld_u32(&st->pbuf);
        const float* p = pbuf ? s.p1 : s.p0;
        const double alpha = ld_f64(&st->alpha);
        const float af = float(alpha);
        double rr = 0, rzn = 0;
#pragma unroll
        for (int k = 0; k < PER_THREAD; k++) {
            const uint32_t c = chunk * kScanChunk + k * THREADS + threadIdx.x;
            if (c >= s.nc) continue;
            const uint32_t inf = s.info[c];
            if (!in_system(inf)) continue;
            const float pc = p[c];
            s.x64[c] += alpha * double(pc);
            const float rn = s.r[c] - af * s.Ap[c];
            s.r[c] = rn;
            const float z = rn / float((inf >> 8) & 7u);
            rr += double(rn) * double(rn);
            rzn += double(rn) * double(z);
        }
        block_sum2(rr, rzn, sh);
        if (arrive_last(s, chunk, nchunks, rr, rzn, &st->arrive, &last)) {
            sum_partials(s, nchunks, rr, rzn, sh);
            if (threadIdx.x == 0) {
                st->arrive = 0;
                st->iters += 1;
                st->since += 1;
                st->rr = rr;
                st->rzn = rzn;
                const double tol2 = s.rtol * s.rtol * st->bb;
                if (rr <= tol2 || st->since >= s.restart || st->iters >= s.max_iter) {
                    st->restart_now = 1;
                } else {
                    st->beta = rzn / st->rz;
                    st->rz = rzn;
                    st->fresh = 0;
                }
            }
        }
    }
}

// -------------------------------------------------------------------------- finish / condition
__global__ void __launch_bounds__(THREADS) k_pcg_finish(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (s.solver != 1) continue;
#pragma unroll
        for (int k = 0; k < PER_THREAD; k++) {
            const uint32_t c = (item - w.base[si]) * kScanChunk + k * THREADS + threadIdx.x;
            if (c < s.nc) s.pressure[c] = float(s.x64[c]);
        }
    }
}

__global__ void k_pcg_cond(const SimDev* sims, int n_sims, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned any = 0;
    for (int i = 0; i < n_sims; i++) {
        const SimDev& s = sims[i];
        if (s.solver == 1 && !__ldcg(&s.pcg->done)) any = 1;
    }
    cudaGraphSetConditional(h, any);
}

__global__ void k_pcg_any(const SimDev* sims, int n_sims, uint32_t* flag) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t any = 0;
    for (int i = 0; i < n_sims; i++) {
        const SimDev& s = sims[i];
        if (s.solver == 1 && !__ldcg(&s.pcg->done)) any = 1;
    }
    *flag = any;
}

// -------------------------------------------------------------------------- launchers
static unsigned grid_of(uint32_t total) {
    const uint32_t cap = uint32_t(sm_count() * 8);
    return total < cap ? (total ? total : 1u) : cap;
}

static inline Work mkw(const StageWork& sw) {
    Work w;
    w.sims = sw.sims;
    w.base = sw.base;
    w.n_sims = sw.n_sims;
    w.total = sw.total;
    return w;
}

cudaError_t launch_pcg_init(const StageWork& chunks, cudaStream_t st) {
    k_pcg_init<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    k_pcg_restart<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

cudaError_t launch_pcg_body(const StageWork& chunks, cudaStream_t st) {
    k_pcg_dir_spmv<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    k_pcg_update<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    k_pcg_restart<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

cudaError_t launch_pcg_dir_spmv(const StageWork& chunks, cudaStream_t st) {
    k_pcg_dir_spmv<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

cudaError_t launch_pcg_update(const StageWork& chunks, cudaStream_t st) {
    k_pcg_update<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

cudaError_t launch_pcg_restart(const StageWork& chunks, cudaStream_t st) {
    k_pcg_restart<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

cudaError_t launch_pcg_cond(const SimDev* sims, int n_sims, cudaGraphConditionalHandle h, cudaStream_t st) {
    k_pcg_cond<<<1, 32, 0, st>>>(sims, n_sims, h);
    return cudaGetLastError();
}

cudaError_t launch_pcg_any(const SimDev* sims, int n_sims, uint32_t* flag, cudaStream_t st) {
    k_pcg_any<<<1, 32, 0, st>>>(sims, n_sims, flag);
    return cudaGetLastError();
}

cudaError_t launch_pcg_finish(const StageWork& chunks, cudaStream_t st) {
    k_pcg_finish<<<grid_of(chunks.total), THREADS, 0, st>>>(mkw(chunks));
    return cudaGetLastError();
}

}  // namespace pxf
