// Device-side data model of the FLIP substep: one SimDev per simulation, packed into a device
// array so that every stage runs as ONE launch over all simulations of a batch (a single drop-in
// simulation is a batch of one).
//
// HBM layout per simulation (x-fastest everywhere, the reference's own indexing,
// shaders/fluid.slang:43-53):
//   particles  pos[N] float4 {x, y, z, bits(pid)}  vel[N] float4 {vx, vy, vz, bits(rank)}
//              A = current state, B = the same particles counting-sorted by cell
//   faces      vel, vel_old: F floats (u block, then v, then w)
//   cells      type u8, start u32 (C + 1, exclusive scan of per-cell counts), count u32,
//              pressure f32, div f32, info u16 (fluid-neighbour mask | non-solid count << 8 |
//              fluid << 15)
//   precision  x2 double-float pair, x64 f64, r z p0 p1 Ap f32, per-chunk partials, and the
//              multigrid levels (type u8, info u16, r z f32 per coarse cell)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pxf {

enum : uint8_t { AIR = 0, FLUID = 1, SOLID = 2 };   // fluid.slang:40

// Per-simulation scalars of the precision (PCG) solver, written by one-block control kernels.
struct PcgState {
    double bb;        // |b|^2
    double rz;        // r.z of the current direction
    double pAp;
    double rr;        // recurrence |r|^2
    double alpha, beta;
    double relres;    // last FP64 restart residual / |b|
    uint32_t iters;   // PCG steps this solve
    uint32_t since;   // steps since the last restart
    uint32_t done;    // converged, capped, broken down or zero rhs
    uint32_t fresh;   // the next direction is p = z
    uint32_t restart_now;
    uint32_t status;  // 0 converged, 1 iteration cap, 2 breakdown, 3 zero rhs
    uint32_t pbuf;    // which of p0 / p1 holds the current direction
    uint32_t zero_x;  // zero right-hand side: the solution is x = 0
    float alpha_hi, alpha_lo;   // alpha as a double-float pair
};

// One level of the multigrid hierarchy (level 0 aliases the simulation's own arrays).
struct MgLevel {
    int nx, ny, nz;
    uint32_t nc;
    uint8_t* type;
    uint16_t* info;
    float* r;
    float* z;
    // System cells of each chunk of `cs` cells (level0_chunk() on level 0, coarse_chunk() below), in ascending order:
    // chunk k owns list[cs k ...], first its red cells ((i + j + k) even), then its black cells;
    // lcnt[2k], lcnt[2k+1] count them.
    uint32_t cs;
    uint32_t* list;
    uint32_t* lcnt;
};
constexpr int kMaxLevels = 12;

struct SimDev {
    int nx, ny, nz;
    uint32_t np;
    float h, dt, flip, inv_h;
    float o[3];
    float g[3];
    uint32_t nu, nv, nw, nf, nc;
    uint32_t iterations;     // red-black GS iterations
    uint32_t solver;         // 0 red-black GS, 1 precision PCG
    uint32_t precond;        // precision PCG preconditioner: 0 multigrid V-cycle, 1 Jacobi
    uint32_t coarse_iters;   // symmetric red-black iterations on the coarsest level
    uint32_t mg_pairs;       // red-black pairs of pre- and of post-smoothing per level
    double rtol;
    uint32_t max_iter, restart;
    float4 *posA, *velA, *posB, *velB;
    float *vel, *vel_old, *pressure, *div;
    uint8_t* type;
    uint32_t *count, *start, *chunk;
    uint16_t* info;
    int32_t *acc, *wacc;     // optional copies of the P2G fixed-point sums
    // precision solver
    float2* x2;              // solution as a double-float pair (hi, lo)
    double* x64;             // FP64 solution, written at restarts and at the end of the solve
    float *r, *z, *p0, *p1, *Ap;
    double* partial;         // one partial sum per list chunk of level 0
    PcgState* pcg;
    int nlev;
    int tail;                // first level handled by the shared-memory tail kernel
    MgLevel lev[kMaxLevels];
    // red-black GS streamed through shared memory (pressure_stream.cu): units of gs_ntx x gs_nty
    // x-y tiles times z segments of gs_zs planes
    float* p_alt;            // second pressure buffer (passes alternate between the two)
    float* rhs;              // div * h * h / dt of the current substep
    uint8_t* gs_cnt;         // non-solid neighbour count of each system cell, 0 elsewhere
    uint32_t* gs_flag;       // per unit: its interior holds a system cell
    uint32_t gs_ntx, gs_nty, gs_nzs, gs_zs;
};

// Work index of one stage over a batch: item i of the stage belongs to simulation s where
// base[s] <= i < base[s + 1].
struct Work {
    const SimDev* sims = nullptr;
    const uint32_t* base = nullptr;     // n_sims + 1 entries, device memory
    int n_sims = 0;
    uint32_t total = 0;
    const uint16_t* sim_of = nullptr;   // simulation of every item (batches of several simulations)
    const uint32_t* act = nullptr;      // the items that have work, built on the device; null: all
    const uint32_t* act_n = nullptr;    // number of entries of act
};

__device__ __forceinline__ int find_sim(const Work& w, uint32_t item) {
    if (w.sim_of) return __ldg(w.sim_of + item);
    int lo = 0, hi = w.n_sims;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(w.base + mid) <= item) lo = mid; else hi = mid;
    }
    return lo;
}

// Items a block-strided loop visits: the compacted list when there is one, else every item.
__device__ __forceinline__ uint32_t work_count(const Work& w) { return w.act ? __ldcg(w.act_n) : w.total; }
__device__ __forceinline__ uint32_t work_item(const Work& w, uint32_t k) { return w.act ? __ldcg(w.act + k) : k; }

// float -> int32, truncating (cvt.rzi.s32.f32: NaN -> 0, saturating).
__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }

// lerp as the GLSL.std.450 FMix definition: a*(1-t) + b*t (no contraction: built -fmad=false).
__device__ __forceinline__ float fmix(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Cell of a position, clamped into the grid (fluid.slang:113).
__device__ __forceinline__ uint32_t cell_of(const SimDev& s, float x, float y, float z) {
    int i = clampi(f2i(floorf((x - s.o[0]) * s.inv_h)), 0, s.nx - 1);
    int j = clampi(f2i(floorf((y - s.o[1]) * s.inv_h)), 0, s.ny - 1);
    int k = clampi(f2i(floorf((z - s.o[2]) * s.inv_h)), 0, s.nz - 1);
    return uint32_t(i) + uint32_t(s.nx) * (uint32_t(j) + uint32_t(s.ny) * uint32_t(k));
}

__device__ __forceinline__ bool wall_or_out(const SimDev& s, int i, int j, int k) {
    return i <= 0 || j <= 0 || k <= 0 || i >= s.nx - 1 || j >= s.ny - 1 || k >= s.nz - 1;
}

// (sum - rhs) / cnt of the red-black update for cnt in 1 .. 6 (rcp[cnt] = RN(1 / cnt)), correctly
// rounded: q0 = x * RN(1/cnt), then one FMA correction with the exact remainder x - q0 * cnt
// (division by a divisor known in advance:
// N. Brisebarre, J.-M. Muller, S. K. Raina, "Accelerating correctly rounded floating-point
// division when the divisor is known in advance", IEEE Trans. Computers 53(8), 2004). Checked
// against IEEE division over every float x for each divisor (tests/div_count_check.c): equal whenever
// x = +0 or 2^-100 <= |x| <= FLT_MAX; other x (tiny, -0, infinite, NaN) take the IEEE division.
__device__ __forceinline__ float div_count(float x, uint32_t cn, const float* __restrict__ rcp) {
    const float d = __uint2float_rn(cn);
    const uint32_t b = __float_as_uint(x);
    if ((b & 0x7fffffffu) - 0x0d800000u <= 0x7f7fffffu - 0x0d800000u || b == 0u) {
        const float r = rcp[cn];
        const float q0 = x * r;
        return __fmaf_rn(__fmaf_rn(-q0, d, x), r, q0);
    }
    return x / d;
}

}  // namespace pxf
