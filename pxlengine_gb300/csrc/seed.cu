// Particle seeding on the device, bit-exact to FluidState::new (crates/pxl-render/src/fluid.rs:119-148).
//
// The reference walks the fill blocks in order and, inside each, the interior cells k, j, i
// (x fastest), keeping a cell when its centre lies inside the block, and draws three lcg()
// values (x, y, z) per particle from ONE generator (fluid.rs:97-100, state 0x9e3779b97f4a7c15 ^ seed).
// A cell's centre test is separable per axis and monotonic in the index, so each block keeps a
// box of cells [i0, i1] x [j0, j1] x [k0, k1]; particle p therefore knows its block, cell and
// draw number 3p directly, and the generator is advanced to draw 3p by affine skip-ahead
// (s -> a s + c composed with itself, mod 2^64). No host-side particle array is built.
#include <cstdint>

#include "pxf_device.cuh"
#include "pxf_kernels.h"
#include "seed.h"

namespace pxf {

namespace {

constexpr uint64_t LCG_A = 6364136223846793005ull;
constexpr uint64_t LCG_C = 1442695040888963407ull;

// State after k steps of s -> A s + C.
__device__ __forceinline__ uint64_t lcg_skip(uint64_t s, uint64_t k) {
    uint64_t ra = 1, rc = 0;           // accumulated map
    uint64_t ba = LCG_A, bc = LCG_C;   // map for 2^bit steps
    while (k) {
        if (k & 1) { rc = ba * rc + bc; ra = ba * ra; }
        bc = ba * bc + bc;
        ba = ba * ba;
        k >>= 1;
    }
    return ra * s + rc;
}

__device__ __forceinline__ float lcg_draw(uint64_t& s) {
    s = s * LCG_A + LCG_C;
    return float(uint32_t(s >> 40)) / float(1u << 24);
}

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// N(0, 1) from a counter (Box-Muller on two 24-bit uniforms).
__device__ __forceinline__ float gauss(uint64_t key) {
    const uint64_t r = splitmix(key);
    const float u1 = (float(uint32_t(r >> 40)) + 1.0f) / 16777217.0f;
    const float u2 = float(uint32_t(r & 0xffffffu)) / 16777216.0f;
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__global__ void k_seed(SeedArgs a, float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ pos0,
                       float4* __restrict__ vel0) {
    for (uint64_t p = a.p_begin + uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < a.p_end;
         p += uint64_t(gridDim.x) * blockDim.x) {
        int b = 0;
        while (b + 1 < a.n_blocks && p >= a.blk[b + 1].first) b++;
        const SeedBlock& B = a.blk[b];
        const uint64_t local = p - B.first;
        const uint64_t cell = local / a.ppc;
        const uint32_t cx = B.hi[0] - B.lo[0] + 1, cy = B.hi[1] - B.lo[1] + 1;
        const uint32_t i = B.lo[0] + uint32_t(cell % cx);
        const uint32_t j = B.lo[1] + uint32_t((cell / cx) % cy);
        const uint32_t k = B.lo[2] + uint32_t(cell / (uint64_t(cx) * cy));
        uint64_t s = lcg_skip(a.rng0, 3 * p);
        const float rx = lcg_draw(s), ry = lcg_draw(s), rz = lcg_draw(s);
        const float px = a.origin[0] + (float(i) + rx) * a.h;
        const float py = a.origin[1] + (float(j) + ry) * a.h;
        const float pz = a.origin[2] + (float(k) + rz) * a.h;
        float v[3] = {B.vel[0], B.vel[1], B.vel[2]};
        if (a.sigma > 0.0f) {
#pragma unroll
            for (int c = 0; c < 3; c++) v[c] += a.sigma * gauss((uint64_t(a.vseed) << 40) ^ (p * 3 + c));
        }
        const float4 P = make_float4(px, py, pz, __uint_as_float(uint32_t(p)));
        const float4 V = make_float4(v[0], v[1], v[2], 0.0f);
        pos[p] = P;
        vel[p] = V;
        if (pos0) { pos0[p] = P; vel0[p] = V; }
    }
}

}  // namespace

// Kept interior index range of one axis: i in [1, n - 2] with min <= origin + (i + 0.5) h <= max.
static bool axis_range(float origin, float h, uint32_t n, float mn, float mx, uint32_t& lo, uint32_t& hi) {
    bool any = false, closed = false;
    for (uint32_t i = 1; i + 1 < n; i++) {
        const float c = origin + (float(i) + 0.5f) * h;
        const bool out = c < mn || c > mx;
        if (!out) {
            if (closed) return false;   // not an interval (cannot happen for h > 0)
            if (!any) lo = i;
            hi = i;
            any = true;
        } else if (any) {
            closed = true;
        }
    }
    if (!any) { lo = 1; hi = 0; }
    return true;
}

bool seed_plan(const float origin[3], float h, const uint32_t n[3], const pxf_fill_block* fill, uint32_t n_fill,
               uint32_t ppc, uint32_t seed, SeedPlan& plan) {
    plan.blocks.assign(n_fill, SeedBlock{});
    plan.ppc = ppc;
    plan.h = h;
    for (int c = 0; c < 3; c++) plan.origin[c] = origin[c];
    plan.rng0 = 0x9e3779b97f4a7c15ull ^ uint64_t(seed);
    uint64_t total = 0;
    for (uint32_t b = 0; b < n_fill; b++) {
        SeedBlock& B = plan.blocks[b];
        uint64_t cells = 1;
        for (int c = 0; c < 3; c++) {
            if (!axis_range(origin[c], h, n[c], fill[b].min[c], fill[b].max[c], B.lo[c], B.hi[c])) return false;
            cells *= (B.hi[c] >= B.lo[c]) ? uint64_t(B.hi[c] - B.lo[c] + 1) : 0ull;
            B.vel[c] = fill[b].velocity[c];
        }
        B.first = total;
        total += cells * ppc;
    }
    plan.total = total;
    return true;
}

cudaError_t launch_seed(const SeedPlan& plan, float4* pos, float4* vel, float4* pos0, float4* vel0, cudaStream_t st) {
    const size_t nb = plan.blocks.size();
    for (size_t g = 0; g < nb; g += kMaxSeedBlocks) {
        SeedArgs a;
        a.n_blocks = int(nb - g < size_t(kMaxSeedBlocks) ? nb - g : size_t(kMaxSeedBlocks));
        for (int b = 0; b < a.n_blocks; b++) a.blk[b] = plan.blocks[g + b];
        a.p_begin = a.blk[0].first;
        a.p_end = (g + a.n_blocks < nb) ? plan.blocks[g + a.n_blocks].first : plan.total;
        a.ppc = plan.ppc;
        a.h = plan.h;
        for (int c = 0; c < 3; c++) a.origin[c] = plan.origin[c];
        a.rng0 = plan.rng0;
        a.sigma = plan.sigma;
        a.vseed = plan.vseed;
        if (a.p_end <= a.p_begin) continue;
        const uint64_t blocks = (a.p_end - a.p_begin + 255) / 256;
        const unsigned grid = blocks < 65535ull * 16 ? unsigned(blocks) : 65535u * 16;
        k_seed<<<grid, 256, 0, st>>>(a, pos, vel, pos0, vel0); note_launch("k_seed", st);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace pxf
