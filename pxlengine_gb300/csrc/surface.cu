// Surface-nets meshing of the liquid (shaders/fluid.slang:222-355, driven per frame by
// crates/pxl-render/src/fluid.rs:308-330), into device vertex / index buffers the library owns.
//
//   s_clear + s_splat -> memset + k_s_splat    (fixed-point density, int atomics: order-free)
//   s_phi             -> k_s_phi
//   s_verts           -> k_s_vcount + k_s_scan + k_s_vemit
//   s_quads           -> k_s_qcount + k_s_scan + k_s_qemit
//
// The reference numbers vertices and triangles with atomic counters, so its order changes from
// run to run. Here a vertex's index is its rank among the surface cells that have one (ascending
// cell index) and a quad's position its rank among the valid quads (ascending node, then axis):
// the same mesh as a set, in one fixed order, which a serial restatement reproduces exactly.
// Overflow follows the reference: a vertex whose index reaches max_verts is dropped (its cell
// keeps no vertex), a quad whose triangles would pass max_tris is dropped, and the counters still
// count every vertex and every valid quad.
//
// Arithmetic follows the shader in FP32 without contraction (-fmad=false): lerp is
// a*(1-t) + b*t, int() truncates, dot products sum x, y, z in that order, normalize(v) is
// v / sqrt(dot(v, v)).
#include <cstdint>

#include "pxf_device.cuh"
#include "pxf_kernels.h"
#include "surface.h"

namespace pxf {

namespace {

constexpr float kSD = 4096.0f;              // fixed-point scale of the density (fluid.slang:39)
constexpr uint32_t kNone = 0xffffffffu;
constexpr uint32_t kSChunk = 2048;          // cells / nodes per scan chunk (256 threads x 8)

__device__ __forceinline__ uint32_t snode(const SurfDev& S, int i, int j, int k) {
    return uint32_t(i) + (S.sx + 1) * (uint32_t(j) + (S.sy + 1) * uint32_t(k));
}

__device__ __forceinline__ float3 f3lerp(float3 a, float3 b, float t) {
    return make_float3(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t);
}

// ---------------------------------------------------------------------------- density + phi
__global__ void __launch_bounds__(256) k_s_splat(SurfDev S, const float4* __restrict__ pos, uint32_t n) {
    const float r = S.radius / S.sh;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const float4 P = pos[p];
        const float gx = (P.x - S.ox) / S.sh, gy = (P.y - S.oy) / S.sh, gz = (P.z - S.oz) / S.sh;
        const int lx = max(f2i(ceilf(gx - r)), 0), ly = max(f2i(ceilf(gy - r)), 0), lz = max(f2i(ceilf(gz - r)), 0);
        const int hx = min(f2i(floorf(gx + r)), int(S.sx)), hy = min(f2i(floorf(gy + r)), int(S.sy)),
                  hz = min(f2i(floorf(gz + r)), int(S.sz));
        const float rr = r * r;
        for (int k = lz; k <= hz; k++)
            for (int j = ly; j <= hy; j++)
                for (int i = lx; i <= hx; i++) {
                    const float dx = float(i) - gx, dy = float(j) - gy, dz = float(k) - gz;
                    const float q = 1.0f - (dx * dx + dy * dy + dz * dz) / rr;
                    if (q > 0.0f) atomicAdd(S.density + snode(S, i, j, k), f2i(q * q * q * kSD));
                }
    }
}

__global__ void __launch_bounds__(256) k_s_phi(SurfDev S) {
    const uint32_t nn = (S.sx + 1) * (S.sy + 1) * (S.sz + 1);
    const int X = int(S.sx), Y = int(S.sy), Z = int(S.sz);
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < nn; id += gridDim.x * blockDim.x) {
        const int i = int(id % (S.sx + 1)), j = int((id / (S.sx + 1)) % (S.sy + 1)),
                  k = int(id / ((S.sx + 1) * (S.sy + 1)));
        float s = 2.0f * float(S.density[id]);
        float wsum = 2.0f;
#pragma unroll
        for (int a = 0; a < 6; a++) {
            int q[3] = {i, j, k};
            q[a >> 1] += (a & 1) ? 1 : -1;
            if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] > X || q[1] > Y || q[2] > Z) continue;
            s += float(S.density[snode(S, q[0], q[1], q[2])]);
            wsum += 1.0f;
        }
        const bool edge = i == 0 || j == 0 || k == 0 || i == X || j == Y || k == Z;
        S.phi[id] = edge ? -1.0f : s / wsum / kSD - S.iso;
    }
}

// ---------------------------------------------------------------------------- vertices
__device__ __forceinline__ uint32_t inside_mask(const SurfDev& S, uint32_t c, float v[8]) {
    const int i = int(c % S.sx), j = int((c / S.sx) % S.sy), k = int(c / (S.sx * S.sy));
    uint32_t inside = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        v[q] = S.phi[snode(S, i + (q & 1), j + ((q >> 1) & 1), k + (q >> 2))];
        if (v[q] > 0.0f) inside |= 1u << q;
    }
    return inside;
}

__device__ __forceinline__ bool has_vertex(uint32_t inside) { return inside != 0u && inside != 255u; }

// Exclusive block prefix of per-thread counts; *total receives the block's sum.
__device__ __forceinline__ uint32_t block_prefix(uint32_t x, uint32_t* total) {
    __shared__ uint32_t ws[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t v = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
    }
    if (lane == 31) ws[wid] = v;
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (int k = 0; k < int(blockDim.x >> 5); k++) {
        if (k < wid) before += ws[k];
        all += ws[k];
    }
    __syncthreads();
    *total = all;
    return before + v - x;
}

__global__ void __launch_bounds__(256) k_s_vcount(SurfDev S) {
    const uint32_t nc = S.sx * S.sy * S.sz;
    const uint32_t nch = (nc + kSChunk - 1) / kSChunk;
    for (uint32_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        uint32_t cnt = 0;
        for (uint32_t q = 0; q < kSChunk / 256; q++) {
            const uint32_t c = ch * kSChunk + threadIdx.x * (kSChunk / 256) + q;
            float v[8];
            if (c < nc && has_vertex(inside_mask(S, c, v))) cnt++;
        }
        uint32_t total;
        block_prefix(cnt, &total);
        if (threadIdx.x == 0) S.vchunk[ch] = total;
    }
}

// Exclusive scan of n chunk counts in place (one block); *out_total receives the sum.
__global__ void __launch_bounds__(1024) k_s_scan(uint32_t* chunks, uint32_t n, uint32_t* out_total) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n ? chunks[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t t = wsum[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            wsum[lane] = t;
        }
        __syncthreads();
        const uint32_t before = (wid ? wsum[wid - 1] : 0u) + carry;
        if (i < n) chunks[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) *out_total = carry;
}

__global__ void __launch_bounds__(256) k_s_vemit(SurfDev S) {
    const uint32_t nc = S.sx * S.sy * S.sz;
    const uint32_t nch = (nc + kSChunk - 1) / kSChunk;
    constexpr uint32_t PER = kSChunk / 256;
    for (uint32_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        const uint32_t c0 = ch * kSChunk + threadIdx.x * PER;
        uint32_t flags = 0, cnt = 0;
        for (uint32_t q = 0; q < PER; q++) {
            float v[8];
            if (c0 + q < nc && has_vertex(inside_mask(S, c0 + q, v))) {
                flags |= 1u << q;
                cnt++;
            }
        }
        uint32_t total;
        uint32_t idx = S.vchunk[ch] + block_prefix(cnt, &total);
        for (uint32_t q = 0; q < PER; q++) {
            const uint32_t c = c0 + q;
            if (c >= nc) break;
            if (!(flags & (1u << q))) {
                S.cell_vert[c] = kNone;
                continue;
            }
            const uint32_t my = idx++;
            if (my >= S.max_verts) {
                S.cell_vert[c] = kNone;
                continue;
            }
            float v[8];
            inside_mask(S, c, v);
            // vertex = mean of the edge crossings
            float3 sum = make_float3(0.f, 0.f, 0.f);
            float ncross = 0.0f;
#pragma unroll
            for (int e = 0; e < 12; e++) {
                const int axis = e >> 2, bits = e & 3;
                const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
                int a0 = 0;
                if (bits & 1) a0 |= 1 << o1;
                if (bits & 2) a0 |= 1 << o2;
                const int a1 = a0 | (1 << axis);
                if ((v[a0] > 0.0f) == (v[a1] > 0.0f)) continue;
                const float t = v[a0] / (v[a0] - v[a1]);
                const float3 p0 = make_float3(float(a0 & 1), float((a0 >> 1) & 1), float(a0 >> 2));
                const float3 p1 = make_float3(float(a1 & 1), float((a1 >> 1) & 1), float(a1 >> 2));
                const float3 l = f3lerp(p0, p1, t);
                sum.x += l.x;
                sum.y += l.y;
                sum.z += l.z;
                ncross += 1.0f;
            }
            const float3 local = make_float3(sum.x / ncross, sum.y / ncross, sum.z / ncross);
            // trilinear gradient of phi at the vertex; the normal points out of the liquid
            float3 grad = make_float3(0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                // w = lerp(1 - local, local, o) with o in {0, 1}: exactly local or 1 - local
                const bool ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
                const float3 ww = make_float3(ox ? local.x : 1.0f - local.x, oy ? local.y : 1.0f - local.y,
                                              oz ? local.z : 1.0f - local.z);
                const float sx = ox ? 1.0f : -1.0f, sy = oy ? 1.0f : -1.0f, sz = oz ? 1.0f : -1.0f;
                grad.x += v[k] * (sx * ww.y * ww.z);
                grad.y += v[k] * (sy * ww.x * ww.z);
                grad.z += v[k] * (sz * ww.x * ww.y);
            }
            const int ci = int(c % S.sx), cj = int((c / S.sx) % S.sy), ck = int(c / (S.sx * S.sy));
            const float px = S.ox + (float(ci) + local.x) * S.sh;
            const float py = S.oy + (float(cj) + local.y) * S.sh;
            const float pz = S.oz + (float(ck) + local.z) * S.sh;
            const float gx = grad.x + 0.0f, gy = grad.y + 1e-9f, gz = grad.z + 0.0f;
            const float len = sqrtf(gx * gx + gy * gy + gz * gz);
            S.verts[2 * size_t(my)] = make_float4(px, py, pz, 0.0f);
            S.verts[2 * size_t(my) + 1] = make_float4(-(gx / len), -(gy / len), -(gz / len), 0.0f);
            S.cell_vert[c] = my;
        }
    }
}

// ---------------------------------------------------------------------------- quads
// Quads of node `id` (bit a set: the edge along axis a yields a quad), with their four vertices.
__device__ __forceinline__ uint32_t node_quads(const SurfDev& S, uint32_t id, bool* in0_out, uint32_t vq[3][4]) {
    const int X = int(S.sx), Y = int(S.sy), Z = int(S.sz);
    const int n[3] = {int(id % (S.sx + 1)), int((id / (S.sx + 1)) % (S.sy + 1)), int(id / ((S.sx + 1) * (S.sy + 1)))};
    const bool in0 = S.phi[id] > 0.0f;
    *in0_out = in0;
    uint32_t mask = 0;
    const int lim[3] = {X, Y, Z};
    for (int axis = 0; axis < 3; axis++) {
        int m[3] = {n[0], n[1], n[2]};
        m[axis] += 1;
        if (m[axis] > lim[axis]) continue;
        if (in0 == (S.phi[snode(S, m[0], m[1], m[2])] > 0.0f)) continue;
        const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
        const int offs[4][2] = {{-1, -1}, {0, -1}, {0, 0}, {-1, 0}};
        bool ok = true;
        for (int k = 0; k < 4 && ok; k++) {
            int c[3] = {n[0], n[1], n[2]};
            c[o1] += offs[k][0];
            c[o2] += offs[k][1];
            if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= X || c[1] >= Y || c[2] >= Z) { ok = false; break; }
            const uint32_t cv = S.cell_vert[uint32_t(c[0]) + S.sx * (uint32_t(c[1]) + S.sy * uint32_t(c[2]))];
            if (cv == kNone) { ok = false; break; }
            vq[axis][k] = cv;
        }
        if (ok) mask |= 1u << axis;
    }
    return mask;
}

__global__ void __launch_bounds__(256) k_s_qcount(SurfDev S) {
    const uint32_t nn = (S.sx + 1) * (S.sy + 1) * (S.sz + 1);
    const uint32_t nch = (nn + kSChunk - 1) / kSChunk;
    for (uint32_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        uint32_t cnt = 0;
        for (uint32_t q = 0; q < kSChunk / 256; q++) {
            const uint32_t id = ch * kSChunk + threadIdx.x * (kSChunk / 256) + q;
            if (id >= nn) break;
            bool in0;
            uint32_t vq[3][4];
            cnt += __popc(node_quads(S, id, &in0, vq));
        }
        uint32_t total;
        block_prefix(cnt, &total);
        if (threadIdx.x == 0) S.qchunk[ch] = total;
    }
}

__global__ void __launch_bounds__(256) k_s_qemit(SurfDev S) {
    const uint32_t nn = (S.sx + 1) * (S.sy + 1) * (S.sz + 1);
    const uint32_t nch = (nn + kSChunk - 1) / kSChunk;
    constexpr uint32_t PER = kSChunk / 256;
    for (uint32_t ch = blockIdx.x; ch < nch; ch += gridDim.x) {
        const uint32_t n0 = ch * kSChunk + threadIdx.x * PER;
        uint32_t cnt = 0;
        for (uint32_t q = 0; q < PER; q++) {
            if (n0 + q >= nn) break;
            bool in0;
            uint32_t vq[3][4];
            cnt += __popc(node_quads(S, n0 + q, &in0, vq));
        }
        uint32_t total;
        uint32_t quad = S.qchunk[ch] + block_prefix(cnt, &total);
        for (uint32_t q = 0; q < PER; q++) {
            if (n0 + q >= nn) break;
            bool in0;
            uint32_t vq[3][4];
            const uint32_t mask = node_quads(S, n0 + q, &in0, vq);
            for (int axis = 0; axis < 3; axis++) {
                if (!(mask & (1u << axis))) continue;
                const uint32_t t = 2 * quad++;   // first triangle of this quad
                if (t + 2 > S.max_tris) continue;
                uint32_t* b = S.indices + size_t(t) * 3;
                const uint32_t* v = vq[axis];
                if (in0) {
                    b[0] = v[0]; b[1] = v[1]; b[2] = v[2];
                    b[3] = v[0]; b[4] = v[2]; b[5] = v[3];
                } else {
                    b[0] = v[0]; b[1] = v[2]; b[2] = v[1];
                    b[3] = v[0]; b[4] = v[3]; b[5] = v[2];
                }
            }
        }
    }
}

__global__ void k_s_finish(uint32_t* counters) {
    if (threadIdx.x == 0 && blockIdx.x == 0) counters[1] = 2u * counters[1];   // quads -> triangles
}

unsigned grid_cap(uint64_t items) {
    const uint64_t cap = uint64_t(sm_count()) * 8u;
    return unsigned(items < cap ? (items ? items : 1) : cap);
}

}  // namespace

cudaError_t launch_surface(const SurfDev& S, const float4* pos, uint32_t np, cudaStream_t st) {
    const uint64_t nn = uint64_t(S.sx + 1) * (S.sy + 1) * (S.sz + 1);
    const uint64_t nc = uint64_t(S.sx) * S.sy * S.sz;
    cudaError_t e = cudaMemsetAsync(S.density, 0, nn * sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(S.counters, 0, 4 * sizeof(uint32_t), st)) != cudaSuccess) return e;
    if (np) {
        k_s_splat<<<grid_cap((np + 255) / 256), 256, 0, st>>>(S, pos, np); note_launch("k_s_splat", st);
    }
    k_s_phi<<<grid_cap((nn + 255) / 256), 256, 0, st>>>(S); note_launch("k_s_phi", st);
    const uint32_t vch = uint32_t((nc + kSChunk - 1) / kSChunk), qch = uint32_t((nn + kSChunk - 1) / kSChunk);
    k_s_vcount<<<grid_cap(vch), 256, 0, st>>>(S); note_launch("k_s_vcount", st);
    k_s_scan<<<1, 1024, 0, st>>>(S.vchunk, vch, S.counters + 0); note_launch("k_s_scan", st);
    k_s_vemit<<<grid_cap(vch), 256, 0, st>>>(S); note_launch("k_s_vemit", st);
    k_s_qcount<<<grid_cap(qch), 256, 0, st>>>(S); note_launch("k_s_qcount", st);
    k_s_scan<<<1, 1024, 0, st>>>(S.qchunk, qch, S.counters + 1); note_launch("k_s_scan", st);
    k_s_qemit<<<grid_cap(qch), 256, 0, st>>>(S); note_launch("k_s_qemit", st);
    k_s_finish<<<1, 32, 0, st>>>(S.counters); note_launch("k_s_finish", st);
    return cudaGetLastError();
}

uint32_t surface_chunks(uint64_t items) { return uint32_t((items + kSChunk - 1) / kSChunk); }

}  // namespace pxf
