// FLIP substep kernels for sm_103a. Every kernel walks a packed work index (pxf_device.cuh) so
// one launch serves a whole batch of simulations with uneven grids.
//
// Stage map against the reference (shaders/fluid.slang, schedule crates/pxl-render/src/fluid.rs:289-303):
//   clear_grid + cell half of normalize_grid  -> k_scan_chunks / k_scan_sims / k_scan_apply
//   p2g + face half of normalize_grid + forces -> k_scatter (counting sort) + k_p2g (tiled gather)
//   compute_divergence                         -> k_divergence
//   pressure_rb                                -> k_pressure_rb
//   project                                    -> k_project
//   g2p_advect                                 -> k_g2p (also bins the advected particle for the
//                                                 next substep's counting sort)
//
// All arithmetic that the reference performs in FP32 is done here in the same order with no
// contraction (the library is compiled with -fmad=false), so the integer P2G sums, cell counts and
// flags are bit-exact and the FP32 fields follow the same rounding as the CPU restatement.
#include "pxf_device.cuh"
#include "pxf_kernels.h"

#include <algorithm>
#include <cstdlib>

namespace pxf {

constexpr uint32_t SCAN_CHUNK = 2048;   // cells per scan work item (256 threads x 8)

// P2G packs a face's two int32 sums into one 64-bit shared atomic: acc in the high word, wacc in
// the low word. Every wacc term is int(w * 65536) with 0 <= w <= 1 and a face collects terms from
// the particles of 18 cells, so with at most 3640 particles per cell (18 * 3640 * 65536 < 2^32) the
// low word never carries into the high word and both words equal the reference's wrapping int32
// sums. Binnings with a denser cell use two 32-bit atomics instead.
constexpr uint32_t kPackedMaxPerCell = 3640;

// ------------------------------------------------------------------ counting sort: scan + classify
// Per-chunk sums of the per-cell particle counts.
__global__ void __launch_bounds__(256) k_scan_chunks(Work w) {
    __shared__ uint32_t red[8];
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t chunk = item - w.base[si];
        const uint32_t c0 = chunk * SCAN_CHUNK;
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            uint32_t c = c0 + k * 256 + threadIdx.x;
            if (c < s.nc) sum += s.count[c];
        }
        sum = __reduce_add_sync(0xffffffffu, sum);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int k = 0; k < 8; k++) t += red[k];
            s.chunk[chunk] = t;
        }
        __syncthreads();
    }
}

// Exclusive scan of the chunk sums, one block per simulation.
__global__ void __launch_bounds__(1024) k_scan_sims(const SimDev* sims, int n_sims) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    for (int si = blockIdx.x; si < n_sims; si += gridDim.x) {
        const SimDev s = sims[si];
        const uint32_t nchunks = (s.nc + SCAN_CHUNK - 1) / SCAN_CHUNK;
        if (threadIdx.x == 0) {
            carry = 0;
            s.chunk[nchunks] = 0;   // dense-cell flag of this binning (raised by k_scan_apply)
        }
        __syncthreads();
        for (uint32_t base = 0; base < nchunks; base += 1024) {
            const uint32_t i = base + threadIdx.x;
            const uint32_t v = i < nchunks ? s.chunk[i] : 0u;
            const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            uint32_t x = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += y;
            }
            if (lane == 31) wsum[wid] = x;
            __syncthreads();
            if (wid == 0) {
                uint32_t t = wsum[lane];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
                    if (lane >= d) t += y;
                }
                wsum[lane] = t;
            }
            __syncthreads();
            const uint32_t before = (wid ? wsum[wid - 1] : 0u) + carry;
            if (i < nchunks) s.chunk[i] = before + x - v;
            __syncthreads();
            if (threadIdx.x == 1023) carry = before + x;
            __syncthreads();
        }
        if (threadIdx.x == 0) s.start[s.nc] = carry;
        __syncthreads();
    }
}

// start = exclusive scan of count; count := 0 for the next binning; cell type and the pressure
// reset of normalize_grid (fluid.slang:125-131).
// Counts are read and starts, flags and resets written in coalesced passes (cell k*256 + tid of the
// chunk); the exclusive scan runs over each thread's 8 consecutive cells staged in shared memory
// (one padding word per 32 keeps those reads free of bank conflicts).
__global__ void __launch_bounds__(256) k_scan_apply(Work w) {
    __shared__ uint32_t wsum[8];
    __shared__ uint32_t sv[SCAN_CHUNK + SCAN_CHUNK / 32];   // counts, then exclusive starts
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t chunk = item - w.base[si];
        const uint32_t cbase = chunk * SCAN_CHUNK;
        auto slot = [](uint32_t o) { return o + (o >> 5); };
        uint32_t vk[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t o = uint32_t(k) * 256 + threadIdx.x;
            vk[k] = cbase + o < s.nc ? s.count[cbase + o] : 0u;
            sv[slot(o)] = vk[k];
        }
        __syncthreads();
        uint32_t v[8];
        uint32_t tsum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = sv[slot(threadIdx.x * 8 + k)];
            tsum += v[k];
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t x = tsum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        uint32_t before = s.chunk[chunk];
        for (int k = 0; k < wid; k++) before += wsum[k];
        before += x - tsum;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sv[slot(threadIdx.x * 8 + k)] = before;
            before += v[k];
        }
        __syncthreads();
        const uint32_t nxy = uint32_t(s.nx) * uint32_t(s.ny);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t o = uint32_t(k) * 256 + threadIdx.x;
            const uint32_t c = cbase + o;
            if (c >= s.nc) continue;
            s.start[c] = sv[slot(o)];
            s.count[c] = 0;
            if (vk[k] > kPackedMaxPerCell) atomicOr(&s.chunk[(s.nc + SCAN_CHUNK - 1) / SCAN_CHUNK], 1u);
            const int i = int(c % uint32_t(s.nx));
            const int j = int((c / uint32_t(s.nx)) % uint32_t(s.ny));
            const int kk = int(c / nxy);
            const uint8_t t = wall_or_out(s, i, j, kk) ? SOLID : (vk[k] > 0 ? FLUID : AIR);
            s.type[c] = t;
            if (t != FLUID) {
                s.pressure[c] = 0.0f;
                if (s.x2) {
                    s.x2[c] = make_float2(0.0f, 0.0f);
                    s.x64[c] = 0.0;
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ counting sort: scatter
// B[start[cell] + rank] = A. The cell is recomputed from the position with the same expression
// that produced the rank, so it matches bit for bit.
// Four items per block pass (grid-strided), every load of the four issued before any store, so
// each thread keeps four particles in flight.
__global__ void __launch_bounds__(256) k_scatter(Work w) {
    constexpr int U = 4;
    for (uint32_t item0 = blockIdx.x; item0 < w.total; item0 += U * gridDim.x) {
        float4 P[U], V[U];
        const SimDev* sp[U];
        uint32_t idx[U];
        bool live[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint32_t item = item0 + u * gridDim.x;
            live[u] = false;
            sp[u] = w.sims;
            idx[u] = 0;
            if (item >= w.total) continue;
            const int si = find_sim(w, item);
            sp[u] = w.sims + si;
            idx[u] = (item - w.base[si]) * 256 + threadIdx.x;
            live[u] = idx[u] < sp[u]->np;
            if (live[u]) {
                P[u] = sp[u]->posA[idx[u]];
                V[u] = sp[u]->velA[idx[u]];
            }
        }
        uint32_t dst[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            dst[u] = 0xffffffffu;
            if (!live[u]) continue;
            const SimDev& s = *sp[u];
            dst[u] = s.start[cell_of(s, P[u].x, P[u].y, P[u].z)] + __float_as_uint(V[u].w);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (!live[u] || dst[u] >= sp[u]->np) continue;   // always below np when the ranks come from the last binning
            sp[u]->posB[dst[u]] = P[u];
            sp[u]->velB[dst[u]] = V[u];
        }
    }
}

// Binning of the current particles (first substep and after a host write): count + rank.
__global__ void __launch_bounds__(256) k_bin(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t i = (item - w.base[si]) * 256 + threadIdx.x;
        const bool live = i < s.np;
        uint32_t c = 0xffffffffu;
        if (live) {
            const float4 P = s.posA[i];
            c = cell_of(s, P.x, P.y, P.z);
        }
        const unsigned active = __ballot_sync(0xffffffffu, live);
        if (live) {
            const unsigned peers = __match_any_sync(active, c);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&s.count[c], uint32_t(__popc(peers)));
            base = __shfl_sync(peers, base, leader);
            const uint32_t rank = base + __popc(peers & ((1u << lane) - 1u));
            s.velA[i].w = __uint_as_float(rank);
        }
    }
}

// ------------------------------------------------------------------ P2G (tiled gather)
// One work item = one TX x TY x TZ tile of cells. The tile's particles plus a one-cell halo are
// contiguous per x-row in the sorted array, so each warp streams whole rows. Every particle's
// 24 face contributions are the reference's int32 fixed-point terms (fluid.slang:97-111); the
// tile owns its faces, so the integer sums live in shared memory and never touch global atomics.
// The epilogue is normalize_grid's face half and forces (fluid.slang:119-124, 142-151).
template <int TX, int TY, int TZ>
struct P2GTile {
    static constexpr int FU = (TX + 1) * TY * TZ;
    static constexpr int FV = TX * (TY + 1) * TZ;
    static constexpr int FW = TX * TY * (TZ + 1);
    static constexpr int NF = FU + FV + FW;
    static constexpr int SMEM = NF * 2 * 4;
    static constexpr int NR = (TY + 2) * (TZ + 2);   // x-rows of the tile and its halo
    static_assert(NR <= 128, "the row scan uses the block's first four warps");
};

template <int TX, int TY, int TZ, bool PACKED>
__device__ __forceinline__ void p2g_tile(const SimDev& s, int* __restrict__ sacc, int* __restrict__ swac,
                                         unsigned long long* __restrict__ spk, const int org[3], const int E[3][3],
                                         bool strided, bool by_rows, const uint32_t* __restrict__ s_rb,
                                         const uint32_t* __restrict__ s_rs) {
    using T = P2GTile<TX, TY, TZ>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int sbase[3] = {0, T::FU, T::FU + T::FV};
    const float SW = 65536.0f;
    // The 24 fixed-point face terms of particle j, added to the owned faces in shared memory.
    auto particle = [&](uint32_t j) {
        {
            const float4 P = s.posB[j];
            const float4 V = s.velB[j];
            const float x[3] = {P.x, P.y, P.z};
            const float vv[3] = {V.x, V.y, V.z};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                // Box of this component's owned faces: SDX x SDY x (TZ + (c == 2)) in shared memory.
                const int SDX = c == 0 ? TX + 1 : TX;
                const int SDY = c == 1 ? TY + 1 : TY;
                int lb[3];
                float wt[3][2];
                bool ok[3][2];
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    float gq = (x[a] - s.o[a]) * s.inv_h - 0.5f;
                    if (a == c) gq += 0.5f;
                    const int b = f2i(floorf(gq));
                    const float f = gq - float(b);
                    // fmix(1 - f, f, 0) and fmix(1 - f, f, 1) (fluid.slang's lerp weights) equal
                    // 1 - f and f for every finite f up to the sign of a zero, which the integer
                    // terms drop, and both forms are NaN for a NaN f; an infinite f comes from an
                    // infinite position, whose saturated cell index owns no face of any tile.
                    wt[a][0] = 1.0f - f;
                    wt[a][1] = f;
                    lb[a] = b - org[a];
                    ok[a][0] = unsigned(lb[a]) < unsigned(E[c][a]);
                    ok[a][1] = unsigned(lb[a] + 1) < unsigned(E[c][a]);
                }
                if (!((ok[0][0] | ok[0][1]) & (ok[1][0] | ok[1][1]) & (ok[2][0] | ok[2][1]))) continue;
                // w = (wx * wy) * wz, the reference's product order
                const float wxy[2][2] = {{wt[0][0] * wt[1][0], wt[0][0] * wt[1][1]},
                                         {wt[0][1] * wt[1][0], wt[0][1] * wt[1][1]}};
                const int base = sbase[c] + lb[0] + SDX * (lb[1] + SDY * lb[2]);
                const float v = vv[c];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
                    if (!(ok[0][ox] & ok[1][oy] & ok[2][oz])) continue;
                    const float wgt = wxy[ox][oy] * wt[2][oz];
                    const int idx = base + ox + SDX * oy + SDX * SDY * oz;
                    const int ta = f2i(wgt * v * SW);
                    const int tw = f2i(wgt * SW);
                    if (PACKED) {
                        atomicAdd(&spk[idx], (static_cast<unsigned long long>(static_cast<uint32_t>(ta)) << 32) |
                                                 static_cast<uint32_t>(tw));
                    } else {
                        atomicAdd(&sacc[idx], ta);
                        atomicAdd(&swac[idx], tw);
                    }
                }
            }
        }
    };
    // The tile's rows (its cells plus the one-cell halo, x-rows of the sorted particle array)
    // concatenated: list position q of row r is s_rs[r] + (q - s_rb[r]).
    // strided: each lane takes a contiguous part of its warp's share, so at any step the lanes of
    // a warp sit in different cells and rarely hit the same face; otherwise lanes take
    // consecutive particles (coalesced loads).
    if (by_rows) {
        // whole rows per warp (uniformly dense tiles)
        for (int rr = warp; rr < T::NR; rr += nw) {
            const uint32_t pb = s_rs[rr], n = s_rb[rr + 1] - s_rb[rr];
            const uint32_t per = (n + 31) / 32;
            for (uint32_t t = 0; t < per; t++) {
                const uint32_t o = strided ? uint32_t(lane) * per + t : t * 32 + uint32_t(lane);
                if (o < n) particle(pb + o);
            }
        }
        return;
    }
    // an equal slice of the list per warp, so a dense row spreads over all warps
    const uint32_t total = s_rb[T::NR];
    const uint32_t qa = uint32_t(uint64_t(total) * uint32_t(warp) / uint32_t(nw));
    const uint32_t qb = uint32_t(uint64_t(total) * uint32_t(warp + 1) / uint32_t(nw));
    const uint32_t per = (qb - qa + 31) / 32;
    uint32_t q = strided ? qa + uint32_t(lane) * per : qa + uint32_t(lane);
    const uint32_t qend = strided ? min(q + per, qb) : qb;
    const uint32_t step = strided ? 1u : 32u;
    int r = 0;
    {
        int hi = T::NR;   // largest r with s_rb[r] <= q
        while (hi - r > 1) {
            const int mid = (r + hi) >> 1;
            if (s_rb[mid] <= q) r = mid; else hi = mid;
        }
    }
    uint32_t row_end = s_rb[r + 1], row_off = s_rs[r] - s_rb[r];
    for (; q < qend; q += step) {
        while (q >= row_end) {
            r++;
            row_end = s_rb[r + 1];
            row_off = s_rs[r] - s_rb[r];
        }
        particle(q + row_off);
    }
}

// order: null = item order; otherwise the k-th block takes tile order[k].
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(256, 3) k_p2g(Work w, int strided, int pack, const uint32_t* __restrict__ order) {
    using T = P2GTile<TX, TY, TZ>;
    extern __shared__ unsigned long long smem64[];
    __shared__ uint32_t s_rb[T::NR + 1], s_rs[T::NR], s_wt[4];
    unsigned long long* spk = smem64;
    int* sacc = reinterpret_cast<int*>(smem64);
    int* swac = sacc + T::NF;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t k = blockIdx.x; k < w.total; k += gridDim.x) {
        const uint32_t item = order ? __ldg(order + k) : k;
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t t = item - w.base[si];
        const int ntx = (s.nx + TX - 1) / TX, nty = (s.ny + TY - 1) / TY;
        const int x0 = int(t % uint32_t(ntx)) * TX;
        const int y0 = int((t / uint32_t(ntx)) % uint32_t(nty)) * TY;
        const int z0 = int(t / uint32_t(ntx * nty)) * TZ;
        // Particle range of every row and the rows' offsets in the concatenated list (a scan
        // over the first four warps).
        uint32_t len = 0;
        if (threadIdx.x < T::NR) {
            const int yy = y0 - 1 + int(threadIdx.x) % (TY + 2), zz = z0 - 1 + int(threadIdx.x) / (TY + 2);
            uint32_t pb = 0;
            if (yy >= 0 && yy < s.ny && zz >= 0 && zz < s.nz) {
                const int xa = max(x0 - 1, 0), xb = min(x0 + TX, s.nx - 1);
                const uint32_t rowc = uint32_t(s.nx) * (uint32_t(yy) + uint32_t(s.ny) * uint32_t(zz));
                pb = s.start[rowc + xa];
                len = s.start[rowc + xb + 1] - pb;
            }
            s_rs[threadIdx.x] = pb;
        }
        uint32_t inc = len;
        if (threadIdx.x < 128) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (lane == 31) s_wt[warp] = inc;
        }
        __syncthreads();
        if (threadIdx.x < T::NR) {
            uint32_t pre = 0;
            for (int k2 = 0; k2 < warp; k2++) pre += s_wt[k2];
            s_rb[threadIdx.x + 1] = pre + inc;
            if (threadIdx.x == 0) s_rb[0] = 0;
        }
        const int n[3] = {s.nx, s.ny, s.nz};
        const int org[3] = {x0, y0, z0};
        const int TT[3] = {TX, TY, TZ};
        // Owned face box per component: full tile, plus the upper boundary face on the own axis
        // for the last tile along that axis.
        int E[3][3];
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (a == c) E[c][a] = (org[a] + TT[a] >= n[a]) ? (n[a] + 1 - org[a]) : TT[a];
                else E[c][a] = min(TT[a], n[a] - org[a]);
            }
        const int sbase[3] = {0, T::FU, T::FU + T::FV};
        const int sdx[3] = {TX + 1, TX, TX};
        const int sdy[3] = {TY, TY + 1, TY};
        const bool packed = pack && __ldg(s.chunk + (s.nc + SCAN_CHUNK - 1) / SCAN_CHUNK) == 0;
        for (int i = threadIdx.x; i < T::NF; i += blockDim.x) spk[i] = 0ull;   // also zeroes sacc / swac
        __syncthreads();
        if (packed) p2g_tile<TX, TY, TZ, true>(s, sacc, swac, spk, org, E, strided & 1, (strided & 2) != 0, s_rb, s_rs);
        else p2g_tile<TX, TY, TZ, false>(s, sacc, swac, spk, org, E, strided & 1, (strided & 2) != 0, s_rb, s_rs);
        __syncthreads();

        // Epilogue: normalize + forces for the owned faces.
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int ex = E[c][0], ey = E[c][1], ez = E[c][2];
            const int cnt = ex * ey * ez;
            const uint32_t fdx = uint32_t(s.nx + (c == 0)), fdy = uint32_t(s.ny + (c == 1));
            const uint32_t fbase = c == 0 ? 0u : (c == 1 ? s.nu : s.nu + s.nv);
            const float gdt = s.g[c] * s.dt;
            for (int idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                const int lx = idx % ex, ly = (idx / ex) % ey, lz = idx / (ex * ey);
                const int si2 = sbase[c] + lx + sdx[c] * (ly + sdy[c] * lz);
                int a, wv;
                if (packed) {
                    const unsigned long long pk = spk[si2];
                    a = static_cast<int>(static_cast<uint32_t>(pk >> 32));
                    wv = static_cast<int>(static_cast<uint32_t>(pk));
                } else {
                    a = sacc[si2];
                    wv = swac[si2];
                }
                const float v = wv > 0 ? float(a) / float(wv) : 0.0f;
                const int fx = x0 + lx, fy = y0 + ly, fz = z0 + lz;
                const uint32_t fi = fbase + uint32_t(fx) + fdx * (uint32_t(fy) + fdy * uint32_t(fz));
                s.vel_old[fi] = v;
                int lo[3] = {fx, fy, fz};
                lo[c] -= 1;
                const bool solid = wall_or_out(s, lo[0], lo[1], lo[2]) || wall_or_out(s, fx, fy, fz);
                s.vel[fi] = solid ? 0.0f : v + gdt;
                if (s.acc) { s.acc[fi] = a; s.wacc[fi] = wv; }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ P2G tile order
// Bucket of every tile (leading zeros of its own cells' particle count) and the bucket sizes:
// one warp per tile, lanes over the tile's x-rows.
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(256) k_tile_weigh(Work w, uint32_t* __restrict__ bucket, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kOrderBuckets];
    for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (item < w.total) {
        const int si = find_sim(w, item);
        const SimDev& s = w.sims[si];
        const int nx = s.nx, ny = s.ny, nz = s.nz;
        const uint32_t* __restrict__ start = s.start;
        const uint32_t t = item - w.base[si];
        const int ntx = (nx + TX - 1) / TX, nty = (ny + TY - 1) / TY;
        const int x0 = int(t % uint32_t(ntx)) * TX;
        const int y0 = int((t / uint32_t(ntx)) % uint32_t(nty)) * TY;
        const int z0 = int(t / uint32_t(ntx * nty)) * TZ;
        const int x1 = min(x0 + TX, nx);
        uint32_t weight = 0;
        for (int r = lane; r < TY * TZ; r += 32) {
            const int y = y0 + r % TY, z = z0 + r / TY;
            if (y < ny && z < nz) {
                const uint32_t rowc = uint32_t(nx) * (uint32_t(y) + uint32_t(ny) * uint32_t(z));
                weight += __ldg(start + rowc + x1) - __ldg(start + rowc + x0);
            }
        }
        weight = __reduce_add_sync(0xffffffffu, weight);
        if (lane == 0) {
            const uint32_t b = uint32_t(__clz(weight));
            bucket[item] = b;
            atomicAdd(&sh[b], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Buckets of the 32x8x8 tiles and of the four 32x4x4 tiles inside each, for the automatic
// shape pick: one warp per large tile, two x-rows per lane, a sum per quarter.
__global__ void __launch_bounds__(256) k_tile_weigh_pair(Work big, Work small, uint32_t* __restrict__ bucket_big,
                                                         uint32_t* __restrict__ hist_big,
                                                         uint32_t* __restrict__ bucket_small,
                                                         uint32_t* __restrict__ hist_small) {
    __shared__ uint32_t shb[kOrderBuckets], shs[kOrderBuckets];
    for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x) shb[i] = shs[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (item < big.total) {
        const int si = find_sim(big, item);
        const SimDev& s = big.sims[si];
        const int nx = s.nx, ny = s.ny, nz = s.nz;
        const uint32_t* __restrict__ start = s.start;
        const uint32_t t = item - big.base[si];
        const uint32_t ntx = uint32_t((nx + 31) / 32), pty = uint32_t((ny + 7) / 8);
        const uint32_t px = t % ntx, py = (t / ntx) % pty, pz = t / (ntx * pty);
        const int x0 = int(px) * 32, x1 = min(x0 + 32, nx);
        uint32_t q[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int r = lane + 32 * h;              // row r: y offset r % 8, z offset r / 8
            const int y = int(py) * 8 + (r & 7), z = int(pz) * 8 + (r >> 3);
            uint32_t wr = 0;
            if (y < ny && z < nz) {
                const uint32_t rowc = uint32_t(nx) * (uint32_t(y) + uint32_t(ny) * uint32_t(z));
                wr = __ldg(start + rowc + x1) - __ldg(start + rowc + x0);
            }
            const int quarter = ((r & 7) >= 4 ? 1 : 0) + ((r >> 3) >= 4 ? 2 : 0);
#pragma unroll
            for (int k = 0; k < 4; k++) q[k] += quarter == k ? wr : 0u;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) q[k] = __reduce_add_sync(0xffffffffu, q[k]);
        if (lane == 0) {
            const uint32_t b = uint32_t(__clz(q[0] + q[1] + q[2] + q[3]));
            bucket_big[item] = b;
            atomicAdd(&shb[b], 1u);
        }
        if (lane < 4) {
            const uint32_t sy = 2u * py + uint32_t(lane & 1), sz = 2u * pz + uint32_t(lane >> 1);
            const uint32_t nty = uint32_t((ny + 3) / 4), ntz = uint32_t((nz + 3) / 4);
            if (sy < nty && sz < ntz) {
                const uint32_t wq = lane == 0 ? q[0] : lane == 1 ? q[1] : lane == 2 ? q[2] : q[3];
                const uint32_t b = uint32_t(__clz(wq));
                bucket_small[small.base[si] + px + ntx * (sy + nty * sz)] = b;
                atomicAdd(&shs[b], 1u);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kOrderBuckets; i += blockDim.x) {
        if (shb[i]) atomicAdd(&hist_big[i], shb[i]);
        if (shs[i]) atomicAdd(&hist_small[i], shs[i]);
    }
}

// Places every tile after the tiles of the heavier buckets: one global reservation per bucket
// and block, shared-memory ranks inside the block.
__global__ void __launch_bounds__(256) k_tile_place(uint32_t total, const uint32_t* __restrict__ bucket,
                                                    uint32_t* __restrict__ hist, uint32_t* __restrict__ order) {
    __shared__ uint32_t off[kOrderBuckets], cnt[kOrderBuckets];
    if (threadIdx.x < kOrderBuckets) {
        cnt[threadIdx.x] = 0;
        off[threadIdx.x] = hist[threadIdx.x];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0;
        for (int i = 0; i < kOrderBuckets; i++) {
            const uint32_t c = off[i];
            off[i] = a;
            a += c;
        }
    }
    __syncthreads();
    const uint32_t item = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t b = 0, rank = 0;
    if (item < total) {
        b = bucket[item];
        rank = atomicAdd(&cnt[b], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kOrderBuckets && cnt[threadIdx.x])
        off[threadIdx.x] += atomicAdd(&hist[kOrderBuckets + threadIdx.x], cnt[threadIdx.x]);
    __syncthreads();
    if (item < total) order[off[b] + rank] = item;
}

// ------------------------------------------------------------------ divergence
// fluid.slang:153-165, plus the per-cell neighbour record used by both pressure solvers.
__global__ void __launch_bounds__(256) k_divergence(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t c = (item - w.base[si]) * 256 + threadIdx.x;
        if (c >= s.nc) continue;
        const uint32_t nx = uint32_t(s.nx), ny = uint32_t(s.ny), nxy = nx * ny;
        const int i = int(c % nx), j = int((c / nx) % ny), k = int(c / nxy);
        float d = 0.0f;
        uint16_t info = 0;
        if (s.type[c] == FLUID) {
            // u faces: (i, j, k) and (i+1, j, k); v faces base nu; w faces base nu + nv.
            const uint32_t ui = uint32_t(i) + (nx + 1) * (uint32_t(j) + ny * uint32_t(k));
            const uint32_t vi = s.nu + uint32_t(i) + nx * (uint32_t(j) + (ny + 1) * uint32_t(k));
            const uint32_t wi = s.nu + s.nv + c;
            d += s.vel[ui + 1] - s.vel[ui];
            d += s.vel[vi + nx] - s.vel[vi];
            d += s.vel[wi + nxy] - s.vel[wi];
            // Neighbours -x, +x, -y, +y, -z, +z (fluid.slang:173-180). A fluid cell is never on
            // the wall layer, so every neighbour is inside the grid.
            const int64_t off[6] = {-1, 1, -int64_t(nx), int64_t(nx), -int64_t(nxy), int64_t(nxy)};
            uint32_t mask = 0, cnt = 0;
#pragma unroll
            for (int q = 0; q < 6; q++) {
                const uint8_t t = s.type[int64_t(c) + off[q]];
                if (t != SOLID) cnt++;
                if (t == FLUID) mask |= 1u << q;
            }
            info = uint16_t(mask | (cnt << 8) | 0x8000u);
        }
        s.div[c] = d * s.inv_h;
        s.info[c] = info;
    }
}

// ------------------------------------------------------------------ red-black Gauss-Seidel
// fluid.slang:167-182: one colour per launch; iteration `it` is skipped by simulations with fewer
// pressure iterations than the batch maximum.
__global__ void __launch_bounds__(256) k_pressure_rb(Work w, uint32_t parity, uint32_t it) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        if (it >= s.iterations || s.solver != 0) continue;
        const uint32_t hx = (uint32_t(s.nx) + 1) >> 1;
        const uint32_t q = (item - w.base[si]) * 256 + threadIdx.x;
        const uint32_t row = q / hx;
        if (row >= uint32_t(s.ny) * uint32_t(s.nz)) continue;
        const uint32_t ny = uint32_t(s.ny);
        const uint32_t j = row % ny, k = row / ny;
        const uint32_t i = 2 * (q - row * hx) + ((j + k + parity) & 1u);
        if (i >= uint32_t(s.nx)) continue;
        const uint32_t nx = uint32_t(s.nx), nxy = nx * ny;
        const uint32_t c = i + nx * row;
        const uint32_t inf = s.info[c];
        if (!(inf & 0x8000u)) continue;
        const float* p = s.pressure;
        float sum = 0.0f;
        if (inf & 1u) sum += p[c - 1];
        if (inf & 2u) sum += p[c + 1];
        if (inf & 4u) sum += p[c - nx];
        if (inf & 8u) sum += p[c + nx];
        if (inf & 16u) sum += p[c - nxy];
        if (inf & 32u) sum += p[c + nxy];
        const float cnt = float((inf >> 8) & 7u);
        if (cnt > 0.0f) s.pressure[c] = (sum - s.div[c] * s.h * s.h / s.dt) / cnt;
    }
}

// ------------------------------------------------------------------ project
// fluid.slang:184-197. With the precision solver the pressure difference comes from the FP64
// solution.
// One thread per cell: the u, v and w faces on the cell's low side (and, in the last cell of a
// row, column or layer, the face on its high side, which touches the outside and becomes 0).
// Every face is updated once with the reference's arithmetic; consecutive threads touch
// consecutive cells and faces.
__device__ __forceinline__ void project_face(const SimDev& s, uint32_t id, int c, int fx, int fy, int fz) {
    int lo[3] = {fx, fy, fz};
    lo[c] -= 1;
    if (wall_or_out(s, lo[0], lo[1], lo[2]) || wall_or_out(s, fx, fy, fz)) {
        s.vel[id] = 0.0f;
        return;
    }
    const uint32_t nx = uint32_t(s.nx), ny = uint32_t(s.ny);
    const uint32_t cb = uint32_t(fx) + nx * (uint32_t(fy) + ny * uint32_t(fz));
    const uint32_t ca = uint32_t(lo[0]) + nx * (uint32_t(lo[1]) + ny * uint32_t(lo[2]));
    const uint8_t ta = s.type[ca], tb = s.type[cb];
    if (ta == FLUID || tb == FLUID) {
        float dp;
        if (s.solver == 0) {
            const float pa = ta == FLUID ? s.pressure[ca] : 0.0f;
            const float pb = tb == FLUID ? s.pressure[cb] : 0.0f;
            dp = pb - pa;
        } else {
            const double pa = ta == FLUID ? s.x64[ca] : 0.0;
            const double pb = tb == FLUID ? s.x64[cb] : 0.0;
            dp = float(pb - pa);
        }
        s.vel[id] -= s.dt * s.inv_h * dp;
    }
}

__global__ void __launch_bounds__(256) k_project(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev& s = w.sims[si];
        const uint32_t c = (item - w.base[si]) * 256 + threadIdx.x;
        if (c >= s.nc) continue;
        const uint32_t nx = uint32_t(s.nx), ny = uint32_t(s.ny), nz = uint32_t(s.nz);
        const int i = int(c % nx), j = int((c / nx) % ny), k = int(c / (nx * ny));
        const uint32_t fu = uint32_t(i) + (nx + 1) * (uint32_t(j) + ny * uint32_t(k));
        const uint32_t fv = s.nu + uint32_t(i) + nx * (uint32_t(j) + (ny + 1) * uint32_t(k));
        const uint32_t fw = s.nu + s.nv + c;
        project_face(s, fu, 0, i, j, k);
        project_face(s, fv, 1, i, j, k);
        project_face(s, fw, 2, i, j, k);
        if (uint32_t(i) == nx - 1) project_face(s, fu + 1, 0, i + 1, j, k);
        if (uint32_t(j) == ny - 1) project_face(s, fv + nx, 1, i, j + 1, k);
        if (uint32_t(k) == nz - 1) project_face(s, fw + nx * ny, 2, i, j, k + 1);
    }
}

// ------------------------------------------------------------------ G2P + advection + binning
// fluid.slang:67-84 (trilinear sampling with clamped indices) and 199-220. Both buffers are
// sampled with one index/weight computation; when every tap lies inside the face grid the clamp
// is the identity and the taps use constant offsets (same values, same summation order).
struct Taps {
    float w[8];
    uint32_t idx[8];
};

__device__ __forceinline__ void face_taps(const SimDev& s, int c, float x, float y, float z, Taps& t) {
    const float xs[3] = {x, y, z};
    const int n[3] = {s.nx, s.ny, s.nz};
    int b[3], d[3];
    float wt[3][2];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float g = (xs[a] - s.o[a]) * s.inv_h - 0.5f;
        if (a == c) g += 0.5f;
        b[a] = f2i(floorf(g));
        const float f = g - float(b[a]);
        // fmix(1 - f, f, 0) and fmix(1 - f, f, 1) (fluid.slang's lerp weights) are exactly 1 - f
        // and f: f = g - floor(g) is +0 <= f < 1 or NaN (never infinite), so f * 0 is +0 or NaN,
        // (1 - f) * 0 likewise, and adding +0 to 1 - f (never -0) or to f changes no bit.
        wt[a][0] = 1.0f - f;
        wt[a][1] = f;
        d[a] = n[a] + (a == c) - 1;
    }
    const uint32_t fdx = uint32_t(d[0] + 1), fdy = uint32_t(d[1] + 1);
    const bool inside = b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && b[0] < d[0] && b[1] < d[1] && b[2] < d[2];
    const float wxy[2][2] = {{wt[0][0] * wt[1][0], wt[0][0] * wt[1][1]}, {wt[0][1] * wt[1][0], wt[0][1] * wt[1][1]}};
    if (inside) {
        const uint32_t base = uint32_t(b[0]) + fdx * (uint32_t(b[1]) + fdy * uint32_t(b[2]));
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
            t.w[k] = wxy[ox][oy] * wt[2][oz];
            t.idx[k] = base + uint32_t(ox) + fdx * uint32_t(oy) + fdx * fdy * uint32_t(oz);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
            const int qx = clampi(b[0] + ox, 0, d[0]);
            const int qy = clampi(b[1] + oy, 0, d[1]);
            const int qz = clampi(b[2] + oz, 0, d[2]);
            t.w[k] = wxy[ox][oy] * wt[2][oz];
            t.idx[k] = uint32_t(qx) + fdx * (uint32_t(qy) + fdy * uint32_t(qz));
        }
    }
}

__device__ __forceinline__ float gather(const float* __restrict__ buf, const Taps& t) {
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) acc += t.w[k] * __ldg(buf + t.idx[k]);
    return acc;
}

__global__ void __launch_bounds__(256, 4) k_g2p(Work w) {
    // The particle records of the thread's next item are loaded before the current one is
    // processed, so their HBM latency overlaps the current gathers.
    float4 Pn = make_float4(0, 0, 0, 0), Vn = Pn;
    if (blockIdx.x < w.total) {
        const int si = find_sim(w, blockIdx.x);
        const uint32_t i = (blockIdx.x - w.base[si]) * 256 + threadIdx.x;
        if (i < w.sims[si].np) {
            Pn = w.sims[si].posB[i];
            Vn = w.sims[si].velB[i];
        }
    }
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev s = w.sims[si];
        const uint32_t i = (item - w.base[si]) * 256 + threadIdx.x;
        const bool live = i < s.np;
        uint32_t cell = 0xffffffffu;
        float4 P = Pn, V = Vn;
        {
            const uint32_t nx_item = item + gridDim.x;
            if (nx_item < w.total) {
                const int sn = find_sim(w, nx_item);
                const uint32_t in = (nx_item - w.base[sn]) * 256 + threadIdx.x;
                if (in < w.sims[sn].np) {
                    Pn = w.sims[sn].posB[in];
                    Vn = w.sims[sn].velB[in];
                }
            }
        }
        if (live) {
            const float* fvel[3] = {s.vel, s.vel + s.nu, s.vel + s.nu + s.nv};
            const float* fold[3] = {s.vel_old, s.vel_old + s.nu, s.vel_old + s.nu + s.nv};
            float pic[3], old[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                Taps t;
                face_taps(s, c, P.x, P.y, P.z, t);
                pic[c] = gather(fvel[c], t);
                old[c] = gather(fold[c], t);
            }
            const float pv[3] = {V.x, V.y, V.z};
            float x[3] = {P.x, P.y, P.z};
            float v[3], mid[3];
            const float hdt = 0.5f * s.dt;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float fl = pv[a] + pic[a] - old[a];
                v[a] = fmix(pic[a], fl, s.flip);
                mid[a] = x[a] + hdt * pic[a];
            }
            float sv[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                Taps t;
                face_taps(s, c, mid[0], mid[1], mid[2], t);
                sv[c] = gather(fvel[c], t);
            }
            const int n[3] = {s.nx, s.ny, s.nz};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                x[a] += s.dt * sv[a];
                const float lo = s.o[a] + s.h * 1.001f;
                const float hi = s.o[a] + s.h * (float(n[a]) - 1.001f);
                // max(v, 0) / min(v, 0) as (v < 0 ? 0 : v) / (0 < v ? 0 : v): NaN and -0 pass through.
                if (x[a] < lo) { x[a] = lo; v[a] = v[a] < 0.0f ? 0.0f : v[a]; }
                if (x[a] > hi) { x[a] = hi; v[a] = 0.0f < v[a] ? 0.0f : v[a]; }
            }
            P.x = x[0]; P.y = x[1]; P.z = x[2];
            V.x = v[0]; V.y = v[1]; V.z = v[2];
            cell = cell_of(s, x[0], x[1], x[2]);
        }
        // Bin for the next substep: warp-aggregated count per cell.
        const unsigned active = __ballot_sync(0xffffffffu, live);
        if (live) {
            const unsigned peers = __match_any_sync(active, cell);
            const int lane = threadIdx.x & 31;
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&s.count[cell], uint32_t(__popc(peers)));
            base = __shfl_sync(peers, base, leader);
            V.w = __uint_as_float(base + __popc(peers & ((1u << lane) - 1u)));
            s.posA[i] = P;
            s.velA[i] = V;
        }
    }
}

// ------------------------------------------------------------------ particle I/O
// Current particles -> reference AoS layout [x, y, z, 0, vx, vy, vz, 0] in seeding order.
__global__ void k_gather_aos(SimDev s, float4* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.np; i += gridDim.x * blockDim.x) {
        const float4 P = s.posA[i];
        const float4 V = s.velA[i];
        const uint32_t pid = __float_as_uint(P.w);
        if (pid < s.np) {
            out[2 * pid] = make_float4(P.x, P.y, P.z, 0.0f);
            out[2 * pid + 1] = make_float4(V.x, V.y, V.z, 0.0f);
        }
    }
}

// Reference AoS layout -> current particles; particle i keeps id i.
__global__ void k_scatter_aos(SimDev s, const float4* __restrict__ in) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.np; i += gridDim.x * blockDim.x) {
        const float4 P = in[2 * i];
        const float4 V = in[2 * i + 1];
        s.posA[i] = make_float4(P.x, P.y, P.z, __uint_as_float(i));
        s.velA[i] = make_float4(V.x, V.y, V.z, 0.0f);
    }
}

// Per-cell counts of the last binning, from the scan (start[c + 1] - start[c]).
__global__ void k_counts_from_start(SimDev s, uint32_t* __restrict__ out) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < s.nc; c += gridDim.x * blockDim.x)
        out[c] = s.start[c + 1] - s.start[c];
}

// ------------------------------------------------------------------ launchers
thread_local uint64_t g_kernel_launches = 0;
thread_local LaunchLog* g_launch_log = nullptr;

__global__ void k_hold(long long cycles) {
    const long long t0 = clock64();
    while (clock64() - t0 < cycles) {
    }
}

cudaError_t launch_hold(long long cycles, cudaStream_t st) {
    k_hold<<<1, 32, 0, st>>>(cycles);
    return cudaGetLastError();
}

static int g_sm_count = 0;

int sm_count() {
    if (!g_sm_count) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}

// Blocks per launch: every item its own block up to the cap (PXF_GRID_CAP blocks per SM,
// default 8), beyond which blocks loop over items.
int grid_cap_per_sm() {
    static const int cap = [] { const char* v = std::getenv("PXF_GRID_CAP"); int c = v ? std::atoi(v) : 8; return c > 0 ? c : 8; }();
    return cap;
}

static unsigned grid_for(uint32_t total, int per_sm) {
    if (per_sm == 8) per_sm = grid_cap_per_sm();
    const uint32_t cap = uint32_t(sm_count() * per_sm);
    return total < cap ? (total ? total : 1u) : cap;
}

static inline Work mk(const StageWork& sw) {
    Work w;
    w.sims = sw.sims;
    w.base = sw.base;
    w.n_sims = sw.n_sims;
    w.total = sw.total;
    return w;
}

template <int TX, int TY, int TZ>
static cudaError_t launch_p2g_t(const StageWork& sw, int lanes, const uint32_t* order, cudaStream_t st) {
    using T = P2GTile<TX, TY, TZ>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_p2g<TX, TY, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    static const int pack = [] { const char* v = std::getenv("PXF_P2G_PACKED"); return v ? std::atoi(v) : 0; }();
    // One block per tile: tiles of the liquid hold most of the work and those of the air none, so
    // the block scheduler's dynamic assignment (heaviest tiles first with an order) balances the
    // SMs (a grid-strided loop would not).
    k_p2g<TX, TY, TZ><<<sw.total ? sw.total : 1u, 256, T::SMEM, st>>>(mk(sw), lanes, pack, order);
    note_launch("k_p2g", st);
    return cudaGetLastError();
}

template <int TX, int TY, int TZ>
static cudaError_t launch_tile_weigh_t(const StageWork& sw, const TileOrder& o, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(o.hist, 0, 2 * kOrderBuckets * sizeof(uint32_t), st);
    if (e != cudaSuccess || sw.total == 0) return e;
    k_tile_weigh<TX, TY, TZ><<<(sw.total + 7) / 8, 256, 0, st>>>(mk(sw), o.bucket, o.hist);
    note_launch("k_tile_weigh", st);
    return cudaGetLastError();
}

template <int TX, int TY, int TZ>
static uint32_t p2g_slots_t() {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_p2g<TX, TY, TZ>, 256, P2GTile<TX, TY, TZ>::SMEM);
    return uint32_t(std::max(per_sm, 1)) * uint32_t(std::max(sm_count(), 1));
}

const int kP2GShapes[][3] = {{32, 8, 8}, {32, 4, 4}, {16, 8, 8}, {64, 4, 4}, {16, 4, 4}};
const int kNumP2GShapes = 5;
static_assert(5 <= kMaxP2GShapes, "per-shape tables");

void p2g_shape(int shape, int out[3]) {
    if (shape < 0 || shape >= kNumP2GShapes) shape = 0;
    out[0] = kP2GShapes[shape][0];
    out[1] = kP2GShapes[shape][1];
    out[2] = kP2GShapes[shape][2];
}

cudaError_t launch_p2g(const StageWork& sw, int shape, int lanes, const uint32_t* order, cudaStream_t st) {
    switch (shape) {
        case 1: return launch_p2g_t<32, 4, 4>(sw, lanes, order, st);
        case 2: return launch_p2g_t<16, 8, 8>(sw, lanes, order, st);
        case 3: return launch_p2g_t<64, 4, 4>(sw, lanes, order, st);
        case 4: return launch_p2g_t<16, 4, 4>(sw, lanes, order, st);
        default: return launch_p2g_t<32, 8, 8>(sw, lanes, order, st);
    }
}


cudaError_t launch_tile_weigh(const StageWork& sw, int shape, const TileOrder& o, cudaStream_t st) {
    switch (shape) {
        case 1: return launch_tile_weigh_t<32, 4, 4>(sw, o, st);
        case 2: return launch_tile_weigh_t<16, 8, 8>(sw, o, st);
        case 3: return launch_tile_weigh_t<64, 4, 4>(sw, o, st);
        case 4: return launch_tile_weigh_t<16, 4, 4>(sw, o, st);
        default: return launch_tile_weigh_t<32, 8, 8>(sw, o, st);
    }
}

cudaError_t launch_tile_place(const StageWork& sw, const TileOrder& o, cudaStream_t st) {
    if (sw.total == 0) return cudaSuccess;
    k_tile_place<<<(sw.total + 255) / 256, 256, 0, st>>>(sw.total, o.bucket, o.hist, o.order);
    note_launch("k_tile_place", st);
    return cudaGetLastError();
}

cudaError_t launch_tile_weigh_pair(const StageWork& big, const StageWork& small, const TileOrder& ob,
                                  const TileOrder& os, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(ob.hist, 0, 2 * kOrderBuckets * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(os.hist, 0, 2 * kOrderBuckets * sizeof(uint32_t), st);
    if (e != cudaSuccess || big.total == 0) return e;
    k_tile_weigh_pair<<<(big.total + 7) / 8, 256, 0, st>>>(mk(big), mk(small), ob.bucket, ob.hist, os.bucket, os.hist);
    note_launch("k_tile_weigh", st);
    return cudaGetLastError();
}

cudaError_t launch_tile_order(const StageWork& sw, int shape, const TileOrder& o, cudaStream_t st) {
    cudaError_t e = launch_tile_weigh(sw, shape, o, st);
    return e != cudaSuccess ? e : launch_tile_place(sw, o, st);
}

uint32_t p2g_slots(int shape) {
    switch (shape) {
        case 1: return p2g_slots_t<32, 4, 4>();
        case 2: return p2g_slots_t<16, 8, 8>();
        case 3: return p2g_slots_t<64, 4, 4>();
        case 4: return p2g_slots_t<16, 4, 4>();
        default: return p2g_slots_t<32, 8, 8>();
    }
}

__global__ void k_p2g_pick(const uint32_t* __restrict__ hist, uint32_t fair, cudaGraphConditionalHandle h) {
    // one warp: the heaviest non-empty bucket (buckets 0..31 by lane; none of them: empty tiles)
    const unsigned nonempty = __ballot_sync(0xffffffffu, hist[threadIdx.x] != 0u);
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const bool small = p2g_small_for_bucket(nonempty ? __ffs(nonempty) - 1 : 32, fair);
    cudaGraphSetConditional(h, small ? 0u : 1u);
}

cudaError_t launch_p2g_pick(const uint32_t* hist, uint32_t fair, cudaGraphConditionalHandle h, cudaStream_t st) {
    k_p2g_pick<<<1, 32, 0, st>>>(hist, fair, h);
    note_launch("k_p2g_pick", st);
    return cudaGetLastError();
}

cudaError_t launch_scan(const StageWork& chunks, const SimDev* sims, int n_sims, cudaStream_t st) {
    k_scan_chunks<<<grid_for(chunks.total, 8), 256, 0, st>>>(mk(chunks)); note_launch("k_scan_chunks", st);
    k_scan_sims<<<n_sims, 1024, 0, st>>>(sims, n_sims); note_launch("k_scan_sims", st);
    k_scan_apply<<<grid_for(chunks.total, 8), 256, 0, st>>>(mk(chunks)); note_launch("k_scan_apply", st);
    return cudaGetLastError();
}

cudaError_t launch_scatter(const StageWork& parts, cudaStream_t st) {
    k_scatter<<<grid_for(parts.total, 8), 256, 0, st>>>(mk(parts)); note_launch("k_scatter", st);
    return cudaGetLastError();
}

cudaError_t launch_bin(const StageWork& parts, cudaStream_t st) {
    k_bin<<<grid_for(parts.total, 8), 256, 0, st>>>(mk(parts)); note_launch("k_bin", st);
    return cudaGetLastError();
}

cudaError_t launch_divergence(const StageWork& cells, cudaStream_t st) {
    k_divergence<<<grid_for(cells.total, 8), 256, 0, st>>>(mk(cells)); note_launch("k_divergence", st);
    return cudaGetLastError();
}

cudaError_t launch_pressure_rb(const StageWork& half_cells, uint32_t parity, uint32_t it, cudaStream_t st) {
    k_pressure_rb<<<grid_for(half_cells.total, 8), 256, 0, st>>>(mk(half_cells), parity, it); note_launch("k_pressure_rb", st);
    return cudaGetLastError();
}

cudaError_t launch_project(const StageWork& cells, cudaStream_t st) {
    k_project<<<grid_for(cells.total, 8), 256, 0, st>>>(mk(cells)); note_launch("k_project", st);
    return cudaGetLastError();
}

cudaError_t launch_g2p(const StageWork& parts, cudaStream_t st) {
    k_g2p<<<grid_for(parts.total, 8), 256, 0, st>>>(mk(parts)); note_launch("k_g2p", st);
    return cudaGetLastError();
}

cudaError_t launch_gather_aos(const SimDev& s, float4* out, cudaStream_t st) {
    k_gather_aos<<<grid_for((s.np + 255) / 256, 8), 256, 0, st>>>(s, out); note_launch("k_gather_aos", st);
    return cudaGetLastError();
}

cudaError_t launch_scatter_aos(const SimDev& s, const float4* in, cudaStream_t st) {
    k_scatter_aos<<<grid_for((s.np + 255) / 256, 8), 256, 0, st>>>(s, in); note_launch("k_scatter_aos", st);
    return cudaGetLastError();
}

cudaError_t launch_counts_from_start(const SimDev& s, uint32_t* out, cudaStream_t st) {
    k_counts_from_start<<<grid_for((s.nc + 255) / 256, 8), 256, 0, st>>>(s, out); note_launch("k_counts_from_start", st);
    return cudaGetLastError();
}

}  // namespace pxf
