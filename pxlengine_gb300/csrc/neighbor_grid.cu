// Neighbour grid of agent simulations: a counting sort of agents by hashed cell
// (shaders/sim.slang:5-7, 28-104; driver crates/pxl-render/src/sim.rs:129-146, 230-260).
//
// The reference runs grid_clear -> grid_count -> scan_local -> scan_blocks -> scan_add ->
// grid_scatter and leaves offsets[h] (first slot of cell h), counts[h] and sorted[] (agent ids
// grouped by cell). Here the count pass also hands every agent its rank inside its cell (a
// warp-aggregated atomic, as the FLIP binning does), so the scatter needs no cursor array:
// slot = offsets[cell] + rank. Counts and offsets are integers and equal the reference's; the
// order of the agents inside one cell follows the atomics, as in the reference.
//
// Every buffer, scratch included, belongs to the caller (pxf_grid_scratch_bytes gives its size);
// the library allocates nothing here.
#include <cstdint>
#include <string>

#include "../../include/pxlflip.h"
#include "pxf_device.cuh"

namespace pxf {

void set_global_error_message(const std::string& m);   // pxf_last_error(NULL) (engine.cu)
int sm_count();

namespace {

constexpr uint32_t kChunk = 2048;   // table entries per scan chunk (256 threads x 8)

struct HashGrid {
    const float* agents;
    uint32_t stride;      // floats per agent record; the position is its first three floats
    uint32_t count;
    float cell_size;
    uint32_t mask;        // table_size - 1
};

// sim.slang:28-31: floor(position / cell_size) per axis, the three products xor-ed, masked.
__device__ __forceinline__ uint32_t agent_cell(const HashGrid& g, uint32_t id) {
    const float* p = g.agents + size_t(id) * g.stride;
    const int cx = f2i(floorf(__ldg(p + 0) / g.cell_size));
    const int cy = f2i(floorf(__ldg(p + 1) / g.cell_size));
    const int cz = f2i(floorf(__ldg(p + 2) / g.cell_size));
    return ((uint32_t(cx) * 73856093u) ^ (uint32_t(cy) * 19349663u) ^ (uint32_t(cz) * 83492791u)) & g.mask;
}

__global__ void k_ng_zero(uint32_t* __restrict__ a, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = 0u;
}

// counts[cell] += 1 per agent (grid_count), with the agent's rank inside its cell kept.
__global__ void k_ng_count(HashGrid g, uint32_t* __restrict__ counts, uint32_t* __restrict__ rank) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < g.count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < g.count;
        const uint32_t c = live ? agent_cell(g, i) : 0u;
        const unsigned active = __ballot_sync(0xffffffffu, live);
        if (live) {
            const unsigned peers = __match_any_sync(active, c);
            const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
            uint32_t b = 0;
            if (lane == leader) b = atomicAdd(&counts[c], uint32_t(__popc(peers)));
            b = __shfl_sync(peers, b, leader);
            rank[i] = b + uint32_t(__popc(peers & ((1u << lane) - 1u)));
        }
    }
}

// Per-chunk sums of the counts.
__global__ void __launch_bounds__(256) k_ng_chunks(const uint32_t* __restrict__ counts, uint32_t n,
                                                    uint32_t* __restrict__ chunks) {
    __shared__ uint32_t red[8];
    const uint32_t nchunks = (n + kChunk - 1) / kChunk;
    for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t c = chunk * kChunk + k * 256 + threadIdx.x;
            if (c < n) sum += counts[c];
        }
        sum = __reduce_add_sync(0xffffffffu, sum);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int k = 0; k < 8; k++) t += red[k];
            chunks[chunk] = t;
        }
        __syncthreads();
    }
}

// Exclusive scan of the chunk sums in one block (any number of chunks, carried between passes).
__global__ void __launch_bounds__(1024) k_ng_scan_chunks(uint32_t n, uint32_t* __restrict__ chunks) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const uint32_t nchunks = (n + kChunk - 1) / kChunk;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nchunks; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nchunks ? chunks[i] : 0u;
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
        if (i < nchunks) chunks[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = before + x;
        __syncthreads();
    }
}

// offsets = exclusive scan of counts (scan_local + scan_add).
__global__ void __launch_bounds__(256) k_ng_offsets(const uint32_t* __restrict__ counts, uint32_t n,
                                                     const uint32_t* __restrict__ chunks, uint32_t* __restrict__ offsets) {
    __shared__ uint32_t wsum[8];
    const uint32_t nchunks = (n + kChunk - 1) / kChunk;
    for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
        const uint32_t c0 = chunk * kChunk + threadIdx.x * 8;
        uint32_t v[8];
        uint32_t tsum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = c0 + k < n ? counts[c0 + k] : 0u;
            tsum += v[k];
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t x = tsum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        uint32_t before = chunks[chunk];
        for (int k = 0; k < wid; k++) before += wsum[k];
        before += x - tsum;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (c0 + k < n) {
                offsets[c0 + k] = before;
                before += v[k];
            }
        }
        __syncthreads();
    }
}

// sorted[offsets[cell] + rank] = agent id (grid_scatter).
__global__ void k_ng_scatter(HashGrid g, const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ rank,
                             uint32_t* __restrict__ sorted) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = offsets[agent_cell(g, i)] + rank[i];
        if (slot < g.count) sorted[slot] = i;   // always true when the counts came from this call
    }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

bool pow2(uint32_t x) { return x && !(x & (x - 1)); }

}  // namespace

}  // namespace pxf

extern "C" {

uint32_t pxf_grid_table_size(uint32_t count) {
    // (count * 2).next_power_of_two().clamp(1024, 1 << 23)
    uint64_t t = 1;
    while (t < uint64_t(count) * 2) t <<= 1;
    if (t < 1024) t = 1024;
    if (t > (uint64_t(1) << 23)) t = uint64_t(1) << 23;
    return uint32_t(t);
}

size_t pxf_grid_scratch_bytes(uint32_t count, uint32_t table_size) {
    using namespace pxf;
    const size_t nchunks = (size_t(table_size) + kChunk - 1) / kChunk;
    return align256(4 * size_t(count)) + align256(4 * (nchunks + 1));
}

int pxf_grid_sort(const float* d_agents, uint32_t stride_floats, uint32_t count, float cell_size, uint32_t table_size,
                  uint32_t* d_offsets, uint32_t* d_counts, uint32_t* d_sorted, void* d_scratch, size_t scratch_bytes,
                  void* stream) {
    using namespace pxf;
    if (!d_offsets || !d_counts || (count && (!d_agents || !d_sorted || !d_scratch))) {
        set_global_error_message("NULL argument");
        return PXF_EINVAL;
    }
    if (!pow2(table_size)) {
        set_global_error_message("table_size must be a power of two (the hash is masked with table_size - 1)");
        return PXF_EINVAL;
    }
    if (count && stride_floats < 3) {
        set_global_error_message("an agent record holds at least its three position floats");
        return PXF_EINVAL;
    }
    if (scratch_bytes < pxf_grid_scratch_bytes(count, table_size)) {
        set_global_error_message("scratch buffer smaller than pxf_grid_scratch_bytes(count, table_size)");
        return PXF_EINVAL;
    }
    HashGrid g;
    g.agents = d_agents;
    g.stride = stride_floats;
    g.count = count;
    g.cell_size = cell_size > 1e-6f ? cell_size : 1e-6f;   // sim.rs:181 (cell_size.max(1e-6))
    g.mask = table_size - 1;
    uint32_t* rank = static_cast<uint32_t*>(d_scratch);
    uint32_t* chunks = reinterpret_cast<uint32_t*>(static_cast<char*>(d_scratch) + align256(4 * size_t(count)));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned cap = unsigned(sm_count()) * 8u;
    auto blocks = [cap](uint64_t n, uint64_t per) {
        const uint64_t b = (n + per - 1) / per;
        return unsigned(b == 0 ? 1 : (b < cap ? b : cap));
    };
    const uint32_t nchunks = (table_size + kChunk - 1) / kChunk;
    k_ng_zero<<<blocks(table_size, 256), 256, 0, st>>>(d_counts, table_size);
    if (count) k_ng_count<<<blocks(count, 256), 256, 0, st>>>(g, d_counts, rank);
    k_ng_chunks<<<blocks(nchunks, 1), 256, 0, st>>>(d_counts, table_size, chunks);
    k_ng_scan_chunks<<<1, 1024, 0, st>>>(table_size, chunks);
    k_ng_offsets<<<blocks(nchunks, 1), 256, 0, st>>>(d_counts, table_size, chunks, d_offsets);
    if (count) k_ng_scatter<<<blocks(count, 256), 256, 0, st>>>(g, d_offsets, rank, d_sorted);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error_message(std::string("launch: ") + cudaGetErrorString(e));
        return PXF_ECUDA;
    }
    return PXF_OK;
}

}  // extern "C"
