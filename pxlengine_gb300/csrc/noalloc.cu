// Cell binning of caller-owned particles without any allocation.
//
// Callers that cannot call cudaMalloc (a renderer that owns every device buffer through its
// own allocator or graphics interop, a real-time thread that must not allocate, code running
// while another component captures the device's work) pass their particle buffer and an
// output buffer; the only scratch of the computation, the per-chunk sums of the exclusive scan,
// lives in a fixed array below. The kernels are variants of the counting-sort scan in
// substep.cu that read and write that array instead of a simulation's own scratch buffer.
#include <cstdint>
#include <mutex>
#include <string>
#include <unordered_map>

#include "../../include/pxlflip.h"
#include "pxf_device.cuh"

namespace pxf {

namespace {

constexpr uint32_t kChunk = 2048;                       // cells per scan chunk (256 threads x 8)
constexpr uint32_t kMaxChunks = 8192;                   // -> at most 16,777,216 cells
constexpr uint64_t kMaxCells = uint64_t(kChunk) * kMaxChunks;

// Scratch shared by every call on a device: one 32-bit sum per chunk (32 KiB), held by every GPU
// that loads the library until the process exits. Each call writes every entry it later reads,
// so nothing needs clearing between calls; calls that overlap on the GPU share it and race.
// Host code must not pass `g_scan_chunks` itself to a kernel (on the host that name is only a
// stand-in for the device symbol): it passes the address cudaGetSymbolAddress returns.
static __device__ __align__(256) uint32_t g_scan_chunks[kMaxChunks];

struct Grid {
    int nx, ny, nz;
    float ox, oy, oz, inv_h;
    uint32_t nc;
};

__device__ __forceinline__ uint32_t cell_of_na(const Grid& g, float x, float y, float z) {
    const int i = clampi(f2i(floorf((x - g.ox) * g.inv_h)), 0, g.nx - 1);
    const int j = clampi(f2i(floorf((y - g.oy) * g.inv_h)), 0, g.ny - 1);
    const int k = clampi(f2i(floorf((z - g.oz) * g.inv_h)), 0, g.nz - 1);
    return uint32_t(i) + uint32_t(g.nx) * (uint32_t(j) + uint32_t(g.ny) * uint32_t(k));
}

__global__ void k_na_zero(uint32_t* __restrict__ out, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = 0;
}

// Per-cell particle counts into out[0 .. nc) (warp-aggregated atomics, as in k_bin).
__global__ void k_na_count(Grid g, const float4* __restrict__ parts, uint32_t n, uint32_t* __restrict__ out) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < n;
        uint32_t c = 0;
        if (live) {
            const float4 p = parts[2 * size_t(i)];   // [x, y, z, w, vx, vy, vz, w] records
            c = cell_of_na(g, p.x, p.y, p.z);
        }
        const unsigned active = __ballot_sync(0xffffffffu, live);
        if (live) {
            const unsigned peers = __match_any_sync(active, c);
            if ((threadIdx.x & 31) == unsigned(__ffs(peers) - 1)) atomicAdd(&out[c], uint32_t(__popc(peers)));
        }
    }
}

__global__ void __launch_bounds__(256) k_na_chunks(const uint32_t* __restrict__ counts, uint32_t nc,
                                                    uint32_t* __restrict__ chunks) {
    __shared__ uint32_t red[8];
    const uint32_t nchunks = (nc + kChunk - 1) / kChunk;
    for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t c = chunk * kChunk + k * 256 + threadIdx.x;
            if (c < nc) sum += counts[c];
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

// Exclusive scan of the chunk sums (one block); out[nc] = total.
__global__ void __launch_bounds__(1024) k_na_scan_chunks(uint32_t nc, uint32_t* __restrict__ out,
                                                         uint32_t* __restrict__ chunks) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const uint32_t nchunks = (nc + kChunk - 1) / kChunk;
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
    if (threadIdx.x == 0) out[nc] = carry;
}

// In-place exclusive scan of out[0 .. nc) with the chunk offsets.
__global__ void __launch_bounds__(256) k_na_apply(uint32_t* __restrict__ out, uint32_t nc,
                                                   const uint32_t* __restrict__ chunks) {
    __shared__ uint32_t wsum[8];
    const uint32_t nchunks = (nc + kChunk - 1) / kChunk;
    for (uint32_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
        const uint32_t c0 = chunk * kChunk + threadIdx.x * 8;
        uint32_t v[8];
        uint32_t tsum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = c0 + k < nc ? out[c0 + k] : 0u;
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
            if (c0 + k < nc) {
                out[c0 + k] = before;
                before += v[k];
            }
        }
        __syncthreads();
    }
}

// Device address of g_scan_chunks in each CUDA context. Every context loads the library's device
// code on its own, so the address belongs to a context, not to a device ordinal: a caller may
// have its own (non-primary) context current, or a primary context may have been destroyed and
// created again. The cache is keyed by the context's process-unique id (cuCtxGetId), reached
// through the runtime's driver entry points because the library links no libcuda.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

std::mutex g_mu;
std::unordered_map<unsigned long long, void*> g_scratch_addr;   // context id -> device address
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

int driver_entry(const char* name, unsigned version, void** fn, std::string& err) {
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    const cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, version, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*fn) {
        err = std::string("driver entry point ") + name + " unavailable" +
              (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        cudaGetLastError();
        return PXF_ECUDA;
    }
    return PXF_OK;
}

int current_context_id(unsigned long long* id, bool* have, std::string& err) {
    void* ctx = nullptr;
    if (g_ctx_current(&ctx) != 0) {
        err = "cuCtxGetCurrent failed";
        return PXF_ECUDA;
    }
    *have = ctx != nullptr;
    if (!ctx) return PXF_OK;
    if (g_ctx_id(ctx, id) != 0) {
        err = "cuCtxGetId failed";
        return PXF_ECUDA;
    }
    return PXF_OK;
}

int scratch_for_current_context(void** addr, std::string& err) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx_current || !g_ctx_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (int rc = driver_entry("cuCtxGetCurrent", 4000, &f1, err)) return rc;
        if (int rc = driver_entry("cuCtxGetId", 12000, &f2, err)) return rc;
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    unsigned long long id = 0;
    bool have = false;
    if (int rc = current_context_id(&id, &have, err)) return rc;
    if (have) {
        auto it = g_scratch_addr.find(id);
        if (it != g_scratch_addr.end()) {
            *addr = it->second;
            return PXF_OK;
        }
    }
    // First call in this context (or no context bound yet: the runtime then binds the current
    // device's primary context while it answers).
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_chunks);
    if (e != cudaSuccess || !p) {
        err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return PXF_ECUDA;
    }
    if (!have) {
        if (int rc = current_context_id(&id, &have, err)) return rc;
        if (!have) {
            err = "no CUDA context is current after the scratch lookup";
            return PXF_ECUDA;
        }
    }
    g_scratch_addr[id] = p;
    *addr = p;
    return PXF_OK;
}

}  // namespace

void set_global_error_message(const std::string& m);   // pxf_last_error(NULL) (engine.cu)

}  // namespace pxf

extern "C" {

int pxf_cell_starts_noalloc(const float* d_particles, uint32_t n, const uint32_t dims[3], const float origin[3],
                            float h, uint32_t* d_cell_start, void* stream) {
    using namespace pxf;
    if (!dims || !origin || !d_cell_start || (n && !d_particles)) {
        set_global_error_message("NULL argument");
        return PXF_EINVAL;
    }
    if (!dims[0] || !dims[1] || !dims[2] || !(h > 0.0f)) {
        set_global_error_message("grid dimensions and cell size must be positive");
        return PXF_EINVAL;
    }
    const uint64_t nc = uint64_t(dims[0]) * dims[1] * dims[2];
    if (nc > kMaxCells) {
        set_global_error_message("grid has " + std::to_string(nc) + " cells, more than the " + std::to_string(kMaxCells) +
                                 " cells the fixed scratch of pxf_cell_starts_noalloc supports");
        return PXF_EINVAL;
    }
    // Set-up on the first call in each CUDA context (the context current on the calling thread,
    // else the current device's primary context): the device address of the scratch array.
    void* scratch = nullptr;
    std::string err;
    const int rc = scratch_for_current_context(&scratch, err);
    if (rc != PXF_OK) {
        set_global_error_message(err);
        return rc;
    }
    uint32_t* chunks = static_cast<uint32_t*>(scratch);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Grid g;
    g.nx = int(dims[0]);
    g.ny = int(dims[1]);
    g.nz = int(dims[2]);
    g.ox = origin[0];
    g.oy = origin[1];
    g.oz = origin[2];
    g.inv_h = 1.0f / h;
    g.nc = uint32_t(nc);
    const uint32_t nchunks = uint32_t((nc + kChunk - 1) / kChunk);
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    const unsigned cap = unsigned(sms) * 8u;
    const unsigned gz = unsigned((nc + 1 + 255) / 256) < cap ? unsigned((nc + 1 + 255) / 256) : cap;
    k_na_zero<<<gz ? gz : 1u, 256, 0, st>>>(d_cell_start, uint32_t(nc + 1));
    if (n) {
        const uint64_t blocks = (uint64_t(n) + 255) / 256;   // 64-bit: no wrap for n near 2^32
        const unsigned gp = blocks < cap ? unsigned(blocks) : cap;
        k_na_count<<<gp, 256, 0, st>>>(g, reinterpret_cast<const float4*>(d_particles), n, d_cell_start);
    }
    const unsigned gc = nchunks < cap ? nchunks : cap;
    k_na_chunks<<<gc, 256, 0, st>>>(d_cell_start, g.nc, chunks);
    k_na_scan_chunks<<<1, 1024, 0, st>>>(g.nc, d_cell_start, chunks);
    k_na_apply<<<gc, 256, 0, st>>>(d_cell_start, g.nc, chunks);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error_message(std::string("launch: ") + cudaGetErrorString(e));
        return PXF_ECUDA;
    }
    return PXF_OK;
}

}  // extern "C"
