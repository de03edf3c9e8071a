// Red-black Gauss-Seidel pressure solve (shaders/fluid.slang:167-182, host loop
// crates/pxl-render/src/fluid.rs:295-300) with two iterations per pass over HBM.
//
// The reference sweeps the whole grid once per colour: 2 x iterations passes over pressure,
// divergence and cell flags. Here one block owns a unit: an x-y tile of kTX x kTY cells and a
// segment of planes along z. It streams the planes of its tile plus a halo of kH = 4 cells (and
// kH planes above and below the segment) through a ring of planes in shared memory and runs the
// four half sweeps of two iterations as a wavefront: when plane z arrives, half sweep 1 (red)
// updates plane z - 1, half sweep 2 (black) plane z - 2, half sweep 3 (red) plane z - 3 and half
// sweep 4 (black) plane z - 4, which is then final and written back. A cell's update reads only
// cells of the other colour, so every update sees exactly the values the reference's order gives
// it, and each half sweep spoils at most one more cell of the halo: after four half sweeps the
// tile interior and the segment's planes are exact. Result: the reference's bits, with one read of
// pressure, right-hand side and neighbour count and one write of pressure per two iterations.
//
// Pressure is double-buffered per pass (a unit reads its halo while its neighbours write their
// interiors): pass j reads buffer j & 1 and writes the other (buffer 0 = pressure, 1 = p_alt).
// k_gs_prep copies pressure into p_alt, evaluates the right-hand side div * h * h / dt (the
// reference's expression and order), stores each system cell's non-solid neighbour count and
// flags the units whose interior holds a system cell; the other units never change and are
// skipped. k_gs_finish copies the result back when a simulation's last pass wrote p_alt.
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "pxf_device.cuh"
#include "pxf_kernels.h"

namespace pxf {

namespace {

constexpr int kLX = kGsLoadX;            // loaded columns of a tile (x): one warp's 32 cell pairs
constexpr int kLY = kGsLoadY;            // loaded rows (y): one warp per row
constexpr int kH = kGsHalo;              // halo: one cell per half sweep
constexpr int kTX = kLX - 2 * kH;        // tile interior
constexpr int kTY = kLY - 2 * kH;
constexpr int kPairs = kLX / 2;          // 32: lane = cell pair
constexpr int kThreads = 32 * kLY;
constexpr int kRing = 8;                 // planes z - 4 .. z + 3 in shared memory
constexpr int kPlane = kLY * kLX;        // floats per plane: rows of [even cells | odd cells]
constexpr int kCntPlane = kLY * 16;      // 32-bit words of counts per plane (4 cells each)
constexpr int kSmemFloats = 2 * kRing * kPlane + kRing * kCntPlane + 1;   // pressure, rhs, counts; + 1 slack
static_assert(kPairs == 32, "a warp covers one loaded row");
static_assert(kH == 2 * kGsIters, "one halo cell per half sweep");
static_assert(kGsIters == 2, "the register ring holds the planes of four half sweeps");

__device__ __forceinline__ void dep_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

struct Unit {
    int x0, y0, z0, z1;   // interior: [x0, x0 + kTX) x [y0, y0 + kTY) x [z0, z1), clipped to the grid below
};

__device__ __forceinline__ Unit unit_of(const SimDev& s, uint32_t u) {
    Unit t;
    const uint32_t tx = u % s.gs_ntx;
    const uint32_t ty = (u / s.gs_ntx) % s.gs_nty;
    const uint32_t zs = u / (s.gs_ntx * s.gs_nty);
    t.x0 = int(tx) * kTX;
    t.y0 = int(ty) * kTY;
    t.z0 = int(zs) * int(s.gs_zs);
    t.z1 = min(t.z0 + int(s.gs_zs), s.nz);
    return t;
}

__device__ __forceinline__ bool system_cell(uint32_t info) { return (info & 0x8000u) && (info & 0x700u); }

// Register and shared-memory slot of plane z - k at unrolled step OFF (planes count from the
// unit's first loaded plane).
__host__ __device__ constexpr int slot_of(int off, int k) { return ((off - k) % kRing + kRing) % kRing; }

// 4-byte asynchronous copy global -> shared; an `in` of false fills the word with zeros.
__device__ __forceinline__ void cp4(void* dst, const void* src, bool in) {
    const uint32_t d = uint32_t(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(in ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

}  // namespace

// ------------------------------------------------------------------ set-up of a solve
// One block per unit: p_alt = pressure, rhs = div * h * h / dt and the non-solid neighbour count
// of every system cell (0 elsewhere) over the unit's interior, and the unit's flag = does the
// interior hold a system cell (fluid with a non-solid neighbour). One warp per x-row.
__global__ void __launch_bounds__(256) k_gs_prep(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev& s = w.sims[si];
        const uint32_t u = item - w.base[si];
        const Unit t = unit_of(s, u);
        const int xe = min(t.x0 + kTX, s.nx), ye = min(t.y0 + kTY, s.ny);
        const int wx = xe - t.x0, wy = ye - t.y0;
        const float h = s.h, dt = s.dt;
        const size_t nx = size_t(s.nx), nxy = nx * size_t(s.ny);
        const float* __restrict__ pr = s.pressure;
        const float* __restrict__ dv = s.div;
        const uint16_t* __restrict__ inf = s.info;
        float* __restrict__ pa = s.p_alt;
        float* __restrict__ rh = s.rhs;
        uint8_t* __restrict__ cn = s.gs_cnt;
        bool mine = false;
        // one warp per x-row of the interior, lanes along x
        const uint32_t rows = uint32_t(wy) * uint32_t(t.z1 - t.z0);
        const int lane = int(threadIdx.x) & 31;
        for (uint32_t row = threadIdx.x >> 5; row < rows; row += blockDim.x >> 5) {
            const uint32_t y = uint32_t(t.y0) + row % uint32_t(wy), z = uint32_t(t.z0) + row / uint32_t(wy);
            const size_t c0 = size_t(t.x0) + nx * size_t(y) + nxy * size_t(z);
            for (int x = lane; x < wx; x += 32) {
                const size_t c = c0 + size_t(x);
                const uint32_t i = inf[c];
                const bool sys = system_cell(i);
                pa[c] = pr[c];
                rh[c] = dv[c] * h * h / dt;
                cn[c] = sys ? uint8_t((i >> 8) & 7u) : uint8_t(0);
                mine |= sys;
            }
        }
        const int any = __syncthreads_or(mine);
        if (threadIdx.x == 0) s.gs_flag[u] = uint32_t(any != 0);
    }
}

// ------------------------------------------------------------------ one pass: two iterations
// pass: index of the pass (buffer parity); it0: first iteration of the pass.
//
// Warp w owns loaded row w, lane l the cell pair (2l, 2l + 1) of that row in every plane. In
// shared memory a plane's row is stored as [even cells | odd cells], so the cells one half sweep
// reads (all of the other colour) lie in consecutive words for consecutive lanes. Planes arrive
// by asynchronous copies three planes ahead. The -z and +z neighbours of a cell belong to the
// same thread, and so do all of a cell's updates, so the thread keeps its own pair of the planes
// z - 5 .. z in registers; other threads read a cell only as an in-plane neighbour, and every
// in-plane neighbour a half sweep of step z reads was written before the barrier that ends step
// z - 1. One barrier per plane. In step z every half sweep updates the cell of x parity
// (y + z + 1) & 1 of the thread's pair (half sweep hs updates plane z - hs with colour hs - 1),
// the same for the whole warp. The plane loop is unrolled kRing times, so every ring slot
// (registers and shared memory) is a constant.
//
// Every fluid neighbour's pressure is added in the reference's order (-x, +x, -y, +y, -z, +z);
// the others hold +0 (non-fluid cells are reset to 0 before the solve and never updated, cells
// outside the grid read 0), and adding +0 to a sum that starts at +0 changes no bit.
__global__ void __launch_bounds__(kThreads, 1) k_gs_pass(Work w, uint32_t pass, uint32_t it0) {
    extern __shared__ float sp[];   // pressure ring [kRing][kLY][2][kPairs], rhs ring the same, count ring
    __shared__ float rcp[8];        // RN(1 / cnt)
    if (threadIdx.x < 8) rcp[threadIdx.x] = threadIdx.x ? 1.0f / float(threadIdx.x) : 0.0f;
    const uint32_t item = blockIdx.x;
    const int si = find_sim(w, item);
    const SimDev& s = w.sims[si];
    const uint32_t u = item - w.base[si];
    const bool run = s.solver == 0 && it0 < s.iterations && __ldg(s.gs_flag + u) != 0u;
    if (!run) {
        dep_wait();
        return;
    }
    const int nhs = 2 * int(min(uint32_t(kGsIters), s.iterations - it0));   // half sweeps of this pass
    const Unit t = unit_of(s, u);
    const int nx = s.nx, ny = s.ny, nz = s.nz;
    const int zlo = max(t.z0 - kH, 0), zhi = min(t.z1 + kH, nz);
    const int lane = int(threadIdx.x) & 31, ly = int(threadIdx.x) >> 5;
    const int X = t.x0 - kH + 2 * lane;
    const int Y = t.y0 - kH + ly;
    const bool rin = Y >= 0 && Y < ny;
    const bool in0 = rin && X >= 0 && X < nx;           // cell 2l inside the grid
    const bool in1 = rin && X + 1 >= 0 && X + 1 < nx;   // cell 2l + 1 inside the grid
    const bool upd_row = rin && ly >= 1 && ly <= kLY - 2;
    const bool upd0 = upd_row && lane >= 1;             // cell 2l is not on the loaded border
    const bool upd1 = upd_row && lane <= kPairs - 2;    // cell 2l + 1 is not on the loaded border
    const bool out_row = rin && ly >= kH && ly < kLY - kH && lane >= kH / 2 && lane < kPairs - kH / 2;
    const bool full = in0 && in1 && (nx & 1) == 0;      // aligned pair inside the grid
    // counts travel as 32-bit words of four cells: lanes 0 .. 15 copy the row's 16 words (a word
    // starts on a multiple of 4 cells when nx is: the loaded row starts at x0 - 4, x0 a multiple
    // of 56), else every lane fetches its own pair's two bytes
    const bool cwords = (nx & 3) == 0;
    const int Xw = t.x0 - kH + 4 * (lane & 15);
    const bool cw_in = cwords && lane < 16 && rin && Xw >= 0 && Xw < nx;
    const float* __restrict__ pin = (pass & 1u) ? s.p_alt : s.pressure;
    float* __restrict__ pout = (pass & 1u) ? s.pressure : s.p_alt;
    const float* __restrict__ grhs = s.rhs;
    const uint8_t* __restrict__ gcnt = s.gs_cnt;
    const uint32_t nxy = uint32_t(nx) * uint32_t(ny);
    const uint32_t rowY = uint32_t(rin ? Y : 0) * uint32_t(nx);
    const uint32_t e0 = rowY + uint32_t(in0 ? X : 0);       // element of cell 2l, plane 0
    const uint32_t e1 = rowY + uint32_t(in1 ? X + 1 : 0);
    const uint32_t ew = rowY + uint32_t(cw_in ? Xw : 0);
    float* const srow = sp + ly * kLX;
    float* const rrow = sp + kRing * kPlane + ly * kLX;                                   // read by this thread only
    uint32_t* const crow = reinterpret_cast<uint32_t*>(sp + 2 * kRing * kPlane) + ly * 16;   // count words of the row

    // Plane z into ring slot `sl` (zeros outside the grid and beyond the loaded planes), one
    // commit group per plane.
    auto issue = [&](int sl, int z) {
        const bool zin = z < zhi;
        const uint32_t o = uint32_t(zin ? z : 0) * nxy;
        cp4(srow + sl * kPlane + lane, pin + e0 + o, zin && in0);
        cp4(srow + sl * kPlane + kPairs + lane, pin + e1 + o, zin && in1);
        cp4(rrow + sl * kPlane + lane, grhs + e0 + o, zin && in0);
        cp4(rrow + sl * kPlane + kPairs + lane, grhs + e1 + o, zin && in1);
        if (cwords && lane < 16) cp4(crow + sl * kCntPlane + lane, gcnt + ew + o, zin && cw_in);
        cp_commit();
    };
    // the pair's counts of plane slot `sl` (two 4-bit fields)
    auto counts = [&](int sl, int z) -> uint32_t {
        if (cwords) {
            const uint32_t wd = crow[sl * kCntPlane + (lane >> 1)] >> (16 * (lane & 1));
            return (wd & 0xfu) | ((wd >> 4) & 0xf0u);
        }
        if (z >= zhi) return 0u;
        const uint32_t o = uint32_t(z) * nxy;
        return (in0 ? uint32_t(__ldg(gcnt + e0 + o)) : 0u) | (in1 ? uint32_t(__ldg(gcnt + e1 + o)) << 4 : 0u);
    };

    float2 P[kRing];   // own pair of plane p in P[(p - zlo) % kRing]
    uint32_t C = 0;    // counts of plane z - k at bits 8 (k - 1) .. 8 k - 1, k = 1 .. 4
#pragma unroll
    for (int k = 0; k < kRing; k++) P[k] = make_float2(0.0f, 0.0f);

    // Right-hand sides and counts are fixed during the solve; pressure is written by the previous pass.
    dep_wait();
    issue(0, zlo);
    issue(1, zlo + 1);
    issue(2, zlo + 2);
    cp_wait<2>();
    __syncthreads();
    P[0] = make_float2(srow[lane], srow[kPairs + lane]);
    uint32_t cnew = counts(0, zlo);   // counts of plane z

    // The half sweeps of step z (unrolled position OFF) for the cells of x parity XB; bit hs of
    // `valid` is set when plane z - hs lies strictly inside the loaded planes.
    auto sweeps = [&](auto off, auto xb, uint32_t valid) {
        constexpr int OFF = decltype(off)::value;
        constexpr int XB = decltype(xb)::value;
        const bool upd = XB ? upd1 : upd0;
#pragma unroll
        for (int hs = 1; hs <= 2 * kGsIters; hs++) {
            if (hs > nhs) break;
            const uint32_t cn = (C >> (8 * (hs - 1) + 4 * XB)) & 0xfu;
            if (!((valid >> hs) & 1u) || !upd || cn == 0u) continue;
            float* const row = srow + slot_of(OFF, hs) * kPlane;
            float sum = 0.0f;
            sum += row[(1 - XB) * kPairs + lane - 1 + XB];   // -x
            sum += row[(1 - XB) * kPairs + lane + XB];       // +x
            sum += row[XB * kPairs + lane - kLX];            // -y
            sum += row[XB * kPairs + lane + kLX];            // +y
            sum += XB ? P[slot_of(OFF, hs + 1)].y : P[slot_of(OFF, hs + 1)].x;   // -z
            sum += XB ? P[slot_of(OFF, hs - 1)].y : P[slot_of(OFF, hs - 1)].x;   // +z
            const float rh = rrow[slot_of(OFF, hs) * kPlane + XB * kPairs + lane];
            const float v = div_count(sum - rh, cn, rcp);
            if (XB) P[slot_of(OFF, hs)].y = v; else P[slot_of(OFF, hs)].x = v;
            row[XB * kPairs + lane] = v;
        }
    };

    // Step z (unrolled position OFF): plane z + 3 requested into the slot of plane z - 5 (which no
    // half sweep of this step reads from shared memory), the half sweeps, the write-back of plane
    // z - nhs, then plane z + 1 is waited for and its own pair and counts read into registers.
    auto step = [&](auto off, int z) {
        constexpr int OFF = decltype(off)::value;
        issue(slot_of(OFF, -3), z + 3);
        const int lo = z - zlo, hi = z - (zhi - 1);   // hs valid: hi < hs < lo
        uint32_t valid = 0;
#pragma unroll
        for (int hs = 1; hs <= 4; hs++) valid |= (hs < lo && hs > hi) ? (1u << hs) : 0u;
        if ((Y + z + 1) & 1) sweeps(off, std::integral_constant<int, 1>{}, valid);
        else sweeps(off, std::integral_constant<int, 0>{}, valid);
        const int qo = z - nhs;
        if (out_row && qo >= t.z0 && qo < t.z1) {
            const float2 v = nhs == 4 ? P[slot_of(OFF, 4)] : P[slot_of(OFF, 2)];
            const uint32_t o = uint32_t(qo) * nxy;
            if (full) {
                __stcg(reinterpret_cast<float2*>(pout + e0 + o), v);
            } else {
                if (in0) pout[e0 + o] = v.x;
                if (in1) pout[e1 + o] = v.y;
            }
        }
        C = (C << 8) | cnew;
        cp_wait<2>();
        __syncthreads();
        constexpr int SN = slot_of(OFF, -1);
        P[SN] = make_float2(srow[SN * kPlane + lane], srow[SN * kPlane + kPairs + lane]);
        cnew = counts(SN, z + 1);
    };

    const int zend = t.z1 - 1 + nhs;
    for (int z = zlo; z <= zend; z += kRing) {
        step(std::integral_constant<int, 0>{}, z);
        if (z + 1 > zend) break;
        step(std::integral_constant<int, 1>{}, z + 1);
        if (z + 2 > zend) break;
        step(std::integral_constant<int, 2>{}, z + 2);
        if (z + 3 > zend) break;
        step(std::integral_constant<int, 3>{}, z + 3);
        if (z + 4 > zend) break;
        step(std::integral_constant<int, 4>{}, z + 4);
        if (z + 5 > zend) break;
        step(std::integral_constant<int, 5>{}, z + 5);
        if (z + 6 > zend) break;
        step(std::integral_constant<int, 6>{}, z + 6);
        if (z + 7 > zend) break;
        step(std::integral_constant<int, 7>{}, z + 7);
    }
    cp_wait<0>();
}

// ------------------------------------------------------------------ end of a solve
// Copies p_alt back into pressure over the active units' interiors of the simulations whose
// last pass wrote p_alt (an odd number of passes).
__global__ void __launch_bounds__(256) k_gs_finish(Work w) {
    for (uint32_t item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int si = find_sim(w, item);
        const SimDev& s = w.sims[si];
        const uint32_t passes = (s.iterations + kGsIters - 1) / kGsIters;
        if (s.solver != 0 || (passes & 1u) == 0) continue;
        const uint32_t u = item - w.base[si];
        if (!__ldg(s.gs_flag + u)) continue;
        const Unit t = unit_of(s, u);
        const int wx = min(t.x0 + kTX, s.nx) - t.x0, wy = min(t.y0 + kTY, s.ny) - t.y0;
        const uint32_t per = uint32_t(wx) * uint32_t(wy), total = per * uint32_t(t.z1 - t.z0);
        for (uint32_t k = threadIdx.x; k < total; k += blockDim.x) {
            const uint32_t z = uint32_t(t.z0) + k / per, r = k % per;
            const uint32_t y = uint32_t(t.y0) + r / uint32_t(wx), x = uint32_t(t.x0) + r % uint32_t(wx);
            const size_t c = size_t(x) + size_t(s.nx) * (size_t(y) + size_t(s.ny) * z);
            s.pressure[c] = s.p_alt[c];
        }
    }
}

// ------------------------------------------------------------------ launches
static size_t pass_smem() { return size_t(kSmemFloats) * sizeof(float); }

cudaError_t gs_stream_attr() {
    return cudaFuncSetAttribute(k_gs_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, int(pass_smem()));
}

cudaError_t launch_gs_stream(const StageWork& units, uint32_t max_iters, cudaStream_t st) {
    if (!units.total || !max_iters) return cudaSuccess;
    const Work w = units;
    const unsigned gp = std::min<unsigned>(units.total, unsigned(sm_count()) * 8u);
    k_gs_prep<<<gp, 256, 0, st>>>(w);
    note_launch("k_gs_prep", st);
    static const bool pdl = [] { const char* v = std::getenv("PXF_PDL"); return !(v && v[0] == '0'); }();
    const uint32_t passes = (max_iters + kGsIters - 1) / kGsIters;
    for (uint32_t j = 0; j < passes; j++) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(units.total);
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = pass_smem();
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaError_t e = cudaLaunchKernelEx(&cfg, k_gs_pass, w, j, j * uint32_t(kGsIters));
        note_launch("k_gs_pass", st);
        if (e != cudaSuccess) return e;
    }
    k_gs_finish<<<gp, 256, 0, st>>>(w);
    note_launch("k_gs_finish", st);
    return cudaGetLastError();
}

}  // namespace pxf
