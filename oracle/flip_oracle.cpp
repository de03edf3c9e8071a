// ORACLE — test infrastructure only.
//
// A CPU restatement of pxlengine's FLIP liquid substep, used as the parity checker for the
// CUDA library and as the timed CPU baseline. Only tests/, __graft_entry__.smoke() and
// bench.py's CPU legs may load this file's library; the product path never does.
//
// Restated from (paths inside the pxlengine project):
//   shaders/fluid.slang:38-220        constants, indexing, clear_grid, p2g, normalize_grid,
//                                     forces, compute_divergence, pressure_rb, project, g2p_advect
//   crates/pxl-render/src/fluid.rs:97-100   lcg
//   crates/pxl-render/src/fluid.rs:119-148  particle seeding
//   crates/pxl-render/src/fluid.rs:158-180  push constants (dt, inv_h)
//   crates/pxl-render/src/fluid.rs:234-236  steps_for_frame
//   crates/pxl-render/src/fluid.rs:289-303  substep schedule
//   crates/pxl-scene/src/lib.rs:121-129     Fluid::grid
//   shaders/fluid.slang:222-355       surface nets: s_clear, s_splat, s_phi, s_verts, s_quads
//   crates/pxl-render/src/fluid.rs:150-156, 308-330  surface grid, iso level, meshing schedule
//
// Parity status: pinned to the reference's own shader. tests/test_oracle_vs_reference.py runs
// shaders/fluid.slang itself on the CPU (compiled by oracle/ref_build.py against
// oracle/slang_shim.h, which binds its built-ins to the semantics below) beside this oracle and
// finds the same bits after every stage of every substep and for the surface pass. The host
// code the shader leaves to Rust (seeding, Fluid::grid, steps_for_frame) is pinned by the
// reference's own unit test (pxl-scene/src/lib.rs:886-899: [32,16,16], h = 0.0625), the
// dam-break particle count in its documentation (139k particles, docs/ROADMAP.md:83; 139,200
// exactly) and an independent pure-Python restatement (tests/golden/make_golden.py).
//
// Semantics fixed here (the shader leaves them to the Slang compiler / Vulkan driver):
//   lerp(a, b, t) = a*(1-t) + b*t      the GLSL.std.450 FMix definition that Slang lowers to
//   int(float)    truncates toward zero; NaN -> 0, out of range saturates (PTX cvt.rzi.s32.f32)
//   no fused multiply-add anywhere (built with -ffp-contract=off), left-to-right evaluation
//   pressure starts at zero (the reference leaves the buffer uninitialised, fluid.rs:204)
//
// Build: see oracle/build.py (g++ -O3 -fopenmp -ffp-contract=off -shared -fPIC).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr uint32_t AIR = 0, FLUID = 1, SOLID = 2;   // fluid.slang:40

// float -> int32 with the GPU's conversion semantics (truncate, NaN -> 0, saturate).
template <class T> inline int32_t to_i32(T f) {
    if (std::isnan(f)) return 0;
    if (f >= T(2147483648.0)) return INT32_MAX;
    if (f <= T(-2147483648.0)) return INT32_MIN;
    return (int32_t)f;
}

// lerp as FMix: a*(1-t) + b*t.
template <class T> inline T fmix(T a, T b, T t) { return a * (T(1) - t) + b * t; }

template <class T> struct Sim {
    // FluidPush (fluid.slang:11-19, fluid.rs:47-72), simulation part.
    uint32_t nx, ny, nz, np;
    T h, dt, flip, inv_h;
    T origin[3], gravity[3];
    uint32_t iterations;
    // Pressure mode: 0 = red-black Gauss-Seidel (reference), 1 = Jacobi-PCG with FP32 vectors,
    // FP64 dot products, FP64 solution and FP64 restart residuals, 2 = Jacobi-PCG entirely in FP64,
    // 3 = as 1 with a multigrid V-cycle preconditioner in FP32 (the CUDA precision solver).
    int pmode = 0;
    uint32_t mg_coarse_iters = 2;    // symmetric red-black iterations on the coarsest level
    uint32_t mg_pairs = 2;           // red-black pairs of pre- and of post-smoothing per level
    double rtol = 1e-6;
    uint32_t max_iter = 2000, restart = 50;
    uint32_t last_iters = 0;
    double last_relres = 0;
    // Buffers (fluid.slang:22-30), x-fastest, faces u then v then w.
    std::vector<T> part;                         // AoS [x,y,z,w, vx,vy,vz,w] per particle
    std::vector<T> vel, vel_old, pressure, divergence;
    std::vector<uint32_t> acc, wacc;             // int32 two's complement, wrapping adds
    std::vector<uint32_t> cell_count, cell_type;
    std::vector<double> xp64;                    // FP64 pressure (pmode 1, 2)

    uint32_t n_u() const { return (nx + 1) * ny * nz; }
    uint32_t n_v() const { return nx * (ny + 1) * nz; }
    uint32_t n_w() const { return nx * ny * (nz + 1); }
    uint32_t n_faces() const { return n_u() + n_v() + n_w(); }
    uint32_t n_cells() const { return nx * ny * nz; }
    void face_dims(uint32_t c, uint32_t d[3]) const {
        d[0] = nx; d[1] = ny; d[2] = nz; d[c] += 1;
    }
    uint32_t face_base(uint32_t c) const { return c == 0 ? 0 : (c == 1 ? n_u() : n_u() + n_v()); }
    uint32_t face_index(uint32_t c, const int f[3]) const {
        uint32_t d[3]; face_dims(c, d);
        return face_base(c) + uint32_t(f[0]) + d[0] * (uint32_t(f[1]) + d[1] * uint32_t(f[2]));
    }
    uint32_t cell_index(const int c[3]) const {
        return uint32_t(c[0]) + nx * (uint32_t(c[1]) + ny * uint32_t(c[2]));
    }
    uint32_t cell_t(const int c[3]) const {
        if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= int(nx) || c[1] >= int(ny) || c[2] >= int(nz))
            return SOLID;
        return cell_type[cell_index(c)];
    }
    void face_coord(uint32_t c, const T x[3], T g[3]) const {
        for (int a = 0; a < 3; a++) g[a] = (x[a] - origin[a]) * inv_h - T(0.5);
        g[c] += T(0.5);
    }
    T sample_face(const std::vector<T>& buf, uint32_t c, const T x[3]) const {
        T g[3]; face_coord(c, x, g);
        uint32_t dd[3]; face_dims(c, dd);
        int d[3] = {int(dd[0]) - 1, int(dd[1]) - 1, int(dd[2]) - 1};
        int b[3]; T f[3];
        for (int a = 0; a < 3; a++) { b[a] = to_i32(std::floor(g[a])); f[a] = g[a] - T(b[a]); }
        T s = 0;
        for (int k = 0; k < 8; k++) {
            int o[3] = {k & 1, (k >> 1) & 1, k >> 2};
            int q[3]; T w3[3];
            for (int a = 0; a < 3; a++) {
                q[a] = std::min(std::max(b[a] + o[a], 0), d[a]);
                w3[a] = fmix(T(1) - f[a], f[a], T(o[a]));
            }
            s += w3[0] * w3[1] * w3[2] * buf[face_index(c, q)];
        }
        return s;
    }

    void alloc() {
        uint32_t F = n_faces(), C = n_cells();
        vel.assign(F, 0); vel_old.assign(F, 0); acc.assign(F, 0); wacc.assign(F, 0);
        cell_count.assign(C, 0); cell_type.assign(C, 0); pressure.assign(C, 0); divergence.assign(C, 0);
        xp64.assign(C, 0.0);
    }

    // fluid.slang:87-91
    void clear_grid() {
        std::fill(acc.begin(), acc.end(), 0u);
        std::fill(wacc.begin(), wacc.end(), 0u);
        std::fill(cell_count.begin(), cell_count.end(), 0u);
    }

    // fluid.slang:93-115. Integer adds are order independent, so the parallel loop matches
    // the serial one bit for bit.
    void p2g() {
        const T SW = T(65536.0);
        const int64_t N = np;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) {
            const T* p = &part[size_t(i) * 8];
            T x[3] = {p[0], p[1], p[2]};
            for (uint32_t c = 0; c < 3; c++) {
                T g[3]; face_coord(c, x, g);
                uint32_t dd[3]; face_dims(c, dd);
                int d[3] = {int(dd[0]) - 1, int(dd[1]) - 1, int(dd[2]) - 1};
                int b[3]; T f[3];
                for (int a = 0; a < 3; a++) { b[a] = to_i32(std::floor(g[a])); f[a] = g[a] - T(b[a]); }
                for (int k = 0; k < 8; k++) {
                    int o[3] = {k & 1, (k >> 1) & 1, k >> 2};
                    int q[3] = {b[0] + o[0], b[1] + o[1], b[2] + o[2]};
                    if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] > d[0] || q[1] > d[1] || q[2] > d[2]) continue;
                    T w3[3];
                    for (int a = 0; a < 3; a++) w3[a] = fmix(T(1) - f[a], f[a], T(o[a]));
                    T w = w3[0] * w3[1] * w3[2];
                    uint32_t fi = face_index(c, q);
                    uint32_t ta = uint32_t(to_i32(w * p[4 + c] * SW));
                    uint32_t tw = uint32_t(to_i32(w * SW));
#pragma omp atomic
                    acc[fi] += ta;
#pragma omp atomic
                    wacc[fi] += tw;
                }
            }
            int cell[3];
            const int nn[3] = {int(nx), int(ny), int(nz)};
            for (int a = 0; a < 3; a++)
                cell[a] = std::min(std::max(to_i32(std::floor((x[a] - origin[a]) * inv_h)), 0), nn[a] - 1);
            uint32_t ci = cell_index(cell);
#pragma omp atomic
            cell_count[ci] += 1u;
        }
    }

    // fluid.slang:117-132
    void normalize_grid() {
        const int64_t F = n_faces(), C = n_cells();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < F; id++) {
            int32_t w = int32_t(wacc[id]);
            T v = w > 0 ? T(int32_t(acc[id])) / T(w) : T(0);
            vel[id] = v;
            vel_old[id] = v;
        }
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            uint32_t i = uint32_t(id) % nx, j = (uint32_t(id) / nx) % ny, k = uint32_t(id) / (nx * ny);
            bool wall = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
            uint32_t t = wall ? SOLID : (cell_count[id] > 0 ? FLUID : AIR);
            cell_type[id] = t;
            if (t != FLUID) { pressure[id] = 0; xp64[id] = 0; }
        }
    }

    // fluid.slang:134-140
    void face_of(uint32_t id, uint32_t& c, int f[3]) const {
        c = id < n_u() ? 0 : (id < n_u() + n_v() ? 1 : 2);
        uint32_t d[3]; face_dims(c, d);
        uint32_t r = id - face_base(c);
        f[0] = int(r % d[0]); f[1] = int((r / d[0]) % d[1]); f[2] = int(r / (d[0] * d[1]));
    }

    // fluid.slang:142-151
    void forces() {
        const int64_t F = n_faces();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < F; id++) {
            uint32_t c; int f[3];
            face_of(uint32_t(id), c, f);
            int lo[3] = {f[0], f[1], f[2]};
            lo[c] -= 1;
            T v = vel[id] + gravity[c] * dt;
            if (cell_t(lo) == SOLID || cell_t(f) == SOLID) v = 0;
            vel[id] = v;
        }
    }

    // fluid.slang:153-165
    void compute_divergence() {
        const int64_t C = n_cells();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            int c[3] = {int(uint32_t(id) % nx), int((uint32_t(id) / nx) % ny), int(uint32_t(id) / (nx * ny))};
            T d = 0;
            if (cell_type[id] == FLUID) {
                for (uint32_t a = 0; a < 3; a++) {
                    int hi[3] = {c[0], c[1], c[2]};
                    hi[a] += 1;
                    d += vel[face_index(a, hi)] - vel[face_index(a, c)];
                }
            }
            divergence[id] = d * inv_h;
        }
    }

    // fluid.slang:167-182, one dispatch (one colour).
    void pressure_rb(uint32_t parity) {
        const int64_t C = n_cells();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            if (cell_type[id] != FLUID) continue;
            int c[3] = {int(uint32_t(id) % nx), int((uint32_t(id) / nx) % ny), int(uint32_t(id) / (nx * ny))};
            if (uint32_t(c[0] + c[1] + c[2]) % 2 != parity) continue;
            T sum = 0, cnt = 0;
            for (int n = 0; n < 6; n++) {
                int q[3] = {c[0], c[1], c[2]};
                q[n >> 1] += (n & 1) ? 1 : -1;
                uint32_t t = cell_t(q);
                if (t == SOLID) continue;
                cnt += 1;
                if (t == FLUID) sum += pressure[cell_index(q)];
            }
            if (cnt > 0) pressure[id] = (sum - divergence[id] * h * h / dt) / cnt;
        }
    }

    // ------------------------------------------------------------------ PCG forms
    // The pressure system of pressure_rb: for fluid cell i, cnt_i p_i - sum_{fluid j} p_j = b_i
    // with b_i = -(div_i h h / dt) and cnt_i the non-solid neighbour count.
    struct Sys {
        std::vector<uint32_t> idx;      // fluid cells
        std::vector<uint8_t> fmask;     // bit n: neighbour n is fluid (n = -x,+x,-y,+y,-z,+z)
        std::vector<double> diag;       // cnt
        std::vector<double> b;
    };
    int64_t nbr_off(int n) const {
        int64_t s[3] = {1, int64_t(nx), int64_t(nx) * ny};
        return (n & 1) ? s[n >> 1] : -s[n >> 1];
    }
    void build_sys(Sys& S) const {
        const uint32_t C = n_cells();
        for (uint32_t id = 0; id < C; id++) {
            if (cell_type[id] != FLUID) continue;
            int c[3] = {int(id % nx), int((id / nx) % ny), int(id / (nx * ny))};
            uint8_t m = 0; int cnt = 0;
            for (int n = 0; n < 6; n++) {
                int q[3] = {c[0], c[1], c[2]};
                q[n >> 1] += (n & 1) ? 1 : -1;
                uint32_t t = cell_t(q);
                if (t == SOLID) continue;
                cnt++;
                if (t == FLUID) m |= uint8_t(1u << n);
            }
            if (cnt == 0) continue;   // isolated fluid cell: pressure_rb leaves it unchanged
            S.idx.push_back(id);
            S.fmask.push_back(m);
            S.diag.push_back(double(cnt));
            // b in the precision of the simulation's own rhs expression.
            T rhs = divergence[id] * h * h / dt;
            S.b.push_back(-double(rhs));
        }
    }
    // y = A x over fluid cells, x given on the full cell grid (double).
    template <class V, class X> void apply_A(const Sys& S, const X& xg, V* y) const {
        const int64_t M = int64_t(S.idx.size());
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < M; k++) {
            uint32_t id = S.idx[k];
            auto s = S.diag[k] * double(xg[id]);
            for (int n = 0; n < 6; n++)
                if (S.fmask[k] & (1u << n)) s -= double(xg[int64_t(id) + nbr_off(n)]);
            y[k] = V(s);
        }
    }

    // ------------------------------------------------------------------ multigrid preconditioner
    // Geometric V-cycle on the cell grid. Level l+1 halves each axis (ceil); a coarse cell is AIR
    // if any child is AIR, else FLUID if any child is FLUID, else SOLID (children outside the
    // fine grid count as SOLID). Each level's operator is the same 7-point system as level 0
    // built from its own types. Smoothing is red-black Gauss-Seidel, mg_pairs pairs per side
    // (pre: red from zero, black, then (red, black) x (mg_pairs - 1); post: the mirror image,
    // (black, red) x mg_pairs, the first black with the coarse correction), restriction sums the children's residuals times 1/2 and prolongation injects
    // the coarse correction into every child, so restriction = prolongation^T / 2 and the cycle
    // is a symmetric operator. The coarsest level (<= 512 cells) runs mg_coarse_iters
    // (default 2) red-black iterations followed by as many black-red iterations from zero.
    struct Level {
        int nx = 0, ny = 0, nz = 0;
        std::vector<uint8_t> type, fmask, cnt;
        std::vector<float> r, z;
        int64_t nc() const { return int64_t(nx) * ny * nz; }
        int64_t off(int n) const {
            const int64_t st[3] = {1, int64_t(nx), int64_t(nx) * ny};
            return (n & 1) ? st[n >> 1] : -st[n >> 1];
        }
    };
    std::vector<Level> mg;

    static void level_info(Level& L) {
        const int64_t C = L.nc();
        L.fmask.assign(C, 0);
        L.cnt.assign(C, 0);
        for (int64_t id = 0; id < C; id++) {
            if (L.type[id] != FLUID) continue;
            int c[3] = {int(id % L.nx), int((id / L.nx) % L.ny), int(id / (int64_t(L.nx) * L.ny))};
            const int n3[3] = {L.nx, L.ny, L.nz};
            uint8_t m = 0, k = 0;
            for (int n = 0; n < 6; n++) {
                int q[3] = {c[0], c[1], c[2]};
                q[n >> 1] += (n & 1) ? 1 : -1;
                uint8_t t = SOLID;
                if (q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < n3[0] && q[1] < n3[1] && q[2] < n3[2])
                    t = L.type[q[0] + int64_t(L.nx) * (q[1] + int64_t(L.ny) * q[2])];
                if (t == SOLID) continue;
                k++;
                if (t == FLUID) m |= uint8_t(1u << n);
            }
            L.fmask[id] = m;
            L.cnt[id] = k;
        }
    }

    void mg_build() {
        mg.clear();
        Level L0;
        L0.nx = int(nx); L0.ny = int(ny); L0.nz = int(nz);
        L0.type.resize(n_cells());
        for (uint32_t i = 0; i < n_cells(); i++) L0.type[i] = uint8_t(cell_type[i]);
        level_info(L0);
        L0.r.assign(L0.nc(), 0.0f);
        L0.z.assign(L0.nc(), 0.0f);
        mg.push_back(std::move(L0));
        while (mg.back().nc() > 512 && mg.back().nx >= 2 && mg.back().ny >= 2 && mg.back().nz >= 2) {
            const Level& F = mg.back();
            Level Cc;
            Cc.nx = (F.nx + 1) / 2; Cc.ny = (F.ny + 1) / 2; Cc.nz = (F.nz + 1) / 2;
            Cc.type.assign(Cc.nc(), SOLID);
            for (int K = 0; K < Cc.nz; K++)
                for (int J = 0; J < Cc.ny; J++)
                    for (int I = 0; I < Cc.nx; I++) {
                        bool air = false, fluid = false;
                        for (int ch = 0; ch < 8; ch++) {
                            int i = 2 * I + (ch & 1), j = 2 * J + ((ch >> 1) & 1), k = 2 * K + (ch >> 2);
                            if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                            uint8_t t = F.type[i + int64_t(F.nx) * (j + int64_t(F.ny) * k)];
                            if (t == AIR) air = true;
                            if (t == FLUID) fluid = true;
                        }
                        Cc.type[I + int64_t(Cc.nx) * (J + int64_t(Cc.ny) * K)] = air ? AIR : (fluid ? FLUID : SOLID);
                    }
            level_info(Cc);
            Cc.r.assign(Cc.nc(), 0.0f);
            Cc.z.assign(Cc.nc(), 0.0f);
            mg.push_back(std::move(Cc));
        }
    }

    static bool in_sys(const Level& L, int64_t id) { return L.type[id] == FLUID && L.cnt[id] > 0; }

    // One red-black half sweep of A z = r on level L. first: the other colour is zero.
    static void smooth(Level& L, int color, bool first) {
        const int64_t C = L.nc();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            if (!in_sys(L, id)) continue;
            int i = int(id % L.nx), j = int((id / L.nx) % L.ny), k = int(id / (int64_t(L.nx) * L.ny));
            if (((i + j + k) & 1) != color) continue;
            float s = L.r[id];
            if (!first) {
                for (int n = 0; n < 6; n++)
                    if (L.fmask[id] & (1u << n)) s += L.z[id + L.off(n)];
            }
            L.z[id] = s / float(L.cnt[id]);
        }
    }

    static float resid(const Level& L, int64_t id) {
        float az = float(L.cnt[id]) * L.z[id];
        for (int n = 0; n < 6; n++)
            if (L.fmask[id] & (1u << n)) az -= L.z[id + L.off(n)];
        return L.r[id] - az;
    }

    void restrict_to(int l) {
        const Level& F = mg[l];
        Level& Cc = mg[l + 1];
        const int64_t C = Cc.nc();
#pragma omp parallel for schedule(static)
        for (int64_t P = 0; P < C; P++) {
            float s = 0.0f;
            if (in_sys(Cc, P)) {
                int I = int(P % Cc.nx), J = int((P / Cc.nx) % Cc.ny), K = int(P / (int64_t(Cc.nx) * Cc.ny));
                for (int ch = 0; ch < 8; ch++) {
                    int i = 2 * I + (ch & 1), j = 2 * J + ((ch >> 1) & 1), k = 2 * K + (ch >> 2);
                    if (i >= F.nx || j >= F.ny || k >= F.nz) continue;
                    int64_t id = i + int64_t(F.nx) * (j + int64_t(F.ny) * k);
                    if (in_sys(F, id)) s += resid(F, id);
                }
            }
            Cc.r[P] = 0.5f * s;
        }
    }

    void prolong_from(int l) {
        Level& F = mg[l];
        const Level& Cc = mg[l + 1];
        const int64_t C = F.nc();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            if (!in_sys(F, id)) continue;
            int i = int(id % F.nx), j = int((id / F.nx) % F.ny), k = int(id / (int64_t(F.nx) * F.ny));
            int64_t P = (i >> 1) + int64_t(Cc.nx) * ((j >> 1) + int64_t(Cc.ny) * (k >> 1));
            if (in_sys(Cc, P)) F.z[id] += Cc.z[P];
        }
    }

    void vcycle(int l) {
        Level& L = mg[l];
        if (l + 1 == int(mg.size())) {
            std::fill(L.z.begin(), L.z.end(), 0.0f);
            for (uint32_t it = 0; it < mg_coarse_iters; it++) { smooth(L, 0, false); smooth(L, 1, false); }
            for (uint32_t it = 0; it < mg_coarse_iters; it++) { smooth(L, 1, false); smooth(L, 0, false); }
            return;
        }
        smooth(L, 0, true);
        smooth(L, 1, false);
        for (uint32_t x = 1; x < mg_pairs; x++) { smooth(L, 0, false); smooth(L, 1, false); }
        restrict_to(l);
        vcycle(l + 1);
        prolong_from(l);
        smooth(L, 1, false);
        smooth(L, 0, false);
        for (uint32_t x = 1; x < mg_pairs; x++) { smooth(L, 1, false); smooth(L, 0, false); }
    }

    // Jacobi-preconditioned CG as a state machine shared by both PCG forms and mirrored by the
    // CUDA precision solver:
    //   restart: r = b - A x in FP64; converged if |r| <= rtol |b| (or iteration cap reached);
    //            otherwise rz = r.z with z = r / cnt, and the next direction is p = z
    //   step:    p = z + beta p; Ap = A p; alpha = rz / p.Ap; x += alpha p; r -= alpha Ap
    //            restart when the recurrence |r| <= rtol |b|, every `restart` steps, or at the cap
    // V is the vector type of r, p, Ap (float for the precision form, double for the FP64 form);
    // x and every dot product are FP64.
    template <class V> void pcg_run(bool use_mg) {
        Sys S; build_sys(S);
        const int64_t M = int64_t(S.idx.size());
        const uint32_t C = n_cells();
        std::vector<V> r(M), z(M), p(M, V(0)), Ap(M), pg(C, V(0)), cnt(M);
        std::vector<double> rd(M);
        for (int64_t k = 0; k < M; k++) cnt[k] = V(S.diag[k]);
        double bb = 0;
#pragma omp parallel for schedule(static) reduction(+ : bb)
        for (int64_t k = 0; k < M; k++) bb += S.b[k] * S.b[k];
        last_iters = 0; last_relres = 0;
        if (M == 0 || bb == 0) {
            for (int64_t k = 0; k < M; k++) xp64[S.idx[k]] = 0;
            finish_pcg(S);
            return;
        }
        if (use_mg) mg_build();
        // z = M^-1 r
        auto precond = [&]() {
            if (!use_mg) {
#pragma omp parallel for schedule(static)
                for (int64_t k = 0; k < M; k++) z[k] = r[k] / cnt[k];
                return;
            }
            Level& L0 = mg[0];
            std::fill(L0.r.begin(), L0.r.end(), 0.0f);
            for (int64_t k = 0; k < M; k++) L0.r[S.idx[k]] = float(r[k]);
            vcycle(0);
            for (int64_t k = 0; k < M; k++) z[k] = V(L0.z[S.idx[k]]);
        };
        auto dot_rz = [&]() {
            double t = 0;
#pragma omp parallel for schedule(static) reduction(+ : t)
            for (int64_t k = 0; k < M; k++) t += double(r[k]) * double(z[k]);
            return t;
        };
        const double tol2 = rtol * rtol * bb;
        uint32_t it = 0, since = 0;
        double rz = 0, beta = 0;
        bool fresh = true, done = false;
        auto do_restart = [&]() {
            apply_A(S, xp64, rd.data());
            double rr = 0;
#pragma omp parallel for schedule(static) reduction(+ : rr)
            for (int64_t k = 0; k < M; k++) { rd[k] = S.b[k] - rd[k]; rr += rd[k] * rd[k]; r[k] = V(rd[k]); }
            last_relres = std::sqrt(rr / bb);
            if (rr <= tol2 || it >= max_iter) { done = true; return; }
            precond();
            rz = dot_rz();
            fresh = true; since = 0;
        };
        do_restart();
        while (!done) {
            const V bv = V(beta);
            const bool fr = fresh;
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < M; k++) {
                p[k] = fr ? z[k] : V(z[k] + bv * p[k]);
                pg[S.idx[k]] = p[k];
            }
            fresh = false;
            double pAp = 0;
#pragma omp parallel for schedule(static) reduction(+ : pAp)
            for (int64_t k = 0; k < M; k++) {
                int64_t id = S.idx[k];
                V s = cnt[k] * pg[id];
                for (int n = 0; n < 6; n++)
                    if (S.fmask[k] & (1u << n)) s -= pg[id + nbr_off(n)];
                Ap[k] = s;
                pAp += double(p[k]) * double(s);
            }
            if (!(pAp > 0)) break;   // breakdown (non-SPD or NaN): stop with the current x
            const double alpha = rz / pAp;
            const V av = V(alpha);
            double rr = 0;
#pragma omp parallel for schedule(static) reduction(+ : rr)
            for (int64_t k = 0; k < M; k++) {
                xp64[S.idx[k]] += alpha * double(p[k]);
                r[k] = r[k] - av * Ap[k];
                rr += double(r[k]) * double(r[k]);
            }
            it++; since++;
            if (rr <= tol2 || since >= restart || it >= max_iter) {
                do_restart();
            } else {
                precond();
                const double rzn = dot_rz();
                beta = rzn / rz;
                rz = rzn;
            }
        }
        last_iters = it;
        finish_pcg(S);
    }
    void pcg_mixed() { pcg_run<float>(false); }
    void pcg_fp64() { pcg_run<double>(false); }
    void pcg_mg() { pcg_run<float>(true); }
    void finish_pcg(const Sys&) {
        const int64_t C = n_cells();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < C; id++) {
            if (cell_type[id] != FLUID) xp64[id] = 0;
            pressure[id] = T(xp64[id]);
        }
    }

    // fluid.slang:184-197. In the PCG forms the pressure difference is taken in FP64 from the
    // FP64 solution; in the reference form it is the shader's FP32 expression.
    void project() {
        const int64_t F = n_faces();
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < F; id++) {
            uint32_t c; int f[3];
            face_of(uint32_t(id), c, f);
            int lo[3] = {f[0], f[1], f[2]};
            lo[c] -= 1;
            uint32_t ta = cell_t(lo), tb = cell_t(f);
            if (ta == SOLID || tb == SOLID) { vel[id] = 0; continue; }
            if (ta == FLUID || tb == FLUID) {
                if (pmode == 0) {
                    T pa = ta == FLUID ? pressure[cell_index(lo)] : T(0);
                    T pb = tb == FLUID ? pressure[cell_index(f)] : T(0);
                    vel[id] -= dt * inv_h * (pb - pa);
                } else {
                    double pa = ta == FLUID ? xp64[cell_index(lo)] : 0.0;
                    double pb = tb == FLUID ? xp64[cell_index(f)] : 0.0;
                    vel[id] -= dt * inv_h * T(pb - pa);
                }
            }
        }
    }

    // fluid.slang:199-220
    void g2p_advect() {
        const int64_t N = np;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) {
            T* pp = &part[size_t(i) * 8];
            T x[3] = {pp[0], pp[1], pp[2]};
            T pic[3], old[3], v[3], mid[3], s[3];
            for (uint32_t c = 0; c < 3; c++) pic[c] = sample_face(vel, c, x);
            for (uint32_t c = 0; c < 3; c++) old[c] = sample_face(vel_old, c, x);
            for (int a = 0; a < 3; a++) {
                T fl = pp[4 + a] + pic[a] - old[a];
                v[a] = fmix(pic[a], fl, flip);
                mid[a] = x[a] + T(0.5) * dt * pic[a];
            }
            for (uint32_t c = 0; c < 3; c++) s[c] = sample_face(vel, c, mid);
            const T nn[3] = {T(nx), T(ny), T(nz)};
            for (int a = 0; a < 3; a++) {
                x[a] += dt * s[a];
                T lo = origin[a] + h * T(1.001f);
                T hi = origin[a] + h * (nn[a] - T(1.001f));
                if (x[a] < lo) { x[a] = lo; v[a] = std::max(v[a], T(0)); }
                if (x[a] > hi) { x[a] = hi; v[a] = std::min(v[a], T(0)); }
            }
            for (int a = 0; a < 3; a++) { pp[a] = x[a]; pp[4 + a] = v[a]; }
        }
    }

    void pressure_solve() {
        if (pmode == 0) {
            for (uint32_t it = 0; it < iterations; it++)
                for (uint32_t parity = 0; parity < 2; parity++) pressure_rb(parity);
        } else if (pmode == 1) {
            pcg_mixed();
        } else if (pmode == 3) {
            pcg_mg();
        } else {
            pcg_fp64();
        }
    }

    // fluid.rs:289-303
    void substep() {
        clear_grid();
        p2g();
        normalize_grid();
        forces();
        compute_divergence();
        pressure_solve();
        project();
        g2p_advect();
    }
};

struct Handle {
    int dbl;
    Sim<float>* f = nullptr;
    Sim<double>* d = nullptr;
};

template <class T> Sim<T>* make_sim(const uint32_t n[3], float h, float dt, float flip, const float origin[3],
                                    const float gravity[3], uint32_t iters, const float* particles, uint32_t np) {
    auto* s = new Sim<T>();
    s->nx = n[0]; s->ny = n[1]; s->nz = n[2]; s->np = np;
    s->h = T(h); s->dt = T(dt); s->flip = T(flip);
    // inv_h is computed in FP32 like the host driver (fluid.rs:166) for both precisions.
    s->inv_h = T(1.0f / h);
    for (int a = 0; a < 3; a++) { s->origin[a] = T(origin[a]); s->gravity[a] = T(gravity[a]); }
    s->iterations = iters;
    s->part.resize(size_t(np) * 8);
    for (size_t i = 0; i < size_t(np) * 8; i++) s->part[i] = T(particles[i]);
    s->alloc();
    return s;
}

template <class T> int sim_stage(Sim<T>* s, int stage) {
    switch (stage) {
        case 0: s->clear_grid(); break;
        case 1: s->p2g(); break;
        case 2: s->normalize_grid(); break;
        case 3: s->forces(); break;
        case 4: s->compute_divergence(); break;
        case 5: s->pressure_solve(); break;
        case 6: s->project(); break;
        case 7: s->g2p_advect(); break;
        default: return -1;
    }
    return 0;
}

// which: 0 particles (AoS 8), 1 vel, 2 vel_old, 3 acc, 4 wacc, 5 cell_count, 6 cell_type,
//        7 pressure, 8 divergence, 9 FP64 pressure
template <class T> int sim_io(Sim<T>* s, int which, void* buf, size_t bytes, bool write) {
    void* src = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: src = s->part.data(); n = s->part.size() * sizeof(T); break;
        case 1: src = s->vel.data(); n = s->vel.size() * sizeof(T); break;
        case 2: src = s->vel_old.data(); n = s->vel_old.size() * sizeof(T); break;
        case 3: src = s->acc.data(); n = s->acc.size() * 4; break;
        case 4: src = s->wacc.data(); n = s->wacc.size() * 4; break;
        case 5: src = s->cell_count.data(); n = s->cell_count.size() * 4; break;
        case 6: src = s->cell_type.data(); n = s->cell_type.size() * 4; break;
        case 7: src = s->pressure.data(); n = s->pressure.size() * sizeof(T); break;
        case 8: src = s->divergence.data(); n = s->divergence.size() * sizeof(T); break;
        case 9: src = s->xp64.data(); n = s->xp64.size() * 8; break;
        default: return -1;
    }
    if (bytes != n) return -2;
    if (write) std::memcpy(src, buf, n);
    else std::memcpy(buf, src, n);
    return 0;
}

float lcg(uint64_t* s) {
    *s = *s * 6364136223846793005ull + 1442695040888963407ull;
    return float(*s >> 40) / float(1ull << 24);
}

}  // namespace

extern "C" {

int orc_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// crates/pxl-scene/src/lib.rs:123-128. Vec3::round is round-half-away-from-zero.
int orc_grid(const float bounds[6], uint32_t resolution, uint32_t out_n[3], float* out_h) {
    float size[3] = {bounds[3] - bounds[0], bounds[4] - bounds[1], bounds[5] - bounds[2]};
    float mx = std::max(std::max(size[0], size[1]), size[2]);
    float h = mx / float(resolution);
    for (int a = 0; a < 3; a++) {
        float n = std::round(size[a] / h);
        n = std::max(n, 4.0f);
        out_n[a] = n >= 4294967296.0f ? UINT32_MAX : uint32_t(n);
    }
    *out_h = h;
    return 0;
}

float orc_lcg(uint64_t* state) { return lcg(state); }

// crates/pxl-render/src/fluid.rs:119-148. fill: n_fill records of 9 floats (min, max, velocity).
// Writes up to `cap` particles (8 floats each) to out (may be NULL) and returns the count.
int64_t orc_seed(const float bounds[6], uint32_t resolution, const float* fill, uint32_t n_fill,
                 uint32_t ppc, uint32_t seed, float* out, int64_t cap) {
    uint32_t n[3]; float h;
    orc_grid(bounds, resolution, n, &h);
    const float* origin = bounds;
    uint64_t rng = 0x9e3779b97f4a7c15ull ^ uint64_t(seed);
    int64_t count = 0;
    for (uint32_t bi = 0; bi < n_fill; bi++) {
        const float* b = fill + 9 * bi;
        for (uint32_t k = 1; k + 1 < n[2]; k++)
            for (uint32_t j = 1; j + 1 < n[1]; j++)
                for (uint32_t i = 1; i + 1 < n[0]; i++) {
                    float c[3] = {origin[0] + (float(i) + 0.5f) * h, origin[1] + (float(j) + 0.5f) * h,
                                  origin[2] + (float(k) + 0.5f) * h};
                    bool out_of = false;
                    for (int a = 0; a < 3; a++) if (c[a] < b[a] || c[a] > b[3 + a]) out_of = true;
                    if (out_of) continue;
                    for (uint32_t q = 0; q < ppc; q++) {
                        float px = origin[0] + (float(i) + lcg(&rng)) * h;
                        float py = origin[1] + (float(j) + lcg(&rng)) * h;
                        float pz = origin[2] + (float(k) + lcg(&rng)) * h;
                        if (out && count < cap) {
                            float* o = out + 8 * count;
                            o[0] = px; o[1] = py; o[2] = pz; o[3] = 0;
                            o[4] = b[6]; o[5] = b[7]; o[6] = b[8]; o[7] = 0;
                        }
                        count++;
                    }
                }
    }
    return count;
}

// crates/pxl-render/src/fluid.rs:234-236
uint64_t orc_steps_for_frame(double warmup, double fps, uint32_t substeps, double frame) {
    double v = std::round((warmup + frame / fps) * fps * double(substeps));
    v = std::max(v, 0.0);
    return v >= 18446744073709551616.0 ? UINT64_MAX : uint64_t(v);
}

// fluid.rs:164: dt = (1 / (fps * substeps)) in f64, cast to f32.
float orc_dt(double fps, uint32_t substeps) { return float(1.0 / (fps * double(substeps))); }

void* orc_sim_new(int dbl, const uint32_t n[3], float h, float dt, float flip, const float origin[3],
                  const float gravity[3], uint32_t iters, const float* particles, uint32_t np) {
    auto* hd = new Handle();
    hd->dbl = dbl;
    if (dbl) hd->d = make_sim<double>(n, h, dt, flip, origin, gravity, iters, particles, np);
    else hd->f = make_sim<float>(n, h, dt, flip, origin, gravity, iters, particles, np);
    return hd;
}

void orc_sim_free(void* p) {
    auto* hd = static_cast<Handle*>(p);
    if (!hd) return;
    delete hd->f;
    delete hd->d;
    delete hd;
}

// mode 0 red-black GS, 1 mixed-precision PCG, 2 FP64 PCG.
int orc_sim_set_pressure(void* p, int mode, double rtol, uint32_t max_iter, uint32_t restart) {
    auto* hd = static_cast<Handle*>(p);
    auto set = [&](auto* s) { s->pmode = mode; s->rtol = rtol; s->max_iter = max_iter; s->restart = restart ? restart : 50; };
    if (hd->dbl) set(hd->d); else set(hd->f);
    return 0;
}

int orc_sim_set_mg(void* p, uint32_t coarse_iters, uint32_t pairs) {
    auto* hd = static_cast<Handle*>(p);
    if (pairs == 0) pairs = 1;
    if (hd->dbl) { hd->d->mg_coarse_iters = coarse_iters; hd->d->mg_pairs = pairs; }
    else { hd->f->mg_coarse_iters = coarse_iters; hd->f->mg_pairs = pairs; }
    return 0;
}

int orc_sim_pcg_stats(void* p, uint32_t* iters, double* relres) {
    auto* hd = static_cast<Handle*>(p);
    if (hd->dbl) { *iters = hd->d->last_iters; *relres = hd->d->last_relres; }
    else { *iters = hd->f->last_iters; *relres = hd->f->last_relres; }
    return 0;
}

int orc_sim_stage(void* p, int stage) {
    auto* hd = static_cast<Handle*>(p);
    return hd->dbl ? sim_stage(hd->d, stage) : sim_stage(hd->f, stage);
}

int orc_sim_step(void* p, uint32_t n) {
    auto* hd = static_cast<Handle*>(p);
    for (uint32_t i = 0; i < n; i++) {
        if (hd->dbl) hd->d->substep(); else hd->f->substep();
    }
    return 0;
}

// Surface nets of particles[n] (AoS, 8 floats each) on a surface grid of sdims cells (nodes one
// more per axis). Vertices are numbered by ascending surface cell, triangles by ascending node and
// axis (a serial order; the reference's follows its atomic counters). Outputs: density and phi per
// node, cell_vert per cell, verts[max_verts][8], indices[max_tris][3], counts = {vertices,
// triangles} before the caps.
int orc_surface_nets(const float* particles, int64_t n, const uint32_t sdims[3], float sh, float radius, float iso,
                     const float origin[3], uint32_t max_verts, uint32_t max_tris, int32_t* density, float* phi,
                     uint32_t* cell_vert, float* verts, uint32_t* indices, uint32_t counts[2]) {
    const int X = int(sdims[0]), Y = int(sdims[1]), Z = int(sdims[2]);
    const int64_t NX = X + 1, NY = Y + 1, nn = NX * NY * (Z + 1), nc = int64_t(X) * Y * Z;
    const float SD = 4096.0f;
    const uint32_t NONE = 0xffffffffu;
    auto node = [&](int i, int j, int k) { return int64_t(i) + NX * (int64_t(j) + NY * int64_t(k)); };
    // s_clear
    std::fill(density, density + nn, 0);
    // s_splat (integer sums: the order of the additions does not matter)
    const float r = radius / sh;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; p++) {
        const float* P = particles + 8 * p;
        const float gx = (P[0] - origin[0]) / sh, gy = (P[1] - origin[1]) / sh, gz = (P[2] - origin[2]) / sh;
        const int lx = std::max(to_i32(std::ceil(gx - r)), 0), ly = std::max(to_i32(std::ceil(gy - r)), 0),
                  lz = std::max(to_i32(std::ceil(gz - r)), 0);
        const int hx = std::min(to_i32(std::floor(gx + r)), X), hy = std::min(to_i32(std::floor(gy + r)), Y),
                  hz = std::min(to_i32(std::floor(gz + r)), Z);
        for (int k = lz; k <= hz; k++)
            for (int j = ly; j <= hy; j++)
                for (int i = lx; i <= hx; i++) {
                    const float dx = float(i) - gx, dy = float(j) - gy, dz = float(k) - gz;
                    const float q = 1.0f - (dx * dx + dy * dy + dz * dz) / (r * r);
                    if (q > 0.0f) {
                        const int32_t add = to_i32(q * q * q * SD);
                        int32_t* d = density + node(i, j, k);
#pragma omp atomic
                        *d += add;
                    }
                }
    }
    // s_phi
#pragma omp parallel for schedule(static)
    for (int64_t id = 0; id < nn; id++) {
        const int i = int(id % NX), j = int((id / NX) % NY), k = int(id / (NX * NY));
        float sum = 2.0f * float(density[id]);
        float wsum = 2.0f;
        for (int a = 0; a < 6; a++) {
            int q[3] = {i, j, k};
            q[a >> 1] += (a & 1) ? 1 : -1;
            if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] > X || q[1] > Y || q[2] > Z) continue;
            sum += float(density[node(q[0], q[1], q[2])]);
            wsum += 1.0f;
        }
        const bool edge = i == 0 || j == 0 || k == 0 || i == X || j == Y || k == Z;
        phi[id] = edge ? -1.0f : sum / wsum / SD - iso;
    }
    // s_verts, serially in cell order
    uint32_t nv = 0;
    for (int64_t c = 0; c < nc; c++) {
        const int ci = int(c % X), cj = int((c / X) % Y), ck = int(c / (int64_t(X) * Y));
        float v[8];
        uint32_t inside = 0;
        for (int q = 0; q < 8; q++) {
            v[q] = phi[node(ci + (q & 1), cj + ((q >> 1) & 1), ck + (q >> 2))];
            if (v[q] > 0.0f) inside |= 1u << q;
        }
        cell_vert[c] = NONE;
        if (inside == 0 || inside == 255) continue;
        const uint32_t idx = nv++;
        if (idx >= max_verts) continue;
        float sx = 0, sy = 0, sz = 0, cnt = 0;
        for (int e = 0; e < 12; e++) {
            const int axis = e >> 2, bits = e & 3, o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
            int a0 = 0;
            if (bits & 1) a0 |= 1 << o1;
            if (bits & 2) a0 |= 1 << o2;
            const int a1 = a0 | (1 << axis);
            if ((v[a0] > 0.0f) == (v[a1] > 0.0f)) continue;
            const float t = v[a0] / (v[a0] - v[a1]);
            sx += fmix(float(a0 & 1), float(a1 & 1), t);
            sy += fmix(float((a0 >> 1) & 1), float((a1 >> 1) & 1), t);
            sz += fmix(float(a0 >> 2), float(a1 >> 2), t);
            cnt += 1.0f;
        }
        const float lx = sx / cnt, ly = sy / cnt, lz = sz / cnt;
        float gx = 0, gy = 0, gz = 0;
        for (int k = 0; k < 8; k++) {
            const bool ox = k & 1, oy = (k >> 1) & 1, oz = k >> 2;
            const float wx = ox ? lx : 1.0f - lx, wy = oy ? ly : 1.0f - ly, wz = oz ? lz : 1.0f - lz;
            const float qx = ox ? 1.0f : -1.0f, qy = oy ? 1.0f : -1.0f, qz = oz ? 1.0f : -1.0f;
            gx += v[k] * (qx * wy * wz);
            gy += v[k] * (qy * wx * wz);
            gz += v[k] * (qz * wx * wy);
        }
        gx = gx + 0.0f;
        gy = gy + 1e-9f;
        gz = gz + 0.0f;
        const float len = std::sqrt(gx * gx + gy * gy + gz * gz);
        float* o = verts + 8 * size_t(idx);
        o[0] = origin[0] + (float(ci) + lx) * sh;
        o[1] = origin[1] + (float(cj) + ly) * sh;
        o[2] = origin[2] + (float(ck) + lz) * sh;
        o[3] = 0.0f;
        o[4] = -(gx / len);
        o[5] = -(gy / len);
        o[6] = -(gz / len);
        o[7] = 0.0f;
        cell_vert[c] = idx;
    }
    // s_quads, serially in node order, then axis
    uint32_t nq = 0;
    const int lim[3] = {X, Y, Z};
    for (int64_t id = 0; id < nn; id++) {
        const int nd[3] = {int(id % NX), int((id / NX) % NY), int(id / (NX * NY))};
        const bool in0 = phi[id] > 0.0f;
        for (int axis = 0; axis < 3; axis++) {
            int m[3] = {nd[0], nd[1], nd[2]};
            m[axis] += 1;
            if (m[axis] > lim[axis]) continue;
            if (in0 == (phi[node(m[0], m[1], m[2])] > 0.0f)) continue;
            const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
            const int offs[4][2] = {{-1, -1}, {0, -1}, {0, 0}, {-1, 0}};
            uint32_t q[4];
            bool ok = true;
            for (int k = 0; k < 4 && ok; k++) {
                int c[3] = {nd[0], nd[1], nd[2]};
                c[o1] += offs[k][0];
                c[o2] += offs[k][1];
                if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= X || c[1] >= Y || c[2] >= Z) { ok = false; break; }
                q[k] = cell_vert[int64_t(c[0]) + int64_t(X) * (int64_t(c[1]) + int64_t(Y) * c[2])];
                if (q[k] == NONE) ok = false;
            }
            if (!ok) continue;
            const uint32_t t = 2 * nq++;
            if (t + 2 > max_tris) continue;
            uint32_t* b = indices + size_t(t) * 3;
            if (in0) {
                b[0] = q[0]; b[1] = q[1]; b[2] = q[2]; b[3] = q[0]; b[4] = q[2]; b[5] = q[3];
            } else {
                b[0] = q[0]; b[1] = q[2]; b[2] = q[1]; b[3] = q[0]; b[4] = q[3]; b[5] = q[2];
            }
        }
    }
    counts[0] = nv;
    counts[1] = 2 * nq;
    return 0;
}

int orc_sim_read(void* p, int which, void* out, size_t bytes) {
    auto* hd = static_cast<Handle*>(p);
    return hd->dbl ? sim_io(hd->d, which, out, bytes, false) : sim_io(hd->f, which, out, bytes, false);
}

int orc_sim_write(void* p, int which, const void* in, size_t bytes) {
    auto* hd = static_cast<Handle*>(p);
    void* b = const_cast<void*>(in);
    return hd->dbl ? sim_io(hd->d, which, b, bytes, true) : sim_io(hd->f, which, b, bytes, true);
}

}  // extern "C"
