// pxlengine's own FLIP shader (shaders/fluid.slang) run on the CPU — test infrastructure only.
//
// oracle/ref_build.py turns the shader's source, where it lies in the reference checkout, into
// fluid_slang.inc (four mechanical edits: the [shader(...)] and [numthreads(...)] attributes and
// the SV_DispatchThreadID semantic are dropped, `out T x` parameters become `T& x`) and compiles
// this file with oracle/slang_shim.h force-included. Every kernel below is the shader's own
// function; this file only plays the host's part of crates/pxl-render/src/fluid.rs:
// FluidPush from FluidState::new (fluid.rs:153-176), zeroed buffers (the reference allocates
// them without initial data; zero is what the oracle and the library assume), the substep schedule of
// fluid_advance (fluid.rs:278-300: clear, p2g, normalize, forces, divergence, iterations x
// {parity 0, 1} pressure_rb, project, g2p_advect) and the surface pass (fluid.rs:308-318:
// s_clear, s_splat, s_phi, s_verts, s_quads), each dispatch as ceil(n / 256) groups of 256
// invocations. Invocations of one dispatch do not depend on each other except through
// InterlockedAdd: integer sums (order-free; those dispatches run on all host threads, OpenMP) and,
// in s_verts / s_quads, the order in which vertices and triangles take their slots (those two run
// one invocation after another, in ascending index, the order the oracle and the library number
// them in).
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

namespace ref {
#include "fluid_slang.inc"
}  // namespace ref

namespace {

struct RefSim {
    ref::FluidPush push{};
    uint32_t iterations = 0;
    std::vector<ref::Particle> particles;
    std::vector<float> vel, vel_old, pressure, divergence;
    std::vector<int> acc, wacc;
    std::vector<uint> cell_count, cell_type;
};

uint64_t groups(uint64_t n) { return (n + 255) / 256; }

void bind(RefSim& s) {
    static_cast<ref::FluidPush&>(ref::pc) = s.push;
    ref::particles.p = s.particles.data();
    ref::vel.p = s.vel.data();
    ref::vel_old.p = s.vel_old.data();
    ref::acc.p = s.acc.data();
    ref::wacc.p = s.wacc.data();
    ref::cell_count.p = s.cell_count.data();
    ref::cell_type.p = s.cell_type.data();
    ref::pressure.p = s.pressure.data();
    ref::divergence.p = s.divergence.data();
}

template <class K> void dispatch(K kernel, uint64_t n) {
    const int64_t total = int64_t(groups(n) * 256);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < total; i++) kernel(uint3(uint(i), 0u, 0u));
}

template <class K> void dispatch_in_order(K kernel, uint64_t n) {
    const uint64_t total = groups(n) * 256;
    for (uint64_t i = 0; i < total; i++) kernel(uint3(uint(i), 0u, 0u));
}

void stage(RefSim& s, int k) {
    bind(s);
    const uint64_t faces = s.vel.size(), cells = s.pressure.size(), parts = s.particles.size();
    const uint64_t fc = faces > cells ? faces : cells;
    switch (k) {
        case 0: dispatch(ref::clear_grid, fc); break;
        case 1: dispatch(ref::p2g, parts); break;
        case 2: dispatch(ref::normalize_grid, fc); break;
        case 3: dispatch(ref::forces, faces); break;
        case 4: dispatch(ref::compute_divergence, cells); break;
        case 5:
            for (uint32_t it = 0; it < s.iterations; it++)
                for (uint parity = 0; parity < 2; parity++) {
                    s.push.parity = parity;
                    ref::pc.parity = parity;
                    dispatch(ref::pressure_rb, cells);
                }
            break;
        case 6: dispatch(ref::project, faces); break;
        case 7: dispatch(ref::g2p_advect, parts); break;
        default: break;
    }
}

}  // namespace

extern "C" {

void* ref_sim_new(const uint32_t dims[3], float h, float dt, float flip, const float origin[3], const float gravity[3],
                  uint32_t iterations, const float* particles, uint32_t n) {
    auto* s = new RefSim;
    ref::FluidPush& p = s->push;
    p.nx = dims[0];
    p.ny = dims[1];
    p.nz = dims[2];
    p.n_particles = n;
    p.h = h;
    p.dt = dt;
    p.flip = flip;
    p.inv_h = 1.0f / h;
    p.origin = float3(origin[0], origin[1], origin[2]);
    p.gravity = float3(gravity[0], gravity[1], gravity[2]);
    s->iterations = iterations;
    const uint64_t nx = dims[0], ny = dims[1], nz = dims[2];
    const uint64_t faces = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1), cells = nx * ny * nz;
    s->particles.resize(n);
    std::memcpy(s->particles.data(), particles, size_t(n) * sizeof(ref::Particle));
    s->vel.assign(faces, 0.0f);
    s->vel_old.assign(faces, 0.0f);
    s->acc.assign(faces, 0);
    s->wacc.assign(faces, 0);
    s->cell_count.assign(cells, 0u);
    s->cell_type.assign(cells, 0u);
    s->pressure.assign(cells, 0.0f);
    s->divergence.assign(cells, 0.0f);
    return s;
}

void ref_sim_free(void* p) { delete static_cast<RefSim*>(p); }

// Host threads the dispatches use (n > 0 sets them first).
int ref_num_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

// Stages numbered as the oracle's: 0 clear, 1 p2g, 2 normalize, 3 forces, 4 divergence,
// 5 pressure (every iteration), 6 project, 7 g2p.
int ref_sim_stage(void* p, int k) {
    if (k < 0 || k > 7) return -1;
    stage(*static_cast<RefSim*>(p), k);
    return 0;
}

void ref_sim_step(void* p, uint32_t n) {
    auto& s = *static_cast<RefSim*>(p);
    for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < 8; k++) stage(s, k);
}

// which: 0 particles (8 floats each), 1 vel, 2 vel_old, 3 acc, 4 wacc, 5 cell_count,
// 6 cell_type, 7 pressure, 8 divergence (the oracle's selectors).
int ref_sim_read(void* p, int which, void* out, size_t bytes) {
    auto& s = *static_cast<RefSim*>(p);
    const void* src = nullptr;
    size_t n = 0;
    switch (which) {
        case 0: src = s.particles.data(); n = s.particles.size() * sizeof(ref::Particle); break;
        case 1: src = s.vel.data(); n = s.vel.size() * 4; break;
        case 2: src = s.vel_old.data(); n = s.vel_old.size() * 4; break;
        case 3: src = s.acc.data(); n = s.acc.size() * 4; break;
        case 4: src = s.wacc.data(); n = s.wacc.size() * 4; break;
        case 5: src = s.cell_count.data(); n = s.cell_count.size() * 4; break;
        case 6: src = s.cell_type.data(); n = s.cell_type.size() * 4; break;
        case 7: src = s.pressure.data(); n = s.pressure.size() * 4; break;
        case 8: src = s.divergence.data(); n = s.divergence.size() * 4; break;
        default: return -1;
    }
    if (bytes != n) return -2;
    std::memcpy(out, src, n);
    return 0;
}

// The surface pass of particles[n] on a grid of sdims cells: density and phi per node, cell_vert
// per cell, verts[2 * max_verts] float4 (position, normal), indices[3 * max_tris], counters.
int ref_surface_nets(const float* particles, uint32_t n, const uint32_t sdims[3], float sh, float radius, float iso,
                     const float origin[3], uint32_t max_verts, uint32_t max_tris, int32_t* density, float* phi,
                     uint32_t* cell_vert, float* verts, uint32_t* indices, uint32_t counters[2]) {
    ref::FluidPush p{};
    p.n_particles = n;
    p.origin = float3(origin[0], origin[1], origin[2]);
    p.sx = sdims[0];
    p.sy = sdims[1];
    p.sz = sdims[2];
    p.max_verts = max_verts;
    p.sh = sh;
    p.radius = radius;
    p.iso = iso;
    p.vbase = 0;
    p.ibase = 0;
    p.max_tris = max_tris;
    const uint64_t snodes = uint64_t(sdims[0] + 1) * (sdims[1] + 1) * (sdims[2] + 1);
    const uint64_t scells = uint64_t(sdims[0]) * sdims[1] * sdims[2];
    std::vector<ref::Particle> parts(n);
    std::memcpy(parts.data(), particles, size_t(n) * sizeof(ref::Particle));
    static_cast<ref::FluidPush&>(ref::pc) = p;
    ref::particles.p = parts.data();
    ref::density.p = density;
    ref::phi.p = phi;
    ref::cell_vert.p = cell_vert;
    ref::counters.p = counters;
    ref::out_verts.p = reinterpret_cast<float4*>(verts);
    ref::out_indices.p = indices;
    dispatch(ref::s_clear, snodes > scells ? snodes : scells);
    dispatch(ref::s_splat, n);
    dispatch(ref::s_phi, snodes);
    dispatch_in_order(ref::s_verts, scells);
    dispatch_in_order(ref::s_quads, snodes);
    return 0;
}

}  // extern "C"
