// pxlengine's own agent neighbour grid (shaders/sim.slang:28-104) run on the CPU — test
// infrastructure only.
//
// oracle/ref_build.py turns the shader's source, where it lies in the reference checkout, into
// sim_slang.inc (the edits of fluid_slang.inc plus `groupshared` dropped: the array is shared by
// the host threads that run one workgroup) and compiles this file with oracle/slang_shim.h
// force-included. Every kernel is the shader's own function; this file plays the host's part of
// crates/pxl-render/src/sim.rs: SimPush from grid_push (sim.rs:178-186: cell_size clamped to at
// least 1e-6, n_blocks = table_size / 1024), the buffers of SimState::new (sim.rs:129-141) and the
// dispatch sequence of sim_advance (sim.rs:258-270): grid_clear over ceil(table / 256) groups,
// grid_count over ceil(count / 256), scan_local over max(n_blocks, 1), scan_blocks over one group,
// scan_add over max(n_blocks, 1), grid_scatter over ceil(count / 256). Kernels that synchronise
// a workgroup (GroupMemoryBarrierWithGroupSync) run each group as a team of 256 OpenMP threads,
// one per invocation; the others run their invocations on all host threads. grid_count and
// grid_scatter use InterlockedAdd (atomic): counts are exact, and the order of the agents inside
// one cell follows the atomics, as on a GPU.
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

namespace refsim {
#include "sim_slang.inc"
}  // namespace refsim

namespace {

uint64_t groups_of(uint64_t n) { return (n + 255) / 256; }

template <class K> void dispatch(K kernel, uint64_t groups) {
    const int64_t total = int64_t(groups * 256);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < total; i++) kernel(uint3(uint(i), 0u, 0u));
}

// One team of 256 host threads per workgroup, one thread per invocation (barriers inside).
template <class K> bool dispatch_teams(K kernel, uint64_t groups) {
    omp_set_dynamic(0);
    bool ok = true;
    for (uint64_t g = 0; g < groups && ok; g++) {
#pragma omp parallel num_threads(256)
        {
            if (omp_get_num_threads() != 256) {
#pragma omp single
                ok = false;
            } else {
                kernel(uint3(uint(g), 0u, 0u), uint3(uint(omp_get_thread_num()), 0u, 0u));
            }
        }
    }
    return ok;
}

}  // namespace

extern "C" {

// The neighbour grid of `count` agents (16 floats each: position, size, velocity, age, colour,
// data): offsets[table_size], counts[table_size], sorted[count]. 0 on success, -1 when a
// workgroup could not get its 256 host threads.
int ref_grid_sort(const float* agents, uint32_t count, float cell_size, uint32_t table_size, uint32_t* offsets,
                  uint32_t* counts, uint32_t* sorted) {
    refsim::SimPush p{};
    p.count = count;
    p.table_size = table_size;
    p.cell_size = cell_size > 1e-6f ? cell_size : 1e-6f;
    p.n_blocks = table_size / 1024;
    static_cast<refsim::SimPush&>(refsim::pc) = p;
    std::vector<refsim::Agent> a(count);
    if (count) std::memcpy(a.data(), agents, size_t(count) * sizeof(refsim::Agent));
    std::vector<uint> cursor(table_size), block_sums(table_size / 1024 > 1 ? table_size / 1024 : 1);
    refsim::agents.p = a.data();
    refsim::offsets.p = offsets;
    refsim::counts.p = counts;
    refsim::sorted.p = sorted;
    refsim::cursor.p = cursor.data();
    refsim::block_sums.p = block_sums.data();
    const uint64_t blocks = p.n_blocks > 1 ? p.n_blocks : 1;
    dispatch(refsim::grid_clear, groups_of(table_size));
    dispatch(refsim::grid_count, groups_of(count));
    if (!dispatch_teams(refsim::scan_local, blocks)) return -1;
    if (!dispatch_teams([](uint3, uint3 t) { refsim::scan_blocks(t); }, 1)) return -1;
    if (!dispatch_teams(refsim::scan_add, blocks)) return -1;
    dispatch(refsim::grid_scatter, groups_of(count));
    return 0;
}

}  // extern "C"
