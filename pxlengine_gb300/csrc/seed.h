// Device seeding plan (seed.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pxlflip.h"

namespace pxf {

constexpr int kMaxSeedBlocks = 32;

struct SeedBlock {
    uint64_t first;      // index of the block's first particle
    uint32_t lo[3], hi[3];
    float vel[3];
};

// Arguments of one seeding launch: up to kMaxSeedBlocks consecutive fill blocks covering the
// particle range [p_begin, p_end). Draw numbers stay global, so launches compose exactly.
struct SeedArgs {
    SeedBlock blk[kMaxSeedBlocks];
    int n_blocks;
    uint64_t p_begin, p_end;
    uint32_t ppc;
    float h;
    float origin[3];
    uint64_t rng0;
    float sigma;         // N(0, sigma) velocity jitter (0: none)
    uint32_t vseed;
};

struct SeedPlan {
    std::vector<SeedBlock> blocks;
    uint32_t ppc = 0;
    float h = 0;
    float origin[3] = {0, 0, 0};
    uint64_t rng0 = 0;
    uint64_t total = 0;
    float sigma = 0;
    uint32_t vseed = 0;
};

// Per-block kept cell boxes and particle offsets (the reference's loop order).
bool seed_plan(const float origin[3], float h, const uint32_t n[3], const pxf_fill_block* fill, uint32_t n_fill,
               uint32_t ppc, uint32_t seed, SeedPlan& plan);
// Writes plan.total particles to pos/vel (and to pos0/vel0 when given).
cudaError_t launch_seed(const SeedPlan& plan, float4* pos, float4* vel, float4* pos0, float4* vel0, cudaStream_t st);

}  // namespace pxf
