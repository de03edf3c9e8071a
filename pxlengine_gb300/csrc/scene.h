// Scene-JSON `fluids` front end: strict parsing with the reference's defaults and validation
// messages (crates/pxl-scene/src/lib.rs:49-129, 624-627, 634-648, 650-735).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pxlflip.h"

namespace pxf {

struct FluidCfg {
    std::string name;
    float bounds[2][3] = {{0, 0, 0}, {0, 0, 0}};
    uint32_t resolution = 64;
    std::vector<pxf_fill_block> fill;
    uint32_t particles_per_cell = 8;
    uint32_t substeps = 8;
    float flip = 0.95f;
    float gravity[3] = {0.0f, -9.81f, 0.0f};
    uint32_t pressure_iterations = 80;
    uint32_t surface_refine = 2;
    float particle_radius = 2.0f;
    float warmup = 0.0f;
    uint32_t max_triangles = 2000000;

    void from_desc(const pxf_fluid_desc& d);
    void to_desc(pxf_fluid_desc& d) const;   // d.name / d.fill point into this object
};

struct SceneFluids {
    std::vector<FluidCfg> fluids;
    uint32_t seed = 0;     // render.seed
    float fps = 24.0f;     // render.fps
};

// Fluid::grid (crates/pxl-scene/src/lib.rs:123-128).
void fluid_grid(const float bounds[2][3], uint32_t resolution, uint32_t n[3], float& h);

// The fluid checks of Scene::validate (crates/pxl-scene/src/lib.rs:710-735). Returns false and
// sets msg on failure. lift: accept grids beyond the scene limits (benchmark entry only).
bool validate_fluid(const FluidCfg& f, uint32_t index, bool lift, std::string& msg);

// Scene::from_json restricted to what the liquid path reads: version, camera presence,
// render.seed / render.fps and the fluids block. Returns false and sets msg on failure.
bool parse_scene(const char* text, SceneFluids& out, std::string& msg);

}  // namespace pxf
