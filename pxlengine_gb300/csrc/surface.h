// Surface-nets meshing (shaders/fluid.slang:222-355) into library-owned device buffers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pxf {

// Device view of one simulation's surface grid and mesh buffers.
struct SurfDev {
    uint32_t sx, sy, sz;          // surface cells per axis (grid cells x surface_refine)
    float sh;                     // surface cell size
    float radius;                 // splat radius (particle_radius x sh)
    float iso;                    // iso level
    float ox, oy, oz;             // grid origin
    uint32_t max_verts, max_tris; // both the fluid's max_triangles (fluid.rs:171-175)
    int32_t* density;             // (sx+1)(sy+1)(sz+1) nodes, fixed point x 4096
    float* phi;                   // nodes: smoothed density - iso (> 0 inside)
    uint32_t* cell_vert;          // sx sy sz cells: vertex index or 0xffffffff
    float4* verts;                // 2 per vertex: (x, y, z, 0), (nx, ny, nz, 0)
    uint32_t* indices;            // 3 per triangle, vertex indices
    uint32_t* vchunk;             // per 2048-cell chunk: vertices, then their exclusive scan
    uint32_t* qchunk;             // per 2048-node chunk: quads, then their exclusive scan
    uint32_t* counters;           // [0] vertices, [1] triangles (before the caps)
};

// Density splat, phi, vertices, quads for the particles pos[0..np).
cudaError_t launch_surface(const SurfDev& S, const float4* pos, uint32_t np, cudaStream_t st);
uint32_t surface_chunks(uint64_t items);

}  // namespace pxf
