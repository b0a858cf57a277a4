// oracle.hpp — CPU restatement of volview's progressive path-tracing path.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product library links this code; it
// is the checker that tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline compare the CUDA path against.
//
// Parity status: the host math (transfer function, LUT, density normalisation)
// is pinned by the reference's own unit tests (crates/render/src/transfer.rs:
// 130-149). The shader math is pinned against the reference's shaders compiled
// as CPU code by oracle/build_ref.py (golden fixtures under tests/golden/).
#pragma once
#include "glsl.hpp"
#include "../include/volpt.h"

namespace vvo {
GLSL_USING

// The reference's std140 uniform block, member for member
// (crates/render/src/renderer.rs:43-74 = shaders/common.glsl:4-33).
struct Uniforms {
    mat4 world_to_index;
    vec4 eye, forward, right, up, dims;
    uvec4 flags;
    vec4 labels, light_dir, ambient, material;
    uvec4 lighting;
    vec4 light_cells;
    uvec4 clip;
    vec4 clip_planes[3];
    vec4 clip_normals[3];
    vec4 subsurface;
    uvec4 path;
    vec4 env, lens, finish, tissue;
    vec4 tf_bucket_max[16];
    vec4 label_colors[256];
    vec4 label_materials[256];
    vec4 label_density[256];
    vec4 label_surface[256];
    vec4 label_optics[256];
};
#ifndef VVO_FP64
static_assert(sizeof(Uniforms) == VV_UNIFORMS_BYTES, "std140 layout");
#endif

// Geometry derived from a volume (volio Volume + renderer.rs:819-834).
struct Geometry {
    mat4 world_to_index;  // f64 inverse, cast to f32
    mat4 index_to_world;
    vec3 dims;
    vec3 bounds_lo, bounds_hi;
    float min_spacing, max_spacing;
    vec3 center;
    float diagonal;
};

// Device-side inputs of the shaders, as x-fastest arrays.
struct Scene {
    ivec3 dims;
    const void* density = nullptr;       // R16_UNORM, or the precision variant's format
    int density_format = 0;              // VV_DENSITY_*
    const int8_t* normals = nullptr;     // RGBA8_SNORM
    const uint16_t* mask = nullptr;      // RG16_UNORM (final, blurred), or the precision variant's format
    int mask_format = 0;                 // VV_MASK_*
    const uint8_t* labels = nullptr;     // R8_UINT; 1 voxel placeholder if absent
    ivec3 label_dims = ivec3(1, 1, 1);
    const float* majorant = nullptr;     // R32F over the brick grid
    ivec3 brick_dims;
    const uint16_t* tf_lut = nullptr;    // RGBA16F, 4096 entries
    const float* preint = nullptr;       // RGBA32F, 4096 entries
    const uint16_t* env_rad = nullptr;   // light map radiance, RGBA16F, env_dims
    const float* env_table = nullptr;    // light map sampling table, RG32F, (env_dims.x + 1) x env_dims.y
    ivec2 env_dims = ivec2(1, 1);
};

}  // namespace vvo
