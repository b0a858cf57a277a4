// oracle_api64.cpp — the path tracer's restatement in double precision
// (test infrastructure): the FP64 oracle, the reference that the precision
// variant's storage formats are measured against.
//
// The same source as the FP32 oracle (oracle_shaders.cpp), compiled with
// `float` defined as `double` (prelude.hpp): every product, sum, texture
// filter weight and decoded texel is a double, the pixel sums accumulate in
// double, the constants keep the shaders' single-precision values, and the
// inputs (the std140 uniform block, the stored volumes, tables and LUT) keep
// their layouts. Built into oracle/_build/liboracle64.so by build_oracle.py.
#define VVO_FP64 1
#include "prelude.hpp"
#include "oracle_shaders.cpp"

namespace {
using namespace vvo;

// The std140 block (4-byte floats and uints, renderer.rs:43-74) into the
// double-precision instance's Uniforms, member by member in block order.
Uniforms from_std140(const void* p) {
    const uint8_t* b = (const uint8_t*)p;
    size_t o = 0;
    Uniforms u;
    auto v4 = [&](vec4& d) {
        f32 t[4];
        std::memcpy(t, b + o, 16);
        o += 16;
        d = vec4(t[0], t[1], t[2], t[3]);
    };
    auto u4 = [&](uvec4& d) {
        uint32_t t[4];
        std::memcpy(t, b + o, 16);
        o += 16;
        d = uvec4(t[0], t[1], t[2], t[3]);
    };
    for (int c = 0; c < 4; c++) v4(u.world_to_index.c[c]);
    v4(u.eye); v4(u.forward); v4(u.right); v4(u.up); v4(u.dims);
    u4(u.flags);
    v4(u.labels); v4(u.light_dir); v4(u.ambient); v4(u.material);
    u4(u.lighting);
    v4(u.light_cells);
    u4(u.clip);
    for (int i = 0; i < 3; i++) v4(u.clip_planes[i]);
    for (int i = 0; i < 3; i++) v4(u.clip_normals[i]);
    v4(u.subsurface);
    u4(u.path);
    v4(u.env); v4(u.lens); v4(u.finish); v4(u.tissue);
    for (int i = 0; i < 16; i++) v4(u.tf_bucket_max[i]);
    for (int i = 0; i < 256; i++) v4(u.label_colors[i]);
    for (int i = 0; i < 256; i++) v4(u.label_materials[i]);
    for (int i = 0; i < 256; i++) v4(u.label_density[i]);
    for (int i = 0; i < 256; i++) v4(u.label_surface[i]);
    for (int i = 0; i < 256; i++) v4(u.label_optics[i]);
    (void)o;  // o == VV_UNIFORMS_BYTES
    return u;
}
}  // namespace

extern "C" {

// The device inputs of the shaders (the FP32 oracle's vvo_scene, field for field).
typedef struct vvo64_scene {
    int dims[3];
    const void* density;
    const int8_t* normals;
    const uint16_t* mask;
    const uint8_t* labels;
    int label_dims[3];
    const f32* majorant;
    int brick_dims[3];
    const uint16_t* tf_lut;
    const f32* preint;
    const uint16_t* env_rad;
    const f32* env_table;
    int env_dims[2];
    int density_format;
    int mask_format;
} vvo64_scene;

static Scene scene64(const vvo64_scene* s) {
    Scene sc;
    sc.dims = ivec3(s->dims[0], s->dims[1], s->dims[2]);
    sc.density = s->density;
    sc.normals = s->normals;
    sc.mask = s->mask;
    sc.labels = s->labels;
    sc.label_dims = ivec3(s->label_dims[0], s->label_dims[1], s->label_dims[2]);
    sc.majorant = (const double*)(const void*)s->majorant;  // texel data, decoded as R32F
    sc.brick_dims = ivec3(s->brick_dims[0], s->brick_dims[1], s->brick_dims[2]);
    sc.tf_lut = s->tf_lut;
    sc.preint = (const double*)(const void*)s->preint;
    sc.env_rad = s->env_rad;
    sc.env_table = (const double*)(const void*)s->env_table;
    sc.env_dims = ivec2(s->env_dims[0], s->env_dims[1]);
    sc.density_format = s->density_format;
    sc.mask_format = s->mask_format;
    return sc;
}

long vvo64_real_bytes(void) { return (long)sizeof(float); }  // 8: `float` is double here

// For each listed pixel (x, y pairs), the sums of `count` paths at
// accumulation indices first .. first + count - 1 (pt.comp's per-pixel
// streams): 12 doubles per pixel (radiance sum, background, albedo sums with
// luminance^2, normal sums with depth), accumulated in double.
void vvo64_pt_pixel_sums(const void* u, const vvo64_scene* s, const int* pix, long n, uint32_t first,
                         uint32_t count, double* out, int threads) {
    Uniforms uu = from_std140(u);
    Scene sc = scene64(s);
    Units t = bind_scene(sc);
    parallel_rows(n, threads, [&](long i) {
        Uniforms ui = uu;
        double acc[12] = {0};
        for (uint32_t k = 0; k < count; k++) {
            ui.path.x = first + k;
            Tracer tr{Shading{ui, t}};
            Tracer::PixelResult R = tr.trace_pixel(uint(pix[2 * i]), uint(pix[2 * i + 1]));
            double v[12] = {R.sum.x, R.sum.y, R.sum.z, R.background, R.albedo_sum.x, R.albedo_sum.y, R.albedo_sum.z,
                            R.albedo_sum.w, R.normal_sum.x, R.normal_sum.y, R.normal_sum.z, R.normal_sum.w};
            for (int c = 0; c < 12; c++) acc[c] += v[c];
        }
        std::memcpy(out + 12 * i, acc, sizeof(acc));
    });
}

}  // extern "C"
