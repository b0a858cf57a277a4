// oracle_api.cpp — extern "C" entry points of the CPU oracle (test infrastructure).
#include <cstring>

#include "oracle.hpp"

namespace vvo {
void tf_evaluate(const vv_transfer_function* tf, float hu, float out[4]);
void tf_lut(const vv_transfer_function* tf, float* lut);
void tf_cumulative(const vv_transfer_function* tf, float* out);
uint16_t hu_to_unorm16(int16_t hu);
void bucket_max(const vv_transfer_function* tf, float out[64]);
void tf_lut_half(const vv_transfer_function* tf, uint16_t* out);
Geometry geometry(const vv_volume* v);
void pack_uniforms(const Geometry& G, const float tf_bucket_max[64], bool has_labels, bool has_env_map,
                   float env_peak_u, const vv_frame_params& p, uint32_t accumulated, uint64_t frame,
                   uint32_t width, uint32_t height, Uniforms& u);
int mask_margin(const Geometry& G, const vv_label_params& l);
void normals_pass(const Uniforms& u, const Scene& sc, int8_t* out, int threads);
void mask_passes(const Uniforms& u, const Scene& sc, const uint8_t* soft_data, ivec3 soft_dims, ivec4 soft_push,
                 int margin, int radius, uint16_t* out_a, uint16_t* scratch_b, int threads);
void majorant_pass(const Uniforms& u, const Scene& sc, float* out);
void pt_frame(const Uniforms& u, const Scene& sc, float* accum, float* albedo, float* normal, uint16_t* hdr,
              int y0, int y1, int threads);
void pt_pixel(const Uniforms& u, const Scene& sc, int x, int y, float out[12]);
void pt_pixels(const Uniforms& u, const Scene& sc, const int* pix, long n, float* out, int threads);
void extinction_probe(const Uniforms& u, const Scene& sc, const float* idx, long n, const float dir[3], int smooth,
                      float* out, int threads);
void pt_rows(const Uniforms& u, const Scene& sc, float* accum, float* albedo, float* normal, uint16_t* hdr,
             const int* rows, int nrows, int threads);
void bspline(const Uniforms& u, const Scene& sc, const float* idx, long n, float* out);
void light_samples(const Uniforms& u, const Scene& sc, const uint32_t* seeds, long n, float* out);
void denoise(const Uniforms& u, const float* accum, const float* albedo, const float* normal, uint16_t* hdr,
             float* ping, float* pong, int threads);
void post(const Uniforms& u, const uint16_t* hdr, float* exposure, uint8_t* out);
float env_prepare(int w, int h, const float* pixels, uint16_t* radiance, float* table, uint16_t* diffuse);
}  // namespace vvo

using namespace vvo;

extern "C" {

// The device inputs of the shaders as plain arrays (x-fastest).
typedef struct vvo_scene {
    int dims[3];
    const void* density;
    const int8_t* normals;
    const uint16_t* mask;
    const uint8_t* labels;
    int label_dims[3];
    const float* majorant;
    int brick_dims[3];
    const uint16_t* tf_lut;
    const float* preint;
    const uint16_t* env_rad;
    const float* env_table;
    int env_dims[2];
    int density_format;
    int mask_format;
} vvo_scene;

typedef struct vvo_geometry {
    float world_to_index[16];
    float index_to_world[16];
    float dims[3];
    float bounds_lo[3], bounds_hi[3];
    float min_spacing, max_spacing;
    float center[3];
    float diagonal;
} vvo_geometry;

static Scene to_scene(const vvo_scene* s) {
    Scene sc;
    sc.dims = ivec3(s->dims[0], s->dims[1], s->dims[2]);
    sc.density = s->density;
    sc.normals = s->normals;
    sc.mask = s->mask;
    sc.labels = s->labels;
    sc.label_dims = ivec3(s->label_dims[0], s->label_dims[1], s->label_dims[2]);
    sc.majorant = s->majorant;
    sc.brick_dims = ivec3(s->brick_dims[0], s->brick_dims[1], s->brick_dims[2]);
    sc.tf_lut = s->tf_lut;
    sc.preint = s->preint;
    sc.env_rad = s->env_rad;
    sc.env_table = s->env_table;
    sc.env_dims = ivec2(s->env_dims[0], s->env_dims[1]);
    sc.density_format = s->density_format;
    sc.mask_format = s->mask_format;
    return sc;
}
static const Uniforms& U(const void* p) { return *(const Uniforms*)p; }

long vvo_uniform_size(void) { return (long)sizeof(Uniforms); }

// EnvironmentMap::prepare (environment.rs:57-175) and the RGBA16F uploads
// (renderer.rs:2224-2290): radiance as half RGBA (w x h), the sampling table
// (RG32F, (w + 1) x h), the diffuse convolution (half RGBA, 32 x 16; may be
// NULL); returns peak_u.
float vvo_env_prepare(int w, int h, const float* pixels, uint16_t* radiance, float* table, uint16_t* diffuse) {
    return env_prepare(w, h, pixels, radiance, table, diffuse);
}

void vvo_hu_to_unorm16(const int16_t* hu, long n, uint16_t* out) {
    for (long i = 0; i < n; i++) out[i] = hu_to_unorm16(hu[i]);
}
void vvo_tf_evaluate(const vv_transfer_function* tf, float hu, float out[4]) { tf_evaluate(tf, hu, out); }
void vvo_tf_lut(const vv_transfer_function* tf, float* out) { tf_lut(tf, out); }
void vvo_tf_lut_half(const vv_transfer_function* tf, uint16_t* out) { tf_lut_half(tf, out); }
void vvo_tf_cumulative(const vv_transfer_function* tf, float* out) { tf_cumulative(tf, out); }
void vvo_bucket_max(const vv_transfer_function* tf, float out[64]) { bucket_max(tf, out); }

void vvo_geometry_of(const vv_volume* v, vvo_geometry* out) {
    Geometry G = geometry(v);
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
            out->world_to_index[4 * c + r] = G.world_to_index[c][r];
            out->index_to_world[4 * c + r] = G.index_to_world[c][r];
        }
    for (int r = 0; r < 3; r++) {
        out->dims[r] = G.dims[r];
        out->bounds_lo[r] = G.bounds_lo[r];
        out->bounds_hi[r] = G.bounds_hi[r];
        out->center[r] = G.center[r];
    }
    out->min_spacing = G.min_spacing;
    out->max_spacing = G.max_spacing;
    out->diagonal = G.diagonal;
}

void vvo_pack_uniforms(const vv_volume* vol, const float bucket[64], int has_labels, int has_env_map,
                       float env_peak_u, const vv_frame_params* p, uint32_t accumulated, uint64_t frame,
                       uint32_t width, uint32_t height, void* out) {
    pack_uniforms(geometry(vol), bucket, has_labels != 0, has_env_map != 0, env_peak_u, *p, accumulated, frame,
                  width, height, *(Uniforms*)out);
}
int vvo_mask_margin(const vv_volume* vol, const vv_label_params* l) { return mask_margin(geometry(vol), *l); }

void vvo_normals(const void* u, const vvo_scene* s, int8_t* out, int threads) {
    normals_pass(U(u), to_scene(s), out, threads);
}
void vvo_mask(const void* u, const vvo_scene* s, const uint8_t* soft, const int soft_dims[3],
              const int soft_push[4], int margin, int radius, uint16_t* out_a, uint16_t* scratch_b, int threads) {
    ivec3 sd = soft ? ivec3(soft_dims[0], soft_dims[1], soft_dims[2]) : ivec3(1);
    mask_passes(U(u), to_scene(s), soft, sd, ivec4(soft_push[0], soft_push[1], soft_push[2], soft_push[3]), margin,
                radius, out_a, scratch_b, threads);
}
void vvo_majorant(const void* u, const vvo_scene* s, float* out) { majorant_pass(U(u), to_scene(s), out); }
void vvo_pt_frame(const void* u, const vvo_scene* s, float* accum, float* albedo, float* normal, uint16_t* hdr,
                  int y0, int y1, int threads) {
    pt_frame(U(u), to_scene(s), accum, albedo, normal, hdr, y0, y1, threads);
}
void vvo_pt_rows(const void* u, const vvo_scene* s, float* accum, float* albedo, float* normal, uint16_t* hdr,
                 const int* rows, int nrows, int threads) {
    pt_rows(U(u), to_scene(s), accum, albedo, normal, hdr, rows, nrows, threads);
}
void vvo_pt_pixel(const void* u, const vvo_scene* s, int x, int y, float out[12]) {
    pt_pixel(U(u), to_scene(s), x, y, out);
}
void vvo_pt_pixels(const void* u, const vvo_scene* s, const int* pix, long n, float* out, int threads) {
    pt_pixels(U(u), to_scene(s), pix, n, out, threads);
}
void vvo_extinction(const void* u, const vvo_scene* s, const float* idx, long n, const float* dir, int smooth,
                    float* out, int threads) {
    extinction_probe(U(u), to_scene(s), idx, n, dir, smooth, out, threads);
}
void vvo_bspline(const void* u, const vvo_scene* s, const float* idx, long n, float* out) {
    bspline(U(u), to_scene(s), idx, n, out);
}
void vvo_light_samples(const void* u, const vvo_scene* s, const uint32_t* seeds, long n, float* out) {
    light_samples(U(u), to_scene(s), seeds, n, out);
}
void vvo_denoise(const void* u, const float* accum, const float* albedo, const float* normal, uint16_t* hdr,
                 float* ping, float* pong, int threads) {
    denoise(U(u), accum, albedo, normal, hdr, ping, pong, threads);
}

void vvo_post(const void* u, const uint16_t* hdr, float* exposure, uint8_t* out) { post(U(u), hdr, exposure, out); }

}  // extern "C"
