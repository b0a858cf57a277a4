// oracle_host.cpp — host-side math of the reference's render crate, restated.
//
// TEST INFRASTRUCTURE ONLY (see oracle.hpp). Each function cites the Rust it
// restates. Vector arithmetic follows glam's formulas (normalize multiplies by
// the reciprocal length; Mat3 * Vec3 sums the scaled columns in order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.hpp"

namespace vvo {

static const float HU_MIN = -1024.0f, HU_MAX = 3071.0f;  // transfer.rs:2-3
static const int LUT_SIZE = 4096;                        // transfer.rs:4

// ---- glam-style helpers (f32)
struct g3 { float x, y, z; };
static g3 g_add(g3 a, g3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static g3 g_sub(g3 a, g3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static g3 g_mul(g3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static float g_dot(g3 a, g3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
static g3 g_cross(g3 a, g3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
static g3 g_normalize(g3 a) { return g_mul(a, 1.0f / std::sqrt(g_dot(a, a))); }
static vec4 g4(g3 a, float w) { return vec4(a.x, a.y, a.z, w); }

// transfer.rs:72-86
void tf_evaluate(const vv_transfer_function* tf, float hu, float out[4]) {
    const vv_control_point* p = tf->points;
    auto rgba = [](const vv_control_point& c, float* o) {
        o[0] = c.color[0]; o[1] = c.color[1]; o[2] = c.color[2]; o[3] = c.extinction;
    };
    if (hu <= p[0].hu) { rgba(p[0], out); return; }
    for (uint32_t k = 0; k + 1 < tf->count; k++) {
        if (hu <= p[k + 1].hu) {
            float t = (hu - p[k].hu) / std::fmax(p[k + 1].hu - p[k].hu, 1e-6f);
            float a[4], b[4];
            rgba(p[k], a);
            rgba(p[k + 1], b);
            for (int i = 0; i < 4; i++) out[i] = a[i] + (b[i] - a[i]) * t;
            return;
        }
    }
    rgba(p[tf->count - 1], out);
}

// transfer.rs:90-97
void tf_lut(const vv_transfer_function* tf, float* lut) {
    for (int i = 0; i < LUT_SIZE; i++) {
        float t = float(i) / float(LUT_SIZE - 1);
        tf_evaluate(tf, HU_MIN + t * (HU_MAX - HU_MIN), lut + 4 * i);
    }
}

// transfer.rs:103-117 (f64 trapezoid rule)
void tf_cumulative(const vv_transfer_function* tf, float* out) {
    std::vector<float> lut(4 * LUT_SIZE);
    tf_lut(tf, lut.data());
    auto weighted = [&](int i, double* w) {
        const float* e = &lut[4 * i];
        w[0] = double(e[0] * e[3]); w[1] = double(e[1] * e[3]); w[2] = double(e[2] * e[3]); w[3] = double(e[3]);
    };
    double dx = 1.0 / double(LUT_SIZE - 1);
    double sum[4] = {0, 0, 0, 0};
    for (int c = 0; c < 4; c++) out[c] = 0.0f;
    for (int i = 1; i < LUT_SIZE; i++) {
        double a[4], b[4];
        weighted(i - 1, a);
        weighted(i, b);
        for (int c = 0; c < 4; c++) {
            sum[c] += 0.5 * (a[c] + b[c]) * dx;
            out[4 * i + c] = float(sum[c]);
        }
    }
}

// transfer.rs:121-124: t in [0, 1], scaled to 65535 and rounded half away from zero.
uint16_t hu_to_unorm16(int16_t hu) {
    float t = (float(hu) - HU_MIN) / (HU_MAX - HU_MIN);
    t = std::fmin(std::fmax(t, 0.0f), 1.0f);
    return (uint16_t)std::round(t * 65535.0f);
}

// renderer.rs:2164-2174: the f32 LUT's largest extinction over each 1/64 of the
// density range, including the first entry of the next bucket.
void bucket_max(const vv_transfer_function* tf, float out[64]) {
    std::vector<float> lut(4 * LUT_SIZE);
    tf_lut(tf, lut.data());
    int per = LUT_SIZE / 64;
    for (int b = 0; b < 64; b++) {
        int end = std::min((b + 1) * per + 1, LUT_SIZE);
        float m = 0.0f;
        for (int i = b * per; i < end; i++) m = std::fmax(m, lut[4 * i + 3]);
        out[b] = m;
    }
}

// renderer.rs:2178-2182: the LUT uploaded as RGBA16F (round to nearest even).
void tf_lut_half(const vv_transfer_function* tf, uint16_t* out) {
    std::vector<float> lut(4 * LUT_SIZE);
    tf_lut(tf, lut.data());
    for (int i = 0; i < 4 * LUT_SIZE; i++) out[i] = glsl::float_to_half(lut[i]);
}

// volio::Volume::index_to_world / world_to_index (volume.rs:22-35) and the
// derived extents of Renderer::new (renderer.rs:819-834, 896-901), in f64 then
// cast to f32 as glam's as_mat4/as_vec3 do.
Geometry geometry(const vv_volume* v) {
    double m[9];  // direction * diag(spacing), column-major
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) m[3 * c + r] = v->direction[3 * c + r] * v->spacing[c];
    // Inverse of the affine map [m | origin].
    double a = m[0], b = m[3], c = m[6], d = m[1], e = m[4], f = m[7], g = m[2], h = m[5], k = m[8];
    double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
    double det = a * A + b * B + c * C;
    double inv[9] = {A / det, B / det, C / det,
                     -(b * k - c * h) / det, (a * k - c * g) / det, -(a * h - b * g) / det,
                     (b * f - c * e) / det, -(a * f - c * d) / det, (a * e - b * d) / det};
    // inv is row-major: row r = inv[3r..3r+2]
    double t[3];
    for (int r = 0; r < 3; r++)
        t[r] = -(inv[3 * r] * v->origin[0] + inv[3 * r + 1] * v->origin[1] + inv[3 * r + 2] * v->origin[2]);
    Geometry G;
    for (int col = 0; col < 3; col++) {
        G.world_to_index[col] = vec4(float(inv[col]), float(inv[3 + col]), float(inv[6 + col]), 0.0f);
        G.index_to_world[col] = vec4(float(m[3 * col]), float(m[3 * col + 1]), float(m[3 * col + 2]), 0.0f);
    }
    G.world_to_index[3] = vec4(float(t[0]), float(t[1]), float(t[2]), 1.0f);
    G.index_to_world[3] = vec4(float(v->origin[0]), float(v->origin[1]), float(v->origin[2]), 1.0f);
    G.dims = vec3(float(v->dims[0]), float(v->dims[1]), float(v->dims[2]));
    auto to_world = [&](double x, double y, double z, double* o) {
        for (int r = 0; r < 3; r++) o[r] = m[r] * x + m[3 + r] * y + m[6 + r] * z + v->origin[r];
    };
    double cw[3];
    to_world((v->dims[0] - 1.0) * 0.5, (v->dims[1] - 1.0) * 0.5, (v->dims[2] - 1.0) * 0.5, cw);
    G.center = vec3(float(cw[0]), float(cw[1]), float(cw[2]));
    G.bounds_lo = vec3(3.4028235e38f);
    G.bounds_hi = vec3(-3.4028235e38f);
    for (int i = 0; i < 8; i++) {
        double x = (i & 1) ? v->dims[0] - 0.5 : -0.5;
        double y = (i & 2) ? v->dims[1] - 0.5 : -0.5;
        double z = (i & 4) ? v->dims[2] - 0.5 : -0.5;
        double w[3];
        to_world(x, y, z, w);
        for (int r = 0; r < 3; r++) {
            G.bounds_lo[r] = std::fmin(G.bounds_lo[r], float(w[r]));
            G.bounds_hi[r] = std::fmax(G.bounds_hi[r], float(w[r]));
        }
    }
    G.min_spacing = float(std::fmin(v->spacing[0], std::fmin(v->spacing[1], v->spacing[2])));
    G.max_spacing = float(std::fmax(v->spacing[0], std::fmax(v->spacing[1], v->spacing[2])));
    double ext = 0.0;
    for (int r = 0; r < 3; r++) {
        double x = std::fmax(double(v->dims[r]) - 1.0, 0.0) * v->spacing[r];
        ext += x * x;
    }
    G.diagonal = float(std::sqrt(ext));
    return G;
}

// camera.rs:34-48
static g3 cam_forward(const vv_orbit_camera& c) {
    float sy = std::sin(c.yaw), cy = std::cos(c.yaw), sp = std::sin(c.pitch), cp = std::cos(c.pitch);
    return {cp * sy, cp * cy, -sp};
}
static g3 cam_eye(const vv_orbit_camera& c) {
    return g_sub({c.target[0], c.target[1], c.target[2]}, g_mul(cam_forward(c), c.distance));
}
static void cam_basis(const vv_orbit_camera& c, g3& right, g3& up) {
    g3 f = cam_forward(c);
    right = g_normalize(g_cross(f, {0.0f, 0.0f, 1.0f}));
    up = g_cross(right, f);
}

// renderer.rs:80-87
static float tissue_majorant(const vv_label_params& l, float anisotropy, float limit) {
    float g = std::fmin(std::fmax(anisotropy, 0.0f), 0.95f);
    float largest = 0.0f;
    for (int i = 0; i < 256; i++) {
        if (l.colors[i][3] > 0.5f && !l.ghost[i] && l.optics[i][3] > 0.0f) {
            float m = 0.0f;
            for (int c = 0; c < 3; c++) m = std::fmax(m, l.optics[i][c]);
            largest = std::fmax(largest, m);
        }
    }
    return std::fmin(largest / (1.0f - g), limit);
}

// What `record` writes into the uniform block (renderer.rs:1516-1660), with the
// clip planes of clip_uniforms (renderer.rs:1449-1466).
void pack_uniforms(const Geometry& G, const float tf_bucket_max[64], bool has_labels,
                   bool has_env_map, float env_peak_u, const vv_frame_params& p,
                   uint32_t accumulated, uint64_t frame, uint32_t width, uint32_t height,
                   Uniforms& u) {
    std::memset((void*)&u, 0, sizeof(u));
    const vv_orbit_camera& cam = p.camera;
    g3 right, up;
    cam_basis(cam, right, up);
    g3 fwd = cam_forward(cam), eye = cam_eye(cam);
    float tan_half = std::tan(cam.fov_y / 2.0f);
    float aspect = float(width) / float(height);
    const vv_lighting& L = p.lighting;
    // Lighting::light_direction (renderer.rs:296-306)
    float se = std::sin(L.elevation), ce = std::cos(L.elevation);
    float sa = std::sin(L.azimuth), ca = std::cos(L.azimuth);
    g3 light_dir = g_normalize(g_add(g_add(g_mul(g_mul(g_mul(fwd, -1.0f), ce), ca),
                                           g_mul(g_mul(right, ce), sa)),
                                     g_mul(up, se)));
    int environment = L.environment;
    if (environment == VV_ENV_MAP && !has_env_map) environment = VV_ENV_STUDIO;
    float env_rotation = 0.0f;
    if (has_env_map) {
        float key_phi = std::atan2(std::sin(L.azimuth), -std::cos(L.azimuth));
        env_rotation = (env_peak_u - 0.5f) * 6.28318530717958647692f - key_phi + L.env_rotation;
    }
    const vv_label_params& lab = p.labels;
    u.world_to_index = G.world_to_index;
    u.eye = g4(eye, 1.0f);
    u.forward = g4(fwd, 0.0f);
    u.right = g4(g_mul(g_mul(right, tan_half), aspect), 0.0f);
    u.up = g4(g_mul(up, tan_half), 0.0f);
    u.dims = vec4(G.dims, p.step_mm);
    u.flags = uvec4(uint32_t(frame), p.srgb_encode ? 1u : 0u, width, height);
    float mode = has_labels ? float(lab.mode) : 0.0f;
    u.labels = vec4(mode, lab.tint, lab.extinction, lab.ghost_opacity);
    u.light_dir = g4(light_dir, L.intensity);
    float amb = environment == VV_ENV_STUDIO ? 0.5f * L.ambient : L.ambient;
    u.ambient = vec4(amb, amb, amb, std::exp2(L.exposure));
    u.material = vec4(L.roughness, L.metalness, float(L.tone_mapper), L.light_size);
    u.lighting = uvec4(L.shadows ? 1u : 0u, L.ambient_occlusion ? 1u : 0u, p.preintegrate ? 1u : 0u,
                       uint32_t(environment));
    u.light_cells = vec4(2.0f * G.max_spacing, 4.0f * G.max_spacing, 0.0f, 0.0f);
    // clip_uniforms
    {
        g3 col[3];
        for (int c = 0; c < 3; c++) col[c] = {G.index_to_world[c].x, G.index_to_world[c].y, G.index_to_world[c].z};
        g3 b = {G.index_to_world[3].x, G.index_to_world[3].y, G.index_to_world[3].z};
        uint32_t n = 0;
        for (int i = 0; i < 3; i++) {
            const vv_clip_plane& cp = p.clipping.planes[i];
            if (!cp.enabled) continue;
            float sign = cp.cut_positive ? 1.0f : -1.0f;
            g3 normal = {0.0f, 0.0f, 0.0f};
            (&normal.x)[cp.plane] = 1.0f;
            normal = g_mul(normal, sign);
            // a.transpose() * normal: row r of the transpose is column r of a.
            g3 an = {g_dot(col[0], normal), g_dot(col[1], normal), g_dot(col[2], normal)};
            u.clip_planes[n] = g4(an, sign * cp.position - g_dot(normal, b));
            u.clip_normals[n] = g4(normal, 0.0f);
            n++;
        }
        u.clip = uvec4(n, p.clipping.all ? 1u : 0u, 0u, 0u);
    }
    const vv_path_tracing& pt = p.path_tracing;
    uint32_t skip = p.skip_empty_space ? 1u : 0u;
    if (pt.enabled) {
        u.path = uvec4(accumulated, pt.bounces, std::max(pt.samples_per_frame, 1u), skip);
        float focus = cam.distance;
        if (pt.has_focus) focus = g_dot(g_sub({pt.focus[0], pt.focus[1], pt.focus[2]}, eye), fwd);
        u.lens = vec4(pt.aperture, std::fmax(focus, 1.0f), 0.0f, 0.0f);
    } else {
        u.path = uvec4(0u, 0u, 0u, skip);
    }
    u.env = vec4(env_rotation, p.smooth_sampling ? 1.0f : 0.0f, L.anisotropy, L.chromatic);
    u.finish = vec4(L.bloom, L.vignette, L.grain, L.auto_exposure ? 1.0f : 0.0f);
    for (int i = 0; i < 16; i++)
        u.tf_bucket_max[i] = vec4(tf_bucket_max[4 * i], tf_bucket_max[4 * i + 1], tf_bucket_max[4 * i + 2],
                                  tf_bucket_max[4 * i + 3]);
    u.subsurface = vec4(L.subsurface * L.subsurface_strength, 10.0f / std::fmax(L.scattering_distance, 0.1f),
                        0.7f, 2.0f * G.max_spacing);
    for (int i = 0; i < 256; i++) {
        const float* c = lab.colors[i];
        u.label_colors[i] = vec4(c[0], c[1], c[2], (c[3] > 0.5f && lab.ghost[i]) ? 2.0f : c[3]);
        const float* d = lab.density[i];
        u.label_density[i] = vec4(d[0], d[1], d[2], d[3]);
        const float* m = lab.materials[i];
        u.label_materials[i] = vec4(m[0], m[1], m[3], m[2] * L.subsurface_strength);
        const float* s = lab.surface[i];
        float k = L.surface_detail;
        u.label_surface[i] = vec4(s[0], s[1] * k, s[2] * k, s[3]);
        const float* o = lab.optics[i];
        u.label_optics[i] = vec4(o[0], o[1], o[2], o[3]);
    }
    float limit = 1.0f / (2.0f * G.max_spacing);
    u.tissue = vec4(tissue_majorant(lab, L.anisotropy, limit), limit, 0.0f, 0.0f);
}

// Cut margin of the mask pass in voxels (renderer.rs:1488-1491).
int mask_margin(const Geometry& G, const vv_label_params& l) {
    float m = std::round(l.cut_margin_mm / G.min_spacing);
    m = std::fmin(std::fmax(m, 0.0f), 3.0f);
    return int(m);
}


// ------------------------------------------------------------ light map
// environment.rs:57-130 (EnvironmentMap::prepare without the diffuse
// convolution, which only the ray marcher reads) and the upload of
// renderer.rs:2224-2290 (radiance to RGBA16F after min(60000)). Sums run in
// f64 in the Rust's order; per-texel arithmetic in f32 without contraction.
static float env_luminance(const float* c) { return 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2]; }

// environment.rs:133-175: the normalised radiance box-filtered to at most
// 128 x 64, then convolved with a clamped cosine lobe into 32 x 16 texels, to
// RGBA16F (min 60000) as uploaded. f32 arithmetic in the Rust's order.
static void env_diffuse(int w, int h, const float* rad, uint16_t* out) {
    const float PI_F = 3.14159265358979323846f;
    auto direction = [&](float uu, float vv, float d[3]) {
        float phi = (uu - 0.5f) * 2.0f * PI_F, theta = vv * PI_F;
        d[0] = std::sin(theta) * std::sin(phi);
        d[1] = std::cos(theta);
        d[2] = std::sin(theta) * std::cos(phi);
    };
    int sw = std::min(128, w), sh = std::max(sw / 2, 1);
    std::vector<float> small(6 * (size_t)sw * sh);  // radiance x solid angle rgb, direction xyz
    for (int i = 0; i < sw * sh; i++) {
        int sx = i % sw, sy = i / sw;
        int x0 = sx * w / sw, x1 = std::max((sx + 1) * w / sw, sx * w / sw + 1);
        int y0 = sy * h / sh, y1 = std::max((sy + 1) * h / sh, sy * h / sh + 1);
        float c[3] = {0.0f, 0.0f, 0.0f};
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++)
                for (int k = 0; k < 3; k++) c[k] = c[k] + rad[4 * ((size_t)y * w + x) + k];
        float n = (float)((y1 - y0) * (x1 - x0));
        float uu = ((float)sx + 0.5f) / (float)sw, vv = ((float)sy + 0.5f) / (float)sh;
        float solid = (2.0f * PI_F / (float)sw) * (PI_F / (float)sh) * std::sin(PI_F * vv);
        float* e = small.data() + 6 * (size_t)i;
        for (int k = 0; k < 3; k++) e[k] = c[k] / n * solid;
        direction(uu, vv, e + 3);
    }
    const int dw = 32, dh = 16;
    for (int i = 0; i < dw * dh; i++) {
        float nrm[3];
        direction(((float)(i % dw) + 0.5f) / (float)dw, ((float)(i / dw) + 0.5f) / (float)dh, nrm);
        float c[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < sw * sh; j++) {
            const float* e = small.data() + 6 * (size_t)j;
            float cs = nrm[0] * e[3] + nrm[1] * e[4] + nrm[2] * e[5];
            if (cs > 0.0f)
                for (int k = 0; k < 3; k++) c[k] = c[k] + e[k] * cs;
        }
        for (int k = 0; k < 3; k++) out[4 * i + k] = glsl::float_to_half(std::min(c[k] / PI_F, 60000.0f));
        out[4 * i + 3] = glsl::float_to_half(1.0f);
    }
}

float env_prepare(int w, int h, const float* pixels, uint16_t* radiance, float* table, uint16_t* diffuse) {
    const float PI_F = 3.14159265358979323846f;
    auto sin_theta = [&](int y) { return std::sin(PI_F * ((float)y + 0.5f) / (float)h); };
    // Mean radiance over the sphere (texels weighted by their solid angle).
    double sum[3] = {0.0, 0.0, 0.0}, weight = 0.0;
    for (int y = 0; y < h; y++) {
        float s = sin_theta(y);
        double row[3] = {0.0, 0.0, 0.0};
        for (int x = 0; x < w; x++)
            for (int i = 0; i < 3; i++) row[i] = row[i] + (double)pixels[3 * ((long)y * w + x) + i];
        for (int i = 0; i < 3; i++) sum[i] = sum[i] + row[i] * (double)s;
        weight = weight + (double)s * (double)w;
    }
    float mean_rgb[3] = {(float)(sum[0] / weight), (float)(sum[1] / weight), (float)(sum[2] / weight)};
    float mean = std::max(env_luminance(mean_rgb), 1e-6f);
    std::vector<float> rad_f((size_t)4 * w * h);
    for (long i = 0; i < (long)w * h; i++) {
        for (int c = 0; c < 3; c++) {
            rad_f[4 * i + c] = pixels[3 * i + c] / mean;
            radiance[4 * i + c] = glsl::float_to_half(std::min(rad_f[4 * i + c], 60000.0f));
        }
        rad_f[4 * i + 3] = 1.0f;
        radiance[4 * i + 3] = glsl::float_to_half(1.0f);
    }
    if (diffuse) env_diffuse(w, h, rad_f.data(), diffuse);
    // Importance sampling proportional to luminance x solid angle.
    std::vector<float> f((size_t)w * h);
    for (long i = 0; i < (long)w * h; i++) f[i] = env_luminance(pixels + 3 * i) * sin_theta((int)(i / w));
    std::vector<double> row_sums(h);
    for (int y = 0; y < h; y++) {
        double a = 0.0;
        for (int x = 0; x < w; x++) a = a + (double)f[(long)y * w + x];
        row_sums[y] = a;
    }
    double total = 0.0;
    for (int y = 0; y < h; y++) total = total + row_sums[y];
    total = std::max(total, (double)1e-12L);  // f64 constants: L-suffixed (floats otherwise)
    double marginal = 0.0;
    for (int y = 0; y < h; y++) {
        float* row = table + 2 * (long)y * (w + 1);
        double acc = 0.0;
        for (int x = 0; x < w; x++) {
            acc = acc + (double)f[(long)y * w + x];
            row[2 * x] = row_sums[y] > 0.0 ? (float)(acc / row_sums[y]) : (float)(x + 1) / (float)w;
            row[2 * x + 1] = (float)((double)f[(long)y * w + x] / total);
        }
        row[2 * (w - 1)] = 1.0f;
        marginal = marginal + row_sums[y];
        row[2 * w] = (float)(marginal / total);
        row[2 * w + 1] = (float)(row_sums[y] / total);
    }
    table[2 * ((long)(h - 1) * (w + 1) + w)] = 1.0f;
    // Brightest region: azimuth of the squared-luminance-weighted mean direction.
    double px = 0.0, pz = 0.0;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double l = (double)f[(long)y * w + x];
            float uu = ((float)x + 0.5f) / (float)w, vv = ((float)y + 0.5f) / (float)h;
            float phi = (uu - 0.5f) * 2.0f * PI_F, theta = vv * PI_F;
            float dx = std::sin(theta) * std::sin(phi), dz = std::sin(theta) * std::cos(phi);
            px = px + l * l * (double)dx;
            pz = pz + l * l * (double)dz;
        }
    return 0.5f + (float)(std::atan2(px, pz) / (double)(2.0L * 3.14159265358979323846264338327950288L));
}
}  // namespace vvo
