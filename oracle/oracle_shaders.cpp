// oracle_shaders.cpp — the reference's compute shaders restated on the CPU.
//
// TEST INFRASTRUCTURE ONLY (see oracle.hpp). Each function cites the GLSL it
// restates. Textures are sampled through glsl.hpp's model of the Vulkan
// texture units; the uniform block is the reference's std140 layout.
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.hpp"

namespace vvo {

static const float PI = 3.14159265358979f;
static const int BRICK = 8;                  // common.glsl:57
static const uint SKIN_LABEL = 255u;         // common.glsl:61
static const uint FIRST_CT_LABEL = 250u;     // common.glsl:66
static const float MAX_EXTINCTION = 8.0f;    // pt.comp:34
static const uint MAX_VOLUME_EVENTS = 32u;   // pt.comp:112
static const float BONE_DENSITY = (300.0f + 1024.0f) / 4095.0f;  // common.glsl:250

// Bound textures of one pass.
struct Units {
    sampler3D density, normals, mask, majorant, mask_b;
    usampler3D labels, soft;
    sampler1D tf, preint;
    sampler2D env, env_table;  // light map (bindings 25, 26)
};

static void bind3(glsl::Texture& t, const void* data, glsl::Format f, ivec3 d, glsl::Filter filt) {
    t.data = data; t.format = f; t.w = d.x; t.h = d.y; t.d = d.z; t.filter = filt;
    t.address = glsl::CLAMP_TO_EDGE;
}

static glsl::Format mask_format_of(const Scene& s) {
    static const glsl::Format formats[3] = {glsl::RG16_UNORM, glsl::RG16F, glsl::RG16_BF16};
    return formats[s.mask_format >= 0 && s.mask_format < 3 ? s.mask_format : 0];
}

Units bind_scene(const Scene& s) {
    Units t;
    static const glsl::Format density_formats[4] = {glsl::R16_UNORM, glsl::R16F, glsl::R16_BF16, glsl::R32F};
    bind3(t.density, s.density, density_formats[s.density_format & 3], s.dims, glsl::LINEAR);
    if (s.normals) bind3(t.normals, s.normals, glsl::RGBA8_SNORM, s.dims, glsl::LINEAR);
    if (s.mask) bind3(t.mask, s.mask, mask_format_of(s), s.dims, glsl::LINEAR);
    if (s.majorant) bind3(t.majorant, s.majorant, glsl::R32F, s.brick_dims, glsl::NEAREST);
    if (s.labels) bind3(t.labels, s.labels, glsl::R8_UINT, s.label_dims, glsl::NEAREST);
    if (s.tf_lut) bind3(t.tf, s.tf_lut, glsl::RGBA16F, ivec3(4096, 1, 1), glsl::LINEAR);
    if (s.preint) bind3(t.preint, s.preint, glsl::RGBA32F, ivec3(4096, 1, 1), glsl::NEAREST);
    if (s.env_rad) {
        bind3(t.env, s.env_rad, glsl::RGBA16F, ivec3(s.env_dims.x, s.env_dims.y, 1), glsl::LINEAR);
        bind3(t.env_table, s.env_table, glsl::RG32F, ivec3(s.env_dims.x + 1, s.env_dims.y, 1), glsl::NEAREST);
    }
    return t;
}

// Splits [0, n) over `threads` host threads.
template <class F> static void parallel_rows(long n, int threads, F f) {
    if (threads <= 1) { for (long i = 0; i < n; i++) f(i); return; }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&, t] { for (long i = t; i < n; i += threads) f(i); });
    for (auto& th : pool) th.join();
}

// ============================================================ common.glsl
struct Sample {  // common.glsl:175-185
    vec3 albedo;
    float extinction;
    float roughness;
    float metalness;
    uint label;
    bool ghost;
    float density;
    float subsurface;
    float coat;
};

struct Shading {
    const Uniforms& u;
    const Units& t;

    vec3 index_to_tex(vec3 idx) const { return (idx + 0.5f) / vec3(u.dims.x, u.dims.y, u.dims.z); }
    float density_at_index(vec3 idx) const { return textureLod(t.density, index_to_tex(idx), 0.0f).x; }

    // common.glsl:89-113: per-axis folded B-spline taps (Sigg & Hadwiger).
    struct Taps { vec3 h0, h1, g0, g1, dh0, dh1, dg0, dg1; };
    Taps cubic_taps(vec3 idx) const {
        vec3 i = floor(idx), f = idx - i, f2 = f * f, f3 = f2 * f;
        vec3 w0 = (1.0f - 3.0f * f + 3.0f * f2 - f3) / 6.0f;
        vec3 w1 = (4.0f - 6.0f * f2 + 3.0f * f3) / 6.0f;
        vec3 w2 = (1.0f + 3.0f * f + 3.0f * f2 - 3.0f * f3) / 6.0f;
        vec3 w3 = f3 / 6.0f;
        vec3 d0 = -0.5f * (1.0f - f) * (1.0f - f);
        vec3 d1 = 0.5f * f * (3.0f * f - 4.0f);
        vec3 d2 = 0.5f * (1.0f - f) * (3.0f * f + 1.0f);
        vec3 d3 = 0.5f * f2;
        Taps k;
        k.g0 = w0 + w1;
        k.g1 = w2 + w3;
        k.h0 = i - 1.0f + w1 / k.g0;
        k.h1 = i + 1.0f + w3 / k.g1;
        k.dg0 = d0 + d1;
        k.dg1 = d2 + d3;
        k.dh0 = i - 1.0f + d1 / min(k.dg0, -1e-7f);
        k.dh1 = i + 1.0f + d3 / max(k.dg1, 1e-7f);
        return k;
    }
    // common.glsl:116-122
    float cubic_fetch(vec3 h0, vec3 h1, vec3 g0, vec3 g1) const {
        float a = g0.x * density_at_index(vec3(h0.x, h0.y, h0.z)) + g1.x * density_at_index(vec3(h1.x, h0.y, h0.z));
        float b = g0.x * density_at_index(vec3(h0.x, h1.y, h0.z)) + g1.x * density_at_index(vec3(h1.x, h1.y, h0.z));
        float c = g0.x * density_at_index(vec3(h0.x, h0.y, h1.z)) + g1.x * density_at_index(vec3(h1.x, h0.y, h1.z));
        float d = g0.x * density_at_index(vec3(h0.x, h1.y, h1.z)) + g1.x * density_at_index(vec3(h1.x, h1.y, h1.z));
        return g0.z * (g0.y * a + g1.y * b) + g1.z * (g0.y * c + g1.y * d);
    }
    float density_cubic(vec3 idx) const {  // common.glsl:124-127
        Taps k = cubic_taps(idx);
        return cubic_fetch(k.h0, k.h1, k.g0, k.g1);
    }
    vec3 density_gradient_cubic(vec3 idx) const {  // common.glsl:130-136
        Taps k = cubic_taps(idx);
        return vec3(cubic_fetch(vec3(k.dh0.x, k.h0.y, k.h0.z), vec3(k.dh1.x, k.h1.y, k.h1.z),
                                vec3(k.dg0.x, k.g0.y, k.g0.z), vec3(k.dg1.x, k.g1.y, k.g1.z)),
                    cubic_fetch(vec3(k.h0.x, k.dh0.y, k.h0.z), vec3(k.h1.x, k.dh1.y, k.h1.z),
                                vec3(k.g0.x, k.dg0.y, k.g0.z), vec3(k.g1.x, k.dg1.y, k.g1.z)),
                    cubic_fetch(vec3(k.h0.x, k.h0.y, k.dh0.z), vec3(k.h1.x, k.h1.y, k.dh1.z),
                                vec3(k.g0.x, k.g0.y, k.dg0.z), vec3(k.g1.x, k.g1.y, k.dg1.z)));
    }
    float density_view(vec3 idx) const {  // common.glsl:160-162
        return u.env.y > 0.5f ? density_cubic(idx) : density_at_index(idx);
    }
    vec4 transfer(float d) const {  // common.glsl:170-173
        return textureLod(t.tf, (d * (4096.0f - 1.0f) + 0.5f) / 4096.0f, 0.0f);
    }
    Sample tf_point(float d) const {  // common.glsl:188-191
        vec4 tf = transfer(d);
        return Sample{vec3(tf.x, tf.y, tf.z), tf.w, u.material.x, u.material.y, 0u, false, d, u.subsurface.x, 0.0f};
    }
    bool label_shown(uint l) const { return u.label_colors[l].w > 0.5f; }               // :232
    bool label_ghosted(uint l) const { return l != 0u && u.label_colors[l].w > 1.5f; }  // :236
    bool label_solid(uint l, uint mode) const {                                          // :242
        if (label_ghosted(l)) return false;
        return mode == 1u ? (l == 0u || label_shown(l)) : (l != 0u && label_shown(l));
    }
    // common.glsl:253-290
    Sample with_label(Sample s, uint label, uint mode, bool ghost) const {
        s.label = label;
        s.ghost = ghost;
        if (label == 0u) return s;
        vec4 color = u.label_colors[label];
        vec4 mat = u.label_materials[label];
        vec3 crgb(color.x, color.y, color.z);
        if (mode == 1u) {
            s.albedo = mix(s.albedo, crgb, u.labels.y);
        } else {
            s.albedo = crgb;
            s.extinction = u.labels.z;
            vec4 d = u.label_density[label];
            if (mode == 3u && !ghost && d.w > 0.0f) {
                s.extinction *= smoothstep(d.x, d.y, s.density);
                float tt = clamp((s.density - d.z) / d.w, -1.5f, 1.5f);
                s.albedo = clamp(s.albedo * (1.0f + 0.2f * tt), 0.0f, 1.0f);
                if (d.z > BONE_DENSITY) {
                    float thin = 1.0f - smoothstep(-1.5f, -0.5f, tt);
                    s.albedo *= mix(vec3(1.0f), vec3(0.92f, 0.6f, 0.5f), thin);
                }
            }
        }
        s.roughness = mat.x;
        s.metalness = mat.y;
        s.subsurface = mat.w;
        s.coat = mat.z;
        return s;
    }
    // common.glsl:302-324: nearest voxel, then the cell's 8 corners, then 12 axis
    // neighbours at distance 1 and 2.
    bool drawn_label_near(vec3 idx, uint mode, bool ghost, uint& label) const {
        ivec3 hi = ivec3(int(u.dims.x), int(u.dims.y), int(u.dims.z)) - 1;
        ivec3 nearest = clamp(ivec3(floor(idx + 0.5f)), ivec3(0), hi);
        ivec3 base = ivec3(floor(idx));
        for (int i = 0; i < 21; i++) {
            ivec3 c;
            if (i == 0) {
                c = nearest;
            } else if (i < 9) {
                c = base + ivec3((i - 1) & 1, ((i - 1) >> 1) & 1, (i - 1) >> 2);
            } else {
                int k = i - 9;
                ivec3 d(0);
                d[k % 3] = (k / 3 % 2 == 0 ? 1 : -1) * (k < 6 ? 1 : 2);
                c = nearest + d;
            }
            label = texelFetch(t.labels, clamp(c, ivec3(0), hi), 0).x;
            if (ghost ? label_ghosted(label) : label_solid(label, mode)) return true;
        }
        return false;
    }
    // common.glsl:326-351
    Sample apply_labels(Sample s, vec3 idx) const {
        uint mode = uint(u.labels.x);
        if (mode == 0u) return s;
        vec4 m = textureLod(t.mask, index_to_tex(idx), 0.0f);
        uint label;
        if (m.x < (mode == 3u ? 0.25f : 0.5f)) {
            if (m.y >= 0.5f && drawn_label_near(idx, mode, true, label)) return with_label(s, label, mode, true);
            s.extinction = 0.0f;
            return s;
        }
        if (drawn_label_near(idx, mode, false, label)) return with_label(s, label, mode, false);
        if (mode >= 2u) s.extinction = 0.0f;
        return s;
    }
    // common.glsl:357-373
    float clip_depth(vec3 idx, int& plane) const {
        plane = -1;
        uint count = u.clip.x;
        if (count == 0u) return -1e30f;
        bool all_planes = u.clip.y != 0u;
        float depth = all_planes ? 1e30f : -1e30f;
        for (uint i = 0u; i < count; i++) {
            vec4 cp = u.clip_planes[i];
            float d = dot(vec3(cp.x, cp.y, cp.z), idx) - cp.w;
            if (all_planes ? d < depth : d > depth) {
                depth = d;
                plane = int(i);
            }
        }
        return depth;
    }
    bool is_clipped(vec3 idx) const { int p; return clip_depth(idx, p) > 0.0f; }
    // common.glsl:385-391
    Sample sample_point(vec3 idx) const {
        Sample s = apply_labels(tf_point(density_at_index(idx)), idx);
        if (s.ghost || is_clipped(idx)) s.extinction = 0.0f;
        return s;
    }
    mat3 w2i3() const { return mat3(u.world_to_index); }
    // common.glsl:395-404
    vec3 mask_gradient(vec3 idx, int channel) const {
        vec3 g;
        for (int a = 0; a < 3; a++) {
            vec3 d(0.0f);
            d[a] = 1.0f;
            g[a] = textureLod(t.mask, index_to_tex(idx + d), 0.0f)[channel] -
                   textureLod(t.mask, index_to_tex(idx - d), 0.0f)[channel];
        }
        return transpose(w2i3()) * (0.5f * g);
    }
    // common.glsl:408-417
    vec2 intersect_volume(vec3 origin, vec3 dir) const {
        vec3 lo(-0.5f);
        vec3 hi = vec3(u.dims.x, u.dims.y, u.dims.z) - 0.5f;
        vec3 inv = 1.0f / dir;
        vec3 t0 = (lo - origin) * inv, t1 = (hi - origin) * inv;
        vec3 tmin = min(t0, t1), tmax = max(t0, t1);
        return vec2(max(max(tmin.x, tmin.y), max(tmin.z, 0.0f)), min(min(tmax.x, tmax.y), tmax.z));
    }
    // common.glsl:421-427
    float brick_majorant(vec3 idx) const {
        if (u.path.w == 0u) return 1e30f;
        ivec3 b = ivec3(floor((idx + 0.5f) / float(BRICK)));
        return texelFetch(t.majorant, clamp(b, ivec3(0), textureSize(t.majorant, 0) - 1), 0).x;
    }
    // common.glsl:430-436
    float brick_exit(vec3 idx, vec3 d_idx) const {
        vec3 lo = floor((idx + 0.5f) / float(BRICK)) * float(BRICK) - 0.5f;
        vec3 hi = lo + float(BRICK);
        vec3 d = mix(d_idx, vec3(1e-9f), equal(d_idx, vec3(0.0f)));
        vec3 t_far = max((lo - idx) / d, (hi - idx) / d);
        return max(min(t_far.x, min(t_far.y, t_far.z)), 0.0f);
    }
    // common.glsl:439-442
    vec3 camera_ray(vec2 px) const {
        vec2 ndc = vec2(px.x / float(u.flags.z), px.y / float(u.flags.w)) * 2.0f - 1.0f;
        return normalize(vec3(u.forward.x, u.forward.y, u.forward.z) + ndc.x * vec3(u.right.x, u.right.y, u.right.z) -
                         ndc.y * vec3(u.up.x, u.up.y, u.up.z));
    }
    vec3 background(vec3 dir) const {  // common.glsl:449-455
        if (u.lighting.w >= 1u) return vec3(0.0f);
        float tt = 0.5f + 0.5f * -dir.z;
        return mix(vec3(0.02f, 0.022f, 0.028f), vec3(0.08f, 0.085f, 0.1f), tt);
    }

    // ======================================================== shading.glsl
    static float ggx_distribution(float nh, float a2) {  // shading.glsl:4-7
        float denom = nh * nh * (a2 - 1.0f) + 1.0f;
        return a2 / (PI * denom * denom);
    }
    // shading.glsl:11-27
    static vec3 brdf(vec3 n, vec3 v, vec3 l, vec3 albedo, float roughness, float metalness, vec3& diffuse) {
        vec3 h = normalize(v + l);
        float nv = max(dot(n, v), 1e-4f), nl = max(dot(n, l), 1e-4f);
        float nh = max(dot(n, h), 0.0f), vh = max(dot(v, h), 0.0f);
        float a = max(roughness * roughness, 2e-3f);
        float d = ggx_distribution(nh, a * a);
        float k = a * 0.5f;
        float g = (nv / (nv * (1.0f - k) + k)) * (nl / (nl * (1.0f - k) + k));
        vec3 f0 = mix(vec3(0.028f), albedo, metalness);
        vec3 f = f0 + (1.0f - f0) * pow(1.0f - vh, 5.0f);
        vec3 specular = d * g * f / (4.0f * nv * nl);
        diffuse = (1.0f - f) * (1.0f - metalness) * albedo / PI;
        return specular;
    }
    static float coat_roughness(const Sample& s) { return clamp(0.5f * s.roughness, 0.1f, 0.25f); }  // :32
    static float smith(float nv, float nl, float a) {  // :37
        float k = a * 0.5f;
        return (nv / (nv * (1.0f - k) + k)) * (nl / (nl * (1.0f - k) + k));
    }
    // shading.glsl:45-58
    static vec3 brdf_coated(vec3 n, vec3 v, vec3 l, const Sample& s, vec3& diffuse) {
        vec3 specular = brdf(n, v, l, s.albedo, s.roughness, s.metalness, diffuse);
        if (s.coat <= 0.0f) return specular;
        vec3 h = normalize(v + l);
        float nv = max(dot(n, v), 1e-4f), nl = max(dot(n, l), 1e-4f);
        float a = coat_roughness(s) * coat_roughness(s);
        float f = s.coat * (0.02f + 0.98f * pow(1.0f - max(dot(v, h), 0.0f), 5.0f));
        float coat = ggx_distribution(max(dot(n, h), 0.0f), a * a) * smith(nv, nl, a) * f / (4.0f * nv * nl);
        diffuse *= 1.0f - f;
        return specular * (1.0f - f) + vec3(coat);
    }
    // shading.glsl:73-144
    float surface_frame(vec3 idx, const Sample& s, vec3 v, int cap_plane, float cut, float cap_depth,
                        vec3& n, float& surfaceness) const {
        uint label_mode = uint(u.labels.x);
        vec3 tex = index_to_tex(idx);
        vec4 nw = textureLod(t.normals, tex, 0.0f);
        vec3 nxyz(nw.x, nw.y, nw.z);
        float n_len = length(nxyz);
        n = n_len > 1e-3f ? nxyz / n_len : vec3(0.0f);
        surfaceness = nw.w;
        bool skin = s.label == SKIN_LABEL;
        if (u.env.y > 0.5f && n_len > 1e-3f && (!s.ghost || skin)) {
            vec3 gw = transpose(w2i3()) * density_gradient_cubic(idx);
            float len = length(gw);
            n = len > 1e-7f ? -gw / len : n;
        }
        bool hollow = u.label_density[s.label].w < 0.0f;
        if (skin) {
        } else if (!s.ghost && label_mode == 3u && !hollow) {
            vec3 g = mask_gradient(idx, 0);
            float g_len = length(g);
            vec3 mask_n = g_len > 1e-5f ? -g / g_len : n;
            vec3 blended = mix(mask_n, n, surfaceness);
            n = length(blended) > 1e-3f ? normalize(blended) : mask_n;
            surfaceness = max(surfaceness, clamp(g_len * 4.0f, 0.0f, 1.0f));
        } else if (!s.ghost && (label_mode >= 2u || (label_mode == 1u && textureLod(t.mask, tex, 0.0f).x < 0.98f))) {
            vec3 g = mask_gradient(idx, 0);
            float g_len = length(g);
            float mask_surface = clamp(g_len * 4.0f, 0.0f, 1.0f);
            if (label_mode >= 2u || mask_surface > surfaceness) {
                n = g_len > 1e-5f ? -g / g_len : n;
                surfaceness = label_mode >= 2u ? mask_surface : max(surfaceness, mask_surface);
            }
        }
        if (cap_plane >= 0 && !s.ghost && -cut < cap_depth) {
            vec4 cn = u.clip_normals[cap_plane];
            n = vec3(cn.x, cn.y, cn.z);
            surfaceness = 1.0f;
        }
        if (s.ghost) {
            vec3 g = mask_gradient(idx, 1);
            float g_len = length(g);
            if (!skin || n_len <= 1e-3f) n = g_len > 1e-5f ? -g / g_len : n;
            surfaceness = clamp(g_len * 4.0f, 0.0f, 1.0f);
            float edge_on = pow(1.0f - abs(dot(n, v)), 3.0f);
            return surfaceness * mix(u.labels.w, 1.0f, edge_on);
        }
        return 1.0f;
    }
    bool measured(const Sample& s) const {  // shading.glsl:147-149
        return u.labels.x >= 2.0f && s.label != 0u && !s.ghost && u.label_optics[s.label].w > 0.0f;
    }
    vec3 tissue_sigma(const Sample& s) const {  // shading.glsl:161-168
        vec4 o = u.label_optics[s.label];
        vec3 mu(o.x, o.y, o.z);
        mu = mix(vec3(mu.y), mu, u.env.w);
        mu /= 1.0f - clamp(u.env.z, 0.0f, 0.95f);
        mu *= min(1.0f, u.tissue.y / max(max(mu.x, max(mu.y, mu.z)), 1e-6f));
        float occupancy = clamp(s.extinction / max(u.labels.z, 1e-6f), 0.0f, 1.0f);
        return occupancy * mu;
    }
    // shading.glsl:175-185 (pcg3d)
    static vec3 hash3(ivec3 c) {
        uvec3 v = uvec3(c) * 1664525u + 1013904223u;
        v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
        v ^= v >> 16u;
        v.x += v.y * v.z; v.y += v.z * v.x; v.z += v.x * v.y;
        return vec3(v) * (1.0f / 4294967296.0f);
    }
    static float gradient_at(ivec3 corner, vec3 offset) { return dot(hash3(corner) * 2.0f - 1.0f, offset); }
    // shading.glsl:192-202
    static float gradient_noise(vec3 p) {
        ivec3 i = ivec3(floor(p));
        vec3 f = fract(p);
        vec3 w = f * f * f * (f * (f * 6.0f - 15.0f) + 10.0f);
        const ivec3 X(1, 0, 0), Y(0, 1, 0), Z(0, 0, 1);
        float x00 = mix(gradient_at(i, f), gradient_at(i + X, f - vec3(X)), w.x);
        float x10 = mix(gradient_at(i + Y, f - vec3(Y)), gradient_at(i + X + Y, f - vec3(X + Y)), w.x);
        float x01 = mix(gradient_at(i + Z, f - vec3(Z)), gradient_at(i + X + Z, f - vec3(X + Z)), w.x);
        float x11 = mix(gradient_at(i + Y + Z, f - vec3(Y + Z)), gradient_at(i + X + Y + Z, f - vec3(X + Y + Z)), w.x);
        return 1.7f * mix(mix(x00, x10, w.y), mix(x01, x11, w.y), w.z);
    }
    static float fbm(vec3 p) {  // shading.glsl:205-208
        return (gradient_noise(p) + 0.5f * gradient_noise(p * 2.03f + 17.1f) + 0.25f * gradient_noise(p * 4.07f + 31.7f)) /
               1.75f;
    }
    // shading.glsl:213-237
    static void cellular(vec3 p, float& nearest, float& border, ivec3& cell) {
        ivec3 i = ivec3(floor(p));
        vec3 f = fract(p);
        vec3 d1(8.0f), d2(8.0f);
        cell = i;
        for (int z = -1; z <= 1; z++)
            for (int y = -1; y <= 1; y++)
                for (int x = -1; x <= 1; x++) {
                    ivec3 c = i + ivec3(x, y, z);
                    vec3 d = vec3(float(x), float(y), float(z)) + hash3(c) - f;
                    if (dot(d, d) < dot(d1, d1)) {
                        d2 = d1; d1 = d; cell = c;
                    } else if (dot(d, d) < dot(d2, d2)) {
                        d2 = d;
                    }
                }
        nearest = length(d1);
        border = dot(0.5f * (d1 + d2), normalize(d2 - d1));
    }
    static float lobule_border(vec3 q, ivec3& lobule) {  // shading.glsl:242-248
        vec3 warp(gradient_noise(q * 1.7f), gradient_noise(q * 1.7f + 5.2f), gradient_noise(q * 1.7f + 9.4f));
        float nearest, border;
        cellular(q + 0.2f * warp, nearest, border, lobule);
        return border;
    }
    static float surface_height(vec3 p, vec4 params) {  // shading.glsl:252-261
        vec3 q = p / params.w;
        if (params.x > 1.5f) {
            ivec3 lobule;
            float bulge = smoothstep(0.0f, 0.35f, lobule_border(q, lobule));
            return 0.7f * bulge + 0.3f * fbm(q * 3.0f);
        }
        return 0.6f * fbm(q) + 0.4f * gradient_noise(q * 4.0f);
    }
    vec3 index_to_world(vec3 idx) const {  // shading.glsl:263-265
        vec4 c3 = u.world_to_index[3];
        return inverse(w2i3()) * (idx - vec3(c3.x, c3.y, c3.z));
    }
    bool textured(const Sample& s) const {  // shading.glsl:267-269
        return s.label != 0u && !s.ghost && u.label_surface[s.label].x > 0.5f;
    }
    // shading.glsl:273-324
    void apply_surface_texture(vec3 idx, Sample& s) const {
        if (!textured(s)) return;
        vec4 params = u.label_surface[s.label];
        float amount = params.y;
        vec3 p = index_to_world(idx);
        vec3 q = p / params.w;
        vec3 tint;
        float wet, rough;
        if (params.x > 1.5f) {
            float strength = min(1.0f, 5.0f * amount);
            ivec3 lobule;
            float border = lobule_border(q, lobule);
            float septum = (1.0f - smoothstep(0.0f, 0.06f, border)) * smoothstep(-0.7f, 0.3f, gradient_noise(q * 6.0f));
            float near_septum = 1.0f - smoothstep(0.0f, 0.2f, border);
            float patches = fbm(q * 1.5f);
            float mottle = fbm(q * 4.0f);
            tint = vec3(1.0f + amount * (hash3(lobule).x * 2.0f - 1.0f + 0.5f * mottle));
            tint *= mix(vec3(1.0f), vec3(0.84f, 0.78f, 0.88f), strength * smoothstep(-0.1f, 0.4f, -patches));
            tint *= mix(vec3(1.0f), vec3(0.6f, 0.57f, 0.66f), strength * septum);
            float nearest, unused;
            ivec3 speck;
            cellular(p / 3.0f, nearest, unused, speck);
            vec3 h = hash3(speck + 7919);
            float speck_mask = (h.x < 0.03f + 0.4f * near_septum ? 1.0f : 0.0f) *
                               (1.0f - smoothstep(0.12f, 0.2f, nearest / (0.6f + 0.8f * h.y)));
            tint *= mix(1.0f, 0.2f, strength * speck_mask);
            wet = 1.0f - 0.3f * near_septum;
            rough = 1.0f + 0.2f * mottle;
        } else {
            float patches = fbm(q);
            float grain = gradient_noise(q * 4.0f);
            tint = vec3(1.0f + amount * (0.7f * patches + 0.3f * grain));
            tint *= mix(vec3(1.0f), vec3(0.97f, 0.94f, 1.0f), clamp(-patches, 0.0f, 1.0f) * min(1.0f, 5.0f * amount));
            wet = clamp(0.8f + 0.4f * patches, 0.4f, 1.2f);
            rough = 1.0f + 0.3f * grain;
        }
        s.albedo = clamp(s.albedo * tint, 0.0f, 1.0f);
        s.roughness = clamp(s.roughness * rough, 0.02f, 1.0f);
        s.coat = clamp(s.coat * wet, 0.0f, 1.0f);
    }
    // shading.glsl:328-342
    vec3 bump_normal(vec3 idx, const Sample& s, vec3 n) const {
        if (!textured(s) || u.label_surface[s.label].z <= 0.0f || dot(n, n) < 0.5f) return n;
        vec4 params = u.label_surface[s.label];
        vec3 p = index_to_world(idx);
        float e = 0.02f * params.w;
        float h = surface_height(p, params);
        vec3 g = vec3(surface_height(p + vec3(e, 0.0f, 0.0f), params) - h,
                      surface_height(p + vec3(0.0f, e, 0.0f), params) - h,
                      surface_height(p + vec3(0.0f, 0.0f, e), params) - h) *
                 (params.z / e);
        return normalize(n - (g - dot(g, n) * n));
    }
};

// ================================================================ pt.comp
struct Tracer : Shading {
    uint state = 0;
    uint pcg() {  // pt.comp:44-49
        uint s = state;
        state = state * 747796405u + 2891336453u;
        uint word = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
        return (word >> 22u) ^ word;
    }
    float rand() { return float(pcg() >> 8) * (1.0f / 16777216.0f); }  // pt.comp:51-53

    vec3 fwd() const { return normalize(vec3(u.forward.x, u.forward.y, u.forward.z)); }
    vec3 rgt() const { return normalize(vec3(u.right.x, u.right.y, u.right.z)); }
    vec3 upv() const { return normalize(vec3(u.up.x, u.up.y, u.up.z)); }
    vec3 amb() const { return vec3(u.ambient.x, u.ambient.y, u.ambient.z); }
    vec3 lightdir() const { return vec3(u.light_dir.x, u.light_dir.y, u.light_dir.z); }

    // common.glsl:459-485: light map coordinates, directions and radiance.
    vec2 env_uv(vec3 d) const {
        vec3 f = fwd(), r = rgt(), up = upv();
        float phi = atan(dot(d, r), dot(d, f));
        float theta = acos(clamp(dot(d, up), -1.0f, 1.0f));
        return vec2(fract(0.5f + (phi + u.env.x) / (2.0f * PI)), theta / PI);
    }
    vec3 env_direction(vec2 uv) const {
        float phi = (uv.x - 0.5f) * 2.0f * PI - u.env.x;
        float theta = uv.y * PI;
        vec3 f = fwd(), r = rgt(), up = upv();
        return sin(theta) * (sin(phi) * r + cos(phi) * f) + cos(theta) * up;
    }
    vec3 env_map_radiance(vec3 d) const {
        vec4 c = textureLod(t.env, env_uv(d), 0.0f);
        return amb() * vec3(c.x, c.y, c.z);
    }

    // pt.comp:56-82
    vec3 environment(vec3 d) const {
        if (u.lighting.w == 2u) return env_map_radiance(d);
        if (u.lighting.w == 1u) {
            vec3 f = fwd(), r = rgt(), up = upv();
            float key_side = dot(lightdir(), r) >= 0.0f ? 1.0f : -1.0f;
            vec3 fill = normalize(-f - 0.9f * key_side * r - 0.1f * up);
            vec3 rim = normalize(f + 0.8f * up - 0.4f * key_side * r);
            float fill_lobe = 0.5f * pow(max(dot(d, fill), 0.0f), 6.0f);
            float rim_lobe = 2.5f * pow(max(dot(d, rim), 0.0f), 24.0f);
            vec3 studio = vec3(0.02f) + fill_lobe * vec3(0.95f, 0.98f, 1.05f) + rim_lobe * vec3(0.9f, 0.95f, 1.1f);
            return amb() * studio * (1.0f / 0.106f);
        }
        float up = 0.5f + 0.5f * d.z;
        vec3 sky(0.92f, 0.96f, 1.04f), ground(1.04f, 1.0f, 0.94f);
        return amb() * mix(ground * 0.35f, sky, up) / 0.675f;
    }
    static mat3 basis(vec3 n) {  // pt.comp:85-92
        float s = n.z >= 0.0f ? 1.0f : -1.0f;
        float a = -1.0f / (s + n.z);
        float b = n.x * n.y * a;
        return mat3(vec3(1.0f + s * n.x * n.x * a, s * b, -s * n.x), vec3(b, s + n.y * n.y * a, -n.y), n);
    }
    vec3 sample_light(const mat3& frame) {  // pt.comp:96-102
        float cos_max = cos(u.material.w);
        float cos_t = mix(cos_max, 1.0f, rand());
        float sin_t = sqrt(max(0.0f, 1.0f - cos_t * cos_t));
        float phi = 2.0f * PI * rand();
        return frame * vec3(sin_t * cos(phi), sin_t * sin(phi), cos_t);
    }
    static vec3 single_scattering_albedo(vec3 a) {  // pt.comp:119-123
        a = clamp(a, 0.0f, 0.999f);
        vec3 s = 4.09712f + 4.20863f * a - sqrt(9.59217f + 41.6808f * a + 17.7126f * a * a);
        return 1.0f - s * s;
    }
    vec3 chroma(const Sample& s) const {  // pt.comp:132-139
        if (s.ghost) return vec3(1.0f);
        return mix(vec3(1.0f), vec3(0.62f, 0.77f, 1.0f), clamp(2.0f * s.subsurface, 0.0f, 1.0f) * u.env.w);
    }
    vec3 path_sigma(const Sample& s, float ext) const {  // pt.comp:143-145
        return measured(s) ? tissue_sigma(s) : ext * chroma(s);
    }
    vec3 event_albedo(const Sample& s) const {  // pt.comp:150-153
        vec3 reduced = single_scattering_albedo(s.albedo);
        return measured(s) ? 1.0f - (1.0f - reduced) * (1.0f - clamp(u.env.z, 0.0f, 0.95f)) : reduced;
    }
    float flight_majorant(vec3 p) const {  // pt.comp:157-163
        float m = brick_majorant(p);
        if (m > 0.0f && u.labels.x >= 2.0f) m = max(m, u.tissue.x);
        return min(m, max(MAX_EXTINCTION, max(u.labels.z, u.tissue.x)));
    }
    float phase_hg(float cos_t) const {  // pt.comp:167-171
        float g = u.env.z;
        float d = 1.0f + g * g - 2.0f * g * cos_t;
        return (1.0f - g * g) / (4.0f * PI * d * sqrt(max(d, 1e-8f)));
    }
    vec3 sample_hg(vec3 dir) {  // pt.comp:173-185
        float g = u.env.z;
        float cos_t;
        if (abs(g) < 1e-3f) {
            cos_t = 1.0f - 2.0f * rand();
        } else {
            float q = (1.0f - g * g) / (1.0f - g + 2.0f * g * rand());
            cos_t = clamp((1.0f + g * g - q * q) / (2.0f * g), -1.0f, 1.0f);
        }
        float sin_t = sqrt(max(0.0f, 1.0f - cos_t * cos_t));
        float phi = 2.0f * PI * rand();
        return basis(dir) * vec3(sin_t * cos(phi), sin_t * sin(phi), cos_t);
    }
    static float mis(float a, float b) { return a * a / max(a * a + b * b, 1e-20f); }  // pt.comp:188-190
    static float coat_share(const Sample& s) { return 0.5f * s.coat; }                 // :237
    static float specular_share(const Sample& s) { return mix(0.2f, 1.0f, s.metalness); }  // :241
    static float ggx_pdf(vec3 n, vec3 v, vec3 l, float a) {  // pt.comp:246-250
        vec3 h = normalize(v + l);
        float nh = max(dot(n, h), 0.0f);
        return ggx_distribution(nh, a * a) * nh / (4.0f * max(dot(v, h), 1e-4f));
    }
    vec3 sample_ggx(const mat3& frame, vec3 v, float a) {  // pt.comp:252-260
        float a2 = a * a;
        float phi = 2.0f * PI * rand();
        float xi = rand();
        float cos_t = sqrt((1.0f - xi) / (1.0f + (a2 - 1.0f) * xi));
        float sin_t = sqrt(max(0.0f, 1.0f - cos_t * cos_t));
        vec3 h = frame * vec3(sin_t * cos(phi), sin_t * sin(phi), cos_t);
        return reflect(-v, h);
    }
    static float bsdf_pdf(vec3 n, vec3 v, vec3 l, const Sample& s) {  // pt.comp:263-273
        float nl = dot(n, l);
        if (nl <= 0.0f) return 0.0f;
        float a = max(s.roughness * s.roughness, 2e-3f);
        float share = specular_share(s);
        float base = share * ggx_pdf(n, v, l, a) + (1.0f - share) * nl / PI;
        float coat = coat_share(s);
        return coat * ggx_pdf(n, v, l, coat_roughness(s) * coat_roughness(s)) + (1.0f - coat) * base;
    }
    // pt.comp:277-292
    float extinction_at(vec3 idx, vec3 dir, bool smooth, Sample& s, int& cap_plane, float& cut) const {
        cut = clip_depth(idx, cap_plane);
        if (cut > 0.0f) return 0.0f;
        s = apply_labels(tf_point(smooth ? density_view(idx) : density_at_index(idx)), idx);
        if (s.extinction <= 0.0f) return 0.0f;
        if (s.ghost) {
            vec3 n;
            float surf;
            return s.extinction * surface_frame(idx, s, -dir, cap_plane, cut, 0.0f, n, surf);
        }
        return s.extinction;
    }
    // pt.comp:300-334: delta tracking with the hero channel.
    bool free_flight(vec3 origin, vec3 dir, bool smooth, int hero, vec3& spectral, vec3& idx, Sample& s,
                     int& cap_plane, float& cut) {
        vec3 d_idx = w2i3() * dir;
        vec2 tr = intersect_volume(origin, d_idx);
        float tt = tr.x;
        for (int i = 0; i < 4096 && tt < tr.y; i++) {
            vec3 p = origin + d_idx * tt;
            float majorant = flight_majorant(p);
            float exit = tt + brick_exit(p, d_idx) + 1e-3f;
            if (majorant <= 0.0f) { tt = exit; continue; }
            float next = tt - log(1.0f - rand()) / majorant;
            if (next >= exit) { tt = exit; continue; }
            tt = next;
            idx = origin + d_idx * tt;
            float ext = extinction_at(idx, dir, smooth, s, cap_plane, cut);
            if (ext <= 0.0f) continue;
            vec3 sigma = path_sigma(s, ext);
            if (rand() * majorant < sigma[hero]) {
                spectral *= sigma / sigma[hero];
                return true;
            }
            spectral *= max(majorant - sigma, 0.0f) / (majorant - sigma[hero]);
        }
        return false;
    }
    // pt.comp:193-200: solid-angle pdf of light map direction `d`.
    float env_pdf(vec3 d) const {
        ivec2 size = textureSize(t.env, 0);
        vec2 uv = env_uv(d);
        ivec2 texel = min(ivec2(int(uv.x * float(size.x)), int(uv.y * float(size.y))), size - 1);
        float p = texelFetch(t.env_table, texel, 0).y;
        return p * float(size.x * size.y) / (2.0f * PI * PI * max(sin(uv.y * PI), 1e-6f));
    }
    // pt.comp:204-233: a light map direction by luminance (binary searches of
    // the marginal and the row's conditional CDF).
    vec3 sample_env(float& pdf) {
        ivec2 size = textureSize(t.env, 0);
        float xi = rand();
        int lo = 0, hi = size.y - 1;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (texelFetch(t.env_table, ivec2(size.x, mid), 0).x >= xi) hi = mid;
            else lo = mid + 1;
        }
        int y = lo;
        xi = rand();
        lo = 0;
        hi = size.x - 1;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (texelFetch(t.env_table, ivec2(mid, y), 0).x >= xi) hi = mid;
            else lo = mid + 1;
        }
        float jx = rand();
        float jy = rand();
        vec2 uv = (vec2(float(lo), float(y)) + vec2(jx, jy)) / vec2(float(size.x), float(size.y));
        float p = texelFetch(t.env_table, ivec2(lo, y), 0).y;
        pdf = p * float(size.x * size.y) / (2.0f * PI * PI * max(sin(uv.y * PI), 1e-6f));
        return env_direction(uv);
    }

    // pt.comp:339-371: ratio tracking with Russian roulette.
    vec3 transmittance(vec3 origin, vec3 dir) {
        vec3 d_idx = w2i3() * dir;
        vec2 tr = intersect_volume(origin, d_idx);
        float tt = tr.x;
        vec3 result(1.0f);
        for (int i = 0; i < 4096 && tt < tr.y; i++) {
            float peak = max(result.x, max(result.y, result.z));
            if (peak < 0.1f) {
                if (rand() * 0.1f >= peak) return vec3(0.0f);
                result *= 0.1f / peak;
            }
            vec3 p = origin + d_idx * tt;
            float majorant = flight_majorant(p);
            float exit = tt + brick_exit(p, d_idx) + 1e-3f;
            if (majorant <= 0.0f) { tt = exit; continue; }
            float next = tt - log(1.0f - rand()) / majorant;
            if (next >= exit) { tt = exit; continue; }
            tt = next;
            Sample m = sample_point(origin + d_idx * tt);
            result *= max(1.0f - path_sigma(m, m.extinction) / majorant, 0.0f);
        }
        return result;
    }

    struct PixelResult { vec3 sum; float background; vec4 albedo_sum, normal_sum; };

    // pt.comp:373-553: `samples` paths through pixel (x, y), sharing one stream.
    PixelResult trace_pixel(uint px, uint py) {
        state = (px * 1973u + py * 9277u + u.path.x * 26699u) | 1u;
        pcg();
        uint samples = u.path.z, max_bounces = u.path.y;
        uint volume_limit = uint(float(MAX_VOLUME_EVENTS) / (1.0f - clamp(u.env.z, 0.0f, 0.95f)));
        float step_mm = u.dims.w;
        mat3 light_frame = basis(lightdir());
        vec3 light(u.light_dir.w);
        float cos_light = cos(u.material.w);
        bool area_light = u.material.w > 1e-4f;
        float light_pdf = area_light ? 1.0f / (2.0f * PI * (1.0f - cos_light)) : 0.0f;
        bool env_map = u.lighting.w == 2u;
        mat3 to_index = w2i3();
        vec4 e4 = u.world_to_index * vec4(u.eye.x, u.eye.y, u.eye.z, 1.0f);
        vec3 eye_idx(e4.x, e4.y, e4.z);
        PixelResult R{vec3(0.0f), 0.0f, vec4(0.0f), vec4(0.0f)};
        for (uint i = 0u; i < samples; i++) {
            float jx = rand();
            float jy = rand();
            vec3 dir = camera_ray(vec2(float(px), float(py)) + vec2(jx, jy));
            vec3 origin = eye_idx;
            if (u.lens.x > 0.0f) {
                vec3 eye(u.eye.x, u.eye.y, u.eye.z);
                vec3 focal = eye + dir * (u.lens.y / dot(dir, fwd()));
                float r = u.lens.x * sqrt(rand());
                float phi = 2.0f * PI * rand();
                eye += r * (cos(phi) * rgt() + sin(phi) * upv());
                dir = normalize(focal - eye);
                vec4 o4 = u.world_to_index * vec4(eye, 1.0f);
                origin = vec3(o4.x, o4.y, o4.z);
            }
            vec3 throughput(1.0f), radiance(0.0f);
            int hero = min(int(rand() * 3.0f), 2);
            vec3 spectral(1.0f);
            float last_pdf = 0.0f;
            for (uint bounce = 0u, surfaces = 0u, volumes = 0u; surfaces <= max_bounces && volumes <= volume_limit;
                 bounce++) {
                vec3 idx;
                Sample s;
                int cap_plane;
                float cut;
                if (!free_flight(origin, dir, bounce == 0u, hero, spectral, idx, s, cap_plane, cut)) {
                    if (bounce == 0u) {
                        R.background += 1.0f;
                        R.albedo_sum.x += 1.0f; R.albedo_sum.y += 1.0f; R.albedo_sum.z += 1.0f;
                        R.normal_sum.w += 1e4f;
                    } else {
                        vec3 path_weight = throughput * spectral / dot(spectral, vec3(1.0f / 3.0f));
                        float weight = env_map ? mis(last_pdf, env_pdf(dir)) : 1.0f;
                        radiance += path_weight * environment(dir) * weight;
                        if (area_light && dot(dir, lightdir()) >= cos_light)
                            radiance += path_weight * light * light_pdf * mis(last_pdf, light_pdf);
                    }
                    break;
                }
                vec3 path_weight = throughput * spectral / dot(spectral, vec3(1.0f / 3.0f));
                vec3 v = -dir;
                vec3 n;
                float surfaceness;
                surface_frame(idx, s, v, cap_plane, cut, 1.5f * step_mm, n, surfaceness);
                apply_surface_texture(idx, s);
                bool surface_event = rand() < surfaceness * (1.0f - s.subsurface) && dot(n, n) > 0.5f;
                if (surface_event || bounce == 0u) n = bump_normal(idx, s, n);
                if (bounce == 0u) {
                    R.albedo_sum += vec4(s.albedo, 0.0f);
                    R.normal_sum += vec4(dot(n, v) < 0.0f ? -n : n, length(idx - eye_idx));
                }
                vec3 light_dir = sample_light(light_frame);
                vec3 light_t = transmittance(idx, light_dir);
                float map_pdf = 0.0f;
                vec3 map_dir(0.0f), map_light(0.0f);
                if (env_map) {
                    map_dir = sample_env(map_pdf);
                    map_light = env_map_radiance(map_dir) / max(map_pdf, 1e-8f);
                    if (map_pdf > 0.0f) map_light *= transmittance(idx, map_dir);
                }
                if (surface_event) {
                    n = dot(n, v) < 0.0f ? -n : n;
                    vec3 diffuse;
                    vec3 specular = brdf_coated(n, v, light_dir, s, diffuse);
                    float light_weight = area_light ? mis(light_pdf, bsdf_pdf(n, v, light_dir, s)) : 1.0f;
                    radiance += path_weight * (diffuse + specular) * max(dot(n, light_dir), 0.0f) * light * light_t *
                                light_weight;
                    if (map_pdf > 0.0f && dot(n, map_dir) > 0.0f) {
                        specular = brdf_coated(n, v, map_dir, s, diffuse);
                        radiance += path_weight * (diffuse + specular) * dot(n, map_dir) * map_light *
                                    mis(map_pdf, bsdf_pdf(n, v, map_dir, s));
                    }
                    mat3 frame = basis(n);
                    vec3 l;
                    if (rand() < coat_share(s)) {
                        l = sample_ggx(frame, v, coat_roughness(s) * coat_roughness(s));
                    } else if (rand() < specular_share(s)) {
                        l = sample_ggx(frame, v, max(s.roughness * s.roughness, 2e-3f));
                    } else {
                        float r = sqrt(rand());
                        float phi = 2.0f * PI * rand();
                        l = frame * vec3(r * cos(phi), r * sin(phi), sqrt(max(0.0f, 1.0f - r * r)));
                    }
                    float nl = dot(n, l);
                    if (nl <= 0.0f) break;
                    float pdf = bsdf_pdf(n, v, l, s);
                    specular = brdf_coated(n, v, l, s, diffuse);
                    throughput *= (diffuse + specular) * nl / max(pdf, 1e-6f);
                    last_pdf = pdf;
                    surfaces++;
                    origin = idx + to_index * (n * step_mm);
                    dir = l;
                } else {
                    vec3 albedo = event_albedo(s);
                    float light_phase = phase_hg(dot(dir, light_dir));
                    radiance += path_weight * albedo * light_phase * light * light_t *
                                (area_light ? mis(light_pdf, light_phase) : 1.0f);
                    if (map_pdf > 0.0f) {
                        float phase = phase_hg(dot(dir, map_dir));
                        radiance += path_weight * albedo * phase * map_light * mis(map_pdf, phase);
                    }
                    throughput *= albedo;
                    volumes++;
                    origin = idx;
                    vec3 next = sample_hg(dir);
                    last_pdf = phase_hg(dot(dir, next));
                    dir = next;
                }
                if (bounce >= 2u) {
                    vec3 w = throughput * spectral / dot(spectral, vec3(1.0f / 3.0f));
                    float survive = clamp(max(w.x, max(w.y, w.z)), 0.05f, 1.0f);
                    if (rand() > survive) break;
                    throughput /= survive;
                }
            }
            float peak = max(radiance.x, max(radiance.y, radiance.z));
            radiance = peak > 20.0f ? radiance * (20.0f / peak) : radiance;
            R.sum += radiance;
            float lum = dot(radiance, vec3(0.2126f, 0.7152f, 0.0722f));
            R.albedo_sum.w += lum * lum;
        }
        return R;
    }
};

// ----------------------------------------------------------- volume passes

// normals.comp:14-37
void normals_pass(const Uniforms& u, const Scene& sc, int8_t* out, int threads) {
    Units t = bind_scene(sc);
    ivec3 D = sc.dims;
    mat3 wt = transpose(mat3(u.world_to_index));
    auto d = [&](ivec3 p) { return texelFetch(t.density, clamp(p, ivec3(0), D - 1), 0).x; };
    parallel_rows((long)D.y * D.z, threads, [&](long row) {
        int y = int(row % D.y), z = int(row / D.y);
        for (int x = 0; x < D.x; x++) {
            ivec3 p(x, y, z);
            vec3 g(0.0f);
            for (int a = -1; a <= 1; a++)
                for (int b = -1; b <= 1; b++) {
                    float w = float((2 - abs(a)) * (2 - abs(b)));
                    g.x += w * (d(p + ivec3(1, a, b)) - d(p + ivec3(-1, a, b)));
                    g.y += w * (d(p + ivec3(a, 1, b)) - d(p + ivec3(a, -1, b)));
                    g.z += w * (d(p + ivec3(a, b, 1)) - d(p + ivec3(a, b, -1)));
                }
            g /= 32.0f;
            vec3 gw = wt * g;
            float len = length(gw);
            vec3 n = len > 1e-7f ? -gw / len : vec3(0.0f);
            glsl::encode(out, glsl::RGBA8_SNORM, ((long)z * D.y + y) * D.x + x, vec4(n, clamp(len * 400.0f, 0.0f, 1.0f)));
        }
    });
}

// mask.comp:32-171: binary (or soft) masks, then the separable binomial blur.
struct MaskPass {
    const Uniforms& u;
    Shading sh;
    const Units& t;
    ivec3 D;
    int margin, radius;
    ivec4 soft;  // axes, flip bits | 8 = present
    sampler3D soft_dummy;

    static float soft_score(bool best, bool second, float m) {  // mask.comp:32-37
        const float CERTAIN = 4.0f;
        if (best == second) return best ? CERTAIN : -CERTAIN;
        return best ? min(m, CERTAIN) : -min(m, CERTAIN);
    }
    vec3 can() const { return vec3(float(D[soft.x]), float(D[soft.y]), float(D[soft.z])); }
    vec3 soft_coord(ivec3 p) const {  // mask.comp:40-50
        ivec3 grid = textureSize(t.soft, 0);
        vec3 c = can(), x;
        for (int a = 0; a < 3; a++) {
            float v = float(p[soft[a]]);
            x[a] = ((soft.w >> a) & 1) != 0 ? c[a] - 1.0f - v : v;
        }
        return x * (vec3(grid) - 1.0f) / max(c - 1.0f, vec3(1.0f));
    }
    bool soft_overridden(vec3 x) const { return texelFetch(t.soft, ivec3(round(x)), 0).w != 0u; }
    vec2 soft_masks(ivec3 p, vec3 x) const {  // mask.comp:62-100
        const float SIGMA_CT = 40.0f / 4095.0f, CERTAIN = 4.0f;
        ivec3 grid = textureSize(t.soft, 0);
        vec3 c = can();
        vec3 to_grid = (vec3(grid) - 1.0f) / max(c - 1.0f, vec3(1.0f));
        uint mode = uint(u.labels.x);
        float here = texelFetch(t.density, p, 0).x;
        ivec3 center = ivec3(round(x));
        vec2 sum(0.0f);
        float weights = 0.0f;
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    ivec3 node = clamp(center + ivec3(dx, dy, dz), ivec3(0), grid - 1);
                    vec3 d = vec3(node) - x;
                    float w_space = exp(-dot(d, d) / (2.0f * 0.6f * 0.6f));
                    vec3 cn = vec3(node) / to_grid;
                    vec3 v;
                    for (int a = 0; a < 3; a++) v[soft[a]] = ((soft.w >> a) & 1) != 0 ? c[a] - 1.0f - cn[a] : cn[a];
                    float there = textureLod(t.density, sh.index_to_tex(v), 0.0f).x;
                    float w_ct = exp(-(here - there) * (here - there) / (2.0f * SIGMA_CT * SIGMA_CT));
                    uvec4 q = texelFetch(t.soft, node, 0);
                    float m = float(q.z) / 16.0f;
                    vec2 score(soft_score(sh.label_solid(q.x, mode), sh.label_solid(q.y, mode), m),
                               soft_score(sh.label_ghosted(q.x), sh.label_ghosted(q.y), m));
                    float w = w_space * w_ct + 1e-6f * w_space;
                    sum += w * score;
                    weights += w;
                }
        vec2 s = sum / weights;
        return clamp(0.5f + s / (2.0f * CERTAIN), 0.0f, 1.0f);
    }
    bool label_removed(uint l) const { return l != 0u && (!sh.label_shown(l) || sh.label_ghosted(l)); }
    vec2 binary_masks(ivec3 p) const {  // mask.comp:107-138
        uint mode = uint(u.labels.x);
        uint label = texelFetch(t.labels, p, 0).x;
        vec2 m(float(sh.label_solid(label, mode)), float(sh.label_ghosted(label)));
        if ((soft.w & 8) != 0 && label < FIRST_CT_LABEL) {
            vec3 x = soft_coord(p);
            if (!soft_overridden(x)) m = soft_masks(p, x);
        }
        if (mode == 1u && margin > 0 && label == 0u) {
            for (int a = -margin; a <= margin && m.x > 0.0f; a++)
                for (int b = -margin; b <= margin && m.x > 0.0f; b++)
                    for (int c = -margin; c <= margin; c++) {
                        uint l = texelFetch(t.labels, clamp(p + ivec3(a, b, c), ivec3(0), D - 1), 0).x;
                        if (label_removed(l)) { m.x = 0.0f; break; }
                    }
        }
        return m;
    }
};

void mask_passes(const Uniforms& u, const Scene& sc, const uint8_t* soft_data, ivec3 soft_dims, ivec4 soft_push,
                 int margin, int radius, uint16_t* out_a, uint16_t* scratch_b, int threads) {
    Units t = bind_scene(sc);
    if (soft_data) bind3(t.soft, soft_data, glsl::RGBA8_UINT, soft_dims, glsl::NEAREST);
    else { static const uint8_t zero[4] = {0, 0, 0, 0}; bind3(t.soft, zero, glsl::RGBA8_UINT, ivec3(1), glsl::NEAREST); }
    MaskPass mp{u, Shading{u, t}, t, sc.dims, margin, radius, soft_push, {}};
    ivec3 D = sc.dims;
    long rows = (long)D.y * D.z;
    auto lin = [&](ivec3 p) { return ((long)p.z * D.y + p.y) * D.x + p.x; };
    const glsl::Format mf = mask_format_of(sc);  // the stored mask's format, in every pass
    parallel_rows(rows, threads, [&](long row) {
        int y = int(row % D.y), z = int(row / D.y);
        for (int x = 0; x < D.x; x++)
            glsl::encode(scratch_b, mf, lin(ivec3(x, y, z)), vec4(mp.binary_masks(ivec3(x, y, z)), 0.0f, 0.0f));
    });
    // Passes 1-3: blur along x (B -> A), y (A -> B), z (B -> A) (mask.comp:260-278).
    for (int pass = 1; pass <= 3; pass++) {
        const uint16_t* src = pass == 2 ? out_a : scratch_b;
        uint16_t* dst = pass == 2 ? scratch_b : out_a;
        std::vector<uint16_t> copy;  // the source is read while the destination is written
        parallel_rows(rows, threads, [&](long row) {
            int y = int(row % D.y), z = int(row / D.y);
            for (int x = 0; x < D.x; x++) {
                ivec3 p(x, y, z), axis(0);
                axis[pass - 1] = 1;
                vec2 sum(0.0f);
                float c = 1.0f;
                for (int j = 0; j <= 2 * radius; j++) {
                    ivec3 q = clamp(p + axis * (j - radius), ivec3(0), D - 1);
                    vec4 v = glsl::decode(src, mf, lin(q));
                    sum += c * vec2(v.x, v.y);
                    c = c * float(2 * radius - j) / float(j + 1);
                }
                sum /= exp2(float(2 * radius));
                glsl::encode(dst, mf, lin(p), vec4(sum, 0.0f, 0.0f));
            }
        });
    }
}

// majorant.comp:14-71
void majorant_pass(const Uniforms& u, const Scene& sc, float* out) {
    Units t = bind_scene(sc);
    ivec3 G = sc.brick_dims, D = sc.dims;
    uint mode = uint(u.labels.x);
    auto tf_max = [&](float lo, float hi) {
        int first = clamp(int(lo * 64.0f), 0, 63), last = clamp(int(hi * 64.0f), 0, 63);
        float m = 0.0f;
        for (int b = first; b <= last; b++) m = max(m, u.tf_bucket_max[b / 4][b % 4]);
        return m;
    };
    for (int bz = 0; bz < G.z; bz++)
        for (int by = 0; by < G.y; by++)
            for (int bx = 0; bx < G.x; bx++) {
                ivec3 b(bx, by, bz);
                ivec3 lo = max(b * BRICK - 2, ivec3(0));
                ivec3 hi = min(b * BRICK + BRICK + 1, D - 1);
                float dmin = 1.0f, dmax = 0.0f, mmax = 0.0f;
                for (int z = lo.z; z <= hi.z; z++)
                    for (int y = lo.y; y <= hi.y; y++)
                        for (int x = lo.x; x <= hi.x; x++) {
                            float d = texelFetch(t.density, ivec3(x, y, z), 0).x;
                            dmin = min(dmin, d);
                            dmax = max(dmax, d);
                            if (mode != 0u) {
                                vec4 m = texelFetch(t.mask, ivec3(x, y, z), 0);
                                mmax = max(mmax, max(m.x, m.y));
                            }
                        }
                float bound;
                if (mode == 0u) bound = tf_max(dmin, dmax);
                else if (mmax <= 0.0f) bound = 0.0f;
                else if (mode == 1u) bound = tf_max(dmin, dmax);
                else bound = u.labels.z;
                out[((long)bz * G.y + by) * G.x + bx] = bound;
            }
}

// One accumulate-frame of pt.comp over pixel rows [y0, y1) (pt.comp:554-560).
void pt_frame(const Uniforms& u, const Scene& sc, float* accum, float* albedo, float* normal, uint16_t* hdr,
              int y0, int y1, int threads) {
    Units t = bind_scene(sc);
    int W = int(u.flags.z);
    bool first = u.path.x == 0u;
    parallel_rows(y1 - y0, threads, [&](long r) {
        int y = y0 + int(r);
        Tracer tr{Shading{u, t}};
        for (int x = 0; x < W; x++) {
            Tracer::PixelResult R = tr.trace_pixel(uint(x), uint(y));
            long i = (long)y * W + x;
            vec4 acc = (first ? vec4(0.0f) : vec4(accum[4 * i], accum[4 * i + 1], accum[4 * i + 2], accum[4 * i + 3])) +
                       vec4(R.sum, R.background);
            vec4 alb = (first ? vec4(0.0f) : vec4(albedo[4 * i], albedo[4 * i + 1], albedo[4 * i + 2], albedo[4 * i + 3])) +
                       R.albedo_sum;
            vec4 nor = (first ? vec4(0.0f) : vec4(normal[4 * i], normal[4 * i + 1], normal[4 * i + 2], normal[4 * i + 3])) +
                       R.normal_sum;
            for (int c = 0; c < 4; c++) { accum[4 * i + c] = acc[c]; albedo[4 * i + c] = alb[c]; normal[4 * i + c] = nor[c]; }
            if (hdr) glsl::encode(hdr, glsl::RGBA16F, i, acc / float(u.path.x + u.path.z));
        }
    });
}

// pt.comp over a list of pixel rows (a bounded, spread-out sample of a frame).
void pt_rows(const Uniforms& u, const Scene& sc, float* accum, float* albedo, float* normal, uint16_t* hdr,
             const int* rows, int nrows, int threads) {
    Units t = bind_scene(sc);
    int W = int(u.flags.z);
    bool first = u.path.x == 0u;
    parallel_rows((long)nrows * W, threads, [&](long k) {
        int y = rows[k / W], x = int(k % W);
        Tracer tr{Shading{u, t}};
        Tracer::PixelResult R = tr.trace_pixel(uint(x), uint(y));
        long i = (long)y * W + x;
        vec4 acc = (first ? vec4(0.0f) : vec4(accum[4 * i], accum[4 * i + 1], accum[4 * i + 2], accum[4 * i + 3])) +
                   vec4(R.sum, R.background);
        for (int c = 0; c < 4; c++) {
            accum[4 * i + c] = acc[c];
            albedo[4 * i + c] = (first ? 0.0f : albedo[4 * i + c]) + R.albedo_sum[c];
            normal[4 * i + c] = (first ? 0.0f : normal[4 * i + c]) + R.normal_sum[c];
        }
        if (hdr) glsl::encode(hdr, glsl::RGBA16F, i, acc / float(u.path.x + u.path.z));
    });
}

// One path of pixel (x, y): the same stream as pt_frame's first sample.
void pt_pixel(const Uniforms& u, const Scene& sc, int x, int y, float out[12]) {
    Units t = bind_scene(sc);
    Tracer tr{Shading{u, t}};
    Tracer::PixelResult R = tr.trace_pixel(uint(x), uint(y));
    float v[12] = {R.sum.x, R.sum.y, R.sum.z, R.background, R.albedo_sum.x, R.albedo_sum.y, R.albedo_sum.z,
                   R.albedo_sum.w, R.normal_sum.x, R.normal_sum.y, R.normal_sum.z, R.normal_sum.w};
    std::memcpy(out, v, sizeof(v));
}

// One path each for a list of pixels (x, y pairs), in parallel: pt_pixel's
// result per pixel, at the uniforms' accumulation count.
void pt_pixels(const Uniforms& u, const Scene& sc, const int* pix, long n, float* out, int threads) {
    Units t = bind_scene(sc);
    parallel_rows(n, threads, [&](long i) {
        Tracer tr{Shading{u, t}};
        Tracer::PixelResult R = tr.trace_pixel(uint(pix[2 * i]), uint(pix[2 * i + 1]));
        float v[12] = {R.sum.x, R.sum.y, R.sum.z, R.background, R.albedo_sum.x, R.albedo_sum.y, R.albedo_sum.z,
                       R.albedo_sum.w, R.normal_sum.x, R.normal_sum.y, R.normal_sum.z, R.normal_sum.w};
        std::memcpy(out + 12 * i, v, sizeof(v));
    });
}

// Light map samples (pt.comp:204-233) from random-stream states: texel column
// and row (the draws replayed through the searches), pdf, direction.
void light_samples(const Uniforms& u, const Scene& sc, const uint32_t* seeds, long n, float* out) {
    Units t = bind_scene(sc);
    Tracer tr{Shading{u, t}};
    ivec2 size = textureSize(t.env, 0);
    for (long i = 0; i < n; i++) {
        tr.state = seeds[i];
        float xi = tr.rand();
        int y = 0;
        while (y < size.y - 1 && !(texelFetch(t.env_table, ivec2(size.x, y), 0).x >= xi)) y++;
        xi = tr.rand();
        int x = 0;
        while (x < size.x - 1 && !(texelFetch(t.env_table, ivec2(x, y), 0).x >= xi)) x++;
        tr.state = seeds[i];
        float pdf;
        vec3 d = tr.sample_env(pdf);
        float v[6] = {float(x), float(y), pdf, d.x, d.y, d.z};
        std::memcpy(out + 6 * i, v, sizeof(v));
    }
}

// Cubic B-spline density and gradient at continuous voxel indices (common.glsl:124-136).
void bspline(const Uniforms& u, const Scene& sc, const float* idx, long n, float* out) {
    Units t = bind_scene(sc);
    Shading sh{u, t};
    for (long i = 0; i < n; i++) {
        vec3 p(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]);
        float v = sh.density_cubic(p);
        vec3 g = sh.density_gradient_cubic(p);
        out[4 * i] = v; out[4 * i + 1] = g.x; out[4 * i + 2] = g.y; out[4 * i + 3] = g.z;
    }
}

// The extinction a flight samples at continuous indices idx[3n] (pt.comp:277-292
// with path_sigma, pt.comp:143-145) and the flight majorant of the brick there
// (pt.comp:157-163): out[4n] = sigma (rgb), majorant. `smooth` selects the
// first flight's B-spline density; dir is the flight's direction.
void extinction_probe(const Uniforms& u, const Scene& sc, const float* idx, long n, const float dir[3], int smooth,
                      float* out, int threads) {
    Units t = bind_scene(sc);
    parallel_rows(n, threads, [&](long i) {
        Tracer tr{Shading{u, t}};
        vec3 p(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]);
        Sample s;
        int cap = -1;
        float cut = 0.0f;
        float ext = tr.extinction_at(p, vec3(dir[0], dir[1], dir[2]), smooth != 0, s, cap, cut);
        vec3 sigma = ext > 0.0f ? tr.path_sigma(s, ext) : vec3(0.0f);
        float v[4] = {sigma.x, sigma.y, sigma.z, tr.flight_majorant(p)};
        std::memcpy(out + 4 * i, v, sizeof(v));
    });
}

// ================================================================ denoise.comp
static float lum(vec3 c) { return dot(c, vec3(0.2126f, 0.7152f, 0.0722f)); }

// All passes of record_denoise (renderer.rs:1868-1904; denoise.comp:53-145):
// prepare, 5 a-trous levels with steps 1..16, finish into the HDR image.
void denoise(const Uniforms& u, const float* accum, const float* albedo, const float* normal, uint16_t* hdr,
             float* ping, float* pong, int threads) {
    int W = int(u.flags.z), H = int(u.flags.w);
    float n = float(u.path.x + u.path.z);
    auto at = [&](const float* img, ivec2 p) {
        long i = (long)p.y * W + p.x;
        return vec4(img[4 * i], img[4 * i + 1], img[4 * i + 2], img[4 * i + 3]);
    };
    auto put = [&](float* img, ivec2 p, vec4 v) {
        long i = (long)p.y * W + p.x;
        for (int c = 0; c < 4; c++) img[4 * i + c] = v[c];
    };
    auto mean_albedo = [&](ivec2 p) { vec4 a = at(albedo, p); return max(vec3(a.x, a.y, a.z) / n, vec3(0.02f)); };
    auto mean_normal_depth = [&](ivec2 p) {
        vec4 g = at(normal, p) / n;
        vec3 gx(g.x, g.y, g.z);
        float len = length(gx);
        return vec4(len > 1e-3f ? gx / len : vec3(0.0f), g.w);
    };
    ivec2 size(W, H);
    parallel_rows(H, threads, [&](long y) {
        for (int x = 0; x < W; x++) {
            ivec2 p(x, int(y));
            vec4 a = at(accum, p);
            vec3 radiance = vec3(a.x, a.y, a.z) / n;
            vec3 irradiance = radiance / mean_albedo(p);
            float l = lum(radiance);
            float temporal = max(at(albedo, p).w / n - l * l, 0.0f) / n;
            float s1 = 0.0f, s2 = 0.0f;
            for (int dy = -2; dy <= 2; dy++)
                for (int dx = -2; dx <= 2; dx++) {
                    ivec2 q = clamp(p + ivec2(dx, dy), ivec2(0), size - 1);
                    vec4 aq = at(accum, q);
                    float lq = lum(vec3(aq.x, aq.y, aq.z) / n);
                    s1 += lq;
                    s2 += lq * lq;
                }
            float spatial = max(s2 / 25.0f - (s1 / 25.0f) * (s1 / 25.0f), 0.0f);
            float variance = max(temporal, spatial * min(1.0f, 4.0f / n));
            float al = lum(mean_albedo(p));
            put(ping, p, vec4(irradiance, variance / (al * al)));
        }
    });
    const float kernel[3] = {3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
    for (int level = 0; level < 5; level++) {
        bool from_pong = level % 2 != 0;
        const float* src = from_pong ? pong : ping;
        float* dst = from_pong ? ping : pong;
        int stp = 1 << level;
        parallel_rows(H, threads, [&](long y) {
            for (int x = 0; x < W; x++) {
                ivec2 p(x, int(y));
                vec4 center = at(src, p);
                vec4 geometry = mean_normal_depth(p);
                vec3 gxyz(geometry.x, geometry.y, geometry.z);
                vec3 alb = mean_albedo(p);
                float l_center = lum(vec3(center.x, center.y, center.z));
                float bv = 0.0f;
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        ivec2 q = clamp(p + ivec2(dx, dy), ivec2(0), size - 1);
                        bv += at(src, q).w * float((2 - abs(dx)) * (2 - abs(dy))) / 16.0f;
                    }
                float sigma_l = 4.0f * sqrt(max(bv, 0.0f)) + 1e-4f;
                vec3 sum(0.0f);
                float variance = 0.0f, weights = 0.0f;
                for (int dy = -2; dy <= 2; dy++)
                    for (int dx = -2; dx <= 2; dx++) {
                        ivec2 q = p + ivec2(dx, dy) * stp;
                        if (any(lessThan(q, ivec2(0))) || any(greaterThanEqual(q, size))) continue;
                        vec4 c = at(src, q);
                        vec4 g = mean_normal_depth(q);
                        vec3 gq(g.x, g.y, g.z);
                        float w_normal = pow(max(dot(gxyz, gq), 0.0f), 64.0f);
                        if (dot(gxyz, gxyz) < 0.5f || dot(gq, gq) < 0.5f)
                            w_normal = float(dot(gxyz, gxyz) < 0.5f && dot(gq, gq) < 0.5f);
                        float w_depth = exp(-abs(geometry.w - g.w) / (0.02f * geometry.w + 1e-3f));
                        vec3 da = alb - mean_albedo(q);
                        float w_albedo = exp(-dot(da, da) / 0.01f);
                        float w_lum = exp(-abs(l_center - lum(vec3(c.x, c.y, c.z))) / sigma_l);
                        float w = kernel[abs(dx)] * kernel[abs(dy)] * w_normal * w_depth * w_albedo * w_lum;
                        sum += w * vec3(c.x, c.y, c.z);
                        variance += w * w * c.w;
                        weights += w;
                    }
                vec4 filtered = weights > 0.0f ? vec4(sum / weights, variance / (weights * weights)) : center;
                put(dst, p, filtered);
            }
        });
    }
    // Finish: 5 levels end in pong (level 4 reads ping) (renderer.rs:1902).
    const float* last = pong;
    parallel_rows(H, threads, [&](long y) {
        for (int x = 0; x < W; x++) {
            ivec2 p(x, int(y));
            vec4 c = at(last, p);
            float bg = at(accum, p).w / n;
            glsl::encode(hdr, glsl::RGBA16F, (long)y * W + x, vec4(vec3(c.x, c.y, c.z) * mean_albedo(p), bg));
        }
    });
}

// ===================================================== bloom.comp, tonemap.comp
// record_post (renderer.rs:1817-1866): bloom passes 0-6 (pass 1 is the
// auto-exposure metering, one workgroup of 64 invocations), then tone mapping.
// `exposure` is the adapted exposure texel, read and updated.
void post(const Uniforms& u, const uint16_t* hdr, float* exposure, uint8_t* out) {
    int W = int(u.flags.z), H = int(u.flags.w);
    int qw = (W + 3) / 4, qh = (H + 3) / 4, ew = (qw + 1) / 2, eh = (qh + 1) / 2;
    std::vector<uint16_t> A(4 * qw * qh), B(4 * qw * qh), Cc(4 * ew * eh), D(4 * ew * eh);
    auto ld = [](const uint16_t* img, int w, int x, int y) { return glsl::decode(img, glsl::RGBA16F, (long)y * w + x); };
    auto st = [](uint16_t* img, int w, int x, int y, vec4 v) { glsl::encode(img, glsl::RGBA16F, (long)y * w + x, v); };
    // Pass 0 (bloom.comp:333-351)
    for (int y = 0; y < qh; y++)
        for (int x = 0; x < qw; x++) {
            vec3 sum(0.0f);
            float weights = 0.0f, coverage = 0.0f;
            for (int dy = 0; dy < 4; dy++)
                for (int dx = 0; dx < 4; dx++) {
                    vec4 h = ld(hdr, W, min(x * 4 + dx, W - 1), min(y * 4 + dy, H - 1));
                    float w = 1.0f / (1.0f + lum(vec3(h.x, h.y, h.z)));
                    sum += vec3(h.x, h.y, h.z) * w;
                    weights += w;
                    coverage += 1.0f - h.w;
                }
            st(A.data(), qw, x, y, vec4(sum / weights, coverage / 16.0f));
        }
    // Pass 1 (bloom.comp:294-327): 64 partial sums, then the tree reduction.
    {
        float ls[64], ws[64];
        int n = qw * qh;
        for (int t = 0; t < 64; t++) {
            float s = 0.0f, w = 0.0f;
            for (int i = t; i < n; i += 64) {
                vec4 c = ld(A.data(), qw, i % qw, i / qw);
                s += c.w * log(max(lum(vec3(c.x, c.y, c.z)), 1e-4f));
                w += c.w;
            }
            ls[t] = s;
            ws[t] = w;
        }
        for (int stride = 32; stride > 0; stride >>= 1)
            for (int t = 0; t < stride; t++) {
                ls[t] += ls[t + stride];
                ws[t] += ws[t + stride];
            }
        float target = ws[0] > 1.0f ? clamp(0.24f / exp(ls[0] / ws[0]), 0.25f, 4.0f) : 1.0f;
        float previous = *exposure;
        *exposure = previous <= 0.0f ? target : exp(mix(log(previous), log(target), 0.15f));
    }
    // Passes 2-6 (bloom.comp:276-285, 352-367)
    const float k[5] = {0.2270f, 0.1945f, 0.1216f, 0.0540f, 0.0162f};
    auto blur = [&](const uint16_t* src, uint16_t* dst, int w, int h, int ax, int ay) {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                vec4 s = ld(src, w, x, y) * k[0];
                for (int i = 1; i < 5; i++)
                    s += k[i] * (ld(src, w, clamp(x + ax * i, 0, w - 1), clamp(y + ay * i, 0, h - 1)) +
                                 ld(src, w, clamp(x - ax * i, 0, w - 1), clamp(y - ay * i, 0, h - 1)));
                st(dst, w, x, y, s);
            }
    };
    blur(A.data(), B.data(), qw, qh, 1, 0);
    blur(B.data(), A.data(), qw, qh, 0, 1);
    for (int y = 0; y < eh; y++)
        for (int x = 0; x < ew; x++) {
            vec4 s(0.0f);
            for (int i = 0; i < 4; i++) s += ld(A.data(), qw, min(x * 2 + (i & 1), qw - 1), min(y * 2 + (i >> 1), qh - 1));
            st(Cc.data(), ew, x, y, s * 0.25f);
        }
    blur(Cc.data(), D.data(), ew, eh, 1, 0);
    blur(D.data(), Cc.data(), ew, eh, 0, 1);
    // tonemap.comp:47-85
    sampler2D narrow, wide;
    narrow.data = A.data(); narrow.format = glsl::RGBA16F; narrow.w = qw; narrow.h = qh; narrow.filter = glsl::LINEAR;
    wide.data = Cc.data(); wide.format = glsl::RGBA16F; wide.w = ew; wide.h = eh; wide.filter = glsl::LINEAR;
    const mat3 inset(0.842479062253094f, 0.0423282422610123f, 0.0423756549057051f, 0.0784335999999992f,
                     0.878468636469772f, 0.0784336f, 0.0792237451477643f, 0.0791661274605434f, 0.879142973793104f);
    const mat3 outset(1.19687900512017f, -0.0528968517574562f, -0.0529716355144438f, -0.0980208811401368f,
                      1.15190312990417f, -0.0980434501171241f, -0.0990297440797205f, -0.0989611768448433f,
                      1.15107367264116f);
    auto agx = [&](vec3 c) {
        const float min_ev = -12.47393f, max_ev = 4.026069f;
        c = inset * c;
        c = clamp(log2(max(c, 1e-10f)), min_ev, max_ev);
        c = (c - min_ev) / (max_ev - min_ev);
        vec3 c2 = c * c, c4 = c2 * c2;
        c = 15.5f * c4 * c2 - 40.14f * c4 * c + 31.96f * c4 - 6.868f * c2 * c + 0.4298f * c2 + 0.1191f * c - 0.00232f;
        c = outset * c;
        return pow(clamp(c, 0.0f, 1.0f), vec3(2.2f));
    };
    auto aces = [](vec3 x) { return clamp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f); };
    auto hash01 = [](uint v) {
        uint state = v * 747796405u + 2891336453u;
        uint word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
        return float((word >> 22u) ^ word) * (1.0f / 4294967296.0f);
    };
    Units none;
    Shading sh{u, none};
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            vec4 h = ld(hdr, W, x, y);
            float e = u.ambient.w;
            if (u.finish.w > 0.5f) e *= *exposure;
            vec3 c(h.x, h.y, h.z);
            vec2 uv = (vec2(float(x), float(y)) + 0.5f) / vec2(float(W), float(H));
            if (u.finish.x > 0.0f) {
                vec4 a = textureLod(narrow, uv, 0.0f), b = textureLod(wide, uv, 0.0f);
                vec3 glow = 0.6f * vec3(a.x, a.y, a.z) + 0.4f * vec3(b.x, b.y, b.z);
                c = mix(c, glow, u.finish.x);
            }
            float r = length(uv * 2.0f - 1.0f) * 0.7071f;
            float vignette = 1.0f - u.finish.y * pow(r, 2.5f);
            c *= e * vignette;
            uint op = uint(u.material.z);
            c = op == 1u ? aces(c) : op == 2u ? agx(c) : clamp(c, 0.0f, 1.0f);
            c += h.w * sh.background(sh.camera_ray(vec2(float(x), float(y)) + 0.5f));
            if (u.flags.y != 0u) {
                vec3 cc = clamp(c, 0.0f, 1.0f);
                c = mix(12.92f * cc, 1.055f * pow(cc, vec3(1.0f / 2.4f)) - 0.055f, step(0.0031308f, cc));
            }
            if (u.finish.z > 0.0f) {
                float nn = hash01(uint(x) + 4099u * uint(y)) + hash01(uint(x) * 7919u + uint(y) + 1u) - 1.0f;
                float yl = clamp(dot(c, vec3(0.2126f, 0.7152f, 0.0722f)), 0.0f, 1.0f);
                c = clamp(c + nn * u.finish.z * (0.3f + 2.8f * yl * (1.0f - yl)), 0.0f, 1.0f);
            }
            glsl::encode(out, glsl::RGBA8_UNORM, (long)y * W + x, vec4(c, 1.0f));
        }
}

}  // namespace vvo
