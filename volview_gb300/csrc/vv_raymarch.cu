// vv_raymarch.cu — the real-time ray marcher `record` runs when path tracing is
// off (renderer.rs:1707-1790): the ambient-occlusion volume (shaders/ao.comp),
// the shadow volume swept slice by slice away from the key light
// (shaders/shadow.comp, renderer.rs:1907-1950), and emission-absorption ray
// marching with single scattering (shaders/dvr.comp) into the HDR image.
//
// The lighting volumes are pixel-linear (x fastest) half-precision images at
// half (shadow, RGBA16F) and a quarter (occlusion, R16F) of the CT's resolution,
// sampled with linear filtering and a white border like the reference's border
// sampler. The scene's volumes, labels, tables and the sample model are the
// path tracer's (vv_pt_device.cuh).
#include <cuda_runtime.h>

#include "vv_pt_device.cuh"

namespace vv {
namespace VV_FMT_NS {  // this density format's kernels and launchers
namespace {

__device__ __forceinline__ float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }
__device__ __forceinline__ uint16_t f2h(float f) { return __half_as_ushort(__float2half_rn(f)); }
__device__ __forceinline__ float comp3(f3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ void set3(f3& v, int i, float s) {
    if (i == 0) v.x = s;
    else if (i == 1) v.y = s;
    else v.z = s;
}

// common.glsl:68-74
__device__ __forceinline__ f3 index_to_tex(const PtArgs& A, f3 idx) { return (idx + 0.5f) / U3(A.u.dims); }
__device__ __forceinline__ f3 tex_to_index(const PtArgs& A, f3 tex) { return tex * U3(A.u.dims) - 0.5f; }

// common.glsl:385-391: a shadow-ray sample (ghosts and clipped parts cast no shadow).
__device__ Sample sample_point(const PtArgs& A, f3 idx) {
    Sample s = apply_labels(A, tf_point(A, density_tri(A, idx)), idx);
    int plane;
    if (s.ghost || clip_depth(A, idx, plane) > 0.0f) s.extinction = 0.0f;
    return s;
}

// common.glsl:160-162
__device__ __forceinline__ float density_view(const PtArgs& A, f3 idx) {
    return A.u.env[1] > 0.5f ? density_cubic(A, idx) : density_tri(A, idx);
}

// common.glsl:195-199: the cumulative integrals, interpolated by hand.
__device__ __forceinline__ float4 preint_at(const PtArgs& A, float density) {
    float x = gclamp(density, 0.0f, 1.0f) * 4095.0f;
    int i = min((int)x, 4094);
    float4 a = __ldg(A.preint + i), b = __ldg(A.preint + i + 1);
    float f = x - (float)i;
    return make_float4(mixf(a.x, b.x, f), mixf(a.y, b.y, f), mixf(a.z, b.z, f), mixf(a.w, b.w, f));
}

// common.glsl:206-214: the pre-integrated sample of a segment from `front` to `back`.
__device__ __noinline__ Sample tf_segment(const PtArgs& A, float front, float back) {
    if (fabsf(back - front) < 1e-4f) return tf_point(A, 0.5f * (front + back));
    float4 pb = preint_at(A, back), pf = preint_at(A, front);
    float d = back - front;
    float4 mean = make_float4((pb.x - pf.x) / d, (pb.y - pf.y) / d, (pb.z - pf.z) / d, (pb.w - pf.w) / d);
    f3 albedo;
    if (mean.w > 1e-6f) {
        albedo = mk(mean.x / mean.w, mean.y / mean.w, mean.z / mean.w);
    } else {
        float4 t = transfer(A, back);
        albedo = mk(t.x, t.y, t.z);
    }
    Sample s = tf_point(A, back);
    s.albedo = albedo;
    s.extinction = gmax(mean.w, 0.0f);
    return s;
}

// common.glsl:218-230
__device__ __noinline__ float preint_half_depth(const PtArgs& A, float front, float back) {
    float target = 0.5f * (preint_at(A, front).w + preint_at(A, back).w);
    float lo = 0.0f, hi = 1.0f;
    for (int i = 0; i < 6; i++) {
        float mid = 0.5f * (lo + hi);
        bool before = (preint_at(A, mixf(front, back, mid)).w < target) == (back > front);
        lo = before ? mid : lo;
        hi = before ? hi : mid;
    }
    return 0.5f * (lo + hi);
}

// dvr.comp:14-21: labels applied, measured tissue as dense as the path tracer draws it.
__device__ __noinline__ Sample labelled(const PtArgs& A, Sample s, f3 idx) {
    s = apply_labels(A, s, idx);
    if (measured(A, s)) s.extinction = dot(tissue_sigma(A, s), mk(1.0f / 3.0f));
    return s;
}

// shading.glsl:61-63: interleaved gradient noise.
__device__ __forceinline__ float ign(float px, float py) {
    float a = px * 0.06711056f + py * 0.00583715f;
    float b = 52.9829189f * (a - floorf(a));
    return b - floorf(b);
}

// A lighting volume, sampled as the border sampler does: linear between texel
// centres, texels outside the volume white (1, 1, 1, 1).
struct LightVol {
    const uint16_t* data;  // `channels` halves per texel, x fastest
    int w, h, d, channels;
};
__device__ __forceinline__ float4 lv_texel(const LightVol& v, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0 || x >= v.w || y >= v.h || z >= v.d) return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    long i = ((long)z * v.h + y) * v.w + x;
    if (v.channels == 1) return make_float4(h2f(__ldg(v.data + i)), 0.0f, 0.0f, 1.0f);
    ushort4 t = __ldg((const ushort4*)v.data + i);
    return make_float4(h2f(t.x), h2f(t.y), h2f(t.z), h2f(t.w));
}
__device__ float4 lv_linear(const LightVol& v, f3 tc) {
    float x = tc.x * (float)v.w - 0.5f, y = tc.y * (float)v.h - 0.5f, z = tc.z * (float)v.d - 0.5f;
    int i0 = (int)floorf(x), j0 = (int)floorf(y), k0 = (int)floorf(z);
    float a = x - (float)i0, b = y - (float)j0, c = z - (float)k0;
    float4 r = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
                float w = (di ? a : 1.0f - a) * (dj ? b : 1.0f - b) * (dk ? c : 1.0f - c);
                float4 t = lv_texel(v, i0 + di, j0 + dj, k0 + dk);
                r.x += t.x * w;
                r.y += t.y * w;
                r.z += t.z * w;
                r.w += t.w * w;
            }
    return r;
}
__device__ __forceinline__ float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4mul(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }

// A linear fetch of a lighting texture at texel-space position p (texel i's
// centre at i; the border texel sits at -1 and w).
__device__ __forceinline__ float4 lt_fetch(const LightTex& v, float x, float y, float z) {
    if (v.rgba) return tex3D<float4>(v.tex, x + 1.5f, y + 1.5f, z + 1.5f);
    return make_float4(tex3D<float>(v.tex, x + 1.5f, y + 1.5f, z + 1.5f), 0.0f, 0.0f, 1.0f);
}
__device__ __forceinline__ float4 lt_linear(const LightTex& v, f3 tc) {
    return lt_fetch(v, tc.x * (float)v.w - 0.5f, tc.y * (float)v.h - 0.5f, tc.z * (float)v.d - 0.5f);
}
// common.glsl:141-152: B-spline filtering from 8 linear fetches (folded taps of
// common.glsl:89-108).
__device__ __noinline__ float4 lt_cubic(const LightTex& v, f3 tc) {
    f3 size = mk((float)v.w, (float)v.h, (float)v.d);
    f3 idx = tc * size - 0.5f;
    f3 i = mk(floorf(idx.x), floorf(idx.y), floorf(idx.z));
    f3 f = idx - i, f2 = f * f, f3v = f2 * f;
    f3 w0 = (1.0f - 3.0f * f + 3.0f * f2 - f3v) / 6.0f;
    f3 w1 = (4.0f - 6.0f * f2 + 3.0f * f3v) / 6.0f;
    f3 w2 = (1.0f + 3.0f * f + 3.0f * f2 - 3.0f * f3v) / 6.0f;
    f3 w3 = f3v / 6.0f;
    f3 g0 = w0 + w1, g1 = w2 + w3;
    f3 a = i - 1.0f + w1 / g0, b = i + 1.0f + w3 / g1;  // the folded taps, in texels
    float4 z0 = f4add(f4mul(g0.y, f4add(f4mul(g0.x, lt_fetch(v, a.x, a.y, a.z)), f4mul(g1.x, lt_fetch(v, b.x, a.y, a.z)))),
                      f4mul(g1.y, f4add(f4mul(g0.x, lt_fetch(v, a.x, b.y, a.z)), f4mul(g1.x, lt_fetch(v, b.x, b.y, a.z)))));
    float4 z1 = f4add(f4mul(g0.y, f4add(f4mul(g0.x, lt_fetch(v, a.x, a.y, b.z)), f4mul(g1.x, lt_fetch(v, b.x, a.y, b.z)))),
                      f4mul(g1.y, f4add(f4mul(g0.x, lt_fetch(v, a.x, b.y, b.z)), f4mul(g1.x, lt_fetch(v, b.x, b.y, b.z)))));
    return f4add(f4mul(g0.z, z0), f4mul(g1.z, z1));
}
// common.glsl:154-157
__device__ __forceinline__ float4 lighting_lookup(const PtArgs& A, const LightTex& v, f3 tc) {
    return A.u.env[1] > 0.5f ? lt_cubic(v, tc) : lt_linear(v, tc);
}

// common.glsl:483-486: cosine-weighted mean light map radiance around `n`
// (32 x 16 RGBA16F, linear, clamped to the edge).
__device__ __noinline__ f3 env_map_diffuse(const PtArgs& A, f3 n) {
    float2 uv = env_uv(A, n);
    const int W = 32, H = 16;
    float x = uv.x * (float)W - 0.5f, y = uv.y * (float)H - 0.5f;
    int i0 = (int)floorf(x), j0 = (int)floorf(y);
    float a = x - (float)i0, b = y - (float)j0;
    f3 c = mk(0.0f);
    for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
            int i = clampi(i0 + di, 0, W - 1), j = clampi(j0 + dj, 0, H - 1);
            ushort4 t = __ldg(A.env_diffuse + j * W + i);
            float w = (di ? a : 1.0f - a) * (dj ? b : 1.0f - b);
            c += mk(h2f(t.x), h2f(t.y), h2f(t.z)) * w;
        }
    return U3(A.u.ambient) * c;
}

// dvr.comp:76-96: the first surface a ray meets, bisected between the previous
// sample and this one for where the opacity reaches half of this sample's.
__device__ __noinline__ f3 refine_surface(const PtArgs& A, f3 idx, f3 d_idx, float step_mm, float target) {
    float inside = 0.0f, outside = -step_mm;
    for (int i = 0; i < 5; i++) {
        float mid = 0.5f * (inside + outside);
        f3 at = idx + d_idx * mid;
        bool opaque = labelled(A, tf_point(A, density_view(A, at)), at).extinction >= target;
        inside = opaque ? mid : inside;
        outside = opaque ? outside : mid;
    }
    return idx + d_idx * inside;
}

// dvr.comp:98-141: light reflected and scattered towards the viewer at a
// sample (lighting volumes, BRDF, subsurface, ambient); ghosted structures'
// opacity `alpha` is rescaled to their shell.
__device__ __noinline__ f3 shade_sample(const PtArgs& A, const LightTex& SV, const LightTex& AV, f3 idx, Sample s,
                                        f3 v, int cap_plane, float cut, float step_mm, bool has_grad, f3 grad,
                                        float& alpha) {
    m3 to_index = w2i3(A);
    f3 l = U3(A.u.light_dir);
    float light = A.u.light_dir[3];
    f3 n;
    float surfaceness;
    float extinction_scale = has_grad ? surface_frame<true>(A, idx, s, v, cap_plane, cut, 1.5f * step_mm, n,
                                                            surfaceness, grad)
                                      : surface_frame(A, idx, s, v, cap_plane, cut, 1.5f * step_mm, n, surfaceness);
    apply_surface_texture(A, idx, s);
    if (s.ghost) alpha = 1.0f - expf(-s.extinction * extinction_scale * step_mm);
    f3 shadow_at = index_to_tex(A, idx + mul(to_index, n * (1.5f * A.u.light_cells[0] * surfaceness)));
    f3 ao_at = index_to_tex(A, idx + mul(to_index, n * (A.u.light_cells[1] * surfaceness)));
    float shadow_t = A.u.lighting[0] != 0u ? lighting_lookup(A, SV, shadow_at).w : 1.0f;
    f3 sss_at = index_to_tex(A, idx - mul(to_index, n * (A.u.subsurface[3] * surfaceness)));
    f3 diffused = mk(1.0f);
    if (A.u.lighting[0] != 0u) {
        float4 dl = lighting_lookup(A, SV, sss_at);
        diffused = mk(dl.x, dl.y, dl.z);
    }
    float occlusion = A.u.lighting[1] != 0u ? lighting_lookup(A, AV, ao_at).x : 1.0f;
    n = bump_normal(A, idx, s, n);
    n = dot(n, v) < 0.0f ? -n : n;
    float nl = gmax(dot(n, l), 0.0f);
    f3 diffuse;
    f3 specular = brdf_coated(n, v, l, s, diffuse);
    f3 surface = (specular + diffuse) * (1.0f - s.subsurface) * nl * shadow_t + diffuse * s.subsurface * diffused;
    f3 volume = s.albedo / (4.0f * PI) * mix3(mk(shadow_t), diffused, s.subsurface);
    f3 direct = mix3(volume, surface, surfaceness) * light;
    f3 ambient_light = A.u.lighting[3] == 2u
                           ? mix3(U3(A.u.ambient), env_map_diffuse(A, n), surfaceness * (1.0f - s.subsurface))
                           : U3(A.u.ambient);
    f3 ambient = s.albedo * ambient_light * occlusion;
    return direct + ambient;
}

}  // namespace

// ao.comp: mean transmittance over 16 directions within 15 mm, remapped so a
// flat surface is unoccluded; one thread per occlusion voxel.
__global__ void __launch_bounds__(64) k_ao(const __grid_constant__ PtArgs A, uint16_t* __restrict__ out, int ax, int ay,
                                           int az) {
    int x = blockIdx.x * 4 + (threadIdx.x & 3), y = blockIdx.y * 4 + ((threadIdx.x >> 2) & 3),
        z = blockIdx.z * 4 + (threadIdx.x >> 4);
    if (x >= ax || y >= ay || z >= az) return;
    f3 center = tex_to_index(A, mk(((float)x + 0.5f) / (float)ax, ((float)y + 0.5f) / (float)ay,
                                   ((float)z + 0.5f) / (float)az));
    m3 to_index = w2i3(A);
    const float dt = 15.0f / 8.0f;
    float visible = 0.0f;
    for (int i = 0; i < 16; i++) {
        float zz = 1.0f - ((float)i + 0.5f) * (2.0f / 16.0f);
        float r = sqrtf(1.0f - zz * zz);
        float phi = (float)i * 2.39996323f;
        f3 d = mul(to_index, mk(r * cosf(phi), r * sinf(phi), zz));
        float depth = 0.0f;
        for (int j = 0; j < 8; j++) depth += sample_point(A, center + d * (((float)j + 0.5f) * dt)).extinction * dt;
        visible += expf(-depth);
    }
    out[((long)z * ay + y) * ax + x] = f2h(gmin(2.0f * visible / 16.0f, 1.0f));
}

// shadow.comp: one slice of the shadow volume from the previous one (direct
// transmittance towards the light, and light diffused sideways through tissue).
__global__ void __launch_bounds__(64) k_shadow_slice(const __grid_constant__ PtArgs A, ushort4* __restrict__ vol,
                                                     int sx, int sy, int sz, int axis, int slice) {
    int u_axis = (axis + 1) % 3, v_axis = (axis + 2) % 3;
    int pu = blockIdx.x * 8 + (threadIdx.x & 7), pv = blockIdx.y * 8 + (threadIdx.x >> 3);
    int sdim[3] = {sx, sy, sz};
    int p[3];
    p[axis] = slice;
    p[u_axis] = pu;
    p[v_axis] = pv;
    if (p[0] >= sx || p[1] >= sy || p[2] >= sz || pu >= sdim[u_axis] || pv >= sdim[v_axis]) return;
    f3 sdims = mk((float)sx, (float)sy, (float)sz);
    f3 l_idx = mul(w2i3(A), U3(A.u.light_dir)) * (sdims / U3(A.u.dims));
    float s = 1.0f / gmax(fabsf(comp3(l_idx, axis)), 1e-6f);
    f3 here = mk((float)p[0], (float)p[1], (float)p[2]);
    f3 prev = here + l_idx * s;
    f3 mid_tex = ((here + prev) * 0.5f + 0.5f) / sdims;
    Sample m = sample_point(A, tex_to_index(A, mid_tex));
    LightVol V{(const uint16_t*)vol, sx, sy, sz, 4};
    float4 back = lv_linear(V, (prev + 0.5f) / sdims);
    float direct = back.w * expf(-m.extinction * s);
    f3 axis_u = mk(0.0f), axis_v = mk(0.0f);
    set3(axis_u, u_axis, A.u.subsurface[2]);
    set3(axis_v, v_axis, A.u.subsurface[2]);
    f3 gathered = 0.4f * mk(back.x, back.y, back.z);
    for (int i = 0; i < 4; i++) {
        f3 offset = (i & 1) == 0 ? axis_u : axis_v;
        offset *= i < 2 ? 1.0f : -1.0f;
        float4 t = lv_linear(V, (prev + offset + 0.5f) / sdims);
        gathered += 0.15f * mk(t.x, t.y, t.z);
    }
    f3 chroma = m.albedo / gmax(gmax(m.albedo.x, gmax(m.albedo.y, m.albedo.z)), 1e-4f);
    f3 ie = m.extinction * A.u.subsurface[1] * (1.2f - chroma);
    f3 indirect = gathered * mk(expf(-ie.x * s), expf(-ie.y * s), expf(-ie.z * s));
    vol[((long)p[2] * sy + p[1]) * sx + p[0]] = make_ushort4(f2h(indirect.x), f2h(indirect.y), f2h(indirect.z),
                                                             f2h(direct));
}

// dvr.comp: one ray per pixel, emission-absorption with single scattering.
#ifndef VV_DVR_MIN_BLOCKS
#define VV_DVR_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(64, VV_DVR_MIN_BLOCKS) k_dvr(const __grid_constant__ PtArgs A, const LightTex SV,
                                                               const LightTex AV) {
    int px = blockIdx.x * 8 + (threadIdx.x & 7), py = blockIdx.y * 8 + (threadIdx.x >> 3);
    if (px >= (int)A.u.flags[2] || py >= (int)A.u.flags[3]) return;
    float nx = ((float)px + 0.5f) / (float)A.u.flags[2] * 2.0f - 1.0f;
    float ny = ((float)py + 0.5f) / (float)A.u.flags[3] * 2.0f - 1.0f;
    f3 dir = normalize(U3(A.u.forward) + nx * U3(A.u.right) - ny * U3(A.u.up));
    const float* m4 = A.u.w2i;
    f3 e = U3(A.u.eye);
    f3 o_idx = mk(m4[0] * e.x + m4[4] * e.y + m4[8] * e.z + m4[12], m4[1] * e.x + m4[5] * e.y + m4[9] * e.z + m4[13],
                  m4[2] * e.x + m4[6] * e.y + m4[10] * e.z + m4[14]);
    m3 to_index = w2i3(A);
    f3 d_idx = mul(to_index, dir);
    f3 inv_d = brick_inv_dir(d_idx);
    float2 t = intersect_volume(A, o_idx, d_idx);
    float step_mm = A.u.dims[3];
    bool preintegrate = A.u.lighting[2] != 0u;
    f3 v = -dir;
    f3 radiance = mk(0.0f);
    float transmittance = 1.0f;
    bool refined = false;
    if (t.x < t.y) {
        float tt = t.x + ign((float)px, (float)py) * step_mm;
        float prev_density = density_view(A, o_idx + d_idx * (tt - step_mm));
        for (; tt < t.y && transmittance > 0.01f; tt += step_mm) {
            f3 idx = o_idx + d_idx * tt;
            float maj = A.u.path[3] == 0u ? 1e30f : __ldg(A.majorant + brick_index(A, idx));
            if (maj <= 0.0f) {
                tt += brick_exit(idx, inv_d);
                prev_density = -1.0f;
                continue;
            }
            int cap_plane;
            float cut = clip_depth(A, idx, cap_plane);
            if (cut > 0.0f) {
                prev_density = -1.0f;
                continue;
            }
            // With smooth sampling the gradient comes with the density: a
            // sample shaded where it was taken needs no second read.
            f3 grad = mk(0.0f);
            bool has_grad = A.u.env[1] > 0.5f;
            float density = has_grad ? density_cubic_with_gradient(A, idx, grad) : density_tri(A, idx);
            float front_density = prev_density;
            bool segment = preintegrate && front_density >= 0.0f;
            Sample s = segment ? tf_segment(A, front_density, density) : tf_point(A, density);
            prev_density = density;
            s = labelled(A, s, idx);
            if (s.extinction <= 0.0f) continue;
            float alpha = 1.0f - expf(-s.extinction * step_mm);
            if (segment && alpha > 0.2f && transmittance > 0.5f && s.label == 0u && fabsf(density - front_density) > 1e-4f) {
                idx = idx - d_idx * (step_mm * (1.0f - preint_half_depth(A, front_density, density)));
                has_grad = false;
            } else if (!refined && alpha > 0.2f && transmittance > 0.9f) {
                refined = true;
                idx = refine_surface(A, idx, d_idx, step_mm, 0.5f * s.extinction);
                has_grad = false;
            }
            f3 lit = shade_sample(A, SV, AV, idx, s, v, cap_plane, cut, step_mm, has_grad, grad, alpha);
            radiance += transmittance * alpha * lit;
            transmittance *= 1.0f - alpha;
        }
    }
    A.hdr[(long)py * A.width + px] = make_ushort4(f2h(radiance.x), f2h(radiance.y), f2h(radiance.z), f2h(transmittance));
}

cudaError_t launch_ao(const PtArgs& a, uint16_t* out, int ax, int ay, int az, cudaStream_t s) {
    dim3 g((ax + 3) / 4, (ay + 3) / 4, (az + 3) / 4);
    k_ao<<<g, 64, 0, s>>>(a, out, ax, ay, az);
    return cudaGetLastError();
}

cudaError_t launch_shadow_sweep(const PtArgs& a, ushort4* vol, int sx, int sy, int sz, int axis, int sign,
                                cudaStream_t s, int* launches) {
    int sd[3] = {sx, sy, sz};
    int u_axis = (axis + 1) % 3, v_axis = (axis + 2) % 3;
    dim3 g((sd[u_axis] + 7) / 8, (sd[v_axis] + 7) / 8);
    cudaError_t e = cudaMemsetAsync(vol, 0, (size_t)sx * sy * sz * sizeof(ushort4), s);
    if (e != cudaSuccess) return e;
    int n = sd[axis];
    for (int i = 0; i < n; i++) {
        int slice = sign > 0 ? n - 1 - i : i;
        k_shadow_slice<<<g, 64, 0, s>>>(a, vol, sx, sy, sz, axis, slice);
    }
    *launches += n;
    return cudaGetLastError();
}

// The texture array of a lighting volume: texel (x, y, z) of the volume at
// (x + 1, y + 1, z + 1), white (1, 1, 1, 1) around it.
__global__ void k_pad_lighting(const uint16_t* __restrict__ vol, int channels, int w, int h, int d,
                               cudaSurfaceObject_t surf) {
    int x = blockIdx.x * 8 + (threadIdx.x & 7), y = blockIdx.y * 8 + (threadIdx.x >> 3), z = blockIdx.z;
    if (x >= w + 2 || y >= h + 2 || z >= d + 2) return;
    const uint16_t one = 0x3c00u;  // 1.0 in binary16
    bool inside = x >= 1 && y >= 1 && z >= 1 && x <= w && y <= h && z <= d;
    long i = inside ? ((long)(z - 1) * h + (y - 1)) * w + (x - 1) : 0;
    if (channels == 4) {
        ushort4 t = inside ? __ldg((const ushort4*)vol + i) : make_ushort4(one, one, one, one);
        surf3Dwrite(t, surf, x * (int)sizeof(ushort4), y, z);
    } else {
        uint16_t t = inside ? __ldg(vol + i) : one;
        surf3Dwrite(t, surf, x * (int)sizeof(uint16_t), y, z);
    }
}

cudaError_t launch_pad_lighting(const uint16_t* vol, int channels, int w, int h, int d, cudaSurfaceObject_t surf,
                                cudaStream_t s) {
    dim3 g((w + 2 + 7) / 8, (h + 2 + 7) / 8, d + 2);
    k_pad_lighting<<<g, 64, 0, s>>>(vol, channels, w, h, d, surf);
    return cudaGetLastError();
}

cudaError_t launch_dvr(const PtArgs& a, const LightTex& shadow, const LightTex& ao, cudaStream_t s) {
    dim3 g((a.width + 7) / 8, (a.height + 7) / 8);
    k_dvr<<<g, 64, 0, s>>>(a, shadow, ao);
    return cudaGetLastError();
}

}  // namespace VV_FMT_NS
}  // namespace vv
