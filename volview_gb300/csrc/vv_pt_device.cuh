// vv_pt_device.cuh — the device functions of the path tracer (pt.comp with
// common.glsl and shading.glsl): samplers, label logic, shading, free flight,
// transmittance and the resumable path state. Included by vv_pt.cu.
#pragma once
#include <cuda_runtime.h>

#include "vv_device.cuh"
#include "vv_kernels.h"

// The density storage format this translation unit's samplers read (DF_*):
// the path tracer's and ray marcher's sources are compiled once per format,
// each into its own namespace (vv::fmt0 .. vv::fmt5), so every format runs
// code specialised for it and the reference's format has no format branch.
#ifndef VV_DFMT
#define VV_DFMT 0
#endif
// Builds 4 and 5 store the label mask in the density's format too: FP16
// density and mask, BF16 density and mask (vv_precision::mask_format). The
// others keep the reference's RG16_UNORM mask. VV_DENS is the density format
// the samplers read, VV_MASKF the mask format (MF_*).
#if VV_DFMT == 4
#define VV_DENS 1
#define VV_MASKF 1
#elif VV_DFMT == 5
#define VV_DENS 2
#define VV_MASKF 2
#else
#define VV_DENS VV_DFMT
#define VV_MASKF 0
#endif
// VV_EXACT = 1: the parity build of the path probe (namespace vv::exactN,
// compiled with --fmad=false). Its samplers take the texture-unit model of the
// Vulkan specification that the CPU oracle restates: index_to_tex, then
// linear filtering of decoded texels with weights (1 - a)(1 - b)(1 - c) ... in
// x, y, z order; the cubic B-spline from the reference's 8 folded trilinear
// fetches; the LUT at (d * 4095 + 0.5) / 4096. With every product and sum
// rounded on its own, as the oracle rounds them, a replayed path differs from
// the oracle's only where CUDA's and the C library's transcendental functions
// differ in the last bit. The product samplers (VV_EXACT = 0) filter codes
// directly at the index, with fused multiply-adds: the same filters, rounded
// differently.
#ifndef VV_EXACT
#define VV_EXACT 0
#endif
#define VV_FMT_CAT2(a, b) a##b
#define VV_FMT_CAT(a, b) VV_FMT_CAT2(a, b)
#if VV_EXACT
#define VV_FMT_NS VV_FMT_CAT(exact, VV_DFMT)
#else
#define VV_FMT_NS VV_FMT_CAT(fmt, VV_DFMT)
#endif

namespace vv {
// Internal linkage: every translation unit that includes this header gets its
// own copy of the device functions (some are out of line).
namespace {


constexpr float PI = 3.14159265358979f;
constexpr float MAX_EXTINCTION = 8.0f;       // pt.comp:34
constexpr uint32_t MAX_VOLUME_EVENTS = 32u;  // pt.comp:112
constexpr float BONE_DENSITY = (300.0f + 1024.0f) / 4095.0f;
constexpr uint32_t SKIN_LABEL = 255u;
constexpr float INV65535 = 1.0f / 65535.0f;

struct Sample {
    f3 albedo;
    float extinction, roughness, metalness;
    uint32_t label;
    bool ghost;
    float density, subsurface, coat;
};

__device__ __forceinline__ f3 U3(const float* a) { return mk(a[0], a[1], a[2]); }
__device__ __forceinline__ m3 w2i3(const PtArgs& A) {
    const float* m = A.u.w2i;
    return {mk(m[0], m[1], m[2]), mk(m[4], m[5], m[6]), mk(m[8], m[9], m[10])};
}
__device__ __forceinline__ float4 ldf4(const float4* p) { return __ldg(p); }

// Warp-aggregated event count (counting launches only).
__device__ __forceinline__ void count(const PtArgs& A, int k) {
    if (A.counters) {
        unsigned m = __activemask();
        if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(A.counters + k, (unsigned long long)__popc(m));
    }
}

// ------------------------------------------------------------------ samplers
struct Tri {
    int o[8];
    float fx, fy, fz;
};
__device__ __forceinline__ Tri tri_taps(const Vol& v, f3 p) {
    float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
    int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    Tri t;
    t.fx = p.x - flx;
    t.fy = p.y - fly;
    t.fz = p.z - flz;
    int x0 = offx(clampi(ix, 0, v.nx - 1)), x1 = offx(clampi(ix + 1, 0, v.nx - 1));
    int y0 = offy(v, clampi(iy, 0, v.ny - 1)), y1 = offy(v, clampi(iy + 1, 0, v.ny - 1));
    int z0 = offz(v, clampi(iz, 0, v.nz - 1)), z1 = offz(v, clampi(iz + 1, 0, v.nz - 1));
    t.o[0] = x0 + y0 + z0; t.o[1] = x1 + y0 + z0; t.o[2] = x0 + y1 + z0; t.o[3] = x1 + y1 + z0;
    t.o[4] = x0 + y0 + z1; t.o[5] = x1 + y0 + z1; t.o[6] = x0 + y1 + z1; t.o[7] = x1 + y1 + z1;
    return t;
}
__device__ __forceinline__ float lerpf(float a, float b, float f) { return fmaf(b - a, f, a); }
__device__ __forceinline__ float tri_mix(const float c[8], const Tri& t) {
    float a = lerpf(c[0], c[1], t.fx), b = lerpf(c[2], c[3], t.fx);
    float d = lerpf(c[4], c[5], t.fx), e = lerpf(c[6], c[7], t.fx);
    return lerpf(lerpf(a, b, t.fy), lerpf(d, e, t.fy), t.fz);
}

#if VV_EXACT
// The texel coordinates of a linear 3D lookup at continuous index p, as the
// oracle's texture model computes them: tc = (p + 0.5) / dims (index_to_tex,
// common.glsl:68-70), u = tc * size - 0.5; the eight taps clamped to the edge,
// their weights (1 - a or a) * (1 - b or b) * (1 - c or c), x fastest.
struct TriX {
    int o[8];
    float w[8];
};
__device__ __forceinline__ TriX tri_taps_exact(const PtArgs& A, f3 p) {
    const Vol& v = A.vol;
    float tx = (p.x + 0.5f) / A.u.dims[0], ty = (p.y + 0.5f) / A.u.dims[1], tz = (p.z + 0.5f) / A.u.dims[2];
    float uu = tx * (float)v.nx - 0.5f, vv = ty * (float)v.ny - 0.5f, qq = tz * (float)v.nz - 0.5f;
    int i0 = (int)floorf(uu), j0 = (int)floorf(vv), k0 = (int)floorf(qq);
    float a = uu - (float)i0, b = vv - (float)j0, c = qq - (float)k0;
    TriX t;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int di = k & 1, dj = (k >> 1) & 1, dk = k >> 2;
        t.o[k] = offx(clampi(i0 + di, 0, v.nx - 1)) + offy(v, clampi(j0 + dj, 0, v.ny - 1)) +
                 offz(v, clampi(k0 + dk, 0, v.nz - 1));
        t.w[k] = (di ? a : 1.0f - a) * (dj ? b : 1.0f - b) * (dk ? c : 1.0f - c);
    }
    return t;
}
__device__ __forceinline__ float tri_sum_exact(const float c[8], const TriX& t) {
    float r = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) r = r + c[k] * t.w[k];
    return r;
}
// A density texel as the sampler decodes it: R16_UNORM code / 65535, the
// other formats their value.
__device__ __forceinline__ float density_texel_exact(const void* d, int o) {
    typedef DensityStore<VV_DENS>::type E;
    float x = density_decode<VV_DENS>(__ldg((const E*)d + o));
    return VV_DENS == DF_UNORM16 ? x / 65535.0f : x;
}
__device__ __forceinline__ float density_at_index_exact(const PtArgs& A, f3 p) {
    TriX t = tri_taps_exact(A, p);
    float c[8];
#pragma unroll
    for (int k = 0; k < 8; k++) c[k] = density_texel_exact(A.density, t.o[k]);
    return tri_sum_exact(c, t);
}
// cubic_taps (common.glsl:89-113) of one axis.
struct AxisTaps {
    float h0, h1, g0, g1, dh0, dh1, dg0, dg1;
};
__device__ __forceinline__ AxisTaps cubic_axis_exact(float x) {
    float i = floorf(x), f = x - i, f2 = f * f, f3_ = f2 * f;
    float w0 = (1.0f - 3.0f * f + 3.0f * f2 - f3_) / 6.0f;
    float w1 = (4.0f - 6.0f * f2 + 3.0f * f3_) / 6.0f;
    float w2 = (1.0f + 3.0f * f + 3.0f * f2 - 3.0f * f3_) / 6.0f;
    float w3 = f3_ / 6.0f;
    float d0 = -0.5f * (1.0f - f) * (1.0f - f);
    float d1 = 0.5f * f * (3.0f * f - 4.0f);
    float d2 = 0.5f * (1.0f - f) * (3.0f * f + 1.0f);
    float d3 = 0.5f * f2;
    AxisTaps t;
    t.g0 = w0 + w1;
    t.g1 = w2 + w3;
    t.h0 = i - 1.0f + w1 / t.g0;
    t.h1 = i + 1.0f + w3 / t.g1;
    t.dg0 = d0 + d1;
    t.dg1 = d2 + d3;
    t.dh0 = i - 1.0f + d1 / gmin(t.dg0, -1e-7f);
    t.dh1 = i + 1.0f + d3 / gmax(t.dg1, 1e-7f);
    return t;
}
// cubic_fetch (common.glsl:116-122): the 8-fetch tensor product.
__device__ __forceinline__ float cubic_fetch_exact(const PtArgs& A, f3 h0, f3 h1, f3 g0, f3 g1) {
    float a = g0.x * density_at_index_exact(A, mk(h0.x, h0.y, h0.z)) + g1.x * density_at_index_exact(A, mk(h1.x, h0.y, h0.z));
    float b = g0.x * density_at_index_exact(A, mk(h0.x, h1.y, h0.z)) + g1.x * density_at_index_exact(A, mk(h1.x, h1.y, h0.z));
    float c = g0.x * density_at_index_exact(A, mk(h0.x, h0.y, h1.z)) + g1.x * density_at_index_exact(A, mk(h1.x, h0.y, h1.z));
    float d = g0.x * density_at_index_exact(A, mk(h0.x, h1.y, h1.z)) + g1.x * density_at_index_exact(A, mk(h1.x, h1.y, h1.z));
    return g0.z * (g0.y * a + g1.y * b) + g1.z * (g0.y * c + g1.y * d);
}
#endif

// textureLod(density_tex, index_to_tex(idx)) (common.glsl:76-78), the density
// stored as this translation unit's format (VV_DENS).
__device__ float density_tri(const PtArgs& A, f3 p) {
    count(A, COUNT_TRILINEAR);
#if VV_EXACT
    return density_at_index_exact(A, p);
#else
    typedef DensityStore<VV_DENS>::type E;
    Tri t = tri_taps(A.vol, p);
    float c[8];
#pragma unroll
    for (int k = 0; k < 8; k++) c[k] = density_decode<VV_DENS>(__ldg((const E*)A.density + t.o[k]));
    return tri_mix(c, t) * density_unit<VV_DENS>();
#endif
}

// textureLod(mask_tex, ...).rg
__device__ float2 mask_tri(const PtArgs& A, f3 p) {
    count(A, COUNT_MASK);
#if VV_EXACT
    TriX x = tri_taps_exact(A, p);
    float er[8], eg[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.mask + x.o[k]);
        er[k] = VV_MASKF == MF_UNORM16 ? (float)(m & 0xffffu) / 65535.0f : mask_decode(m & 0xffffu, VV_MASKF);
        eg[k] = VV_MASKF == MF_UNORM16 ? (float)(m >> 16) / 65535.0f : mask_decode(m >> 16, VV_MASKF);
    }
    return make_float2(tri_sum_exact(er, x), tri_sum_exact(eg, x));
#endif
    Tri t = tri_taps(A.vol, p);
    float r[8], g[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.mask + t.o[k]);
        // UNORM16 codes are filtered as integers, then scaled; FP16/BF16 as values.
        r[k] = VV_MASKF == MF_UNORM16 ? (float)(m & 0xffffu) : mask_decode(m & 0xffffu, VV_MASKF);
        g[k] = VV_MASKF == MF_UNORM16 ? (float)(m >> 16) : mask_decode(m >> 16, VV_MASKF);
    }
    const float unit = VV_MASKF == MF_UNORM16 ? INV65535 : 1.0f;
    return make_float2(tri_mix(r, t) * unit, tri_mix(g, t) * unit);
}
__device__ float mask_tri_ch(const PtArgs& A, f3 p, int ch) {
    count(A, COUNT_MASK);
#if VV_EXACT
    TriX x = tri_taps_exact(A, p);
    float c[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.mask + x.o[k]);
        uint32_t code = ch == 0 ? (m & 0xffffu) : (m >> 16);
        c[k] = VV_MASKF == MF_UNORM16 ? (float)code / 65535.0f : mask_decode(code, VV_MASKF);
    }
    return tri_sum_exact(c, x);
#endif
    Tri t = tri_taps(A.vol, p);
    float r[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.mask + t.o[k]);
        uint32_t code = ch == 0 ? (m & 0xffffu) : (m >> 16);
        r[k] = VV_MASKF == MF_UNORM16 ? (float)code : mask_decode(code, VV_MASKF);
    }
    return tri_mix(r, t) * (VV_MASKF == MF_UNORM16 ? INV65535 : 1.0f);
}

// textureLod(normal_tex, ...): RGBA8_SNORM. The volume holds no -128, so the
// decode max(c / 127, -1) is c / 127 and commutes with the interpolation.
__device__ float4 normal_tri(const PtArgs& A, f3 p) {
    count(A, COUNT_NORMAL);
#if VV_EXACT
    TriX q = tri_taps_exact(A, p);
    float c[4][8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.normals + q.o[k]);
#pragma unroll
        for (int ch = 0; ch < 4; ch++) c[ch][k] = gmax((float)(int8_t)((m >> (8 * ch)) & 0xff) / 127.0f, -1.0f);
    }
    return make_float4(tri_sum_exact(c[0], q), tri_sum_exact(c[1], q), tri_sum_exact(c[2], q), tri_sum_exact(c[3], q));
#endif
    Tri t = tri_taps(A.vol, p);
    float x[8], y[8], z[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t m = __ldg(A.normals + t.o[k]);
        x[k] = (float)(int8_t)(m & 0xff);
        y[k] = (float)(int8_t)((m >> 8) & 0xff);
        z[k] = (float)(int8_t)((m >> 16) & 0xff);
        w[k] = (float)(int8_t)(m >> 24);
    }
    const float s = 1.0f / 127.0f;
    return make_float4(tri_mix(x, t) * s, tri_mix(y, t) * s, tri_mix(z, t) * s, tri_mix(w, t) * s);
}

// Cubic B-spline weights of one axis (common.glsl:89-101).
__device__ __forceinline__ void bspline_w(float f, float w[4]) {
    float f2 = f * f, f3_ = f2 * f;
    w[0] = (1.0f - 3.0f * f + 3.0f * f2 - f3_) / 6.0f;
    w[1] = (4.0f - 6.0f * f2 + 3.0f * f3_) / 6.0f;
    w[2] = (1.0f + 3.0f * f + 3.0f * f2 - 3.0f * f3_) / 6.0f;
    w[3] = f3_ / 6.0f;
}
__device__ __forceinline__ void bspline_d(float f, float d[4]) {
    d[0] = -0.5f * (1.0f - f) * (1.0f - f);
    d[1] = 0.5f * f * (3.0f * f - 4.0f);
    d[2] = 0.5f * (1.0f - f) * (3.0f * f + 1.0f);
    d[3] = 0.5f * f * f;
}
struct Cubic {
    int ox[4], oy[4], oz[4];
    float fx, fy, fz;
};
__device__ __forceinline__ Cubic cubic_taps(const Vol& v, f3 p) {
    Cubic c;
    float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
    int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    c.fx = p.x - flx; c.fy = p.y - fly; c.fz = p.z - flz;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        c.ox[k] = offx(clampi(ix - 1 + k, 0, v.nx - 1));
        c.oy[k] = offy(v, clampi(iy - 1 + k, 0, v.ny - 1));
        c.oz[k] = offz(v, clampi(iz - 1 + k, 0, v.nz - 1));
    }
    return c;
}

// density_cubic (common.glsl:124-127) as the 64-tap tensor product.
__device__ __noinline__ float density_cubic(const PtArgs& A, f3 p) {
    count(A, COUNT_CUBIC);
#if VV_EXACT
    AxisTaps x = cubic_axis_exact(p.x), y = cubic_axis_exact(p.y), z = cubic_axis_exact(p.z);
    return cubic_fetch_exact(A, mk(x.h0, y.h0, z.h0), mk(x.h1, y.h1, z.h1), mk(x.g0, y.g0, z.g0), mk(x.g1, y.g1, z.g1));
#endif
    typedef DensityStore<VV_DENS>::type E;
    Cubic c = cubic_taps(A.vol, p);
    float wx[4], wy[4], wz[4];
    bspline_w(c.fx, wx);
    bspline_w(c.fy, wy);
    bspline_w(c.fz, wz);
    float acc = 0.0f;
    // Loops, not 64 unrolled taps: the flight kernels wait on instruction
    // fetch, and the smaller code runs faster (349.7 -> 377.4 M path samples/s
    // with both loops rolled and extinction_unclipped out of line).
#pragma unroll 1
    for (int z = 0; z < 4; z++) {
        float az = 0.0f;
#pragma unroll 1
        for (int y = 0; y < 4; y++) {
            const E* row = (const E*)A.density + c.oz[z] + c.oy[y];
            float r = wx[0] * density_decode<VV_DENS>(__ldg(row + c.ox[0])) +
                      wx[1] * density_decode<VV_DENS>(__ldg(row + c.ox[1])) +
                      wx[2] * density_decode<VV_DENS>(__ldg(row + c.ox[2])) +
                      wx[3] * density_decode<VV_DENS>(__ldg(row + c.ox[3]));
            az = fmaf(wy[y], r, az);
        }
        acc = fmaf(wz[z], az, acc);
    }
    return acc * density_unit<VV_DENS>();
}

// density_gradient_cubic (common.glsl:130-136) from the same 64 voxels; with
// VALUE, also density_cubic's value, with its arithmetic (the value's z-slices
// are the gradient's vz sums), from the same read.
template <bool VALUE> __device__ __forceinline__ f3 density_gradient_cubic_impl(const PtArgs& A, f3 p, float& value) {
    typedef DensityStore<VV_DENS>::type E;
    Cubic c = cubic_taps(A.vol, p);
    float wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
    bspline_w(c.fx, wx); bspline_w(c.fy, wy); bspline_w(c.fz, wz);
    bspline_d(c.fx, dx); bspline_d(c.fy, dy); bspline_d(c.fz, dz);
    float acc = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
    // The ray marcher's value-and-gradient fetch runs its z slices as a loop
    // (measured 32.7 -> 30.9 ms per 1024^2 frame); the path tracer's gradient
    // stays unrolled (rolled: 370 -> 368 M path samples/s).
#pragma unroll(VALUE ? 1 : 4)
    for (int z = 0; z < 4; z++) {
        float vz = 0.0f, gxz = 0.0f, gyz = 0.0f;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const E* row = (const E*)A.density + c.oz[z] + c.oy[y];
            float v0 = density_decode<VV_DENS>(__ldg(row + c.ox[0])), v1 = density_decode<VV_DENS>(__ldg(row + c.ox[1]));
            float v2 = density_decode<VV_DENS>(__ldg(row + c.ox[2])), v3 = density_decode<VV_DENS>(__ldg(row + c.ox[3]));
            float rw = wx[0] * v0 + wx[1] * v1 + wx[2] * v2 + wx[3] * v3;
            float rd = dx[0] * v0 + dx[1] * v1 + dx[2] * v2 + dx[3] * v3;
            vz = fmaf(wy[y], rw, vz);
            gxz = fmaf(wy[y], rd, gxz);
            gyz = fmaf(dy[y], rw, gyz);
        }
        if (VALUE) acc = fmaf(wz[z], vz, acc);
        gx = fmaf(wz[z], gxz, gx);
        gy = fmaf(wz[z], gyz, gy);
        gz = fmaf(dz[z], vz, gz);
    }
    if (VALUE) value = acc * density_unit<VV_DENS>();
    return mk(gx, gy, gz) * density_unit<VV_DENS>();
}
__device__ __noinline__ f3 density_gradient_cubic(const PtArgs& A, f3 p) {
    count(A, COUNT_GRADIENT);
#if VV_EXACT
    AxisTaps x = cubic_axis_exact(p.x), y = cubic_axis_exact(p.y), z = cubic_axis_exact(p.z);
    return mk(cubic_fetch_exact(A, mk(x.dh0, y.h0, z.h0), mk(x.dh1, y.h1, z.h1), mk(x.dg0, y.g0, z.g0),
                                mk(x.dg1, y.g1, z.g1)),
              cubic_fetch_exact(A, mk(x.h0, y.dh0, z.h0), mk(x.h1, y.dh1, z.h1), mk(x.g0, y.dg0, z.g0),
                                mk(x.g1, y.dg1, z.g1)),
              cubic_fetch_exact(A, mk(x.h0, y.h0, z.dh0), mk(x.h1, y.h1, z.dh1), mk(x.g0, y.g0, z.dg0),
                                mk(x.g1, y.g1, z.dg1)));
#endif
    float unused;
    return density_gradient_cubic_impl<false>(A, p, unused);
}
// density_cubic and density_gradient_cubic at one point from one read of the
// 64 voxels, each result that function's.
__device__ __noinline__ float density_cubic_with_gradient(const PtArgs& A, f3 p, f3& grad) {
    count(A, COUNT_CUBIC);
    float v;
    grad = density_gradient_cubic_impl<true>(A, p, v);
    return v;
}

// transfer (common.glsl:170-173): linear LUT lookup at texel centres.
__device__ float4 transfer(const PtArgs& A, float d) {
#if VV_EXACT
    {
        float uu = (d * (4096.0f - 1.0f) + 0.5f) / 4096.0f * 4096.0f - 0.5f;
        int i0 = (int)floorf(uu);
        float a = uu - (float)i0;
        float4 t0 = ldf4(A.lut + clampi(i0, 0, 4095)), t1 = ldf4(A.lut + clampi(i0 + 1, 0, 4095));
        float w0 = 1.0f - a;
        return make_float4(t0.x * w0 + t1.x * a, t0.y * w0 + t1.y * a, t0.z * w0 + t1.z * a, t0.w * w0 + t1.w * a);
    }
#endif
    float u = d * 4095.0f;
    float fl = floorf(u);
    float f = u - fl;
    int i = (int)fl;
    float4 a = ldf4(A.lut + clampi(i, 0, 4095));
    float4 b = ldf4(A.lut + clampi(i + 1, 0, 4095));
    return make_float4(lerpf(a.x, b.x, f), lerpf(a.y, b.y, f), lerpf(a.z, b.z, f), lerpf(a.w, b.w, f));
}

__device__ __forceinline__ uint32_t label_fetch(const PtArgs& A, int x, int y, int z) {
    count(A, COUNT_LABEL);
    return __ldg(A.labels + voff(A.vol, x, y, z));
}

// ------------------------------------------------------------- common.glsl
__device__ __forceinline__ Sample tf_point(const PtArgs& A, float d) {
    float4 tf = transfer(A, d);
    Sample s;
    s.albedo = mk(tf.x, tf.y, tf.z);
    s.extinction = tf.w;
    s.roughness = A.u.material[0];
    s.metalness = A.u.material[1];
    s.label = 0u;
    s.ghost = false;
    s.density = d;
    s.subsurface = A.u.subsurface[0];
    s.coat = 0.0f;
    return s;
}
__device__ __forceinline__ float lab_a(const PtArgs& A, uint32_t l) { return __ldg(&A.tab->colors[l].w); }
__device__ __forceinline__ bool label_shown(const PtArgs& A, uint32_t l) { return lab_a(A, l) > 0.5f; }
__device__ __forceinline__ bool label_ghosted(const PtArgs& A, uint32_t l) { return l != 0u && lab_a(A, l) > 1.5f; }
__device__ __forceinline__ bool label_solid(const PtArgs& A, uint32_t l, uint32_t mode) {
    if (label_ghosted(A, l)) return false;
    return mode == 1u ? (l == 0u || label_shown(A, l)) : (l != 0u && label_shown(A, l));
}

// common.glsl:253-290
__device__ __noinline__ Sample with_label(const PtArgs& A, Sample s, uint32_t label, uint32_t mode, bool ghost) {
    s.label = label;
    s.ghost = ghost;
    if (label == 0u) return s;
    float4 color = ldf4(&A.tab->colors[label]);
    float4 mat = ldf4(&A.tab->materials[label]);
    if (mode == 1u) {
        s.albedo = mix3(s.albedo, mk(color.x, color.y, color.z), A.u.labels[1]);
    } else {
        s.albedo = mk(color.x, color.y, color.z);
        s.extinction = A.u.labels[2];
        if (mode == 3u && !ghost) {
            float4 d = ldf4(&A.tab->density[label]);
            if (d.w > 0.0f) {
                s.extinction *= smoothstepf(d.x, d.y, s.density);
                float t = gclamp((s.density - d.z) / d.w, -1.5f, 1.5f);
                s.albedo = gclamp(s.albedo * (1.0f + 0.2f * t), 0.0f, 1.0f);
                if (d.z > BONE_DENSITY) {
                    float thin = 1.0f - smoothstepf(-1.5f, -0.5f, t);
                    s.albedo *= mix3(mk(1.0f), mk(0.92f, 0.6f, 0.5f), thin);
                }
            }
        }
    }
    s.roughness = mat.x;
    s.metalness = mat.y;
    s.subsurface = mat.w;
    s.coat = mat.z;
    return s;
}

// common.glsl:302-324
__device__ __noinline__ bool drawn_label_near(const PtArgs& A, f3 idx, uint32_t mode, bool ghost, uint32_t& label) {
    int hx = A.vol.nx - 1, hy = A.vol.ny - 1, hz = A.vol.nz - 1;
    int nx = clampi((int)floorf(idx.x + 0.5f), 0, hx), ny = clampi((int)floorf(idx.y + 0.5f), 0, hy),
        nz = clampi((int)floorf(idx.z + 0.5f), 0, hz);
    int bx = (int)floorf(idx.x), by = (int)floorf(idx.y), bz = (int)floorf(idx.z);
#pragma unroll 1
    for (int i = 0; i < 21; i++) {
        int cx, cy, cz;
        if (i == 0) {
            cx = nx; cy = ny; cz = nz;
        } else if (i < 9) {
            cx = bx + ((i - 1) & 1); cy = by + (((i - 1) >> 1) & 1); cz = bz + ((i - 1) >> 2);
        } else {
            int k = i - 9;
            int d = (k / 3 % 2 == 0 ? 1 : -1) * (k < 6 ? 1 : 2);
            int a = k % 3;
            cx = nx + (a == 0 ? d : 0); cy = ny + (a == 1 ? d : 0); cz = nz + (a == 2 ? d : 0);
        }
        label = label_fetch(A, clampi(cx, 0, hx), clampi(cy, 0, hy), clampi(cz, 0, hz));
        if (ghost ? label_ghosted(A, label) : label_solid(A, label, mode)) return true;
    }
    return false;
}

// common.glsl:326-351
__device__ Sample apply_labels(const PtArgs& A, Sample s, f3 idx) {
    uint32_t mode = (uint32_t)A.u.labels[0];
    if (mode == 0u) return s;
    float2 m = mask_tri(A, idx);
    uint32_t label;
    if (m.x < (mode == 3u ? 0.25f : 0.5f)) {
        if (m.y >= 0.5f && drawn_label_near(A, idx, mode, true, label)) return with_label(A, s, label, mode, true);
        s.extinction = 0.0f;
        return s;
    }
    if (drawn_label_near(A, idx, mode, false, label)) return with_label(A, s, label, mode, false);
    if (mode >= 2u) s.extinction = 0.0f;
    return s;
}

// common.glsl:357-373
__device__ __forceinline__ float clip_depth(const PtArgs& A, f3 idx, int& plane) {
    plane = -1;
    uint32_t count = A.u.clip[0];
    if (count == 0u) return -1e30f;
    bool all_planes = A.u.clip[1] != 0u;
    float depth = all_planes ? 1e30f : -1e30f;
    for (uint32_t i = 0u; i < count && i < 3u; i++) {
        const float* cp = A.u.clip_planes + 4 * i;
        float d = cp[0] * idx.x + cp[1] * idx.y + cp[2] * idx.z - cp[3];
        if (all_planes ? d < depth : d > depth) {
            depth = d;
            plane = (int)i;
        }
    }
    return depth;
}

// sample_point (common.glsl:385-391) at an `idx` the caller has found inside
// the kept part (clip_depth(idx) <= 0); clipped points have extinction 0.
__device__ __forceinline__ Sample sample_point_unclipped(const PtArgs& A, f3 idx) {
    Sample s = apply_labels(A, tf_point(A, density_tri(A, idx)), idx);
    if (s.ghost) s.extinction = 0.0f;
    return s;
}

// common.glsl:395-404
__device__ __noinline__ f3 mask_gradient(const PtArgs& A, f3 idx, int ch) {
    f3 g;
    g.x = mask_tri_ch(A, idx + mk(1.0f, 0.0f, 0.0f), ch) - mask_tri_ch(A, idx - mk(1.0f, 0.0f, 0.0f), ch);
    g.y = mask_tri_ch(A, idx + mk(0.0f, 1.0f, 0.0f), ch) - mask_tri_ch(A, idx - mk(0.0f, 1.0f, 0.0f), ch);
    g.z = mask_tri_ch(A, idx + mk(0.0f, 0.0f, 1.0f), ch) - mask_tri_ch(A, idx - mk(0.0f, 0.0f, 1.0f), ch);
    return mul_t(w2i3(A), 0.5f * g);
}

// common.glsl:408-417
__device__ __forceinline__ float2 intersect_volume(const PtArgs& A, f3 o, f3 d) {
    f3 lo = mk(-0.5f), hi = mk(A.u.dims[0] - 0.5f, A.u.dims[1] - 0.5f, A.u.dims[2] - 0.5f);
    f3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    f3 t0 = (lo - o) * inv, t1 = (hi - o) * inv;
    f3 tmin = gmin(t0, t1), tmax = gmax(t0, t1);
    return make_float2(gmax(gmax(tmin.x, tmin.y), gmax(tmin.z, 0.0f)), gmin(gmin(tmax.x, tmax.y), tmax.z));
}

// The brick of continuous index `idx` whose majorant brick_majorant
// (common.glsl:421-428) fetches, as an index into the majorant grid.
__device__ __forceinline__ int brick_index(const PtArgs& A, f3 idx) {
    int bx = clampi((int)floorf((idx.x + 0.5f) * 0.125f), 0, A.vol.bx - 1);
    int by = clampi((int)floorf((idx.y + 0.5f) * 0.125f), 0, A.vol.by - 1);
    int bz = clampi((int)floorf((idx.z + 0.5f) * 0.125f), 0, A.vol.bz - 1);
    return (bz * A.vol.by + by) * A.vol.bx + bx;
}
// The reciprocal of a ray's index-space direction, zero components replaced
// by 1e-9 as brick_exit does (common.glsl:433).
__device__ __forceinline__ f3 brick_inv_dir(f3 d_idx) {
    return mk(1.0f / (d_idx.x == 0.0f ? 1e-9f : d_idx.x), 1.0f / (d_idx.y == 0.0f ? 1e-9f : d_idx.y),
              1.0f / (d_idx.z == 0.0f ? 1e-9f : d_idx.z));
}
// brick_exit (common.glsl:430-436), multiplying by the ray's reciprocal
// direction instead of dividing at every step.
__device__ __forceinline__ float brick_exit(f3 idx, f3 inv_d) {
    f3 lo = mk(floorf((idx.x + 0.5f) * 0.125f) * 8.0f - 0.5f, floorf((idx.y + 0.5f) * 0.125f) * 8.0f - 0.5f,
               floorf((idx.z + 0.5f) * 0.125f) * 8.0f - 0.5f);
    f3 hi = lo + 8.0f;
    f3 t_far = gmax((lo - idx) * inv_d, (hi - idx) * inv_d);
    return gmax(gmin(t_far.x, gmin(t_far.y, t_far.z)), 0.0f);
}

// ------------------------------------------------------------ shading.glsl
__device__ __forceinline__ float ggx_distribution(float nh, float a2) {
    float denom = nh * nh * (a2 - 1.0f) + 1.0f;
    return a2 / (PI * denom * denom);
}
// shading.glsl:11-27
__device__ f3 brdf(f3 n, f3 v, f3 l, f3 albedo, float roughness, float metalness, f3& diffuse) {
    f3 h = normalize(v + l);
    float nv = gmax(dot(n, v), 1e-4f), nl = gmax(dot(n, l), 1e-4f);
    float nh = gmax(dot(n, h), 0.0f), vh = gmax(dot(v, h), 0.0f);
    float a = gmax(roughness * roughness, 2e-3f);
    float d = ggx_distribution(nh, a * a);
    float k = a * 0.5f;
    float g = (nv / (nv * (1.0f - k) + k)) * (nl / (nl * (1.0f - k) + k));
    f3 f0 = mix3(mk(0.028f), albedo, metalness);
    float p5 = powf(1.0f - vh, 5.0f);
    f3 f = f0 + (1.0f - f0) * p5;
    f3 specular = f * (d * g) / (4.0f * nv * nl);
    diffuse = (1.0f - f) * (1.0f - metalness) * albedo / PI;
    return specular;
}
__device__ __forceinline__ float coat_roughness(const Sample& s) { return gclamp(0.5f * s.roughness, 0.1f, 0.25f); }
__device__ __forceinline__ float smith(float nv, float nl, float a) {
    float k = a * 0.5f;
    return (nv / (nv * (1.0f - k) + k)) * (nl / (nl * (1.0f - k) + k));
}
// shading.glsl:45-58
__device__ __noinline__ f3 brdf_coated(f3 n, f3 v, f3 l, const Sample& s, f3& diffuse) {
    f3 specular = brdf(n, v, l, s.albedo, s.roughness, s.metalness, diffuse);
    if (s.coat <= 0.0f) return specular;
    f3 h = normalize(v + l);
    float nv = gmax(dot(n, v), 1e-4f), nl = gmax(dot(n, l), 1e-4f);
    float a = coat_roughness(s) * coat_roughness(s);
    float f = s.coat * (0.02f + 0.98f * powf(1.0f - gmax(dot(v, h), 0.0f), 5.0f));
    float coat = ggx_distribution(gmax(dot(n, h), 0.0f), a * a) * smith(nv, nl, a) * f / (4.0f * nv * nl);
    diffuse *= 1.0f - f;
    return specular * (1.0f - f) + mk(coat);
}

// shading.glsl:73-144
// With GIVEN, `given_grad` is density_gradient_cubic(A, idx), already known.
template <bool GIVEN = false>
__device__ __noinline__ float surface_frame(const PtArgs& A, f3 idx, const Sample& s, f3 v, int cap_plane, float cut,
                               float cap_depth, f3& n, float& surfaceness, f3 given_grad = f3{0.0f, 0.0f, 0.0f}) {
    uint32_t label_mode = (uint32_t)A.u.labels[0];
    float4 nw = normal_tri(A, idx);
    f3 nxyz = mk(nw.x, nw.y, nw.z);
    float n_len = len(nxyz);
    n = n_len > 1e-3f ? nxyz / n_len : mk(0.0f);
    surfaceness = nw.w;
    bool skin = s.label == SKIN_LABEL;
    if (A.u.env[1] > 0.5f && n_len > 1e-3f && (!s.ghost || skin)) {
        f3 gw = mul_t(w2i3(A), GIVEN ? given_grad : density_gradient_cubic(A, idx));
        float l = len(gw);
        n = l > 1e-7f ? -gw / l : n;
    }
    bool hollow = __ldg(&A.tab->density[s.label].w) < 0.0f;
    if (skin) {
    } else if (!s.ghost && label_mode == 3u && !hollow) {
        f3 g = mask_gradient(A, idx, 0);
        float g_len = len(g);
        f3 mask_n = g_len > 1e-5f ? -g / g_len : n;
        f3 blended = mix3(mask_n, n, surfaceness);
        n = len(blended) > 1e-3f ? normalize(blended) : mask_n;
        surfaceness = gmax(surfaceness, gclamp(g_len * 4.0f, 0.0f, 1.0f));
    } else if (!s.ghost && (label_mode >= 2u || (label_mode == 1u && mask_tri_ch(A, idx, 0) < 0.98f))) {
        f3 g = mask_gradient(A, idx, 0);
        float g_len = len(g);
        float mask_surface = gclamp(g_len * 4.0f, 0.0f, 1.0f);
        if (label_mode >= 2u || mask_surface > surfaceness) {
            n = g_len > 1e-5f ? -g / g_len : n;
            surfaceness = label_mode >= 2u ? mask_surface : gmax(surfaceness, mask_surface);
        }
    }
    if (cap_plane >= 0 && !s.ghost && -cut < cap_depth) {
        n = U3(A.u.clip_normals + 4 * cap_plane);
        surfaceness = 1.0f;
    }
    if (s.ghost) {
        f3 g = mask_gradient(A, idx, 1);
        float g_len = len(g);
        if (!skin || n_len <= 1e-3f) n = g_len > 1e-5f ? -g / g_len : n;
        surfaceness = gclamp(g_len * 4.0f, 0.0f, 1.0f);
        float edge_on = powf(1.0f - fabsf(dot(n, v)), 3.0f);
        return surfaceness * mixf(A.u.labels[3], 1.0f, edge_on);
    }
    return 1.0f;
}

// shading.glsl:147-168
__device__ __forceinline__ bool measured(const PtArgs& A, const Sample& s) {
    return A.u.labels[0] >= 2.0f && s.label != 0u && !s.ghost && __ldg(&A.tab->optics[s.label].w) > 0.0f;
}
__device__ __noinline__ f3 tissue_sigma(const PtArgs& A, const Sample& s) {
    float4 o = ldf4(&A.tab->optics[s.label]);
    f3 mu = mix3(mk(o.y), mk(o.x, o.y, o.z), A.u.env[3]);
    mu /= 1.0f - gclamp(A.u.env[2], 0.0f, 0.95f);
    mu *= gmin(1.0f, A.u.tissue[1] / gmax(maxc(mu), 1e-6f));
    float occupancy = gclamp(s.extinction / gmax(A.u.labels[2], 1e-6f), 0.0f, 1.0f);
    return occupancy * mu;
}

// shading.glsl:175-185 (pcg3d)
__device__ __forceinline__ f3 hash3(int cx, int cy, int cz) {
    uint32_t x = (uint32_t)cx * 1664525u + 1013904223u;
    uint32_t y = (uint32_t)cy * 1664525u + 1013904223u;
    uint32_t z = (uint32_t)cz * 1664525u + 1013904223u;
    x += y * z; y += z * x; z += x * y;
    x ^= x >> 16u; y ^= y >> 16u; z ^= z >> 16u;
    x += y * z; y += z * x; z += x * y;
    const float s = 1.0f / 4294967296.0f;
    return mk((float)x * s, (float)y * s, (float)z * s);
}
__device__ __forceinline__ float gradient_at(int cx, int cy, int cz, f3 off) {
    f3 h = hash3(cx, cy, cz);
    return dot(h * 2.0f - 1.0f, off);
}
// shading.glsl:192-202
__device__ __noinline__ float gradient_noise(f3 p) {
    float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
    int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    f3 f = mk(p.x - flx, p.y - fly, p.z - flz);
    f3 w = f * f * f * (f * (f * 6.0f - 15.0f) + 10.0f);
    float x00 = mixf(gradient_at(ix, iy, iz, f), gradient_at(ix + 1, iy, iz, f - mk(1, 0, 0)), w.x);
    float x10 = mixf(gradient_at(ix, iy + 1, iz, f - mk(0, 1, 0)), gradient_at(ix + 1, iy + 1, iz, f - mk(1, 1, 0)), w.x);
    float x01 = mixf(gradient_at(ix, iy, iz + 1, f - mk(0, 0, 1)), gradient_at(ix + 1, iy, iz + 1, f - mk(1, 0, 1)), w.x);
    float x11 = mixf(gradient_at(ix, iy + 1, iz + 1, f - mk(0, 1, 1)), gradient_at(ix + 1, iy + 1, iz + 1, f - mk(1, 1, 1)), w.x);
    return 1.7f * mixf(mixf(x00, x10, w.y), mixf(x01, x11, w.y), w.z);
}
__device__ float fbm(f3 p) {
    return (gradient_noise(p) + 0.5f * gradient_noise(p * 2.03f + 17.1f) + 0.25f * gradient_noise(p * 4.07f + 31.7f)) /
           1.75f;
}
// shading.glsl:213-237
__device__ __noinline__ void cellular(f3 p, float& nearest, float& border, int cell[3]) {
    float flx = floorf(p.x), fly = floorf(p.y), flz = floorf(p.z);
    int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    f3 f = mk(p.x - flx, p.y - fly, p.z - flz);
    f3 d1 = mk(8.0f), d2 = mk(8.0f);
    cell[0] = ix; cell[1] = iy; cell[2] = iz;
    for (int z = -1; z <= 1; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                f3 d = mk((float)x, (float)y, (float)z) + hash3(ix + x, iy + y, iz + z) - f;
                if (dot(d, d) < dot(d1, d1)) {
                    d2 = d1; d1 = d;
                    cell[0] = ix + x; cell[1] = iy + y; cell[2] = iz + z;
                } else if (dot(d, d) < dot(d2, d2)) {
                    d2 = d;
                }
            }
    nearest = len(d1);
    border = dot(0.5f * (d1 + d2), normalize(d2 - d1));
}
__device__ float lobule_border(f3 q, int lobule[3]) {
    f3 warp = mk(gradient_noise(q * 1.7f), gradient_noise(q * 1.7f + 5.2f), gradient_noise(q * 1.7f + 9.4f));
    float nearest, border;
    cellular(q + 0.2f * warp, nearest, border, lobule);
    return border;
}
__device__ __noinline__ float surface_height(f3 p, float4 params) {
    f3 q = p / params.w;
    if (params.x > 1.5f) {
        int lobule[3];
        float bulge = smoothstepf(0.0f, 0.35f, lobule_border(q, lobule));
        return 0.7f * bulge + 0.3f * fbm(q * 3.0f);
    }
    return 0.6f * fbm(q) + 0.4f * gradient_noise(q * 4.0f);
}
// shading.glsl:263-265: inverse(mat3(world_to_index)) * (idx - translation).
__device__ __noinline__ f3 index_to_world(const PtArgs& A, f3 idx) {
    m3 m = w2i3(A);
    float a00 = m.c0.x, a01 = m.c0.y, a02 = m.c0.z, a10 = m.c1.x, a11 = m.c1.y, a12 = m.c1.z;
    float a20 = m.c2.x, a21 = m.c2.y, a22 = m.c2.z;
    float b01 = a22 * a11 - a12 * a21, b11 = -a22 * a10 + a12 * a20, b21 = a21 * a10 - a11 * a20;
    float det = a00 * b01 + a01 * b11 + a02 * b21;
    m3 inv = {mk(b01, -a22 * a01 + a02 * a21, a12 * a01 - a02 * a11) / det,
              mk(b11, a22 * a00 - a02 * a20, -a12 * a00 + a02 * a10) / det,
              mk(b21, -a21 * a00 + a01 * a20, a11 * a00 - a01 * a10) / det};
    return mul(inv, idx - mk(A.u.w2i[12], A.u.w2i[13], A.u.w2i[14]));
}
__device__ __forceinline__ bool textured(const PtArgs& A, const Sample& s) {
    return s.label != 0u && !s.ghost && __ldg(&A.tab->surface[s.label].x) > 0.5f;
}
// shading.glsl:273-324
__device__ __noinline__ void apply_surface_texture(const PtArgs& A, f3 idx, Sample& s) {
    if (!textured(A, s)) return;
    float4 params = ldf4(&A.tab->surface[s.label]);
    float amount = params.y;
    f3 p = index_to_world(A, idx);
    f3 q = p / params.w;
    f3 tint;
    float wet, rough;
    if (params.x > 1.5f) {
        float strength = gmin(1.0f, 5.0f * amount);
        int lobule[3];
        float border = lobule_border(q, lobule);
        float septum = (1.0f - smoothstepf(0.0f, 0.06f, border)) * smoothstepf(-0.7f, 0.3f, gradient_noise(q * 6.0f));
        float near_septum = 1.0f - smoothstepf(0.0f, 0.2f, border);
        float patches = fbm(q * 1.5f);
        float mottle = fbm(q * 4.0f);
        tint = mk(1.0f + amount * (hash3(lobule[0], lobule[1], lobule[2]).x * 2.0f - 1.0f + 0.5f * mottle));
        tint *= mix3(mk(1.0f), mk(0.84f, 0.78f, 0.88f), strength * smoothstepf(-0.1f, 0.4f, -patches));
        tint *= mix3(mk(1.0f), mk(0.6f, 0.57f, 0.66f), strength * septum);
        float nearest, unused;
        int speck[3];
        cellular(p / 3.0f, nearest, unused, speck);
        f3 h = hash3(speck[0] + 7919, speck[1] + 7919, speck[2] + 7919);
        float speck_mask = (h.x < 0.03f + 0.4f * near_septum ? 1.0f : 0.0f) *
                           (1.0f - smoothstepf(0.12f, 0.2f, nearest / (0.6f + 0.8f * h.y)));
        tint *= mixf(1.0f, 0.2f, strength * speck_mask);
        wet = 1.0f - 0.3f * near_septum;
        rough = 1.0f + 0.2f * mottle;
    } else {
        float patches = fbm(q);
        float grain = gradient_noise(q * 4.0f);
        tint = mk(1.0f + amount * (0.7f * patches + 0.3f * grain));
        tint *= mix3(mk(1.0f), mk(0.97f, 0.94f, 1.0f), gclamp(-patches, 0.0f, 1.0f) * gmin(1.0f, 5.0f * amount));
        wet = gclamp(0.8f + 0.4f * patches, 0.4f, 1.2f);
        rough = 1.0f + 0.3f * grain;
    }
    s.albedo = gclamp(s.albedo * tint, 0.0f, 1.0f);
    s.roughness = gclamp(s.roughness * rough, 0.02f, 1.0f);
    s.coat = gclamp(s.coat * wet, 0.0f, 1.0f);
}
// shading.glsl:328-342
__device__ __noinline__ f3 bump_normal(const PtArgs& A, f3 idx, const Sample& s, f3 n) {
    if (!textured(A, s) || __ldg(&A.tab->surface[s.label].z) <= 0.0f || dot(n, n) < 0.5f) return n;
    float4 params = ldf4(&A.tab->surface[s.label]);
    f3 p = index_to_world(A, idx);
    float e = 0.02f * params.w;
    float h = surface_height(p, params);
    f3 g = mk(surface_height(p + mk(e, 0.0f, 0.0f), params) - h, surface_height(p + mk(0.0f, e, 0.0f), params) - h,
              surface_height(p + mk(0.0f, 0.0f, e), params) - h) *
           (params.z / e);
    return normalize(n - (g - dot(g, n) * n));
}

// ------------------------------------------------------------------ pt.comp
struct Rng {
    uint32_t s;
    __device__ __forceinline__ uint32_t pcg() {  // pt.comp:44-49
        uint32_t st = s;
        s = s * 747796405u + 2891336453u;
        uint32_t word = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
        return (word >> 22u) ^ word;
    }
    __device__ __forceinline__ float rand() { return (float)(pcg() >> 8) * (1.0f / 16777216.0f); }
};

// Per-launch constants derived from the uniforms (pt.comp:381-397).
struct Consts {
    m3 light_frame;
    f3 light_dir;
    float light;
    float cos_light, light_pdf;
    bool area_light;
    uint32_t volume_limit, max_bounces;
    float step_mm;
    f3 eye_idx;
};

__device__ __forceinline__ m3 basis(f3 n) {  // pt.comp:85-92
    float s = n.z >= 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (s + n.z);
    float b = n.x * n.y * a;
    return {mk(1.0f + s * n.x * n.x * a, s * b, -s * n.x), mk(b, s + n.y * n.y * a, -n.y), n};
}

__device__ __noinline__ Consts make_consts(const PtArgs& A) {
    Consts c;
    c.light_dir = U3(A.u.light_dir);
    c.light_frame = basis(c.light_dir);
    c.light = A.u.light_dir[3];
    c.cos_light = cosf(A.u.material[3]);
    c.area_light = A.u.material[3] > 1e-4f;
    c.light_pdf = c.area_light ? 1.0f / (2.0f * PI * (1.0f - c.cos_light)) : 0.0f;
    c.volume_limit = (uint32_t)((float)MAX_VOLUME_EVENTS / (1.0f - gclamp(A.u.env[2], 0.0f, 0.95f)));
    c.max_bounces = A.u.path[1];
    c.step_mm = A.u.dims[3];
    const float* m = A.u.w2i;
    f3 e = U3(A.u.eye);
    c.eye_idx = mk(m[0] * e.x + m[4] * e.y + m[8] * e.z + m[12], m[1] * e.x + m[5] * e.y + m[9] * e.z + m[13],
                   m[2] * e.x + m[6] * e.y + m[10] * e.z + m[14]);
    return c;
}

// common.glsl:459-481: light map coordinates of a world direction (the map is
// fixed to the camera: centre column ahead, top row above) and back.
__device__ __forceinline__ float2 env_uv(const PtArgs& A, f3 d) {
    f3 f = normalize(U3(A.u.forward)), r = normalize(U3(A.u.right)), up = normalize(U3(A.u.up));
    float phi = atan2f(dot(d, r), dot(d, f));
    float theta = acosf(gclamp(dot(d, up), -1.0f, 1.0f));
    float x = 0.5f + (phi + A.u.env[0]) / (2.0f * PI);
    return make_float2(x - floorf(x), theta / PI);
}
__device__ __forceinline__ f3 env_direction(const PtArgs& A, float2 uv) {
    float phi = (uv.x - 0.5f) * 2.0f * PI - A.u.env[0];
    float theta = uv.y * PI;
    f3 f = normalize(U3(A.u.forward)), r = normalize(U3(A.u.right)), up = normalize(U3(A.u.up));
    return sinf(theta) * (sinf(phi) * r + cosf(phi) * f) + cosf(theta) * up;
}
// common.glsl:483-486: the light map's radiance towards `d`, filtered as the
// sampler does (linear between texel centres, CLAMP_TO_EDGE, RGBA16F texels).
__device__ __noinline__ f3 env_map_radiance(const PtArgs& A, f3 d) {
    float2 uv = env_uv(A, d);
    float x = uv.x * (float)A.env_w - 0.5f, y = uv.y * (float)A.env_h - 0.5f;
    int i0 = (int)floorf(x), j0 = (int)floorf(y);
    float a = x - (float)i0, b = y - (float)j0;
    f3 c = mk(0.0f);
    for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
            int i = clampi(i0 + di, 0, A.env_w - 1), j = clampi(j0 + dj, 0, A.env_h - 1);
            ushort4 t = __ldg(A.env_rad + (long)j * A.env_w + i);
            float w = (di ? a : 1.0f - a) * (dj ? b : 1.0f - b);
            c += mk(__half2float(__ushort_as_half(t.x)), __half2float(__ushort_as_half(t.y)),
                    __half2float(__ushort_as_half(t.z))) * w;
        }
    return U3(A.u.ambient) * c;
}
// pt.comp:193-200: solid-angle pdf of light map direction `d`.
__device__ __noinline__ float env_pdf(const PtArgs& A, f3 d) {
    float2 uv = env_uv(A, d);
    int tx = min((int)(uv.x * (float)A.env_w), A.env_w - 1), ty = min((int)(uv.y * (float)A.env_h), A.env_h - 1);
    float p = __ldg(&A.env_table[(long)ty * (A.env_w + 1) + tx].y);
    return p * (float)(A.env_w * A.env_h) / (2.0f * PI * PI * gmax(sinf(uv.y * PI), 1e-6f));
}

// pt.comp:56-82
__device__ __noinline__ f3 environment(const PtArgs& A, f3 d) {
    if (A.u.lighting[3] == 2u) return env_map_radiance(A, d);
    f3 amb = U3(A.u.ambient);
    if (A.u.lighting[3] >= 1u) {
        f3 f = normalize(U3(A.u.forward)), r = normalize(U3(A.u.right)), up = normalize(U3(A.u.up));
        float key_side = dot(U3(A.u.light_dir), r) >= 0.0f ? 1.0f : -1.0f;
        f3 fill = normalize(-f - 0.9f * key_side * r - 0.1f * up);
        f3 rim = normalize(f + 0.8f * up - 0.4f * key_side * r);
        float fill_lobe = 0.5f * powf(gmax(dot(d, fill), 0.0f), 6.0f);
        float rim_lobe = 2.5f * powf(gmax(dot(d, rim), 0.0f), 24.0f);
        f3 studio = mk(0.02f) + fill_lobe * mk(0.95f, 0.98f, 1.05f) + rim_lobe * mk(0.9f, 0.95f, 1.1f);
        return amb * studio * (1.0f / 0.106f);
    }
    float up = 0.5f + 0.5f * d.z;
    return amb * mix3(mk(1.04f, 1.0f, 0.94f) * 0.35f, mk(0.92f, 0.96f, 1.04f), up) / 0.675f;
}

__device__ __forceinline__ f3 sample_light(const PtArgs& A, const Consts& C, Rng& rng) {
    float cos_t = mixf(C.cos_light, 1.0f, rng.rand());
    float sin_t = sqrtf(gmax(0.0f, 1.0f - cos_t * cos_t));
    float phi = 2.0f * PI * rng.rand();
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return mul(C.light_frame, mk(sin_t * cp, sin_t * sp, cos_t));
}

// pt.comp:204-223: the light map texel drawn by luminance x solid angle:
// binary search of the marginal CDF over rows, then of the row's conditional
// CDF. Each search starts from its guide bucket's range (PtArgs::env_guide),
// which holds the index the search over the whole CDF finds.
__device__ __forceinline__ void env_texel(const PtArgs& A, Rng& rng, int& x, int& y) {
    const int W = A.env_w;
    const float2* T = A.env_table;
    const uint16_t* G = A.env_guide;
    float xi = rng.rand();
    int k = (int)(xi * (float)A.env_gm);
    int lo = __ldg(G + k), hi = __ldg(G + k + 1);
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (__ldg(&T[(long)mid * (W + 1) + W].x) >= xi) hi = mid;
        else lo = mid + 1;
    }
    y = lo;
    xi = rng.rand();
    const uint16_t* g = G + (A.env_gm + 1) + (long)y * (A.env_gr + 1);
    k = (int)(xi * (float)A.env_gr);
    lo = __ldg(g + k);
    hi = __ldg(g + k + 1);
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (__ldg(&T[(long)y * (W + 1) + mid].x) >= xi) hi = mid;
        else lo = mid + 1;
    }
    x = lo;
}
// pt.comp:204-233: a direction towards the light map: the texel, then a
// uniform point in it, with its solid-angle pdf.
__device__ __noinline__ f3 sample_env(const PtArgs& A, Rng& rng, float& pdf) {
    const int W = A.env_w, H = A.env_h;
    int x, y;
    env_texel(A, rng, x, y);
    float jx = rng.rand();
    float jy = rng.rand();
    float2 uv = make_float2(((float)x + jx) / (float)W, ((float)y + jy) / (float)H);
    float p = __ldg(&A.env_table[(long)y * (W + 1) + x].y);
    pdf = p * (float)(W * H) / (2.0f * PI * PI * gmax(sinf(uv.y * PI), 1e-6f));
    return env_direction(A, uv);
}
__device__ __forceinline__ f3 single_scattering_albedo(f3 a) {
    a = gclamp(a, 0.0f, 0.999f);
    f3 s = mk(4.09712f) + 4.20863f * a - mk(sqrtf(9.59217f + 41.6808f * a.x + 17.7126f * a.x * a.x),
                                            sqrtf(9.59217f + 41.6808f * a.y + 17.7126f * a.y * a.y),
                                            sqrtf(9.59217f + 41.6808f * a.z + 17.7126f * a.z * a.z));
    return 1.0f - s * s;
}
__device__ __forceinline__ f3 chroma(const PtArgs& A, const Sample& s) {
    if (s.ghost) return mk(1.0f);
    return mix3(mk(1.0f), mk(0.62f, 0.77f, 1.0f), gclamp(2.0f * s.subsurface, 0.0f, 1.0f) * A.u.env[3]);
}
__device__ __forceinline__ f3 path_sigma(const PtArgs& A, const Sample& s, float ext) {
    return measured(A, s) ? tissue_sigma(A, s) : ext * chroma(A, s);
}
__device__ __forceinline__ f3 event_albedo(const PtArgs& A, const Sample& s) {
    f3 reduced = single_scattering_albedo(s.albedo);
    return measured(A, s) ? 1.0f - (1.0f - reduced) * (1.0f - gclamp(A.u.env[2], 0.0f, 0.95f)) : reduced;
}
// flight_majorant (pt.comp:157-163) of brick `b` (brick_index).
__device__ __forceinline__ float flight_majorant_of(const PtArgs& A, int b) {
    float m = 1e30f;
    if (A.u.path[3] != 0u) {
        count(A, COUNT_MAJORANT);
        m = __ldg(A.majorant + b);
    }
    if (m > 0.0f && A.u.labels[0] >= 2.0f) m = gmax(m, A.u.tissue[0]);
    return gmin(m, gmax(MAX_EXTINCTION, gmax(A.u.labels[2], A.u.tissue[0])));
}
__device__ __forceinline__ float phase_hg(const PtArgs& A, float cos_t) {
    float g = A.u.env[2];
    float d = 1.0f + g * g - 2.0f * g * cos_t;
    return (1.0f - g * g) / (4.0f * PI * d * sqrtf(gmax(d, 1e-8f)));
}
__device__ __noinline__ f3 sample_hg(const PtArgs& A, f3 dir, Rng& rng) {
    float g = A.u.env[2];
    float cos_t;
    if (fabsf(g) < 1e-3f) {
        cos_t = 1.0f - 2.0f * rng.rand();
    } else {
        float q = (1.0f - g * g) / (1.0f - g + 2.0f * g * rng.rand());
        cos_t = gclamp((1.0f + g * g - q * q) / (2.0f * g), -1.0f, 1.0f);
    }
    float sin_t = sqrtf(gmax(0.0f, 1.0f - cos_t * cos_t));
    float phi = 2.0f * PI * rng.rand();
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return mul(basis(dir), mk(sin_t * cp, sin_t * sp, cos_t));
}
__device__ __forceinline__ float mis(float a, float b) { return a * a / gmax(a * a + b * b, 1e-20f); }
__device__ __forceinline__ float coat_share(const Sample& s) { return 0.5f * s.coat; }
__device__ __forceinline__ float specular_share(const Sample& s) { return mixf(0.2f, 1.0f, s.metalness); }
__device__ __forceinline__ float ggx_pdf(f3 n, f3 v, f3 l, float a) {
    f3 h = normalize(v + l);
    float nh = gmax(dot(n, h), 0.0f);
    return ggx_distribution(nh, a * a) * nh / (4.0f * gmax(dot(v, h), 1e-4f));
}
__device__ __noinline__ f3 sample_ggx(const m3& frame, f3 v, float a, Rng& rng) {
    float a2 = a * a;
    float phi = 2.0f * PI * rng.rand();
    float xi = rng.rand();
    float cos_t = sqrtf((1.0f - xi) / (1.0f + (a2 - 1.0f) * xi));
    float sin_t = sqrtf(gmax(0.0f, 1.0f - cos_t * cos_t));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    f3 h = mul(frame, mk(sin_t * cp, sin_t * sp, cos_t));
    f3 i = -v;
    return i - 2.0f * dot(h, i) * h;
}
__device__ __noinline__ float bsdf_pdf(f3 n, f3 v, f3 l, const Sample& s) {
    float nl = dot(n, l);
    if (nl <= 0.0f) return 0.0f;
    float a = gmax(s.roughness * s.roughness, 2e-3f);
    float share = specular_share(s);
    float base = share * ggx_pdf(n, v, l, a) + (1.0f - share) * nl / PI;
    float coat = coat_share(s);
    float cr = coat_roughness(s);
    return coat * ggx_pdf(n, v, l, cr * cr) + (1.0f - coat) * base;
}

// pt.comp:277-292
// extinction_at (pt.comp:277-292) after its clip test: the caller has found
// `idx` inside the kept part (cut = clip_depth(idx) <= 0).
__device__ __noinline__ float extinction_unclipped(const PtArgs& A, f3 idx, f3 dir, bool smooth, Sample& s, int& cap_plane,
                                      float& cut) {
    float d = (smooth && A.u.env[1] > 0.5f) ? density_cubic(A, idx) : density_tri(A, idx);
    s = apply_labels(A, tf_point(A, d), idx);
    if (s.extinction <= 0.0f) return 0.0f;
    if (s.ghost) {
        f3 n;
        float surf;
        return s.extinction * surface_frame(A, idx, s, -dir, cap_plane, cut, 0.0f, n, surf);
    }
    return s.extinction;
}

// pt.comp:300-334: delta tracking against the brick majorants, hero channel,
// as a resumable loop: ff_begin sets up the ray, each ff_step is one iteration.
struct Flight {
    f3 d_idx, inv_d;
    float tt, t_end;
    int iter;
    int brick;    // brick whose flight majorant `maj` holds (-1: none yet)
    float maj;
};
enum { FF_CONTINUE = 0, FF_HIT = 1, FF_ESCAPE = 2 };

__device__ __forceinline__ void ff_begin(const PtArgs& A, f3 origin, f3 dir, Flight& F) {
    F.d_idx = mul(w2i3(A), dir);
    float2 tr = intersect_volume(A, origin, F.d_idx);
    F.inv_d = brick_inv_dir(F.d_idx);
    F.tt = tr.x;
    F.t_end = tr.y;
    F.iter = 0;
    F.brick = -1;
}

__device__ __forceinline__ int ff_step(const PtArgs& A, f3 origin, f3 dir, bool smooth, int hero, f3& spectral,
                                       Flight& F, f3& idx, Sample& s, int& cap_plane, float& cut, Rng& rng) {
    // The iterations of pt.comp:307-333 that fetch no voxel run back to back:
    // empty bricks, samples beyond the brick exit, and tentative collisions in
    // the clipped part (extinction_at returns 0 there before any fetch). The
    // step ends at the first tentative collision that needs the volume. The
    // majorant of the brick the ray is in is fetched once per brick.
    float majorant;
    for (;;) {
        if (!(F.iter < 4096 && F.tt < F.t_end)) return FF_ESCAPE;
        f3 p = origin + F.d_idx * F.tt;
        int b = brick_index(A, p);
        if (b != F.brick) {
            F.brick = b;
            F.maj = flight_majorant_of(A, b);
        }
        F.iter++;
        majorant = F.maj;
        float exit = F.tt + brick_exit(p, F.inv_d) + 1e-3f;
        if (majorant <= 0.0f) {
            F.tt = exit;
            continue;
        }
        float next = F.tt - logf(1.0f - rng.rand()) / majorant;
        if (next >= exit) {
            F.tt = exit;
            continue;
        }
        F.tt = next;
        idx = origin + F.d_idx * F.tt;
        cut = clip_depth(A, idx, cap_plane);
        if (cut <= 0.0f) break;
    }
    float ext = extinction_unclipped(A, idx, dir, smooth, s, cap_plane, cut);
    if (ext <= 0.0f) return FF_CONTINUE;
    f3 sigma = path_sigma(A, s, ext);
    float sh = comp(sigma, hero);
    if (rng.rand() * majorant < sh) {
        spectral *= sigma / sh;
        return FF_HIT;
    }
    spectral *= gmax(majorant - sigma, 0.0f) / (majorant - sh);
    return FF_CONTINUE;
}

__device__ bool free_flight(const PtArgs& A, f3 origin, f3 dir, bool smooth, int hero, f3& spectral, f3& idx,
                            Sample& s, int& cap_plane, float& cut, Rng& rng) {
    Flight F;
    ff_begin(A, origin, dir, F);
    for (;;) {
        int r = ff_step(A, origin, dir, smooth, hero, spectral, F, idx, s, cap_plane, cut, rng);
        if (r == FF_HIT) return true;
        if (r == FF_ESCAPE) return false;
    }
}

// pt.comp:339-371 as a resumable loop: tr_begin sets up the shadow ray, each
// tr_step is one iteration; the estimate is in Shadow::result.
struct Shadow {
    f3 d_idx, inv_d, result;
    float tt, t_end;
    int iter;
};
__device__ __forceinline__ void tr_begin(const PtArgs& A, f3 origin, f3 dir, Shadow& T) {
    T.d_idx = mul(w2i3(A), dir);
    float2 tr = intersect_volume(A, origin, T.d_idx);
    T.inv_d = brick_inv_dir(T.d_idx);
    T.tt = tr.x;
    T.t_end = tr.y;
    T.iter = 0;
    T.result = mk(1.0f);
}
// Returns false when the estimate is final.
__device__ __forceinline__ bool tr_step(const PtArgs& A, f3 origin, Shadow& T, Rng& rng) {
    // One iteration of pt.comp:345-370 per call. Samples in the clipped part
    // need no fetch: sample_point's extinction is 0 there, path_sigma is 0 and
    // the estimate is multiplied by exactly 1.
    if (!(T.iter < 4096 && T.tt < T.t_end)) return false;
    T.iter++;
    float peak = maxc(T.result);
    if (peak < 0.1f) {
        if (rng.rand() * 0.1f >= peak) {
            T.result = mk(0.0f);
            return false;
        }
        T.result *= 0.1f / peak;
    }
    f3 p = origin + T.d_idx * T.tt;
    float majorant = flight_majorant_of(A, brick_index(A, p));
    float exit = T.tt + brick_exit(p, T.inv_d) + 1e-3f;
    if (majorant <= 0.0f) {
        T.tt = exit;
        return true;
    }
    float next = T.tt - logf(1.0f - rng.rand()) / majorant;
    if (next >= exit) {
        T.tt = exit;
        return true;
    }
    T.tt = next;
    f3 q = origin + T.d_idx * T.tt;
    int plane;
    if (clip_depth(A, q, plane) > 0.0f) return true;
    Sample m = sample_point_unclipped(A, q);
    T.result *= gmax(1.0f - path_sigma(A, m, m.extinction) / majorant, 0.0f);
    return true;
}

// pt.comp:339-371: ratio tracking with Russian roulette.
__device__ __noinline__ f3 transmittance(const PtArgs& A, f3 origin, f3 dir, Rng& rng) {
    Shadow T;
    tr_begin(A, origin, dir, T);
    while (tr_step(A, origin, T, rng)) {
    }
    return T.result;
}

// ------------------------------------------------------------- path state
struct Path {
    Rng rng;
    f3 origin, dir, throughput, radiance, spectral;
    float last_pdf;
    int hero;
    uint32_t bounce, surfaces, volumes;
};
struct PixelSums {
    f3 sum;
    float background;
    float4 albedo, normal;
};

// pt.comp:404-426: camera ray (with thin lens) and the path's initial state.
__device__ __noinline__ void start_path(const PtArgs& A, const Consts& C, Path& P, uint32_t px, uint32_t py) {
    count(A, COUNT_PATH);
    float jx = P.rng.rand();
    float jy = P.rng.rand();
    float nx = ((float)px + jx) / (float)A.u.flags[2] * 2.0f - 1.0f;
    float ny = ((float)py + jy) / (float)A.u.flags[3] * 2.0f - 1.0f;
    f3 dir = normalize(U3(A.u.forward) + nx * U3(A.u.right) - ny * U3(A.u.up));
    f3 origin = C.eye_idx;
    if (A.u.lens[0] > 0.0f) {
        f3 eye = U3(A.u.eye);
        f3 focal = eye + dir * (A.u.lens[1] / dot(dir, normalize(U3(A.u.forward))));
        float r = A.u.lens[0] * sqrtf(P.rng.rand());
        float phi = 2.0f * PI * P.rng.rand();
        float sp, cp;
        sincosf(phi, &sp, &cp);
        eye += r * (cp * normalize(U3(A.u.right)) + sp * normalize(U3(A.u.up)));
        dir = normalize(focal - eye);
        const float* m = A.u.w2i;
        origin = mk(m[0] * eye.x + m[4] * eye.y + m[8] * eye.z + m[12], m[1] * eye.x + m[5] * eye.y + m[9] * eye.z + m[13],
                    m[2] * eye.x + m[6] * eye.y + m[10] * eye.z + m[14]);
    }
    P.origin = origin;
    P.dir = dir;
    P.throughput = mk(1.0f);
    P.radiance = mk(0.0f);
    P.hero = min((int)(P.rng.rand() * 3.0f), 2);
    P.spectral = mk(1.0f);
    P.last_pdf = 0.0f;
    P.bounce = 0u;
    P.surfaces = 0u;
    P.volumes = 0u;
}

// What one scattering vertex carries from stage to stage.
struct Vertex {
    f3 idx;
    Sample s;
    int cap_plane;
    float cut;
    f3 n;
    bool surface_event;
    f3 light_dir;
    f3 light_t;
    f3 map_dir, map_light;  // the light map's sample (lighting.w == 2), map_light / pdf x transmittance
    float map_pdf;          // 0: no light map sample
};

// The bounce loop (pt.comp:427-545) in four stages, in the order the
// reference consumes random numbers: extend (free flight) / shade up to the
// light sample / shadow ray / shade after it. bounce_step runs them in one
// go; the wavefront kernels run each stage over a queue of paths.

// Stage 1: the loop condition and free flight (pt.comp:427-433). Returns true
// at a scattering vertex; false when the path leaves the loop (`escaped` tells
// whether free flight left the volume, see stage_escape).
__device__ __forceinline__ bool stage_extend(const PtArgs& A, const Consts& C, Path& P, Vertex& V, bool& escaped) {
    escaped = false;
    if (!(P.surfaces <= C.max_bounces && P.volumes <= C.volume_limit)) return false;
    count(A, COUNT_VERTEX);
    if (free_flight(A, P.origin, P.dir, P.bounce == 0u, P.hero, P.spectral, V.idx, V.s, V.cap_plane, V.cut, P.rng))
        return true;
    escaped = true;
    return false;
}

// A path that left the volume: background coverage at the first bounce, else
// the environment and the key light, MIS-weighted (pt.comp:434-446).
__device__ __noinline__ void stage_escape(const PtArgs& A, const Consts& C, Path& P, PixelSums& S) {
    if (P.bounce == 0u) {
        S.background += 1.0f;
        S.albedo.x += 1.0f; S.albedo.y += 1.0f; S.albedo.z += 1.0f;
        S.normal.w += 1e4f;
    } else {
        float weight = A.u.lighting[3] == 2u ? mis(P.last_pdf, env_pdf(A, P.dir)) : 1.0f;
        f3 path_weight = P.throughput * P.spectral / dot(P.spectral, mk(1.0f / 3.0f));
        P.radiance += path_weight * environment(A, P.dir) * weight;
        if (C.area_light && dot(P.dir, C.light_dir) >= C.cos_light)
            P.radiance += path_weight * (C.light * C.light_pdf * mis(P.last_pdf, C.light_pdf));
    }
}

// Stage 2: surface frame, texture, event choice, guides, light sample (pt.comp:448-465).
__device__ __noinline__ void stage_shade(const PtArgs& A, const Consts& C, Path& P, PixelSums& S, Vertex& V) {
    f3 v = -P.dir;
    float surfaceness;
    surface_frame(A, V.idx, V.s, v, V.cap_plane, V.cut, 1.5f * C.step_mm, V.n, surfaceness);
    apply_surface_texture(A, V.idx, V.s);
    V.surface_event = P.rng.rand() < surfaceness * (1.0f - V.s.subsurface) && dot(V.n, V.n) > 0.5f;
    if (V.surface_event || P.bounce == 0u) V.n = bump_normal(A, V.idx, V.s, V.n);
    if (P.bounce == 0u) {
        S.albedo.x += V.s.albedo.x; S.albedo.y += V.s.albedo.y; S.albedo.z += V.s.albedo.z;
        f3 nn = dot(V.n, v) < 0.0f ? -V.n : V.n;
        S.normal.x += nn.x; S.normal.y += nn.y; S.normal.z += nn.z;
        S.normal.w += len(V.idx - C.eye_idx);
    }
    V.light_dir = sample_light(A, C, P.rng);
}

// The light map's next-event sample after the key light's shadow ray
// (pt.comp:467-476), before its own shadow ray.
__device__ __noinline__ void sample_map_light(const PtArgs& A, Rng& rng, Vertex& V) {
    V.map_dir = sample_env(A, rng, V.map_pdf);
    V.map_light = env_map_radiance(A, V.map_dir) / gmax(V.map_pdf, 1e-8f);
}
__device__ __noinline__ void map_shadow(const PtArgs& A, Path& P, Vertex& V) {
    sample_map_light(A, P.rng, V);
    if (V.map_pdf > 0.0f) V.map_light *= transmittance(A, V.idx, V.map_dir, P.rng);
}

// Stage 3: the shadow rays towards the light sample and the light map's
// sample (pt.comp:466-476).
__device__ __forceinline__ void stage_shadow(const PtArgs& A, Path& P, Vertex& V) {
    V.light_t = transmittance(A, V.idx, V.light_dir, P.rng);
    V.map_pdf = 0.0f;
    V.map_dir = mk(0.0f);
    V.map_light = mk(0.0f);
    if (A.u.lighting[3] == 2u) map_shadow(A, P, V);
}

// The light map's next-event contributions (pt.comp:484-488, 525-528).
__device__ __noinline__ f3 map_surface_term(const Vertex& V, f3 n, f3 v, f3 path_weight) {
    f3 diffuse;
    f3 specular = brdf_coated(n, v, V.map_dir, V.s, diffuse);
    return path_weight * (diffuse + specular) * dot(n, V.map_dir) * V.map_light *
           mis(V.map_pdf, bsdf_pdf(n, v, V.map_dir, V.s));
}
__device__ __noinline__ f3 map_volume_term(const PtArgs& A, const Vertex& V, f3 dir, f3 path_weight, f3 albedo) {
    float phase = phase_hg(A, dot(dir, V.map_dir));
    return path_weight * albedo * phase * V.map_light * mis(V.map_pdf, phase);
}

// Stage 4: light contribution, next direction, Russian roulette (pt.comp:478-545).
// Returns true when the path continues.
__device__ __noinline__ bool stage_scatter(const PtArgs& A, const Consts& C, Path& P, Vertex& V) {
    f3 path_weight = P.throughput * P.spectral / dot(P.spectral, mk(1.0f / 3.0f));
    f3 v = -P.dir;
    const Sample& s = V.s;
    if (V.surface_event) {
        f3 n = dot(V.n, v) < 0.0f ? -V.n : V.n;
        f3 diffuse;
        f3 specular = brdf_coated(n, v, V.light_dir, s, diffuse);
        float light_weight = C.area_light ? mis(C.light_pdf, bsdf_pdf(n, v, V.light_dir, s)) : 1.0f;
        P.radiance += path_weight * (diffuse + specular) * (gmax(dot(n, V.light_dir), 0.0f) * C.light) * V.light_t *
                      light_weight;
        if (V.map_pdf > 0.0f && dot(n, V.map_dir) > 0.0f) P.radiance += map_surface_term(V, n, v, path_weight);
        m3 frame = basis(n);
        f3 l;
        if (P.rng.rand() < coat_share(s)) {
            float cr = coat_roughness(s);
            l = sample_ggx(frame, v, cr * cr, P.rng);
        } else if (P.rng.rand() < specular_share(s)) {
            l = sample_ggx(frame, v, gmax(s.roughness * s.roughness, 2e-3f), P.rng);
        } else {
            float r = sqrtf(P.rng.rand());
            float phi = 2.0f * PI * P.rng.rand();
            float sp, cp;
            sincosf(phi, &sp, &cp);
            l = mul(frame, mk(r * cp, r * sp, sqrtf(gmax(0.0f, 1.0f - r * r))));
        }
        float nl = dot(n, l);
        if (nl <= 0.0f) return false;
        float pdf = bsdf_pdf(n, v, l, s);
        specular = brdf_coated(n, v, l, s, diffuse);
        P.throughput *= (diffuse + specular) * (nl / gmax(pdf, 1e-6f));
        P.last_pdf = pdf;
        P.surfaces++;
        P.origin = V.idx + mul(w2i3(A), n * C.step_mm);
        P.dir = l;
    } else {
        f3 albedo = event_albedo(A, s);
        float light_phase = phase_hg(A, dot(P.dir, V.light_dir));
        P.radiance += path_weight * albedo * (light_phase * C.light) * V.light_t *
                      (C.area_light ? mis(C.light_pdf, light_phase) : 1.0f);
        if (V.map_pdf > 0.0f) P.radiance += map_volume_term(A, V, P.dir, path_weight, albedo);
        P.throughput *= albedo;
        P.volumes++;
        P.origin = V.idx;
        f3 next = sample_hg(A, P.dir, P.rng);
        P.last_pdf = phase_hg(A, dot(P.dir, next));
        P.dir = next;
    }
    if (P.bounce >= 2u) {
        f3 w = P.throughput * P.spectral / dot(P.spectral, mk(1.0f / 3.0f));
        float survive = gclamp(maxc(w), 0.05f, 1.0f);
        if (P.rng.rand() > survive) return false;
        P.throughput /= survive;
    }
    P.bounce++;
    return true;
}

// One iteration of the bounce loop (pt.comp:427-545). Returns false when the
// path ends (a `break`, or the loop condition fails next).
__device__ bool bounce_step(const PtArgs& A, const Consts& C, Path& P, PixelSums& S) {
    Vertex V;
    bool escaped;
    if (!stage_extend(A, C, P, V, escaped)) {
        if (escaped) stage_escape(A, C, P, S);
        return false;
    }
    stage_shade(A, C, P, S, V);
    stage_shadow(A, P, V);
    return stage_scatter(A, C, P, V);
}

// pt.comp:546-551: firefly clamp and the luminance^2 guide.
__device__ __forceinline__ void finish_path(Path& P, PixelSums& S) {
    float peak = maxc(P.radiance);
    f3 r = peak > 20.0f ? P.radiance * (20.0f / peak) : P.radiance;
    S.sum += r;
    float lum = dot(r, mk(0.2126f, 0.7152f, 0.0722f));
    S.albedo.w += lum * lum;
}

__device__ __forceinline__ uint32_t seed_of(uint32_t px, uint32_t py, uint32_t accumulated) {
    return (px * 1973u + py * 9277u + accumulated * 26699u) | 1u;
}

__device__ __forceinline__ ushort4 to_half4(float4 v) {
    return make_ushort4(__half_as_ushort(__float2half_rn(v.x)), __half_as_ushort(__float2half_rn(v.y)),
                        __half_as_ushort(__float2half_rn(v.z)), __half_as_ushort(__float2half_rn(v.w)));
}

// pt.comp:554-560: add the pixel's sums to the accumulation images. With
// several frames in flight for one pixel the adds are atomic.
__device__ void accumulate(const PtArgs& A, uint32_t px, uint32_t py, const PixelSums& S, bool atomic_add,
                           bool write_hdr, float n_total) {
    count(A, COUNT_PIXEL);
    long i = (long)py * A.width + px;
    float4 acc = make_float4(S.sum.x, S.sum.y, S.sum.z, S.background);
    if (atomic_add) {
        atomicAdd(&A.accum[i], acc);
        atomicAdd(&A.albedo[i], S.albedo);
        atomicAdd(&A.normal[i], S.normal);
    } else {
        float4 a = A.accum[i], b = A.albedo[i], c = A.normal[i];
        a = make_float4(a.x + acc.x, a.y + acc.y, a.z + acc.z, a.w + acc.w);
        A.accum[i] = a;
        A.albedo[i] = make_float4(b.x + S.albedo.x, b.y + S.albedo.y, b.z + S.albedo.z, b.w + S.albedo.w);
        A.normal[i] = make_float4(c.x + S.normal.x, c.y + S.normal.y, c.z + S.normal.z, c.w + S.normal.w);
        if (write_hdr) A.hdr[i] = to_half4(make_float4(a.x / n_total, a.y / n_total, a.z / n_total, a.w / n_total));
    }
}

}  // namespace
}  // namespace vv
