// vv_post.cu — what runs after the accumulate-frame: the edge-avoiding a-trous
// denoiser (shaders/denoise.comp, renderer.rs:1868-1904) and the camera
// finishing + tone mapping of the readback (shaders/bloom.comp,
// shaders/tonemap.comp, renderer.rs:1817-1866).
//
// All images are pixel-linear RGBA (float4 accumulation and denoiser
// ping/pong, half4 HDR and bloom images, uchar4 output). Each pass is an
// L2/HBM-bound stencil over a 1024^2 image (16 MiB per float4 image).
#include <cuda_runtime.h>

#include "vv_device.cuh"
#include "vv_kernels.h"

namespace vv {

__device__ __forceinline__ float lum(float r, float g, float b) { return r * 0.2126f + g * 0.7152f + b * 0.0722f; }
__device__ __forceinline__ float4 h4(ushort4 v) {
    return make_float4(__half2float(__ushort_as_half(v.x)), __half2float(__ushort_as_half(v.y)),
                       __half2float(__ushort_as_half(v.z)), __half2float(__ushort_as_half(v.w)));
}
__device__ __forceinline__ ushort4 to_h4(float4 v) {
    return make_ushort4(__half_as_ushort(__float2half_rn(v.x)), __half_as_ushort(__float2half_rn(v.y)),
                        __half_as_ushort(__float2half_rn(v.z)), __half_as_ushort(__float2half_rn(v.w)));
}
__device__ __forceinline__ float samples_of(const PostArgs& a) { return (float)(a.u.path[0] + a.u.path[2]); }

__device__ __forceinline__ f3 mean_albedo(const PostArgs& a, int i, float n) {
    float4 g = a.albedo[i];
    return mk(gmax(g.x / n, 0.02f), gmax(g.y / n, 0.02f), gmax(g.z / n, 0.02f));
}
__device__ __forceinline__ float4 mean_normal_depth(const PostArgs& a, int i, float n) {
    float4 g = a.normal[i];
    f3 v = mk(g.x / n, g.y / n, g.z / n);
    float l = len(v);
    f3 nn = l > 1e-3f ? v / l : mk(0.0f);
    return make_float4(nn.x, nn.y, nn.z, g.w / n);
}

// denoise.comp:62-86 (pass 0): demodulated irradiance and its variance.
__global__ void k_denoise_prepare(const PostArgs a) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    int W = (int)a.width, H = (int)a.height;
    if (x >= W || y >= H) return;
    float n = samples_of(a);
    int i = y * W + x;
    float4 acc = a.accum[i];
    f3 radiance = mk(acc.x / n, acc.y / n, acc.z / n);
    f3 alb = mean_albedo(a, i, n);
    f3 irr = radiance / alb;
    float l = lum(radiance.x, radiance.y, radiance.z);
    float temporal = gmax(a.albedo[i].w / n - l * l, 0.0f) / n;
    float s1 = 0.0f, s2 = 0.0f;
    for (int dy = -2; dy <= 2; dy++)
        for (int dx = -2; dx <= 2; dx++) {
            int qx = clampi(x + dx, 0, W - 1), qy = clampi(y + dy, 0, H - 1);
            float4 q = a.accum[qy * W + qx];
            float lq = lum(q.x / n, q.y / n, q.z / n);
            s1 += lq;
            s2 += lq * lq;
        }
    float spatial = gmax(s2 / 25.0f - (s1 / 25.0f) * (s1 / 25.0f), 0.0f);
    float variance = gmax(temporal, spatial * gmin(1.0f, 4.0f / n));
    // The edge-stopping guides every level reads at every tap, computed once.
    a.guide_nd[i] = mean_normal_depth(a, i, n);
    a.guide_alb[i] = make_float4(alb.x, alb.y, alb.z, 0.0f);
    float al = lum(alb.x, alb.y, alb.z);
    a.ping[i] = make_float4(irr.x, irr.y, irr.z, variance / (al * al));
}

// denoise.comp:96-144: one a-trous level, 5x5 B3 taps `step` pixels apart.
__global__ void k_denoise_level(const PostArgs a, int step, int from_pong) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    int W = (int)a.width, H = (int)a.height;
    if (x >= W || y >= H) return;
    const float4* src = from_pong ? a.pong : a.ping;
    float4* dst = from_pong ? a.ping : a.pong;
    int i = y * W + x;
    float4 center = src[i];
    float4 geo = a.guide_nd[i];
    f3 gxyz = mk(geo.x, geo.y, geo.z);
    float4 ga = a.guide_alb[i];
    f3 alb = mk(ga.x, ga.y, ga.z);
    float l_center = lum(center.x, center.y, center.z);
    float bv = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
            int qx = clampi(x + dx, 0, W - 1), qy = clampi(y + dy, 0, H - 1);
            bv += src[qy * W + qx].w * (float)((2 - abs(dx)) * (2 - abs(dy))) / 16.0f;
        }
    float sigma_l = 4.0f * sqrtf(gmax(bv, 0.0f)) + 1e-4f;
    const float kernel[3] = {3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
    f3 sum = mk(0.0f);
    float variance = 0.0f, weights = 0.0f;
    bool center_flat = dot(gxyz, gxyz) < 0.5f;
    for (int dy = -2; dy <= 2; dy++)
        for (int dx = -2; dx <= 2; dx++) {
            int qx = x + dx * step, qy = y + dy * step;
            if (qx < 0 || qy < 0 || qx >= W || qy >= H) continue;
            int j = qy * W + qx;
            float4 c = src[j];
            float4 g = a.guide_nd[j];
            f3 gq = mk(g.x, g.y, g.z);
            float w_normal = powf(gmax(dot(gxyz, gq), 0.0f), 64.0f);
            bool q_flat = dot(gq, gq) < 0.5f;
            if (center_flat || q_flat) w_normal = (center_flat && q_flat) ? 1.0f : 0.0f;
            float w_depth = expf(-fabsf(geo.w - g.w) / (0.02f * geo.w + 1e-3f));
            float4 gb = a.guide_alb[j];
            f3 da = alb - mk(gb.x, gb.y, gb.z);
            float w_albedo = expf(-dot(da, da) / 0.01f);
            float w_lum = expf(-fabsf(l_center - lum(c.x, c.y, c.z)) / sigma_l);
            float w = kernel[abs(dx)] * kernel[abs(dy)] * w_normal * w_depth * w_albedo * w_lum;
            sum += w * mk(c.x, c.y, c.z);
            variance += w * w * c.w;
            weights += w;
        }
    dst[i] = weights > 0.0f ? make_float4(sum.x / weights, sum.y / weights, sum.z / weights,
                                          variance / (weights * weights))
                            : center;
}

// denoise.comp:89-94: remodulate into the HDR image.
__global__ void k_denoise_finish(const PostArgs a, int from_pong) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    int W = (int)a.width, H = (int)a.height;
    if (x >= W || y >= H) return;
    float n = samples_of(a);
    int i = y * W + x;
    float4 c = (from_pong ? a.pong : a.ping)[i];
    float4 ga = a.guide_alb[i];
    f3 alb = mk(ga.x, ga.y, ga.z);
    a.hdr[i] = to_h4(make_float4(c.x * alb.x, c.y * alb.y, c.z * alb.z, a.accum[i].w / n));
}

__global__ void k_hdr_resolve(const PostArgs a, float n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)(a.width * a.height)) return;
    float4 v = a.accum[i];
    a.hdr[i] = to_h4(make_float4(v.x / n, v.y / n, v.z / n, v.w / n));
}

// The pass's sums into the accumulation (pt.comp:554-559 for the pass's
// frames), then the HDR store of its last frame (pt.comp:560). A single-frame
// pass's own sums are that frame's, so the totals are the reference's to the bit.
__global__ void k_merge(const PostArgs a, const float4* __restrict__ pacc, const float4* __restrict__ palb,
                        const float4* __restrict__ pnor, float n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)(a.width * a.height)) return;
    float4 v = a.accum[i], pv = pacc[i];
    v = make_float4(v.x + pv.x, v.y + pv.y, v.z + pv.z, v.w + pv.w);
    float4* acc = (float4*)a.accum;
    float4* alb = (float4*)a.albedo;
    float4* nor = (float4*)a.normal;
    acc[i] = v;
    float4 b = alb[i], pb = palb[i];
    alb[i] = make_float4(b.x + pb.x, b.y + pb.y, b.z + pb.z, b.w + pb.w);
    float4 c = nor[i], pc = pnor[i];
    nor[i] = make_float4(c.x + pc.x, c.y + pc.y, c.z + pc.z, c.w + pc.w);
    a.hdr[i] = to_h4(make_float4(v.x / n, v.y / n, v.z / n, v.w / n));
}

// One running sum (4 channels) plus a pass's sums, as PreciseSums says.
__device__ __forceinline__ float4 merge_sum(float4* total, float4* comp, double* wide, float4 add,
                                            const PreciseSums& ps, int i) {
    float4 t = total[i];
    float a[4] = {add.x, add.y, add.z, add.w}, v[4] = {t.x, t.y, t.z, t.w};
    if (ps.wide_mode == 0) {
        if (ps.kahan) {
            float4 cv = comp[i];
            float c[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {  // Kahan: y = a - c, t = v + y, c = (t - v) - y
                float y = __fsub_rn(a[k], c[k]);
                float s = __fadd_rn(v[k], y);
                c[k] = __fsub_rn(__fsub_rn(s, v[k]), y);
                v[k] = s;
            }
            comp[i] = make_float4(c[0], c[1], c[2], c[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) v[k] = __fadd_rn(v[k], a[k]);
        }
    } else {
        double w[4];
        if (ps.wide_mode == 1) {  // the FP32 sum, corrected by its compensation
            float4 cv = ps.kahan ? comp[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            float c[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
            for (int k = 0; k < 4; k++) w[k] = (double)v[k] - (double)c[k];
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) w[k] = wide[4 * (long)i + k];
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            w[k] += (double)a[k];
            wide[4 * (long)i + k] = w[k];
            v[k] = (float)w[k];
        }
    }
    float4 r = make_float4(v[0], v[1], v[2], v[3]);
    total[i] = r;
    return r;
}

__global__ void k_merge_precise(const PostArgs a, const float4* __restrict__ pacc, const float4* __restrict__ palb,
                                const float4* __restrict__ pnor, const PreciseSums ps, double n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)(a.width * a.height)) return;
    float4 v = merge_sum((float4*)a.accum, ps.comp[0], ps.wide[0], pacc[i], ps, i);
    merge_sum((float4*)a.albedo, ps.comp[1], ps.wide[1], palb[i], ps, i);
    merge_sum((float4*)a.normal, ps.comp[2], ps.wide[2], pnor[i], ps, i);
    if (ps.wide_mode != 0) {
        const double* w = ps.wide[0] + 4 * (long)i;
        a.hdr[i] = to_h4(make_float4((float)(w[0] / n), (float)(w[1] / n), (float)(w[2] / n), (float)(w[3] / n)));
    } else {
        float nf = (float)n;
        a.hdr[i] = to_h4(make_float4(v.x / nf, v.y / nf, v.z / nf, v.w / nf));
    }
}

cudaError_t launch_merge_precise(const PostArgs& a, const float4* accum, const float4* albedo, const float4* normal,
                                 const PreciseSums& ps, double n, cudaStream_t s) {
    int N = (int)(a.width * a.height);
    k_merge_precise<<<(N + 255) / 256, 256, 0, s>>>(a, accum, albedo, normal, ps, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------------- bloom
// bloom.comp pass 0: Karis-weighted 4x4 average of the HDR image, with coverage.
__global__ void k_bloom_down4(const PostArgs a) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= a.bw[0] || y >= a.bh[0]) return;
    int W = (int)a.width, H = (int)a.height;
    f3 sum = mk(0.0f);
    float weights = 0.0f, coverage = 0.0f;
    for (int dy = 0; dy < 4; dy++)
        for (int dx = 0; dx < 4; dx++) {
            int qx = min(x * 4 + dx, W - 1), qy = min(y * 4 + dy, H - 1);
            float4 h = h4(a.hdr[qy * W + qx]);
            float w = 1.0f / (1.0f + lum(h.x, h.y, h.z));
            sum += mk(h.x, h.y, h.z) * w;
            weights += w;
            coverage += 1.0f - h.w;
        }
    a.bloom[0][y * a.bw[0] + x] = to_h4(make_float4(sum.x / weights, sum.y / weights, sum.z / weights, coverage / 16.0f));
}

// bloom.comp pass 1 (auto exposure), in two kernels. The terms of the
// exposure sums, one thread per pixel of A (coverage-weighted log luminance,
// coverage), into `terms` (a float2 per pixel).
__global__ void k_exposure_terms(const PostArgs a, float2* terms) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.bw[0] * a.bh[0]) return;
    float4 c = h4(a.bloom[0][i]);
    float l = logf(gmax(lum(c.x, c.y, c.z), 1e-4f));
    terms[i] = make_float2(__fmul_rn(c.w, l), c.w);
}

// The sums themselves, in the workgroup's order (thread t adds pixels t,
// t + 64, ... in turn, then a tree over the 64 partial sums), so the result
// is the one-workgroup shader's to the bit.
__global__ void k_exposure(const PostArgs a, const float2* terms) {
    __shared__ float log_sum[64], weight_sum[64];
    int t = threadIdx.x;
    int n = a.bw[0] * a.bh[0];
    float s = 0.0f, w = 0.0f;
    for (int i = t; i < n; i += 64) {
        float2 term = terms[i];
        s += term.x;
        w += term.y;
    }
    log_sum[t] = s;
    weight_sum[t] = w;
    __syncthreads();
    for (int stride = 32; stride > 0; stride >>= 1) {
        if (t < stride) {
            log_sum[t] += log_sum[t + stride];
            weight_sum[t] += weight_sum[t + stride];
        }
        __syncthreads();
    }
    if (t == 0) {
        const float KEY = 0.24f, ADAPT = 0.15f;
        float target = weight_sum[0] > 1.0f ? gclamp(KEY / expf(log_sum[0] / weight_sum[0]), 0.25f, 4.0f) : 1.0f;
        float previous = a.exposure[0];
        float adapted = previous <= 0.0f ? target : expf(mixf(logf(previous), logf(target), ADAPT));
        a.exposure[0] = adapted;
    }
}

// bloom.comp:277-285: 9-tap Gaussian along one axis.
__global__ void k_bloom_blur(const ushort4* src, ushort4* dst, int w, int h, int ax, int ay) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= w || y >= h) return;
    const float k[5] = {0.2270f, 0.1945f, 0.1216f, 0.0540f, 0.0162f};
    float4 c = h4(src[y * w + x]);
    float4 s = make_float4(c.x * k[0], c.y * k[0], c.z * k[0], c.w * k[0]);
    for (int i = 1; i < 5; i++) {
        int px = clampi(x + ax * i, 0, w - 1), py = clampi(y + ay * i, 0, h - 1);
        int mx = clampi(x - ax * i, 0, w - 1), my = clampi(y - ay * i, 0, h - 1);
        float4 p = h4(src[py * w + px]), m = h4(src[my * w + mx]);
        s.x += k[i] * (p.x + m.x);
        s.y += k[i] * (p.y + m.y);
        s.z += k[i] * (p.z + m.z);
        s.w += k[i] * (p.w + m.w);
    }
    dst[y * w + x] = to_h4(s);
}

// bloom.comp pass 4: 2x2 average of A into C.
__global__ void k_bloom_down2(const PostArgs a) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= a.bw[2] || y >= a.bh[2]) return;
    float4 s = make_float4(0, 0, 0, 0);
    for (int i = 0; i < 4; i++) {
        int qx = min(x * 2 + (i & 1), a.bw[0] - 1), qy = min(y * 2 + (i >> 1), a.bh[0] - 1);
        float4 c = h4(a.bloom[0][qy * a.bw[0] + qx]);
        s.x += c.x; s.y += c.y; s.z += c.z; s.w += c.w;
    }
    a.bloom[2][y * a.bw[2] + x] = to_h4(make_float4(s.x * 0.25f, s.y * 0.25f, s.z * 0.25f, s.w * 0.25f));
}

// Linear filtering of a half4 image at normalised uv (CLAMP_TO_EDGE).
__device__ float4 bilinear(const ushort4* img, int w, int h, float u, float v) {
    float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    float fx0 = floorf(x), fy0 = floorf(y);
    int x0 = (int)fx0, y0 = (int)fy0;
    float fx = x - fx0, fy = y - fy0;
    int xa = clampi(x0, 0, w - 1), xb = clampi(x0 + 1, 0, w - 1);
    int ya = clampi(y0, 0, h - 1), yb = clampi(y0 + 1, 0, h - 1);
    float4 c00 = h4(img[ya * w + xa]), c10 = h4(img[ya * w + xb]), c01 = h4(img[yb * w + xa]), c11 = h4(img[yb * w + xb]);
    auto l = [](float p, float q, float f) { return p * (1.0f - f) + q * f; };
    return make_float4(l(l(c00.x, c10.x, fx), l(c01.x, c11.x, fx), fy), l(l(c00.y, c10.y, fx), l(c01.y, c11.y, fx), fy),
                       l(l(c00.z, c10.z, fx), l(c01.z, c11.z, fx), fy), l(l(c00.w, c10.w, fx), l(c01.w, c11.w, fx), fy));
}

__device__ __forceinline__ float aces1(float x) {
    return gclamp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
}
// tonemap.comp:27-45 (AgX base look)
__device__ f3 agx(f3 c) {
    const float in_[9] = {0.842479062253094f, 0.0423282422610123f, 0.0423756549057051f, 0.0784335999999992f,
                          0.878468636469772f, 0.0784336f, 0.0792237451477643f, 0.0791661274605434f, 0.879142973793104f};
    const float out_[9] = {1.19687900512017f, -0.0528968517574562f, -0.0529716355144438f, -0.0980208811401368f,
                           1.15190312990417f, -0.0980434501171241f, -0.0990297440797205f, -0.0989611768448433f,
                           1.15107367264116f};
    const float min_ev = -12.47393f, max_ev = 4.026069f;
    m3 inset = {mk(in_[0], in_[1], in_[2]), mk(in_[3], in_[4], in_[5]), mk(in_[6], in_[7], in_[8])};
    m3 outset = {mk(out_[0], out_[1], out_[2]), mk(out_[3], out_[4], out_[5]), mk(out_[6], out_[7], out_[8])};
    c = mul(inset, c);
    c = mk(gclamp(log2f(gmax(c.x, 1e-10f)), min_ev, max_ev), gclamp(log2f(gmax(c.y, 1e-10f)), min_ev, max_ev),
           gclamp(log2f(gmax(c.z, 1e-10f)), min_ev, max_ev));
    c = (c - min_ev) / (max_ev - min_ev);
    f3 c2 = c * c, c4 = c2 * c2;
    c = 15.5f * c4 * c2 - 40.14f * c4 * c + 31.96f * c4 - 6.868f * c2 * c + 0.4298f * c2 + 0.1191f * c - 0.00232f;
    c = mul(outset, c);
    c = gclamp(c, 0.0f, 1.0f);
    return mk(powf(c.x, 2.2f), powf(c.y, 2.2f), powf(c.z, 2.2f));
}
__device__ __forceinline__ float srgb1(float c) {
    c = gclamp(c, 0.0f, 1.0f);
    return c < 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ float hash01(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (float)((word >> 22u) ^ word) * (1.0f / 4294967296.0f);
}
__device__ __forceinline__ uint8_t unorm8(float f) { return (uint8_t)rintf(gclamp(f, 0.0f, 1.0f) * 255.0f); }

// tonemap.comp:47-85
__global__ void k_tonemap(const PostArgs a) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    int W = (int)a.width, H = (int)a.height;
    if (x >= W || y >= H) return;
    float4 hdr = h4(a.hdr[y * W + x]);
    float exposure = a.u.ambient[3];
    if (a.u.finish[3] > 0.5f) exposure *= a.exposure[0];
    f3 c = mk(hdr.x, hdr.y, hdr.z);
    float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
    if (a.u.finish[0] > 0.0f) {
        float4 n4 = bilinear(a.bloom[0], a.bw[0], a.bh[0], u, v);
        float4 w4 = bilinear(a.bloom[2], a.bw[2], a.bh[2], u, v);
        f3 glow = 0.6f * mk(n4.x, n4.y, n4.z) + 0.4f * mk(w4.x, w4.y, w4.z);
        c = mix3(c, glow, a.u.finish[0]);
    }
    float ux = u * 2.0f - 1.0f, uy = v * 2.0f - 1.0f;
    float r = sqrtf(ux * ux + uy * uy) * 0.7071f;
    float vignette = 1.0f - a.u.finish[1] * powf(r, 2.5f);
    c = c * (exposure * vignette);
    uint32_t op = (uint32_t)a.u.material[2];
    if (op == 1u) c = mk(aces1(c.x), aces1(c.y), aces1(c.z));
    else if (op == 2u) c = agx(c);
    else c = gclamp(c, 0.0f, 1.0f);
    // background(camera_ray(pixel + 0.5)) (common.glsl:439-455)
    if (a.u.lighting[3] < 1u) {
        float nx = ((float)x + 0.5f) / (float)W * 2.0f - 1.0f, ny = ((float)y + 0.5f) / (float)H * 2.0f - 1.0f;
        f3 dir = normalize(mk(a.u.forward[0], a.u.forward[1], a.u.forward[2]) +
                           nx * mk(a.u.right[0], a.u.right[1], a.u.right[2]) - ny * mk(a.u.up[0], a.u.up[1], a.u.up[2]));
        float t = 0.5f + 0.5f * -dir.z;
        c += hdr.w * mix3(mk(0.02f, 0.022f, 0.028f), mk(0.08f, 0.085f, 0.1f), t);
    }
    if (a.u.flags[1] != 0u) c = mk(srgb1(c.x), srgb1(c.y), srgb1(c.z));
    if (a.u.finish[2] > 0.0f) {
        float n = hash01((uint32_t)x + 4099u * (uint32_t)y) + hash01((uint32_t)x * 7919u + (uint32_t)y + 1u) - 1.0f;
        float yl = gclamp(lum(c.x, c.y, c.z), 0.0f, 1.0f);
        c = gclamp(c + n * a.u.finish[2] * (0.3f + 2.8f * yl * (1.0f - yl)), 0.0f, 1.0f);
    }
    a.out[y * W + x] = make_uchar4(unorm8(c.x), unorm8(c.y), unorm8(c.z), 255);
}

static dim3 grid16(int w, int h) { return dim3((w + 15) / 16, (h + 15) / 16); }

cudaError_t launch_denoise(const PostArgs& a, cudaStream_t s, int* launches) {
    dim3 g = grid16(a.width, a.height);
    k_denoise_prepare<<<g, 256, 0, s>>>(a);
    for (int level = 0; level < 5; level++) k_denoise_level<<<g, 256, 0, s>>>(a, 1 << level, level % 2);
    k_denoise_finish<<<g, 256, 0, s>>>(a, 5 % 2);
    *launches += 7;
    return cudaGetLastError();
}

cudaError_t launch_post(const PostArgs& a, cudaStream_t s, int* launches) {
    k_bloom_down4<<<grid16(a.bw[0], a.bh[0]), 256, 0, s>>>(a);
    // The exposure terms go to the denoiser's ping image, free after the denoiser.
    int npx = a.bw[0] * a.bh[0];
    k_exposure_terms<<<(npx + 255) / 256, 256, 0, s>>>(a, (float2*)a.ping);
    k_exposure<<<1, 64, 0, s>>>(a, (const float2*)a.ping);
    k_bloom_blur<<<grid16(a.bw[0], a.bh[0]), 256, 0, s>>>(a.bloom[0], a.bloom[1], a.bw[0], a.bh[0], 1, 0);
    k_bloom_blur<<<grid16(a.bw[0], a.bh[0]), 256, 0, s>>>(a.bloom[1], a.bloom[0], a.bw[0], a.bh[0], 0, 1);
    k_bloom_down2<<<grid16(a.bw[2], a.bh[2]), 256, 0, s>>>(a);
    k_bloom_blur<<<grid16(a.bw[2], a.bh[2]), 256, 0, s>>>(a.bloom[2], a.bloom[3], a.bw[2], a.bh[2], 1, 0);
    k_bloom_blur<<<grid16(a.bw[2], a.bh[2]), 256, 0, s>>>(a.bloom[3], a.bloom[2], a.bw[2], a.bh[2], 0, 1);
    k_tonemap<<<grid16(a.width, a.height), 256, 0, s>>>(a);
    *launches += 9;
    return cudaGetLastError();
}

cudaError_t launch_merge(const PostArgs& a, const float4* accum, const float4* albedo, const float4* normal, float n,
                         cudaStream_t s) {
    int N = (int)(a.width * a.height);
    k_merge<<<(N + 255) / 256, 256, 0, s>>>(a, accum, albedo, normal, n);
    return cudaGetLastError();
}

cudaError_t launch_hdr_resolve(const PostArgs& a, float n, cudaStream_t s) {
    int N = (int)(a.width * a.height);
    k_hdr_resolve<<<(N + 255) / 256, 256, 0, s>>>(a, n);
    return cudaGetLastError();
}

}  // namespace vv
