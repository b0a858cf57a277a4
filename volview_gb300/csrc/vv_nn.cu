// vv_nn.cu — the learned denoiser's operators: 3x3 convolutions as implicit
// GEMMs on the FP16 tensor cores (tcgen05 for the shapes vv_nn_tc.cu takes,
// mma.sync m16n8k16 for the rest, FP32 accumulation), their
// weight and bias gradients, and the element-wise parts of a U-Net (ReLU, 2x2
// average pooling, nearest upsampling, channel concatenation), its input
// features from the path tracer's accumulation, an L1 loss in log radiance and
// Adam.
//
// Tensors are NHWC: pixel-major, channels innermost, FP16 activations and
// weights. Channel counts are multiples of 16 on the reduction side and of 8
// on the output side, and image widths multiples of 16, so that a warp's 16
// output pixels are 16 consecutive pixels of one row and every fragment load
// is an aligned 32-bit word. Weights are [cout][3][3][cin].
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/volpt_nn.h"

namespace vv {
namespace nn {

// vv_nn_tc.cu: the tcgen05 convolution; false when the shape is not one it takes.
bool conv3x3_tc(const __half* x, int n, int h, int w, int cin, const __half* wt, const float* bias, int cout,
                int relu, __half* y, cudaStream_t s, cudaError_t* err);

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __half* p) { return __ldg((const unsigned int*)p); }
__device__ __forceinline__ uint32_t pack(__half lo, __half hi) {
    return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

// y = act(conv3x3(x, w) + bias). A block of CONV_WARPS warps takes as many
// 16-pixel row segments, one per warp, and NT x 8 of the cout output channels
// (from blockIdx.y * NT * 8: small images split their channels over several
// blocks so that the grid covers the GPU). For each of the 9 taps the block
// first copies that tap's weights of its channels (NT x 8 x CIN) into shared
// memory, rows padded to CIN + 8 halves so that the B fragment loads of a warp
// fall in distinct banks; each warp then reduces over CIN in steps of 16 on the
// tensor cores, its A fragments (the input pixels at the tap's offset, zeros
// outside the image: same padding) read as aligned 32-bit words.
// Fragment layouts of m16n8k16 (g = lane / 4, t = lane % 4): A row g / g + 8,
// columns 2t, 2t + 1 / + 8; B column g, rows 2t, 2t + 1 / + 8; C row g / g + 8,
// columns 2t, 2t + 1.
constexpr int CONV_WARPS = 8;
template <int NT>
__global__ void __launch_bounds__(CONV_WARPS * 32) k_conv3x3(const __half* __restrict__ x, int n, int h, int w, int cin,
                                                             const __half* __restrict__ wt,
                                                             const float* __restrict__ bias, int relu,
                                                             __half* __restrict__ y, int cout) {
    extern __shared__ __align__(16) unsigned char smem[];
    __half* sw = (__half*)smem;
    const int stride = cin + 8;  // halves per staged weight row
    const int co0 = blockIdx.y * NT * 8;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long tile = (long)blockIdx.x * CONV_WARPS + (threadIdx.x >> 5);  // 16-pixel tile
    const long pixels = (long)n * h * w;
    const bool active = tile * 16 < pixels;
    const long p0 = active ? tile * 16 : 0;
    const int img = (int)(p0 / ((long)h * w));
    const int rem = (int)(p0 - (long)img * h * w);
    const int py = rem / w, px0 = rem % w;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const int chunks = NT * 8 * (cin / 8);  // 16-byte pieces of one tap's weights of the block's channels
    for (int tap = 0; tap < 9; tap++) {
        __syncthreads();  // the previous tap's weights are no longer read
        for (int i = threadIdx.x; i < chunks; i += CONV_WARPS * 32) {
            int co = i / (cin / 8), c8 = i % (cin / 8);
            *(uint4*)(sw + co * stride + c8 * 8) =
                __ldg((const uint4*)(wt + ((long)(co0 + co) * 9 + tap) * cin + c8 * 8));
        }
        __syncthreads();
        if (!active) continue;
        const int sy = py + tap / 3 - 1;
        const int sx0 = px0 + g + tap % 3 - 1, sx1 = sx0 + 8;
        const bool row_in = sy >= 0 && sy < h;
        const bool in0 = row_in && sx0 >= 0 && sx0 < w, in1 = row_in && sx1 >= 0 && sx1 < w;
        const __half* r0 = x + (((long)img * h + (row_in ? sy : 0)) * w + (in0 ? sx0 : 0)) * cin;
        const __half* r1 = x + (((long)img * h + (row_in ? sy : 0)) * w + (in1 ? sx1 : 0)) * cin;
        for (int c0 = 0; c0 < cin; c0 += 16) {
            uint32_t a[4];
            a[0] = in0 ? ld32(r0 + c0 + 2 * t) : 0u;
            a[1] = in1 ? ld32(r1 + c0 + 2 * t) : 0u;
            a[2] = in0 ? ld32(r0 + c0 + 8 + 2 * t) : 0u;
            a[3] = in1 ? ld32(r1 + c0 + 8 + 2 * t) : 0u;
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const __half* wr = sw + (j * 8 + g) * stride + c0 + 2 * t;
                uint32_t b[2] = {*(const uint32_t*)wr, *(const uint32_t*)(wr + 8)};
                mma16816(acc[j], a, b);
            }
        }
    }
    if (!active) return;
    __half* o0 = y + (p0 + g) * cout + co0;
    __half* o1 = y + (p0 + g + 8) * cout + co0;
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const int co = j * 8 + 2 * t;
        float b0 = bias ? bias[co0 + co] : 0.0f, b1 = bias ? bias[co0 + co + 1] : 0.0f;
        float v[4] = {acc[j][0] + b0, acc[j][1] + b1, acc[j][2] + b0, acc[j][3] + b1};
        if (relu)
            for (int k = 0; k < 4; k++) v[k] = fmaxf(v[k], 0.0f);
        *(uint32_t*)(o0 + co) = pack(__float2half_rn(v[0]), __float2half_rn(v[1]));
        *(uint32_t*)(o1 + co) = pack(__float2half_rn(v[2]), __float2half_rn(v[3]));
    }
}

// wt_t[ci][8 - tap][co] = w[co][tap][ci]: the weights of the convolution
// that carries dy back to dx (3x3 flipped, channels swapped).
__global__ void k_flip_weights(const __half* __restrict__ w, int cout, int cin, __half* __restrict__ wt) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long total = (long)cout * 9 * cin;
    if (i >= total) return;
    int ci = (int)(i % cin), tap = (int)((i / cin) % 9), co = (int)(i / ((long)cin * 9));
    wt[((long)ci * 9 + (8 - tap)) * cout + co] = w[i];
}

// dw[co][tap][ci] += sum over pixels of dy[p][co] * x[p + tap offset][ci]: a
// GEMM (co x ci, reduced over pixels) on the tensor cores. A warp takes 16
// output channels, NT x 8 input channels and one tap, and reduces a chunk of
// CHUNK 16-pixel row segments before adding into the FP32 gradient.
template <int NT>
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const __half* __restrict__ x, const __half* __restrict__ dy,
                                                       int n, int h, int w, int cin, int cout, int chunk,
                                                       float* __restrict__ dw) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int tap = blockIdx.z, dyo = tap / 3 - 1, dxo = tap % 3 - 1;
    const int co_tiles = (cout + 15) / 16;
    const int co0 = (blockIdx.y % co_tiles) * 16, ci0 = (blockIdx.y / co_tiles) * NT * 8;
    const long tiles = (long)n * h * w / 16;
    const long first = ((long)blockIdx.x * 4 + (threadIdx.x >> 5)) * chunk;
    if (first >= tiles) return;
    const long last = first + chunk < tiles ? first + chunk : tiles;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const bool cg0 = co0 + g < cout, cg1 = co0 + g + 8 < cout;
    const __half zero = __float2half_rn(0.0f);
    for (long tile = first; tile < last; tile++) {
        const long p0 = tile * 16;
        const int img = (int)(p0 / ((long)h * w));
        const int rem = (int)(p0 - (long)img * h * w);
        const int py = rem / w, px0 = rem % w;
        // A: dy rows (channels) g / g + 8, columns (pixels) 2t, 2t + 1 / + 8.
        const __half* d = dy + p0 * cout;
        int k0 = 2 * t, k1 = 2 * t + 8;
        uint32_t a[4];
        a[0] = pack(cg0 ? d[(long)k0 * cout + co0 + g] : zero, cg0 ? d[(long)(k0 + 1) * cout + co0 + g] : zero);
        a[1] = pack(cg1 ? d[(long)k0 * cout + co0 + g + 8] : zero, cg1 ? d[(long)(k0 + 1) * cout + co0 + g + 8] : zero);
        a[2] = pack(cg0 ? d[(long)k1 * cout + co0 + g] : zero, cg0 ? d[(long)(k1 + 1) * cout + co0 + g] : zero);
        a[3] = pack(cg1 ? d[(long)k1 * cout + co0 + g + 8] : zero, cg1 ? d[(long)(k1 + 1) * cout + co0 + g + 8] : zero);
        // B: x at the tap's offset, rows (pixels) 2t, 2t + 1 / + 8, column g.
        const int sy = py + dyo;
        const bool row_in = sy >= 0 && sy < h;
        int sx[4] = {px0 + k0 + dxo, px0 + k0 + 1 + dxo, px0 + k1 + dxo, px0 + k1 + 1 + dxo};
        const __half* src[4];
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            in[q] = row_in && sx[q] >= 0 && sx[q] < w;
            src[q] = x + (((long)img * h + (row_in ? sy : 0)) * w + (in[q] ? sx[q] : 0)) * cin;
        }
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const int ci = ci0 + j * 8 + g;
            if (ci0 + j * 8 >= cin) break;
            uint32_t b[2];
            b[0] = pack(in[0] ? src[0][ci] : zero, in[1] ? src[1][ci] : zero);
            b[1] = pack(in[2] ? src[2][ci] : zero, in[3] ? src[3][ci] : zero);
            mma16816(acc[j], a, b);
        }
    }
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const int ci = ci0 + j * 8 + 2 * t;
        if (ci >= cin) break;
        if (cg0) {
            atomicAdd(&dw[((long)(co0 + g) * 9 + tap) * cin + ci], acc[j][0]);
            atomicAdd(&dw[((long)(co0 + g) * 9 + tap) * cin + ci + 1], acc[j][1]);
        }
        if (cg1) {
            atomicAdd(&dw[((long)(co0 + g + 8) * 9 + tap) * cin + ci], acc[j][2]);
            atomicAdd(&dw[((long)(co0 + g + 8) * 9 + tap) * cin + ci + 1], acc[j][3]);
        }
    }
}

// db[c] += sum over pixels of dy[p][c].
__global__ void k_bias_grad(const __half* __restrict__ dy, long pixels, int c, int chunk, float* __restrict__ db) {
    const int ch = threadIdx.x;
    if (ch >= c) return;
    const long first = (long)blockIdx.x * chunk;
    const long last = first + chunk < pixels ? first + chunk : pixels;
    float s = 0.0f;
    for (long p = first; p < last; p++) s += __half2float(dy[p * c + ch]);
    atomicAdd(&db[ch], s);
}

__global__ void k_relu_backward(__half* __restrict__ dy, const __half* __restrict__ y, long count) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count && !(__half2float(y[i]) > 0.0f)) dy[i] = __float2half_rn(0.0f);
}

// 2x2 average pooling (n, h, w, c) -> (n, h / 2, w / 2, c), and its gradient.
__global__ void k_avgpool2(const __half* __restrict__ x, int n, int h, int w, int c, __half* __restrict__ y) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int ho = h / 2, wo = w / 2;
    if (i >= (long)n * ho * wo * c) return;
    int ch = (int)(i % c);
    long p = i / c;
    int xo = (int)(p % wo), yo = (int)((p / wo) % ho), img = (int)(p / ((long)wo * ho));
    const __half* b = x + (((long)img * h + 2 * yo) * w + 2 * xo) * c + ch;
    float s = __half2float(b[0]) + __half2float(b[c]) + __half2float(b[(long)w * c]) + __half2float(b[(long)w * c + c]);
    y[i] = __float2half_rn(0.25f * s);
}
// k_avgpool2 for channel counts that are a multiple of 8: 8 channels (16
// bytes) per thread from each of the 2x2 inputs, the same sums in the same
// order.
__global__ void k_avgpool2_q(const uint4* __restrict__ x, int n, int h, int w, int q, uint4* __restrict__ y) {
    const int ho = h / 2, wo = w / 2;
    const long total = (long)n * ho * wo * q;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const long p = i / q;
        const int k = (int)(i - p * q);
        const long row = p / wo;  // img * ho + yo
        const int xo = (int)(p - row * wo);
        const long img = row / ho;
        const int yo = (int)(row - img * ho);
        const uint4* b = x + (((img * h + 2 * yo) * w + 2 * xo) * q + k);
        const uint4 v00 = __ldg(b), v01 = __ldg(b + q), v10 = __ldg(b + (long)w * q), v11 = __ldg(b + (long)w * q + q);
        const __half* h00 = (const __half*)&v00;
        const __half* h01 = (const __half*)&v01;
        const __half* h10 = (const __half*)&v10;
        const __half* h11 = (const __half*)&v11;
        uint4 out;
        __half* o = (__half*)&out;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            float sum = __half2float(h00[j]) + __half2float(h01[j]) + __half2float(h10[j]) + __half2float(h11[j]);
            o[j] = __float2half_rn(0.25f * sum);
        }
        y[i] = out;
    }
}
__global__ void k_avgpool2_backward(const __half* __restrict__ dy, int n, int h, int w, int c, __half* __restrict__ dx) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)n * h * w * c) return;
    int ch = (int)(i % c);
    long p = i / c;
    int xx = (int)(p % w), yy = (int)((p / w) % h), img = (int)(p / ((long)w * h));
    dx[i] = __float2half_rn(0.25f * __half2float(dy[(((long)img * (h / 2) + yy / 2) * (w / 2) + xx / 2) * c + ch]));
}

// Nearest 2x upsampling (n, h, w, c) -> (n, 2h, 2w, c), and its gradient.
__global__ void k_upsample2(const __half* __restrict__ x, int n, int h, int w, int c, __half* __restrict__ y) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)n * 4 * h * w * c) return;
    int ch = (int)(i % c);
    long p = i / c;
    int xx = (int)(p % (2 * w)), yy = (int)((p / (2 * w)) % (2 * h)), img = (int)(p / (4L * w * h));
    y[i] = x[(((long)img * h + yy / 2) * w + xx / 2) * c + ch];
}
__global__ void k_upsample2_backward(const __half* __restrict__ dy, int n, int h, int w, int c, __half* __restrict__ dx) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)n * h * w * c) return;
    int ch = (int)(i % c);
    long p = i / c;
    int xx = (int)(p % w), yy = (int)((p / w) % h), img = (int)(p / ((long)w * h));
    const __half* b = dy + (((long)img * 2 * h + 2 * yy) * 2 * w + 2 * xx) * c + ch;
    float s = __half2float(b[0]) + __half2float(b[c]) + __half2float(b[2L * w * c]) + __half2float(b[2L * w * c + c]);
    dx[i] = __float2half_rn(s);
}

// The decoder's input in one pass: y (n, 2h, 2w, 8 qa + 8 qb) = the nearest 2x
// upsampling of a (n, h, w, 8 qa) followed by b (n, 2h, 2w, 8 qb), channel-wise;
// 8 channels (16 bytes) per thread, each source read once, y written once.
__global__ void k_upsample_concat(const uint4* __restrict__ a, int h, int w, int qa, const uint4* __restrict__ b,
                                  int qb, long pixels, uint4* __restrict__ y) {
    const int q = qa + qb;
    const long total = pixels * q, w2 = 2L * w, h2 = 2L * h;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const long p = i / q;
        const int k = (int)(i - p * q);
        uint4 v;
        if (k < qa) {
            const long row = p / w2;  // img * 2h + yy
            const long xx = p - row * w2;
            const long img = row / h2;
            const long yy = row - img * h2;
            v = __ldg(a + ((img * h + (yy >> 1)) * w + (xx >> 1)) * qa + k);
        } else {
            v = __ldg(b + p * qb + (k - qa));
        }
        y[i] = v;
    }
}

// y[p] = a[p] ++ b[p] (channels), and the split of its gradient.
__global__ void k_concat(const __half* __restrict__ a, int ca, const __half* __restrict__ b, int cb, long pixels,
                         __half* __restrict__ y) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = ca + cb;
    if (i >= pixels * c) return;
    long p = i / c;
    int ch = (int)(i % c);
    y[i] = ch < ca ? a[p * ca + ch] : b[p * cb + ch - ca];
}
__global__ void k_split(const __half* __restrict__ dy, int ca, int cb, long pixels, __half* __restrict__ da,
                        __half* __restrict__ db) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = ca + cb;
    if (i >= pixels * c) return;
    long p = i / c;
    int ch = (int)(i % c);
    if (ch < ca) {
        if (da) da[p * ca + ch] = dy[i];
    } else if (db) {
        db[p * cb + ch - ca] = dy[i];
    }
}

// The network's input from an accumulation of `n` paths per pixel (w x h,
// pixel-linear RGBA32F sums as vv_read_accumulation gives them): 16 channels,
// log(1 + radiance), albedo, normal (the guides' means), then zeros.
__global__ void k_features(const float4* __restrict__ accum, const float4* __restrict__ albedo,
                           const float4* __restrict__ normal, float n, long pixels, __half* __restrict__ x) {
    long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixels) return;
    float4 a = accum[p], b = albedo[p], c = normal[p];
    float inv = 1.0f / n;
    float f[16] = {log1pf(fmaxf(a.x * inv, 0.0f)), log1pf(fmaxf(a.y * inv, 0.0f)), log1pf(fmaxf(a.z * inv, 0.0f)),
                   b.x * inv, b.y * inv, b.z * inv, c.x * inv, c.y * inv, c.z * inv, 0, 0, 0, 0, 0, 0, 0};
    uint32_t* o = (uint32_t*)(x + p * 16);
#pragma unroll
    for (int k = 0; k < 8; k++) o[k] = pack(__float2half_rn(f[2 * k]), __float2half_rn(f[2 * k + 1]));
}

// L1 loss of the first 3 of `c` predicted channels against target log
// radiance (3 floats per pixel): loss += sum |p - t| / (3 pixels), and its
// gradient times grad_scale into dpred (zero for the other channels; the
// scale keeps FP16 gradients of large images out of the subnormals).
__global__ void k_l1_loss(const __half* __restrict__ pred, int c, const float* __restrict__ target, long pixels,
                          float grad_scale, float* __restrict__ loss, __half* __restrict__ dpred) {
    long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    float s = 0.0f;
    if (p < pixels) {
        const float scale = grad_scale / (3.0f * (float)pixels);
        for (int k = 0; k < c; k++) {
            float g = 0.0f;
            if (k < 3) {
                float d = __half2float(pred[p * c + k]) - target[p * 3 + k];
                s += fabsf(d);
                g = d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f);
            }
            dpred[p * c + k] = __float2half_rn(g);
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (3.0f * (float)pixels));
}

// Adam (Kingma and Ba) on FP32 master weights, with bias-corrected moments;
// the FP16 copy the convolutions read is rewritten.
__global__ void k_adam(float* __restrict__ w, __half* __restrict__ w16, const float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, long count, float lr, float b1, float b2,
                       float eps, float inv_scale, float c1, float c2) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float g = grad[i] * inv_scale;
    float mi = b1 * m[i] + (1.0f - b1) * g, vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2half_rn(wi);
}

// y += x (FP16, FP32 arithmetic): gradients of a tensor with two consumers.
__global__ void k_add(__half* __restrict__ y, const __half* __restrict__ x, long count) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] = __float2half_rn(__half2float(y[i]) + __half2float(x[i]));
}

// rgb = exp(max(p, 0)) - 1 of the first 3 of `c` predicted channels.
__global__ void k_radiance(const __half* __restrict__ pred, int c, long pixels, float* __restrict__ rgb) {
    long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixels) return;
    for (int k = 0; k < 3; k++) rgb[p * 3 + k] = expm1f(fmaxf(__half2float(pred[p * c + k]), 0.0f));
}

// The network's input over a padded image (wp x hp, zeros outside the w x h
// image) from the renderer's own accumulation images (pixel-linear RGBA32F).
__global__ void k_features_image(const float4* __restrict__ accum, const float4* __restrict__ albedo,
                                 const float4* __restrict__ normal, float n, int w, int h, int wp, int hp,
                                 __half* __restrict__ x) {
    long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long)wp * hp) return;
    int px = (int)(q % wp), py = (int)(q / wp);
    uint32_t* o = (uint32_t*)(x + q * 16);
    if (px >= w || py >= h) {
#pragma unroll
        for (int k = 0; k < 8; k++) o[k] = 0u;
        return;
    }
    long p = (long)py * w + px;
    float4 a = accum[p], b = albedo[p], c = normal[p];
    float inv = 1.0f / n;
    float f[16] = {log1pf(fmaxf(a.x * inv, 0.0f)), log1pf(fmaxf(a.y * inv, 0.0f)), log1pf(fmaxf(a.z * inv, 0.0f)),
                   b.x * inv, b.y * inv, b.z * inv, c.x * inv, c.y * inv, c.z * inv, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 8; k++) o[k] = pack(__float2half_rn(f[2 * k]), __float2half_rn(f[2 * k + 1]));
}

// The HDR store of a denoised image: rgb = exp(max(pred, 0)) - 1 of the
// prediction (padded width wp, c channels), coverage from the accumulation.
__global__ void k_prediction_to_hdr(const __half* __restrict__ pred, int c, int wp, int w, int h,
                                    const float4* __restrict__ accum, float n, ushort4* __restrict__ hdr) {
    long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long)w * h) return;
    long q = (p / w) * wp + p % w;
    const __half* v = pred + q * c;
    float r = expm1f(fmaxf(__half2float(v[0]), 0.0f)), g = expm1f(fmaxf(__half2float(v[1]), 0.0f));
    float b = expm1f(fmaxf(__half2float(v[2]), 0.0f)), a = accum[p].w / n;
    hdr[p] = make_ushort4(__half_as_ushort(__float2half_rn(r)), __half_as_ushort(__float2half_rn(g)),
                          __half_as_ushort(__float2half_rn(b)), __half_as_ushort(__float2half_rn(a)));
}

static inline unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }
static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
// Blocks of 256 threads for a grid-stride loop over n items: enough to fill
// the GPU many times over, capped so that each thread takes a few items.
static inline unsigned grid_for(long n) { return (unsigned)std::min<long>(std::max<long>((n + 255) / 256, 1), 152L * 64); }

}  // namespace nn
}  // namespace vv

using namespace vv::nn;

static vv_status launched() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? VV_OK : VV_ERR_CUDA;
}

extern "C" vv_status vv_nn_conv3x3(const void* x, int n, int h, int w, int cin, const void* weights,
                                   const float* bias, int cout, int relu, void* y, void* stream) {
    if (!x || !weights || !y || n <= 0 || h <= 0 || w <= 0 || w % 16 || cin <= 0 || cin % 16) return VV_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    switch (cout) {
        case 8: case 16: case 32: case 48: case 64: case 80: case 96: case 112: case 144: case 176: break;
        default: return VV_ERR_ARG;
    }
    // Widths that are multiples of 128 with the weights and two segments'
    // input rows in shared memory run on tcgen05 (vv_nn_tc.cu); the rest here.
    cudaError_t te = cudaSuccess;
    if (conv3x3_tc((const __half*)x, n, h, w, cin, (const __half*)weights, bias, cout, relu, (__half*)y, s, &te))
        return te == cudaSuccess ? VV_OK : VV_ERR_CUDA;
    const unsigned g = blocks((long)n * h * w / 16, CONV_WARPS);
    const __half* X = (const __half*)x;
    const __half* W = (const __half*)weights;
    __half* Y = (__half*)y;
    // All of cout per block, unless the grid would not cover the SMs: then the
    // channels split into groups of 6 to 2 tiles of 8 (the largest that
    // divides cout / 8 and gives a block per SM, else the smallest).
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = cout / 8;
    int nt = tiles;
    if ((long)g < sms) {
        const int groups[5] = {6, 5, 4, 3, 2};
        int pick = 0;
        for (int k = 0; k < 5; k++) {
            if (groups[k] >= tiles || tiles % groups[k]) continue;
            pick = groups[k];
            if ((long)g * (tiles / pick) >= sms) break;
        }
        if (pick) nt = pick;
    }
    const size_t smem = (size_t)nt * 8 * (cin + 8) * sizeof(__half);
    if (smem > 48 * 1024) return VV_ERR_ARG;  // one tap's weights staged in shared memory
    const dim3 grid(g, tiles / nt);
    switch (nt) {
        case 1: k_conv3x3<1><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 2: k_conv3x3<2><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 3: k_conv3x3<3><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 4: k_conv3x3<4><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 5: k_conv3x3<5><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 6: k_conv3x3<6><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 8: k_conv3x3<8><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 10: k_conv3x3<10><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 12: k_conv3x3<12><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 14: k_conv3x3<14><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 18: k_conv3x3<18><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        case 22: k_conv3x3<22><<<grid, CONV_WARPS * 32, smem, s>>>(X, n, h, w, cin, W, bias, relu, Y, cout); break;
        default: return VV_ERR_ARG;
    }
    return launched();
}

extern "C" vv_status vv_nn_flip_weights(const void* w, int cout, int cin, void* wt, void* stream) {
    if (!w || !wt || cout <= 0 || cin <= 0) return VV_ERR_ARG;
    long total = (long)cout * 9 * cin;
    k_flip_weights<<<blocks(total, 256), 256, 0, (cudaStream_t)stream>>>((const __half*)w, cout, cin, (__half*)wt);
    return launched();
}

extern "C" vv_status vv_nn_conv3x3_wgrad(const void* x, const void* dy, int n, int h, int w, int cin, int cout,
                                         float* dw, void* stream) {
    if (!x || !dy || !dw || n <= 0 || h <= 0 || w <= 0 || w % 16 || cin <= 0 || cin % 8 || cout <= 0 || cout % 8)
        return VV_ERR_ARG;
    const int NT = 8;  // 64 input channels per warp
    const int chunk = 16;
    long tiles = (long)n * h * w / 16;
    dim3 grid(blocks(tiles, 4 * chunk), ((cout + 15) / 16) * ((cin + NT * 8 - 1) / (NT * 8)), 9);
    k_conv3x3_wgrad<NT><<<grid, 128, 0, (cudaStream_t)stream>>>((const __half*)x, (const __half*)dy, n, h, w, cin,
                                                                 cout, chunk, dw);
    return launched();
}

extern "C" vv_status vv_nn_bias_grad(const void* dy, long pixels, int c, float* db, void* stream) {
    if (!dy || !db || pixels <= 0 || c <= 0 || c > 1024) return VV_ERR_ARG;
    const int chunk = 256;
    k_bias_grad<<<blocks(pixels, chunk), c, 0, (cudaStream_t)stream>>>((const __half*)dy, pixels, c, chunk, db);
    return launched();
}

extern "C" vv_status vv_nn_relu_backward(void* dy, const void* y, long count, void* stream) {
    if (!dy || !y || count < 0) return VV_ERR_ARG;
    if (count == 0) return VV_OK;
    k_relu_backward<<<blocks(count, 256), 256, 0, (cudaStream_t)stream>>>((__half*)dy, (const __half*)y, count);
    return launched();
}

extern "C" vv_status vv_nn_avgpool2(const void* x, int n, int h, int w, int c, void* y, int backward,
                                    void* stream) {
    if (!x || !y || n <= 0 || h <= 0 || w <= 0 || h % 2 || w % 2 || c <= 0) return VV_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    long out = backward ? (long)n * h * w * c : (long)n * (h / 2) * (w / 2) * c;
    if (backward) {
        k_avgpool2_backward<<<blocks(out, 256), 256, 0, s>>>((const __half*)x, n, h, w, c, (__half*)y);
    } else if (c % 8 == 0 && aligned16(x) && aligned16(y)) {
        k_avgpool2_q<<<grid_for(out / 8), 256, 0, s>>>((const uint4*)x, n, h, w, c / 8, (uint4*)y);
    } else {
        k_avgpool2<<<blocks(out, 256), 256, 0, s>>>((const __half*)x, n, h, w, c, (__half*)y);
    }
    return launched();
}

extern "C" vv_status vv_nn_upsample2(const void* x, int n, int h, int w, int c, void* y, int backward,
                                     void* stream) {
    if (!x || !y || n <= 0 || h <= 0 || w <= 0 || c <= 0) return VV_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    long out = backward ? (long)n * h * w * c : 4L * n * h * w * c;
    if (backward) k_upsample2_backward<<<blocks(out, 256), 256, 0, s>>>((const __half*)x, n, h, w, c, (__half*)y);
    else k_upsample2<<<blocks(out, 256), 256, 0, s>>>((const __half*)x, n, h, w, c, (__half*)y);
    return launched();
}

extern "C" vv_status vv_nn_concat(const void* a, int ca, const void* b, int cb, long pixels, void* y,
                                  void* stream) {
    if (!a || !b || !y || ca <= 0 || cb <= 0 || pixels <= 0) return VV_ERR_ARG;
    long total = pixels * (ca + cb);
    k_concat<<<blocks(total, 256), 256, 0, (cudaStream_t)stream>>>((const __half*)a, ca, (const __half*)b, cb,
                                                                   pixels, (__half*)y);
    return launched();
}

extern "C" vv_status vv_nn_upsample_concat(const void* a, int n, int h, int w, int ca, const void* b, int cb,
                                           void* y, void* stream) {
    if (!a || !b || !y || n <= 0 || h <= 0 || w <= 0 || ca <= 0 || cb <= 0) return VV_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const long pixels = 4L * n * h * w;
    if (ca % 8 == 0 && cb % 8 == 0 && aligned16(a) && aligned16(b) && aligned16(y)) {
        k_upsample_concat<<<grid_for(pixels * ((ca + cb) / 8)), 256, 0, s>>>(
            (const uint4*)a, h, w, ca / 8, (const uint4*)b, cb / 8, pixels, (uint4*)y);
        return launched();
    }
    return VV_ERR_ARG;  // other shapes: vv_nn_upsample2, then vv_nn_concat
}

extern "C" vv_status vv_nn_split(const void* dy, int ca, int cb, long pixels, void* da, void* db, void* stream) {
    if (!dy || ca <= 0 || cb <= 0 || pixels <= 0) return VV_ERR_ARG;
    long total = pixels * (ca + cb);
    k_split<<<blocks(total, 256), 256, 0, (cudaStream_t)stream>>>((const __half*)dy, ca, cb, pixels, (__half*)da,
                                                                  (__half*)db);
    return launched();
}

extern "C" vv_status vv_nn_features(const float* accum, const float* albedo, const float* normal, float n,
                                    long pixels, void* x, void* stream) {
    if (!accum || !albedo || !normal || !x || !(n > 0.0f) || pixels <= 0) return VV_ERR_ARG;
    k_features<<<blocks(pixels, 256), 256, 0, (cudaStream_t)stream>>>((const float4*)accum, (const float4*)albedo,
                                                                      (const float4*)normal, n, pixels, (__half*)x);
    return launched();
}

extern "C" vv_status vv_nn_l1_loss(const void* pred, int c, const float* target, long pixels, float grad_scale,
                                   float* loss, void* dpred, void* stream) {
    if (!pred || !target || !loss || !dpred || c < 3 || pixels <= 0 || !(grad_scale > 0.0f)) return VV_ERR_ARG;
    k_l1_loss<<<blocks(pixels, 256), 256, 0, (cudaStream_t)stream>>>((const __half*)pred, c, target, pixels,
                                                                     grad_scale, loss, (__half*)dpred);
    return launched();
}

extern "C" vv_status vv_nn_adam(float* w, void* w16, const float* grad, float* m, float* v, long count, float lr,
                                float beta1, float beta2, float eps, float grad_scale, int step, void* stream) {
    if (!w || !grad || !m || !v || count <= 0 || step < 1 || !(grad_scale > 0.0f)) return VV_ERR_ARG;
    float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<blocks(count, 256), 256, 0, (cudaStream_t)stream>>>(w, (__half*)w16, grad, m, v, count, lr, beta1,
                                                                beta2, eps, 1.0f / grad_scale, c1, c2);
    return launched();
}

extern "C" vv_status vv_nn_add(void* y, const void* x, long count, void* stream) {
    if (!y || !x || count < 0) return VV_ERR_ARG;
    if (count == 0) return VV_OK;
    k_add<<<blocks(count, 256), 256, 0, (cudaStream_t)stream>>>((__half*)y, (const __half*)x, count);
    return launched();
}

extern "C" vv_status vv_nn_features_image(const float* accum, const float* albedo, const float* normal, float n,
                                          int w, int h, int wp, int hp, void* x, void* stream) {
    if (!accum || !albedo || !normal || !x || !(n > 0.0f) || w <= 0 || h <= 0 || wp < w || hp < h) return VV_ERR_ARG;
    k_features_image<<<blocks((long)wp * hp, 256), 256, 0, (cudaStream_t)stream>>>(
        (const float4*)accum, (const float4*)albedo, (const float4*)normal, n, w, h, wp, hp, (__half*)x);
    return launched();
}

extern "C" vv_status vv_nn_prediction_to_hdr(const void* pred, int c, int wp, int w, int h, const float* accum,
                                             float n, void* hdr, void* stream) {
    if (!pred || !accum || !hdr || c < 3 || w <= 0 || h <= 0 || wp < w || !(n > 0.0f)) return VV_ERR_ARG;
    k_prediction_to_hdr<<<blocks((long)w * h, 256), 256, 0, (cudaStream_t)stream>>>(
        (const __half*)pred, c, wp, w, h, (const float4*)accum, n, (ushort4*)hdr);
    return launched();
}

extern "C" vv_status vv_nn_radiance(const void* pred, int c, long pixels, float* rgb, void* stream) {
    if (!pred || !rgb || c < 3 || pixels <= 0) return VV_ERR_ARG;
    k_radiance<<<blocks(pixels, 256), 256, 0, (cudaStream_t)stream>>>((const __half*)pred, c, pixels, rgb);
    return launched();
}
