// vv_volume.cu — the per-volume passes: density upload, normals, label masks,
// brick majorants, and the unbricking copy used by readback.
//
// These passes are HBM-bound integer/FP stencils. Their arithmetic uses
// round-to-nearest intrinsics (__fmul_rn, __fadd_rn, ...) in the order the
// reference shaders evaluate it, so that their outputs match the reference bit
// for bit (the normals and masks are quantised, and a fused multiply-add could
// move a value across a rounding boundary).
#include <cuda_runtime.h>

#include <cuda_bf16.h>

#include "vv_device.cuh"
#include "vv_kernels.h"

namespace vv {

static const float HU_MIN = -1024.0f, HU_MAX = 3071.0f;

// hu_to_unorm16 (crates/render/src/transfer.rs:121-124) into the bricked
// layout; one thread per bricked element, reading the x-fastest source. The
// precision variants store the same normalised density t as FP16 or BF16
// (rounded to nearest even) or FP32 instead of round(t * 65535).
__global__ void k_density(const int16_t* __restrict__ hu, void* __restrict__ out, Vol v) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= vol_elems(v)) return;
    int x, y, z;
    vcoord(v, e, x, y, z);
    float t = 0.0f;
    if (x < v.nx && y < v.ny && z < v.nz) {
        float h = (float)hu[((long)z * v.ny + y) * v.nx + x];
        t = __fdiv_rn(__fsub_rn(h, HU_MIN), __fsub_rn(HU_MAX, HU_MIN));
        t = fminf(fmaxf(t, 0.0f), 1.0f);
    }
    switch (v.dfmt) {
        case DF_FP16: ((uint16_t*)out)[e] = __half_as_ushort(__float2half_rn(t)); break;
        case DF_BF16: ((uint16_t*)out)[e] = __bfloat16_as_ushort(__float2bfloat16_rn(t)); break;
        case DF_FP32: ((float*)out)[e] = t; break;
        default: ((uint16_t*)out)[e] = (uint16_t)roundf(__fmul_rn(t, 65535.0f));
    }
}

__device__ __forceinline__ float dens(const void* d, const Vol& v, int x, int y, int z) {
    x = clampi(x, 0, v.nx - 1);
    y = clampi(y, 0, v.ny - 1);
    z = clampi(z, 0, v.nz - 1);
    return density_texel(d, v.dfmt, voff(v, x, y, z));
}

__device__ __forceinline__ int8_t to_snorm8(float f) {
    return (int8_t)rintf(__fmul_rn(fminf(fmaxf(f, -1.0f), 1.0f), 127.0f));
}

// normals.comp:14-37: 3x3x3 Sobel, /32, world transform, -g/|g| and clamp(|g|*400).
__global__ void k_normals(const void* __restrict__ d, uint32_t* __restrict__ out, Vol v, m3 w) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= vol_elems(v)) return;
    int x, y, z;
    vcoord(v, e, x, y, z);
    if (x >= v.nx || y >= v.ny || z >= v.nz) { out[e] = 0; return; }
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++) {
            float wt = (float)((2 - abs(a)) * (2 - abs(b)));
            gx = __fadd_rn(gx, __fmul_rn(wt, __fsub_rn(dens(d, v, x + 1, y + a, z + b), dens(d, v, x - 1, y + a, z + b))));
            gy = __fadd_rn(gy, __fmul_rn(wt, __fsub_rn(dens(d, v, x + a, y + 1, z + b), dens(d, v, x + a, y - 1, z + b))));
            gz = __fadd_rn(gz, __fmul_rn(wt, __fsub_rn(dens(d, v, x + a, y + b, z + 1), dens(d, v, x + a, y + b, z - 1))));
        }
    gx = __fdiv_rn(gx, 32.0f);
    gy = __fdiv_rn(gy, 32.0f);
    gz = __fdiv_rn(gz, 32.0f);
    // transpose(mat3(world_to_index)) * g
    auto dotrn = [](f3 c, float p, float q, float r) {
        return __fadd_rn(__fadd_rn(__fmul_rn(c.x, p), __fmul_rn(c.y, q)), __fmul_rn(c.z, r));
    };
    float wx = dotrn(w.c0, gx, gy, gz), wy = dotrn(w.c1, gx, gy, gz), wz = dotrn(w.c2, gx, gy, gz);
    float l = __fsqrt_rn(dotrn(mk(wx, wy, wz), wx, wy, wz));
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (l > 1e-7f) {
        nx = __fdiv_rn(-wx, l);
        ny = __fdiv_rn(-wy, l);
        nz = __fdiv_rn(-wz, l);
    }
    float s = fminf(fmaxf(__fmul_rn(l, 400.0f), 0.0f), 1.0f);
    uint32_t q = (uint32_t)(uint8_t)to_snorm8(nx) | ((uint32_t)(uint8_t)to_snorm8(ny) << 8) |
                 ((uint32_t)(uint8_t)to_snorm8(nz) << 16) | ((uint32_t)(uint8_t)to_snorm8(s) << 24);
    out[e] = q;
}

// --------------------------------------------------------------------- masks
struct MaskArgs {
    Vol v;
    const void* density;
    const uint8_t* labels;
    const uint8_t* soft;  // RGBA8 nodes, x-fastest
    int sdims[3];
    int soft_push[4];     // axes, flip bits | 8 = present
    int margin;
    int mode;
    const float4* colors; // label_colors table
    float dims[3];
};

__device__ __forceinline__ bool label_shown(const float4* c, uint32_t l) { return __ldg(&c[l].w) > 0.5f; }
__device__ __forceinline__ bool label_ghosted(const float4* c, uint32_t l) { return l != 0u && __ldg(&c[l].w) > 1.5f; }
__device__ __forceinline__ bool label_solid(const float4* c, uint32_t l, uint32_t mode) {
    if (label_ghosted(c, l)) return false;
    return mode == 1u ? (l == 0u || label_shown(c, l)) : (l != 0u && label_shown(c, l));
}

__device__ __forceinline__ uint8_t label_at(const MaskArgs& A, int x, int y, int z) {
    return __ldg(A.labels + voff(A.v, x, y, z));
}

// Trilinear density at continuous index v (common.glsl:68-78): texel space via
// the normalised coordinate, as the texture unit computes it.
__device__ float density_linear_rn(const MaskArgs& A, float ix, float iy, float iz) {
    float p[3] = {ix, iy, iz};
    int i0[3];
    float fr[3];
    for (int k = 0; k < 3; k++) {
        float tc = __fdiv_rn(__fadd_rn(p[k], 0.5f), A.dims[k]);
        float uu = __fsub_rn(__fmul_rn(tc, A.dims[k]), 0.5f);
        float fl = floorf(uu);
        i0[k] = (int)fl;
        fr[k] = __fsub_rn(uu, fl);
    }
    float r = 0.0f;
    for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
            for (int di = 0; di < 2; di++) {
                float wgt = __fmul_rn(__fmul_rn(di ? fr[0] : __fsub_rn(1.0f, fr[0]), dj ? fr[1] : __fsub_rn(1.0f, fr[1])),
                                      dk ? fr[2] : __fsub_rn(1.0f, fr[2]));
                r = __fadd_rn(r, __fmul_rn(dens(A.density, A.v, i0[0] + di, i0[1] + dj, i0[2] + dk), wgt));
            }
    return r;
}

__device__ __forceinline__ float soft_score(bool best, bool second, float m) {
    const float CERTAIN = 4.0f;
    if (best == second) return best ? CERTAIN : -CERTAIN;
    return best ? fminf(m, CERTAIN) : -fminf(m, CERTAIN);
}

// mask.comp:62-100: joint bilateral upsampling of the soft grid's margins.
__device__ void soft_masks(const MaskArgs& A, int px, int py, int pz, const float xg[3], float& mr, float& mg) {
    const float SIGMA_CT = 40.0f / 4095.0f, CERTAIN = 4.0f;
    const int* ax = A.soft_push;
    int D[3] = {A.v.nx, A.v.ny, A.v.nz};
    float can[3] = {(float)D[ax[0]], (float)D[ax[1]], (float)D[ax[2]]};
    float to_grid[3];
    for (int k = 0; k < 3; k++)
        to_grid[k] = __fdiv_rn(__fsub_rn((float)A.sdims[k], 1.0f), fmaxf(__fsub_rn(can[k], 1.0f), 1.0f));
    float here = dens(A.density, A.v, px, py, pz);
    int center[3] = {(int)roundf(xg[0]), (int)roundf(xg[1]), (int)roundf(xg[2])};
    float sx = 0.0f, sy = 0.0f, wsum = 0.0f;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int node[3] = {clampi(center[0] + dx, 0, A.sdims[0] - 1), clampi(center[1] + dy, 0, A.sdims[1] - 1),
                               clampi(center[2] + dz, 0, A.sdims[2] - 1)};
                float d0 = __fsub_rn((float)node[0], xg[0]), d1 = __fsub_rn((float)node[1], xg[1]),
                      d2 = __fsub_rn((float)node[2], xg[2]);
                float dd = __fadd_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1)), __fmul_rn(d2, d2));
                float w_space = expf(__fdiv_rn(-dd, 2.0f * 0.6f * 0.6f));
                float c[3] = {__fdiv_rn((float)node[0], to_grid[0]), __fdiv_rn((float)node[1], to_grid[1]),
                              __fdiv_rn((float)node[2], to_grid[2])};
                float vv[3];
                for (int a = 0; a < 3; a++)
                    vv[ax[a]] = ((A.soft_push[3] >> a) & 1) != 0 ? __fsub_rn(__fsub_rn(can[a], 1.0f), c[a]) : c[a];
                float there = density_linear_rn(A, vv[0], vv[1], vv[2]);
                float df = __fsub_rn(here, there);
                float w_ct = expf(__fdiv_rn(-__fmul_rn(df, df), __fmul_rn(__fmul_rn(2.0f, SIGMA_CT), SIGMA_CT)));
                const uint8_t* t = A.soft + 4 * (((long)node[2] * A.sdims[1] + node[1]) * A.sdims[0] + node[0]);
                uint32_t best = t[0], second = t[1];
                float m = __fdiv_rn((float)t[2], 16.0f);
                float s0 = soft_score(label_solid(A.colors, best, A.mode), label_solid(A.colors, second, A.mode), m);
                float s1 = soft_score(label_ghosted(A.colors, best), label_ghosted(A.colors, second), m);
                float w = __fadd_rn(__fmul_rn(w_space, w_ct), __fmul_rn(1e-6f, w_space));
                sx = __fadd_rn(sx, __fmul_rn(w, s0));
                sy = __fadd_rn(sy, __fmul_rn(w, s1));
                wsum = __fadd_rn(wsum, w);
            }
    float a = __fdiv_rn(sx, wsum), b = __fdiv_rn(sy, wsum);
    mr = fminf(fmaxf(__fadd_rn(0.5f, __fdiv_rn(a, 2.0f * CERTAIN)), 0.0f), 1.0f);
    mg = fminf(fmaxf(__fadd_rn(0.5f, __fdiv_rn(b, 2.0f * CERTAIN)), 0.0f), 1.0f);
}

// mask.comp:107-138 (pass 0): binary or soft masks, and the tint-mode cut margin.
__global__ void k_mask_binary(MaskArgs A, uint32_t* __restrict__ out) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= vol_elems(A.v)) return;
    int x, y, z;
    vcoord(A.v, e, x, y, z);
    if (x >= A.v.nx || y >= A.v.ny || z >= A.v.nz) { out[e] = 0; return; }
    uint32_t mode = (uint32_t)A.mode;
    uint32_t label = label_at(A, x, y, z);
    float mr = label_solid(A.colors, label, mode) ? 1.0f : 0.0f;
    float mg = label_ghosted(A.colors, label) ? 1.0f : 0.0f;
    if ((A.soft_push[3] & 8) != 0 && label < 250u) {
        // soft_coord (mask.comp:40-50)
        int P[3] = {x, y, z};
        int D[3] = {A.v.nx, A.v.ny, A.v.nz};
        float xg[3];
        for (int a = 0; a < 3; a++) {
            float can = (float)D[A.soft_push[a]];
            float val = (float)P[A.soft_push[a]];
            float s = ((A.soft_push[3] >> a) & 1) != 0 ? __fsub_rn(__fsub_rn(can, 1.0f), val) : val;
            xg[a] = __fdiv_rn(__fmul_rn(s, __fsub_rn((float)A.sdims[a], 1.0f)), fmaxf(__fsub_rn(can, 1.0f), 1.0f));
        }
        int n0 = (int)roundf(xg[0]), n1 = (int)roundf(xg[1]), n2 = (int)roundf(xg[2]);
        n0 = clampi(n0, 0, A.sdims[0] - 1);  // texelFetch inside the grid by construction
        n1 = clampi(n1, 0, A.sdims[1] - 1);
        n2 = clampi(n2, 0, A.sdims[2] - 1);
        uint8_t over = A.soft[4 * (((long)n2 * A.sdims[1] + n1) * A.sdims[0] + n0) + 3];
        if (over == 0) soft_masks(A, x, y, z, xg, mr, mg);
    }
    int m = A.margin;
    if (mode == 1u && m > 0 && label == 0u) {
        for (int a = -m; a <= m && mr > 0.0f; a++)
            for (int b = -m; b <= m && mr > 0.0f; b++)
                for (int c = -m; c <= m; c++) {
                    uint32_t l = label_at(A, clampi(x + a, 0, A.v.nx - 1), clampi(y + b, 0, A.v.ny - 1),
                                          clampi(z + c, 0, A.v.nz - 1));
                    if (l != 0u && (!label_shown(A.colors, l) || label_ghosted(A.colors, l))) {
                        mr = 0.0f;
                        break;
                    }
                }
    }
    out[e] = mask_encode(mr, A.v.mfmt) | (mask_encode(mg, A.v.mfmt) << 16);
}

// mask.comp:260-278 (passes 1-3): binomial blur of radius r along one axis.
__global__ void k_mask_blur(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, Vol v, int axis, int r) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= vol_elems(v)) return;
    int x, y, z;
    vcoord(v, e, x, y, z);
    if (x >= v.nx || y >= v.ny || z >= v.nz) { dst[e] = 0; return; }
    float sx = 0.0f, sy = 0.0f, c = 1.0f;
    for (int j = 0; j <= 2 * r; j++) {
        int q[3] = {x, y, z};
        q[axis] += j - r;
        q[0] = clampi(q[0], 0, v.nx - 1);
        q[1] = clampi(q[1], 0, v.ny - 1);
        q[2] = clampi(q[2], 0, v.nz - 1);
        uint32_t m = __ldg(src + voff(v, q[0], q[1], q[2]));
        sx = __fadd_rn(sx, __fmul_rn(c, mask_decode(m & 0xffffu, v.mfmt)));
        sy = __fadd_rn(sy, __fmul_rn(c, mask_decode(m >> 16, v.mfmt)));
        c = __fdiv_rn(__fmul_rn(c, (float)(2 * r - j)), (float)(j + 1));
    }
    float n = exp2f((float)(2 * r));
    sx = __fdiv_rn(sx, n);
    sy = __fdiv_rn(sy, n);
    dst[e] = mask_encode(sx, v.mfmt) | (mask_encode(sy, v.mfmt) << 16);
}

// majorant.comp:26-71: one thread per brick over the brick and two voxels of border.
__global__ void k_majorant(const void* __restrict__ d, const uint32_t* __restrict__ mask, Vol v, int mode,
                           float label_ext, const float* __restrict__ bucket, float* __restrict__ out) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    int nb = v.bx * v.by * v.bz;
    if (b >= nb) return;
    int bxi = b % v.bx, byi = (b / v.bx) % v.by, bzi = b / (v.bx * v.by);
    int lo[3] = {max(bxi * 8 - 2, 0), max(byi * 8 - 2, 0), max(bzi * 8 - 2, 0)};
    int hi[3] = {min(bxi * 8 + 9, v.nx - 1), min(byi * 8 + 9, v.ny - 1), min(bzi * 8 + 9, v.nz - 1)};
    float dmin = 1.0f, dmax = 0.0f, mmax = 0.0f;
    for (int z = lo[2]; z <= hi[2]; z++) {
        int oz = offz(v, z);
        for (int y = lo[1]; y <= hi[1]; y++) {
            int oyz = oz + offy(v, y);
            for (int x = lo[0]; x <= hi[0]; x++) {
                int o = oyz + offx(x);
                float dv = density_texel(d, v.dfmt, o);
                dmin = gmin(dmin, dv);
                dmax = gmax(dmax, dv);
                if (mode != 0) {
                    uint32_t m = __ldg(mask + o);
                    mmax = gmax(mmax, gmax(mask_decode(m & 0xffffu, v.mfmt), mask_decode(m >> 16, v.mfmt)));
                }
            }
        }
    }
    auto tf_max = [&](float lo_, float hi_) {
        int first = clampi((int)(lo_ * 64.0f), 0, 63), last = clampi((int)(hi_ * 64.0f), 0, 63);
        float m = 0.0f;
        for (int k = first; k <= last; k++) m = gmax(m, bucket[k]);
        return m;
    };
    float bound;
    if (mode == 0) bound = tf_max(dmin, dmax);
    else if (mmax <= 0.0f) bound = 0.0f;
    else if (mode == 1) bound = tf_max(dmin, dmax);
    else bound = label_ext;
    out[b] = bound;
}

// Bricked -> x-fastest copy of `elem`-byte elements.
__global__ void k_unbrick(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, Vol v, int elem) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    long n = (long)v.nx * v.ny * v.nz;
    if (i >= n) return;
    int x = (int)(i % v.nx), y = (int)((i / v.nx) % v.ny), z = (int)(i / ((long)v.nx * v.ny));
    long o = voff(v, x, y, z);
    for (int k = 0; k < elem; k++) dst[i * elem + k] = src[o * elem + k];
}

// x-fastest -> bricked copy of bytes (labels).
__global__ void k_brick_u8(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, Vol v) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= vol_elems(v)) return;
    int x, y, z;
    vcoord(v, e, x, y, z);
    dst[e] = (x < v.nx && y < v.ny && z < v.nz) ? src[((long)z * v.ny + y) * v.nx + x] : 0;
}

static unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_density(const int16_t* hu, void* out, const Vol& v, cudaStream_t s) {
    k_density<<<blocks_for(vol_elems(v), 256), 256, 0, s>>>(hu, out, v);
    return cudaGetLastError();
}
cudaError_t launch_normals(const void* d, uint32_t* out, const Vol& v, const m3& w2i, cudaStream_t s) {
    k_normals<<<blocks_for(vol_elems(v), 256), 256, 0, s>>>(d, out, v, w2i);
    return cudaGetLastError();
}
cudaError_t launch_masks(const MaskLaunch& L, cudaStream_t s) {
    MaskArgs A;
    A.v = L.v;
    A.density = L.density;
    A.labels = L.labels;
    A.soft = L.soft;
    for (int k = 0; k < 3; k++) A.sdims[k] = L.soft_dims[k];
    for (int k = 0; k < 4; k++) A.soft_push[k] = L.soft_push[k];
    A.margin = L.margin;
    A.mode = L.mode;
    A.colors = L.colors;
    A.dims[0] = (float)L.v.nx;
    A.dims[1] = (float)L.v.ny;
    A.dims[2] = (float)L.v.nz;
    unsigned nb = blocks_for(vol_elems(L.v), 256);
    k_mask_binary<<<nb, 256, 0, s>>>(A, L.scratch);
    k_mask_blur<<<nb, 256, 0, s>>>(L.scratch, L.out, L.v, 0, L.radius);
    k_mask_blur<<<nb, 256, 0, s>>>(L.out, L.scratch, L.v, 1, L.radius);
    k_mask_blur<<<nb, 256, 0, s>>>(L.scratch, L.out, L.v, 2, L.radius);
    return cudaGetLastError();
}
cudaError_t launch_majorant(const void* d, const uint32_t* mask, const Vol& v, int mode, float label_ext,
                            const float* bucket, float* out, cudaStream_t s) {
    int nb = v.bx * v.by * v.bz;
    k_majorant<<<blocks_for(nb, 128), 128, 0, s>>>(d, mask, v, mode, label_ext, bucket, out);
    return cudaGetLastError();
}
cudaError_t launch_unbrick(const void* src, void* dst, const Vol& v, int elem, cudaStream_t s) {
    long n = (long)v.nx * v.ny * v.nz;
    k_unbrick<<<blocks_for(n, 256), 256, 0, s>>>((const uint8_t*)src, (uint8_t*)dst, v, elem);
    return cudaGetLastError();
}
cudaError_t launch_brick_u8(const uint8_t* src, uint8_t* dst, const Vol& v, cudaStream_t s) {
    k_brick_u8<<<blocks_for(vol_elems(v), 256), 256, 0, s>>>(src, dst, v);
    return cudaGetLastError();
}

}  // namespace vv
