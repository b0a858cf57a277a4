// vv_device.cuh — device-side building blocks of the GB300 path tracer.
//
// Data layout in HBM: every voxel volume (density R16_UNORM, mask RG16_UNORM,
// normals RGBA8_SNORM, labels R8_UINT) is stored in 8^3-voxel bricks, bricks in
// x-fastest order, each brick made of eight 4^3 sub-bricks (a 4^3 sub-brick of
// 16-bit density is one 128-byte line). The offset of voxel (x, y, z) is a sum of
// per-axis terms (offx + offy + offz), so gathers cost the same address
// arithmetic as a linear layout while 2x2x2 and 4x4x4 neighbourhoods touch
// 2-3x fewer 32-byte sectors.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

namespace vv {

// --------------------------------------------------------------- float3 math
struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__host__ __device__ __forceinline__ f3 mk(float s) { return {s, s, s}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ f3 operator*(float s, f3 a) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator-(float s, f3 a) { return {s - a.x, s - a.y, s - a.z}; }
__host__ __device__ __forceinline__ f3 operator+(float s, f3 a) { return {s + a.x, s + a.y, s + a.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ f3& operator+=(f3& a, f3 b) { a = a + b; return a; }
__host__ __device__ __forceinline__ f3& operator*=(f3& a, f3 b) { a = a * b; return a; }
__host__ __device__ __forceinline__ f3& operator*=(f3& a, float s) { a = a * s; return a; }
__host__ __device__ __forceinline__ f3& operator/=(f3& a, float s) { a = a / s; return a; }
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float len(f3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ f3 normalize(f3 a) { return a / len(a); }
// GLSL min/max: y if y < x (resp. x < y), else x.
__host__ __device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__host__ __device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__host__ __device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__host__ __device__ __forceinline__ f3 gmax(f3 a, float s) { return {gmax(a.x, s), gmax(a.y, s), gmax(a.z, s)}; }
__host__ __device__ __forceinline__ f3 gmin(f3 a, f3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
__host__ __device__ __forceinline__ f3 gmax(f3 a, f3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
__host__ __device__ __forceinline__ f3 gclamp(f3 a, float lo, float hi) {
    return {gclamp(a.x, lo, hi), gclamp(a.y, lo, hi), gclamp(a.z, lo, hi)};
}
__host__ __device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__host__ __device__ __forceinline__ f3 mix3(f3 x, f3 y, float a) { return x * (1.0f - a) + y * a; }
__host__ __device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float t = gclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__host__ __device__ __forceinline__ float comp(f3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__host__ __device__ __forceinline__ float maxc(f3 a) { return gmax(a.x, gmax(a.y, a.z)); }

// Column-major 3x3 matrix.
struct m3 {
    f3 c0, c1, c2;
};
__host__ __device__ __forceinline__ f3 mul(const m3& m, f3 v) { return m.c0 * v.x + m.c1 * v.y + m.c2 * v.z; }
// transpose(m) * v: the dot products of v with the columns.
__host__ __device__ __forceinline__ f3 mul_t(const m3& m, f3 v) { return {dot(m.c0, v), dot(m.c1, v), dot(m.c2, v)}; }

// ------------------------------------------------------------ uniform block
// The scalar head of the reference's std140 uniform block (renderer.rs:43-74),
// 720 bytes: passed to kernels by value (constant bank, uniform across warps).
struct alignas(16) UHead {
    float w2i[16];  // world_to_index, column-major
    float eye[4], forward[4], right[4], up[4], dims[4];
    uint32_t flags[4];
    float labels[4], light_dir[4], ambient[4], material[4];
    uint32_t lighting[4];
    float light_cells[4];
    uint32_t clip[4];
    float clip_planes[12];
    float clip_normals[12];
    float subsurface[4];
    uint32_t path[4];
    float env[4], lens[4], finish[4], tissue[4];
    float tf_bucket_max[64];
};
static_assert(sizeof(UHead) == 720, "uniform head layout");

// The per-label tables that follow the head (5 x 256 vec4), read through L1.
struct LabelTables {
    float4 colors[256];
    float4 materials[256];
    float4 density[256];
    float4 surface[256];
    float4 optics[256];
};
static_assert(sizeof(LabelTables) == 20480, "label table layout");

// ------------------------------------------------------------ bricked volumes
struct Vol {
    int nx, ny, nz;     // voxels
    int bx, by, bz;     // bricks per axis
    int sy, sz;         // element strides of a brick row / brick slab
    int dfmt;           // storage format of the density volume (DF_*)
    int mfmt;           // storage format of the label mask volume's two channels (MF_*)
};

// Density storage formats (vv_precision::density_format): the reference's
// R16_UNORM, or the density itself as FP16, BF16 or FP32.
enum { DF_UNORM16 = 0, DF_FP16 = 1, DF_BF16 = 2, DF_FP32 = 3 };
__host__ __device__ __forceinline__ int density_bytes(int dfmt) { return dfmt == DF_FP32 ? 4 : 2; }
// Label mask storage formats (vv_precision::mask_format): two 16-bit channels
// per voxel as the reference's RG16_UNORM, or as FP16 or BF16 values.
enum { MF_UNORM16 = 0, MF_FP16 = 1, MF_BF16 = 2 };

__host__ __device__ __forceinline__ Vol make_vol(int nx, int ny, int nz) {
    Vol v;
    v.nx = nx; v.ny = ny; v.nz = nz;
    v.bx = (nx + 7) >> 3; v.by = (ny + 7) >> 3; v.bz = (nz + 7) >> 3;
    v.sy = v.bx * 512;
    v.sz = v.bx * v.by * 512;
    v.dfmt = DF_UNORM16;
    v.mfmt = MF_UNORM16;
    return v;
}
__host__ __device__ __forceinline__ long vol_elems(const Vol& v) { return (long)v.bx * v.by * v.bz * 512; }
__host__ __device__ __forceinline__ int offx(int x) { return ((x >> 3) << 9) | ((x & 4) << 4) | (x & 3); }
__host__ __device__ __forceinline__ int offy(const Vol& v, int y) { return (y >> 3) * v.sy + ((y & 4) << 5) + ((y & 3) << 2); }
__host__ __device__ __forceinline__ int offz(const Vol& v, int z) { return (z >> 3) * v.sz + ((z & 4) << 6) + ((z & 3) << 4); }
__host__ __device__ __forceinline__ int voff(const Vol& v, int x, int y, int z) { return offx(x) + offy(v, y) + offz(v, z); }
// Inverse of voff for an element index (for brick-order passes).
__host__ __device__ __forceinline__ void vcoord(const Vol& v, long e, int& x, int& y, int& z) {
    long b = e >> 9;
    int w = (int)(e & 511);
    int sub = w >> 6, in = w & 63;
    int bxi = (int)(b % v.bx), byi = (int)((b / v.bx) % v.by), bzi = (int)(b / ((long)v.bx * v.by));
    x = (bxi << 3) | ((sub & 1) << 2) | (in & 3);
    y = (byi << 3) | (((sub >> 1) & 1) << 2) | ((in >> 2) & 3);
    z = (bzi << 3) | (((sub >> 2) & 1) << 2) | (in >> 4);
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ float unorm16(uint32_t u) { return (float)u / 65535.0f; }

#ifdef __CUDACC__
// One 16-bit mask channel: decode to a float, and the store's conversion
// (UNORM16: clamp, scale, round to nearest even; FP16 and BF16: round to
// nearest even).
__device__ __forceinline__ float mask_decode(uint32_t code, int mfmt) {
    if (mfmt == MF_FP16) return __half2float(__ushort_as_half((unsigned short)code));
    if (mfmt == MF_BF16) return __uint_as_float(code << 16);
    return unorm16(code);
}
__device__ __forceinline__ uint32_t mask_encode(float f, int mfmt) {
    if (mfmt == MF_FP16) return __half_as_ushort(__float2half_rn(f));
    if (mfmt == MF_BF16) {
        uint32_t w = __float_as_uint(f);
        return (w + 0x7fffu + ((w >> 16) & 1u)) >> 16;
    }
    return (uint32_t)rintf(__fmul_rn(fminf(fmaxf(f, 0.0f), 1.0f), 65535.0f));
}
#endif

#ifdef __CUDACC__
// A density element stored as F (its C type: 16 bits, or a float for FP32),
// in the format's filtering units: a UNORM16 code as its integer (filtered,
// then scaled by density_unit = 1/65535, as the path tracer's samplers do),
// the others as the density itself (scale 1).
template <int F> struct DensityStore { typedef uint16_t type; };
template <> struct DensityStore<DF_FP32> { typedef float type; };
template <int F> __device__ __forceinline__ float density_decode(uint16_t v) {
    if (F == DF_FP16) return __half2float(__ushort_as_half(v));
    if (F == DF_BF16) return __uint_as_float((uint32_t)v << 16);
    return (float)v;
}
template <int F> __device__ __forceinline__ float density_decode(float v) { return v; }
template <int F> __device__ __forceinline__ float density_unit() { return F == DF_UNORM16 ? 1.0f / 65535.0f : 1.0f; }
// Element o decoded to a density in [0, 1] (the texel a sampler reads).
__device__ __forceinline__ float density_texel(const void* d, int dfmt, long o) {
    switch (dfmt) {
        case DF_FP16: return density_decode<DF_FP16>(__ldg((const uint16_t*)d + o));
        case DF_BF16: return density_decode<DF_BF16>(__ldg((const uint16_t*)d + o));
        case DF_FP32: return __ldg((const float*)d + o);
        default: return unorm16(__ldg((const uint16_t*)d + o));
    }
}
#endif
__device__ __forceinline__ float snorm8(int c) { return gmax((float)c / 127.0f, -1.0f); }

}  // namespace vv
