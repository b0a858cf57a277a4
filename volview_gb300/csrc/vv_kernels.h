// vv_kernels.h — launch interface between the host renderer and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "vv_device.cuh"

namespace vv {

struct MaskLaunch {
    Vol v;
    const void* density;        // stored as vol.dfmt
    const uint8_t* labels;
    const uint8_t* soft;
    int soft_dims[3];
    int soft_push[4];
    int margin;
    int radius;
    int mode;
    const float4* colors;
    uint32_t* scratch;  // mask B
    uint32_t* out;      // mask A (what rendering samples)
};

// Everything one path-tracing launch reads and writes.
struct PtArgs {
    UHead u;
    const void* density;        // stored as vol.dfmt
    const uint32_t* mask;
    const uint32_t* normals;
    const uint8_t* labels;
    const float* majorant;
    const float4* preint;       // cumulative transfer-function integrals, 4096 (ray marcher)
    const ushort4* env_diffuse; // light map's diffuse convolution, 32 x 16 RGBA16F (ray marcher)
    const ushort4* env_rad;     // light map radiance, RGBA16F, env_w x env_h (lighting.w == 2)
    const float2* env_table;    // light map sampling table, (env_w + 1) x env_h
    // Search guides of the sampling table: for bucket k of `env_gm` (of `env_gr`
    // per row) the first row (column) whose CDF reaches k / env_gm, clamped to
    // the last; the marginal's env_gm + 1 entries, then env_gr + 1 per row.
    const uint16_t* env_guide;
    int env_w, env_h, env_gm, env_gr;
    const float4* lut;          // transfer function, RGBA16F values as float
    const LabelTables* tab;
    Vol vol;
    float4* accum;
    float4* albedo;
    float4* normal;
    ushort4* hdr;
    uint32_t width, height;
    uint32_t frames;            // accumulate-frames in this launch
    uint32_t tiles_x, tiles_y;  // 8x4-pixel tiles
    uint32_t* counter;          // work-item counter, zero at launch
    int32_t* status;            // device status word (0 ok; read by vv_synchronize, written by no kernel)
    int persistent;             // 1: persistent warps with path regeneration
    int write_hdr;              // 1: accum/albedo/normal are the totals and a single-frame pass writes each
                                // pixel's HDR as it finishes; 0: they are the pass's own sums (merged later)
    unsigned long long* counters;  // event counters (COUNT_*), or null
};

// Event counters of a counting launch (for the algorithmic-byte model).
enum {
    COUNT_MAJORANT = 0,   // brick-majorant lookups (free flight and shadow rays), 4 B
    COUNT_CUBIC = 1,      // cubic B-spline densities, 4^3 x 2 B
    COUNT_TRILINEAR = 2,  // trilinear densities, 2^3 x 2 B
    COUNT_MASK = 3,       // trilinear mask lookups, 2^3 x 4 B
    COUNT_LABEL = 4,      // label fetches, 1 B
    COUNT_NORMAL = 5,     // trilinear normal lookups, 2^3 x 4 B
    COUNT_GRADIENT = 6,   // cubic B-spline gradients, 4^3 x 2 B
    COUNT_PIXEL = 7,      // pixel accumulations, 3 x (16 B read + 16 B write) + 8 B
    COUNT_PATH = 8,       // paths started
    COUNT_VERTEX = 9,     // path vertices (bounce-loop iterations)
    COUNT_N = 10
};

cudaError_t launch_density(const int16_t* hu, void* out, const Vol& v, cudaStream_t s);
cudaError_t launch_normals(const void* d, uint32_t* out, const Vol& v, const m3& w2i, cudaStream_t s);
cudaError_t launch_masks(const MaskLaunch& L, cudaStream_t s);
cudaError_t launch_majorant(const void* d, const uint32_t* mask, const Vol& v, int mode, float label_ext,
                            const float* bucket, float* out, cudaStream_t s);
cudaError_t launch_unbrick(const void* src, void* dst, const Vol& v, int elem, cudaStream_t s);
cudaError_t launch_brick_u8(const uint8_t* src, uint8_t* dst, const Vol& v, cudaStream_t s);

// Wavefront tracer state: per slot (path in flight) WF_SLOT_BYTES of records
// (path, accumulation, vertex, shaded vertex, shadow result; vv_wavefront.cu),
// WF_MAP_BYTES more with a light map, the stage queues (slot indices) and
// their counters. A slot's sample count has 20 bits: the wavefront takes
// fewer than WF_MAX_SAMPLES samples per frame.
constexpr int WF_SLOT_BYTES = 288;
constexpr int WF_MAP_BYTES = 16;  // per slot: the light map sample's direction
constexpr uint32_t WF_MAX_SAMPLES = 1u << 20;
enum {
    WF_EXT0 = 0, WF_EXT1 = 1, WF_SHADE = 2, WF_SHADOW = 3, WF_SCATTER = 4,
    WF_ITEMS = 5,     // next (frame, pixel) work item
    WF_TAKE_EXT = 6,  // entries of the extend queue taken so far
    WF_TAKE_SHADOW = 7,  // entries of the shadow queue taken so far
    WF_ESC0 = 8, WF_ESC1 = 9,  // flights that left the volume or hit the bounce limits
    WF_FIRST0 = 10, WF_FIRST1 = 11,  // first flights (bounce 0): a queue of their own
    WF_TAKE_FIRST = 12,  // entries of the first-flight queue taken so far
    WF_STOP = 13,     // 0 while waves run; 1 + the queue index the finishing launch takes over
    WF_MAP = 14,      // light map shadow rays queued by the key light's shadow rays
    WF_TAKE_MAP = 15, // entries of the light map shadow queue taken so far
    WF_COUNTERS = 16
};
struct WfArgs {
    uint32_t capacity;     // slots (and queue entries) allocated
    float4* path;          // 4 x float4 per slot
    float4* acc;           // 4 x float4 per slot
    float4* vtx;           // 4 x float4 per slot
    float4* shd;           // 4 x float4 per slot
    float4* sh;            // 2 x float4 per slot
    float4* mapdir;        // 1 x float4 per slot (light map)
    uint32_t* ext[2];      // later flights
    uint32_t* first[2];    // first flights
    uint32_t* esc[2];
    uint32_t* shade;
    uint32_t* shadow;
    uint32_t* scatter;
    uint32_t* map;         // slots whose light map shadow ray is next
    uint32_t* counts;      // WF_COUNTERS words
    // Later flights binned by the coarse cell of their origin and the octant
    // of their direction: the scatter kernel writes each queued slot's bin
    // beside it, a counting sort orders the queue into `sorted`, which the
    // next wave's later-flight extend reads.
    uint32_t* ext_key[2];
    uint32_t* sorted;
    uint32_t* bin_count;   // nbins counters (zero between waves)
    uint32_t* bin_next;    // nbins insertion points
    uint32_t nbins;
    int cell_shift;        // log2 of a cell's edge in voxels
    int cells_x, cells_y, cells_z;
    uint32_t bin_min;      // queues shorter than this are not ordered (the extend reads them as queued)
    // Batched passes only: each request's next work item (VV_BATCH_MAX words)
    // and its constants derived from the uniforms (VV_BATCH_MAX records of
    // WF_CONSTS_BYTES), written by the pass's first launch.
    uint32_t* items;
    void* consts;
};
// A batched pass (vv_batch_record): the work items of up to VV_BATCH_MAX
// requests share the pass's slots, queues and waves. Each request has its own
// volume, transfer function, uniforms, label tables, masks, majorants, image
// and frame count (its PtArgs) and owns the slots [slot_end[r - 1],
// slot_end[r]) (slot_end[-1] = 0); a slot serves its request for the whole
// pass.
constexpr int VV_BATCH_MAX = 8;
constexpr int WF_CONSTS_BYTES = 256;
struct PtBatch {
    uint32_t n;
    uint32_t slot_end[VV_BATCH_MAX];
    PtArgs a[VV_BATCH_MAX];
};
// A lighting volume as the image loop reads it: a 3D texture of its texels
// inside a one-texel white border, filtered by the texture units (clamped
// addressing onto the border = the reference's white-border sampler).
struct LightTex {
    cudaTextureObject_t tex;
    int w, h, d;  // texels of the volume, border excluded
    int rgba;     // 1: RGBA16F (shadow), 0: R16F (occlusion)
};

// The launchers of the path tracer and the ray marcher (vv_pt.cu,
// vv_wavefront.cu, vv_raymarch.cu), compiled once per storage format:
// namespace vv::fmtN holds those of density format N (DF_*, N < 4) with the
// RG16_UNORM mask, fmt4 and fmt5 those of FP16 and BF16 density with the mask
// in the same format; each build's samplers read its formats with no branch.
#define VV_FORMAT_LAUNCHERS                                                                                      \
    /* One or more accumulate-frames (pt.comp) with the single-kernel tracers. */                                \
    cudaError_t launch_pt(const PtArgs& a, int sms, cudaStream_t s, int* launches);                             \
    /* Accumulate-frames with the wavefront tracer (same results as launch_pt). */                              \
    cudaError_t launch_pt_wavefront(const PtArgs& a, const WfArgs& w, int sms, cudaStream_t s, int* launches);  \
    /* The ray marcher (path tracing off): occlusion volume (R16F), shadow volume */                            \
    /* swept slice by slice (RGBA16F), the image into a.hdr. */                                                  \
    cudaError_t launch_ao(const PtArgs& a, uint16_t* out, int ax, int ay, int az, cudaStream_t s);              \
    cudaError_t launch_shadow_sweep(const PtArgs& a, ushort4* vol, int sx, int sy, int sz, int axis, int sign,  \
                                    cudaStream_t s, int* launches);                                             \
    /* Copies a pixel-linear lighting volume (`channels` halves per texel) into its */                          \
    /* texture array through `surf`, white border included. */                                                   \
    cudaError_t launch_pad_lighting(const uint16_t* vol, int channels, int w, int h, int d,                      \
                                    cudaSurfaceObject_t surf, cudaStream_t s);                                  \
    cudaError_t launch_dvr(const PtArgs& a, const LightTex& shadow, const LightTex& ao, cudaStream_t s);        \
    /* Parity probes: B-spline density and gradient at n continuous indices; light */                           \
    /* map samples; one path per listed pixel at accumulation count a.u.path[0]. */                              \
    cudaError_t launch_bspline_probe(const PtArgs& a, const float* idx, float* out, int n, cudaStream_t s);     \
    cudaError_t launch_light_sample_probe(const PtArgs& a, const uint32_t* seeds, float* out, int n,            \
                                          cudaStream_t s);                                                      \
    cudaError_t launch_pt_pixels(const PtArgs& a, const int* px, float* out, int n, cudaStream_t s);            \
    /* The sampled extinction and the brick's flight majorant at n indices. */                                  \
    cudaError_t launch_extinction_probe(const PtArgs& a, const float* idx, float* out, int n, const float dir[3], \
                                        int smooth, cudaStream_t s);
namespace fmt0 { VV_FORMAT_LAUNCHERS }
namespace fmt1 { VV_FORMAT_LAUNCHERS }
namespace fmt2 { VV_FORMAT_LAUNCHERS }
namespace fmt3 { VV_FORMAT_LAUNCHERS }
namespace fmt4 { VV_FORMAT_LAUNCHERS }  // FP16 density and FP16 mask
namespace fmt5 { VV_FORMAT_LAUNCHERS }  // BF16 density and BF16 mask
// Batched passes run with the reference's storage (R16_UNORM density,
// RG16_UNORM mask): the wavefront of every request of the batch at once.
namespace fmt0 {
cudaError_t launch_pt_wavefront_batch(const PtBatch& b, const WfArgs& w, int sms, cudaStream_t s, int* launches);
}
// The parity build of the single-path probe (vv_pt_exact.cu), per format: the
// oracle's texture-unit arithmetic, no fused multiply-adds.
#define VV_EXACT_LAUNCHERS \
    cudaError_t launch_pt_pixels(const PtArgs& a, const int* px, float* out, int n, cudaStream_t s);
namespace exact0 { VV_EXACT_LAUNCHERS }
namespace exact1 { VV_EXACT_LAUNCHERS }
namespace exact2 { VV_EXACT_LAUNCHERS }
namespace exact3 { VV_EXACT_LAUNCHERS }
namespace exact4 { VV_EXACT_LAUNCHERS }
namespace exact5 { VV_EXACT_LAUNCHERS }

struct PostArgs {
    UHead u;
    uint32_t width, height;
    const float4* accum;
    const float4* albedo;
    const float4* normal;
    float4* ping;
    float4* pong;
    float4* guide_nd;    // denoiser guides per pixel: mean normal (normalised) and depth
    float4* guide_alb;   // mean albedo (floored at 0.02), w unused
    ushort4* hdr;
    ushort4* bloom[4];   // A, B (quarter), C, D (eighth)
    int bw[4], bh[4];
    float* exposure;     // 1 texel, adapted across frames
    uchar4* out;
};
// record_denoise (renderer.rs:1868-1904): 7 passes.
cudaError_t launch_denoise(const PostArgs& a, cudaStream_t s, int* launches);
// record_post (renderer.rs:1817-1866): bloom, exposure, tone mapping.
cudaError_t launch_post(const PostArgs& a, cudaStream_t s, int* launches);
// The merge with precise running sums (vv_precision): Kahan-compensated FP32
// sums and/or FP64 sums once past a sample count.
struct PreciseSums {
    float4* comp[3];  // compensation of accum, albedo, normal (kahan)
    double* wide[3];  // 4 doubles per pixel: the FP64 running sums
    int kahan;
    int wide_mode;    // 0: FP32 sums; 1: FP64 from now on (from the FP32 sums); 2: FP64 sums
};
cudaError_t launch_merge_precise(const PostArgs& a, const float4* accum, const float4* albedo, const float4* normal,
                                 const PreciseSums& ps, double n, cudaStream_t s);
// hdr = accum / n (the HDR store at the end of pt.comp) for batched frames.
cudaError_t launch_hdr_resolve(const PostArgs& a, float n, cudaStream_t s);
// A pass's own sums added to the accumulation images (a.accum/albedo/normal),
// then hdr = accum / n: the end of pt.comp for the pass's last frame.
cudaError_t launch_merge(const PostArgs& a, const float4* accum, const float4* albedo, const float4* normal, float n,
                         cudaStream_t s);

}  // namespace vv
