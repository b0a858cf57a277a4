// vv_pt.cu — the progressive volume path tracer (shaders/pt.comp with
// shaders/common.glsl and shaders/shading.glsl) for sm_103a.
//
// Design:
//  * Voxel volumes are bricked (vv_device.cuh); samplers are software
//    trilinear in FP32 (exact weights, no 8-bit texture-unit fractions).
//  * The cubic B-spline value and gradient are evaluated directly from the 4^3
//    voxel neighbourhood (64 taps, separable weights) instead of the reference's
//    8 (value) + 24 (gradient) trilinear fetches: the same filter
//    (Sigg & Hadwiger fold the same weights into linear fetches), 64 loads
//    instead of 256 for the gradient.
//  * A path is a resumable state (start / one bounce / finish). The persistent
//    kernel keeps every lane busy: when a lane's path ends it takes the next
//    (pixel, frame) work item, found with a warp ballot and one atomicAdd per
//    warp, while the other lanes continue their bounces.
//  * The uniform head is a by-value kernel parameter (constant bank); the
//    per-label tables are read through L1.
#include <cuda_runtime.h>

#include "vv_pt_device.cuh"

namespace vv {
namespace VV_FMT_NS {  // this density format's kernels and launchers

// The reference's shape: one thread per pixel, one frame (8x8 blocks).
__global__ void __launch_bounds__(64, 8) k_pt_frame(const __grid_constant__ PtArgs A) {
    uint32_t px = blockIdx.x * 8 + threadIdx.x % 8, py = blockIdx.y * 8 + threadIdx.x / 8;
    if (px >= A.width || py >= A.height) return;
    Consts C = make_consts(A);
    Path P;
    PixelSums S = {mk(0.0f), 0.0f, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
    P.rng.s = seed_of(px, py, A.u.path[0]);
    P.rng.pcg();
    for (uint32_t k = 0; k < A.u.path[2]; k++) {
        start_path(A, C, P, px, py);
        while (bounce_step(A, C, P, S)) {
        }
        finish_path(P, S);
    }
    accumulate(A, px, py, S, false, A.write_hdr != 0, (float)(A.u.path[0] + A.u.path[2]));
}

// Persistent warps over (frame, 8x4 tile) work items with per-lane path
// regeneration: a lane whose pixel is done takes the next pixel of its warp's
// queue; the warp refills its queue (32 pixels of one tile) with one atomicAdd
// when every lane has drained it.
__global__ void __launch_bounds__(128, 4) k_pt_persistent(const __grid_constant__ PtArgs A) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tiles = A.tiles_x * A.tiles_y;
    const uint32_t items = tiles * A.frames;
    const uint32_t spf = A.u.path[2];
    const bool multi = A.frames > 1;
    Consts C = make_consts(A);
    Path P;
    PixelSums S;
    uint32_t px = 0, py = 0, sample = 0;
    bool active = false;
    // The warp's current item and which of its 32 pixels have been handed out.
    uint32_t item = 0xffffffffu;
    uint32_t taken = 0xffffffffu;  // all taken: fetch a new item first
    bool exhausted = false;
    for (;;) {
        // Lanes without a pixel take the next one from the warp's item.
        uint32_t need = __ballot_sync(0xffffffffu, !active);
        while (need && !exhausted) {
            if (taken == 0xffffffffu) {
                uint32_t it = 0;
                if (lane == 0) it = atomicAdd(A.counter, 1u);
                it = __shfl_sync(0xffffffffu, it, 0);
                if (it >= items) { exhausted = true; break; }
                item = it;
                // pixels outside the image count as taken
                uint32_t t = item % tiles;
                uint32_t tx = t % A.tiles_x, ty = t / A.tiles_x;
                uint32_t mx = tx * 8 + (lane & 7), my = ty * 4 + (lane >> 3);
                taken = __ballot_sync(0xffffffffu, mx >= A.width || my >= A.height);
            }
            uint32_t free_px = ~taken;
            // Match the k-th needy lane with the k-th free pixel.
            int rank = __popc(need & ((1u << lane) - 1u));
            bool mine = (need >> lane) & 1u;
            int nfree = __popc(free_px);
            int nneed = __popc(need);
            int give = min(nfree, nneed);
            if (mine && rank < give) {
                // position of the rank-th set bit of free_px
                uint32_t f = free_px;
                for (int k = 0; k < rank; k++) f &= f - 1u;
                uint32_t slot = __ffs(f) - 1u;
                uint32_t t = item % tiles, frame = item / tiles;
                uint32_t tx = t % A.tiles_x, ty = t / A.tiles_x;
                px = tx * 8 + (slot & 7);
                py = ty * 4 + (slot >> 3);
                uint32_t accumulated = A.u.path[0] + frame * spf;
                P.rng.s = seed_of(px, py, accumulated);
                P.rng.pcg();
                S = {mk(0.0f), 0.0f, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
                sample = 0;
                start_path(A, C, P, px, py);
                active = true;
            }
            // Mark the handed-out pixels taken and the served lanes satisfied.
            uint32_t served = __ballot_sync(0xffffffffu, mine && rank < give);
            uint32_t f = free_px;
            for (int k = 0; k < give; k++) {
                uint32_t bit = f & (0u - f);
                taken |= bit;
                f &= f - 1u;
            }
            need &= ~served;
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) break;
        if (active) {
            if (!bounce_step(A, C, P, S)) {
                finish_path(P, S);
                if (++sample < spf) {
                    start_path(A, C, P, px, py);
                } else {
                    accumulate(A, px, py, S, multi, !multi && A.write_hdr != 0, (float)(A.u.path[0] + spf));
                    active = false;
                }
            }
        }
    }
}

cudaError_t launch_pt(const PtArgs& a, int sms, cudaStream_t s, int* launches) {
    if (!a.persistent) {
        dim3 grid((a.width + 7) / 8, (a.height + 7) / 8);
        k_pt_frame<<<grid, 64, 0, s>>>(a);
        *launches += 1;
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pt_persistent, 128, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    k_pt_persistent<<<sms * per_sm, 128, 0, s>>>(a);
    *launches += 1;
    return cudaGetLastError();
}

// ------------------------------------------------------------- parity probes
__global__ void k_bspline_probe(const __grid_constant__ PtArgs A, const float* idx, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 p = mk(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]);
    float v = density_cubic(A, p);
    f3 g = density_gradient_cubic(A, p);
    out[4 * i] = v; out[4 * i + 1] = g.x; out[4 * i + 2] = g.y; out[4 * i + 3] = g.z;
}
cudaError_t launch_bspline_probe(const PtArgs& a, const float* idx, float* out, int n, cudaStream_t s) {
    k_bspline_probe<<<(n + 127) / 128, 128, 0, s>>>(a, idx, out, n);
    return cudaGetLastError();
}

// The extinction a flight samples at idx (extinction_at, pt.comp:277-292, with
// path_sigma) and the flight majorant of the brick there: out[4n] = sigma.xyz, majorant.
__global__ void k_extinction_probe(const __grid_constant__ PtArgs A, const float* idx, float* out, int n, f3 dir,
                                   int smooth) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 p = mk(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]);
    int cap = -1;
    float cut = clip_depth(A, p, cap);
    Sample s;
    float ext = cut > 0.0f ? 0.0f : extinction_unclipped(A, p, dir, smooth != 0, s, cap, cut);
    f3 sigma = ext > 0.0f ? path_sigma(A, s, ext) : mk(0.0f);
    out[4 * i] = sigma.x; out[4 * i + 1] = sigma.y; out[4 * i + 2] = sigma.z;
    out[4 * i + 3] = flight_majorant_of(A, brick_index(A, p));
}
cudaError_t launch_extinction_probe(const PtArgs& a, const float* idx, float* out, int n, const float dir[3],
                                    int smooth, cudaStream_t s) {
    k_extinction_probe<<<(n + 127) / 128, 128, 0, s>>>(a, idx, out, n, mk(dir[0], dir[1], dir[2]), smooth);
    return cudaGetLastError();
}
__global__ void k_light_sample_probe(const __grid_constant__ PtArgs A, const uint32_t* seeds, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng rng;
    rng.s = seeds[i];
    Rng replay = rng;
    int x, y;
    env_texel(A, replay, x, y);
    float pdf;
    f3 d = sample_env(A, rng, pdf);
    out[6 * i] = (float)x;
    out[6 * i + 1] = (float)y;
    out[6 * i + 2] = pdf;
    out[6 * i + 3] = d.x; out[6 * i + 4] = d.y; out[6 * i + 5] = d.z;
}
cudaError_t launch_light_sample_probe(const PtArgs& a, const uint32_t* seeds, float* out, int n, cudaStream_t s) {
    k_light_sample_probe<<<(n + 127) / 128, 128, 0, s>>>(a, seeds, out, n);
    return cudaGetLastError();
}

#include "vv_pt_probe.cuh"

}  // namespace VV_FMT_NS
}  // namespace vv
