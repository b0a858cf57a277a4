// vv_wavefront.cu — the wavefront path tracer: each bounce of every live path
// runs as four compact stage kernels over compacted queues of path slots.
//
//   extend   free flight to the next scattering vertex (or the escape)
//   shade    surface frame, texture, event choice, guides, light sample
//   shadow   ratio-tracked transmittance towards the light sample
//   scatter  light contribution, next direction, Russian roulette
//
// Every kernel executes one small piece of code for all its lanes, so warps
// stay converged between stages and the instruction working set fits the
// caches (the single-kernel tracer spends most cycles waiting on instruction
// fetch). Paths whose stage ends append themselves to the next stage's queue
// with one warp-aggregated atomicAdd per warp (ballot + popc). The random
// numbers are consumed in the reference's order (pt.comp), so a slot replays
// the same path as the reference-shaped kernel.
//
// Work items are (frame, pixel) pairs; a slot traces one item's samples in
// turn (the reference's per-pixel stream for one frame), then takes the next
// item from a global counter, so the frames of one pixel run in parallel and
// slow pixels do not queue their frames behind each other. With one frame per
// launch each slot owns its pixel and accumulates without atomics. When few
// paths are left, the rest run to completion in one launch of the
// single-kernel tracer (k_wf_finish), instead of many nearly empty waves for
// the longest random walks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "vv_pt_device.cuh"

namespace vv {
namespace VV_FMT_NS {  // this density format's kernels and launchers

// Path state, one record array per producer, indexed by slot. Each record is
// a whole number of 32-byte DRAM sectors and every stage writes whole sectors,
// so a stage reads only what it uses and no sector is left half-written:
//
//   record  bytes  written by            read by
//   PATH    64     scatter, init         extend (all), shade (sector 0)
//   ACC     64     scatter, init; shade  scatter (sector 0 each vertex, all at
//                  (sector 1, bounce 0)  the path's end), shade (bounce 0)
//   VTX     64     extend                shade; scatter (escapes: sector 1)
//   SHD     64     shade                 shadow (sector 0), scatter
//   SH      32     shadow                scatter
//   MAPDIR  16     shadow (light map)    scatter (light map)
//
// PATH: P0 origin.xyz, rng | P1 dir.xyz, bounce | surfaces << 16
//       P2 spectral.xyz, volumes | sample << 10 | hero << 30 | P3 throughput.xyz, last_pdf
// ACC:  A0 radiance.xyz, item | A1 sum.xyz, background | A2 albedo sums | A3 normal sums
// VTX:  V0 idx.xyz, cut | V1 sample albedo.xyz, extinction
//       V2 roughness, metalness, density, subsurface | V3 coat, label word, rng, escape flag
// SHD:  S0 idx.xyz, rng | S1 light direction.xyz, event word
//       S2 albedo.xyz, roughness | S3 shading normal.xyz, metalness
// SH:   H0 light transmittance.xyz, rng | H1 light map radiance / pdf x transmittance.xyz, pdf
// MAPDIR: the light map sample's direction.xyz
//
// The SHD event word is the coat (a float in [0, 1]) for a surface event; for
// a volume event, which needs no coat, roughness, metalness or normal, it is
// EV_VOLUME | label | ghost << 16 (a NaN pattern no coat takes).
enum { PATH_N = 4, ACC_N = 4, VTX_N = 4, SHD_N = 4, SH_N = 2 };
static_assert((PATH_N + ACC_N + VTX_N + SHD_N + SH_N) * 16 == WF_SLOT_BYTES, "slot layout");
static_assert(16 == WF_MAP_BYTES, "light map record");
constexpr uint32_t EV_VOLUME = 0xFFC00000u;
constexpr uint32_t SAMPLE_BITS = 20u;  // samples per frame below 2^20 (WF_MAX_SAMPLES)
static_assert((1u << SAMPLE_BITS) == WF_MAX_SAMPLES, "sample field");

__device__ __forceinline__ float4* rec(float4* base, uint32_t s, int n) { return base + (size_t)s * n; }
__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ f3 xyz(float4 q) { return mk(q.x, q.y, q.z); }
__device__ __forceinline__ uint32_t ubits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float fbits(uint32_t u) { return __uint_as_float(u); }

__device__ __forceinline__ uint32_t path_word(const Path& P, uint32_t sample) {
    return P.volumes | (sample << 10) | ((uint32_t)P.hero << 30);
}
__device__ __forceinline__ void unpack_path_word(uint32_t w, Path& P, uint32_t& sample) {
    P.volumes = w & 1023u;
    sample = (w >> 10) & ((1u << SAMPLE_BITS) - 1u);
    P.hero = (int)(w >> 30);
}
__device__ void load_path(const WfArgs& W, uint32_t s, Path& P, uint32_t& sample) {
    const float4* q = rec(W.path, s, PATH_N);
    float4 a = q[0], b = q[1], c = q[2], d = q[3];
    P.origin = xyz(a);
    P.rng.s = ubits(a.w);
    P.dir = xyz(b);
    P.bounce = ubits(b.w) & 0xffffu;
    P.surfaces = ubits(b.w) >> 16;
    P.spectral = xyz(c);
    unpack_path_word(ubits(c.w), P, sample);
    P.throughput = xyz(d);
    P.last_pdf = d.w;
}
__device__ void store_path(const WfArgs& W, uint32_t s, const Path& P, uint32_t sample) {
    float4* q = rec(W.path, s, PATH_N);
    q[0] = f4(P.origin, fbits(P.rng.s));
    q[1] = f4(P.dir, fbits(P.bounce | (P.surfaces << 16)));
    q[2] = f4(P.spectral, fbits(path_word(P, sample)));
    q[3] = f4(P.throughput, P.last_pdf);
}
// ACC sector 0: the path's radiance, its work item, the pixel's sum and background.
__device__ void load_acc_head(const WfArgs& W, uint32_t s, Path& P, uint32_t& item, PixelSums& S) {
    const float4* q = rec(W.acc, s, ACC_N);
    float4 a = q[0], b = q[1];
    P.radiance = xyz(a);
    item = ubits(a.w);
    S.sum = xyz(b);
    S.background = b.w;
}
__device__ void store_acc_head(const WfArgs& W, uint32_t s, const Path& P, uint32_t item, const PixelSums& S) {
    float4* q = rec(W.acc, s, ACC_N);
    q[0] = f4(P.radiance, fbits(item));
    q[1] = f4(S.sum, S.background);
}
// ACC sector 1: the guides' sums (written at the first bounce and the path's end).
__device__ void load_acc_guides(const WfArgs& W, uint32_t s, PixelSums& S) {
    const float4* q = rec(W.acc, s, ACC_N);
    S.albedo = q[2];
    S.normal = q[3];
}
__device__ void store_acc_guides(const WfArgs& W, uint32_t s, const PixelSums& S) {
    float4* q = rec(W.acc, s, ACC_N);
    q[2] = S.albedo;
    q[3] = S.normal;
}
__device__ __forceinline__ uint32_t label_word(const Sample& s, int cap_plane) {
    return (s.label & 0xffffu) | (s.ghost ? 1u << 16 : 0u) | ((uint32_t)(cap_plane + 1) << 17);
}
__device__ void store_vertex(const WfArgs& W, uint32_t s, const Vertex& V, uint32_t rng) {
    float4* q = rec(W.vtx, s, VTX_N);
    q[0] = f4(V.idx, V.cut);
    q[1] = f4(V.s.albedo, V.s.extinction);
    q[2] = make_float4(V.s.roughness, V.s.metalness, V.s.density, V.s.subsurface);
    q[3] = make_float4(V.s.coat, fbits(label_word(V.s, V.cap_plane)), fbits(rng), 0.0f);
}
__device__ void load_vertex(const WfArgs& W, uint32_t s, Vertex& V, uint32_t& rng) {
    const float4* q = rec(W.vtx, s, VTX_N);
    float4 a = q[0], b = q[1], c = q[2], d = q[3];
    V.idx = xyz(a);
    V.cut = a.w;
    V.s.albedo = xyz(b);
    V.s.extinction = b.w;
    V.s.roughness = c.x;
    V.s.metalness = c.y;
    V.s.density = c.z;
    V.s.subsurface = c.w;
    V.s.coat = d.x;
    uint32_t w = ubits(d.y);
    V.s.label = w & 0xffffu;
    V.s.ghost = (w >> 16) & 1u;
    V.cap_plane = (int)(w >> 17) - 1;
    rng = ubits(d.z);
}
// What scatter needs of the vertex after shade, and shadow of it (sector 0).
__device__ void store_shaded(const WfArgs& W, uint32_t s, const Vertex& V, uint32_t rng) {
    float4* q = rec(W.shd, s, SHD_N);
    uint32_t ev = V.surface_event ? ubits(V.s.coat)
                                  : EV_VOLUME | (V.s.label & 0xffffu) | (V.s.ghost ? 1u << 16 : 0u);
    q[0] = f4(V.idx, fbits(rng));
    q[1] = f4(V.light_dir, fbits(ev));
    q[2] = f4(V.s.albedo, V.s.roughness);
    q[3] = f4(V.n, V.s.metalness);
}
__device__ void load_shaded(const WfArgs& W, uint32_t s, Vertex& V) {
    const float4* q = rec(W.shd, s, SHD_N);
    float4 a = q[0], b = q[1], c = q[2], d = q[3];
    V.idx = xyz(a);
    V.light_dir = xyz(b);
    uint32_t ev = ubits(b.w);
    V.surface_event = (ev & EV_VOLUME) != EV_VOLUME;
    V.s.albedo = xyz(c);
    V.s.roughness = c.w;
    V.n = xyz(d);
    V.s.metalness = d.w;
    if (V.surface_event) {
        V.s.coat = b.w;
        V.s.label = 0u;
        V.s.ghost = false;
    } else {
        V.s.coat = 0.0f;
        V.s.label = ev & 0xffffu;
        V.s.ghost = (ev >> 16) & 1u;
    }
    V.s.extinction = 0.0f;  // not read after shade
    V.s.density = 0.0f;
    V.s.subsurface = 0.0f;
    V.cut = 0.0f;
    V.cap_plane = -1;
}

// Appends `slot` to queue `q` where `pred`; called by all 32 lanes together.
__device__ __forceinline__ void push(uint32_t* q, uint32_t* count, uint32_t slot, bool pred) {
    unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return;
    int lane = (int)(threadIdx.x & 31u);
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) q[base + __popc(m & ((1u << lane) - 1u))] = slot;
}

// push, also writing `key` beside the slot in `keys`.
__device__ __forceinline__ void push_key(uint32_t* q, uint32_t* keys, uint32_t* count, uint32_t slot, uint32_t key,
                                         bool pred) {
    unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return;
    int lane = (int)(threadIdx.x & 31u);
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pred) {
        uint32_t at = base + __popc(m & ((1u << lane) - 1u));
        q[at] = slot;
        keys[at] = key;
    }
}

// The bin of a later flight: the coarse cell of its origin (x fastest), then
// the octant of its direction.
__device__ __forceinline__ uint32_t flight_bin(const WfArgs& W, f3 origin, f3 dir) {
    int cx = min(max((int)floorf(origin.x) >> W.cell_shift, 0), W.cells_x - 1);
    int cy = min(max((int)floorf(origin.y) >> W.cell_shift, 0), W.cells_y - 1);
    int cz = min(max((int)floorf(origin.z) >> W.cell_shift, 0), W.cells_z - 1);
    uint32_t oct = (dir.x < 0.0f ? 1u : 0u) | (dir.y < 0.0f ? 2u : 0u) | (dir.z < 0.0f ? 4u : 0u);
    return ((uint32_t)((cz * W.cells_y + cy) * W.cells_x + cx) << 3) | oct;
}

// A pass serves one request (PtArgs) or a batch of requests on one volume
// (PtBatch). The stage kernels are templates over the two: a slot's request
// (request_of), its arguments (args_of) and its constants (consts_of). For a
// single request these fold to the kernel's own parameter and the constants
// it derives once, so that pass compiles to the same code as without batches.
template <class X> struct IsBatch { static constexpr bool value = false; };
template <> struct IsBatch<PtBatch> { static constexpr bool value = true; };

__device__ __forceinline__ uint32_t request_of(const PtArgs&, uint32_t) { return 0u; }
__device__ __forceinline__ uint32_t request_of(const PtBatch& B, uint32_t slot) {
    uint32_t r = 0;
#pragma unroll 1
    while (r + 1u < B.n && slot >= B.slot_end[r]) r++;
    return r;
}
__device__ __forceinline__ const PtArgs& args_of(const PtArgs& A, uint32_t) { return A; }
__device__ __forceinline__ const PtArgs& args_of(const PtBatch& B, uint32_t r) { return B.a[r]; }
__device__ __forceinline__ uint32_t slot_begin(const PtArgs&, uint32_t) { return 0u; }
__device__ __forceinline__ uint32_t slot_begin(const PtBatch& B, uint32_t r) { return r ? B.slot_end[r - 1] : 0u; }
static_assert(sizeof(Consts) <= WF_CONSTS_BYTES, "batched constants record");
__device__ __forceinline__ const Consts& consts_of(const PtArgs&, const WfArgs&, uint32_t, const Consts& C0) {
    return C0;
}
__device__ __forceinline__ const Consts& consts_of(const PtBatch&, const WfArgs& W, uint32_t r, const Consts&) {
    return *reinterpret_cast<const Consts*>(static_cast<const char*>(W.consts) + (size_t)r * WF_CONSTS_BYTES);
}
// The constants a single-request kernel derives once (a batch reads each
// request's from the table its first launch wrote).
__device__ __forceinline__ Consts kernel_consts(const PtArgs& A) { return make_consts(A); }
__device__ __forceinline__ Consts kernel_consts(const PtBatch&) { return Consts(); }

// The end of a sample path: firefly clamp and sums (pt.comp:546-551), then
// the pixel's next sample in the same slot (pt.comp:403). Returns true when
// the slot has a new path; false when the work item (one pixel of one frame)
// is done and its sums are ready to accumulate.
__device__ bool end_sample(const PtArgs& A, const Consts& C, Path& P, PixelSums& S, uint32_t item, uint32_t& sample) {
    finish_path(P, S);
    if (++sample < A.u.path[2]) {
        uint32_t pixel = item / A.frames;
        start_path(A, C, P, pixel % A.width, pixel / A.width);
        return true;
    }
    return false;
}

// Starts work item `item` (frame item % frames, pixel item / frames).
__device__ void start_item(const PtArgs& A, const Consts& C, uint32_t item, Path& P, PixelSums& S) {
    // Frames vary fastest: the frames of one pixel are neighbouring items, so a
    // warp traces two pixels' nearly identical primary rays (measured at 16
    // frames per pass: 239 -> 267 M path samples/s against pixels fastest).
    uint32_t frame = item % A.frames, pixel = item / A.frames;
    uint32_t px = pixel % A.width, py = pixel / A.width;
    P.rng.s = seed_of(px, py, A.u.path[0] + frame * A.u.path[2]);
    P.rng.pcg();
    S = {mk(0.0f), 0.0f, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
    start_path(A, C, P, px, py);
}
__device__ __forceinline__ void store_new_item(const WfArgs& W, uint32_t slot, const Path& P, uint32_t item,
                                               const PixelSums& S) {
    store_path(W, slot, P, 0u);
    store_acc_head(W, slot, P, item, S);
    store_acc_guides(W, slot, S);
}

// Hands the next work items to the lanes with `need` set (all 32 lanes call
// it together; one atomicAdd per warp). Returns the lane's item, or ~0u.
__device__ __forceinline__ uint32_t take_item(uint32_t* counter, uint32_t total, bool need) {
    unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return ~0u;
    int lane = (int)(threadIdx.x & 31u);
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    uint32_t item = base + __popc(m & ((1u << lane) - 1u));
    return (need && item < total) ? item : ~0u;
}
// take_item in a batched pass: each lane draws from its request's counter,
// one atomicAdd per request present among the warp's needing lanes.
__device__ __forceinline__ uint32_t take_item_of(uint32_t* counters, uint32_t r, uint32_t total, bool need) {
    unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) return ~0u;
    int lane = (int)(threadIdx.x & 31u);
    unsigned grp = __match_any_sync(0xffffffffu, need ? r : 0x80000000u | (uint32_t)lane);
    int leader = __ffs(grp) - 1;
    uint32_t base = 0;
    if (need && lane == leader) base = atomicAdd(&counters[r], (uint32_t)__popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    uint32_t item = base + __popc(grp & ((1u << lane) - 1u));
    return (need && item < total) ? item : ~0u;
}

// A lane whose item ended takes its request's next one and starts it in its slot.
template <class X>
__device__ __forceinline__ bool refill(const X& B, const WfArgs& W, uint32_t r, const Consts& C, uint32_t slot,
                                       bool need) {
    const PtArgs& A = args_of(B, r);
    const uint32_t total = A.frames * A.width * A.height;
    uint32_t item;
    if constexpr (IsBatch<X>::value) item = take_item_of(W.items, r, total, need);
    else item = take_item(&W.counts[WF_ITEMS], total, need);
    if (item == ~0u) return false;
    Path P;
    PixelSums S;
    start_item(A, C, item, P, S);
    store_new_item(W, slot, P, item, S);
    return true;
}

// pt.comp:554-560 for the items that ended in this warp (all 32 lanes call
// it). With several frames in flight the adds are atomic, and the lanes that
// finished frames of the same pixel first add their sums together, so each
// pixel takes one set of atomics per warp: the frames of a pixel are
// neighbouring items and tend to end in the same warp (background pixels all
// in the first wave). With one frame per pass each pixel has one slot, which
// adds to the sums directly. In a batched pass (BATCH) the lanes are grouped
// by request and pixel, and every request's pass sums take atomic adds (into
// sums that start at zero, so one add per pixel is the same as a store).
template <bool BATCH>
__device__ void accumulate_items(const PtArgs& A, bool done, uint32_t item, const PixelSums& S, uint32_t r) {
    uint32_t pixel = item / A.frames;
    if (!BATCH && A.frames == 1u) {
        if (done) accumulate(A, pixel % A.width, pixel / A.width, S, false, A.write_hdr != 0, (float)(A.u.path[0] + A.u.path[2]));
        return;
    }
    if (!__any_sync(0xffffffffu, done)) return;
    int lane = (int)(threadIdx.x & 31u);
    // A batched request's pixels are below 2^28 (checked by the host).
    uint32_t key = BATCH ? (r << 28) | pixel : pixel;
    unsigned grp = __match_any_sync(0xffffffffu, done ? key : 0x80000000u | (uint32_t)lane);
    unsigned biggest = __reduce_max_sync(0xffffffffu, (unsigned)__popc(grp));
    float v[12] = {S.sum.x, S.sum.y, S.sum.z, S.background, S.albedo.x, S.albedo.y,
                   S.albedo.z, S.albedo.w, S.normal.x, S.normal.y, S.normal.z, S.normal.w};
    if (biggest > 1u) {
        // Suffix sums along each group's lanes by pointer jumping: after
        // ceil(log2(size)) rounds the group's lowest lane holds its total.
        unsigned higher = grp & ~((2u << lane) - 1u);
        int next = higher ? __ffs(higher) - 1 : -1;
        int rounds = 32 - __clz((int)biggest - 1);
        for (int k2 = 0; k2 < rounds; k2++) {
            int src = next >= 0 ? next : lane;
#pragma unroll
            for (int k = 0; k < 12; k++) {
                float o = __shfl_sync(0xffffffffu, v[k], src);
                if (next >= 0) v[k] += o;
            }
            int nn = __shfl_sync(0xffffffffu, next, src);
            next = next >= 0 ? nn : -1;
        }
    }
    if (!done) return;
    count(A, COUNT_PIXEL);
    if (lane != __ffs(grp) - 1) return;
    long i = (long)pixel;
    atomicAdd(&A.accum[i], make_float4(v[0], v[1], v[2], v[3]));
    atomicAdd(&A.albedo[i], make_float4(v[4], v[5], v[6], v[7]));
    atomicAdd(&A.normal[i], make_float4(v[8], v[9], v[10], v[11]));
}

// Grid-stride loop over a queue with a warp-uniform bound, so that `push` sees
// all 32 lanes.
#define WF_FOR_EACH(n)                                                                          \
    for (uint32_t base_ = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base_ < (n);          \
         base_ += gridDim.x * blockDim.x)

template <class X>
__global__ void __launch_bounds__(256) k_wf_init(const __grid_constant__ X B, const WfArgs W, uint32_t slots) {
    Consts C0 = kernel_consts(B);
    uint32_t last = ~0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
        const uint32_t r = request_of(B, i);
        const PtArgs& A = args_of(B, r);
        if (IsBatch<X>::value && r != last) {
            C0 = make_consts(A);
            last = r;
        }
        const uint32_t item = i - slot_begin(B, r);  // a request's slots start at its item 0
        Path P;
        PixelSums S;
        start_item(A, C0, item, P, S);
        store_new_item(W, i, P, item, S);
        W.first[0][i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k < WF_COUNTERS; k++) W.counts[k] = 0;
        W.counts[WF_FIRST0] = slots;
        W.counts[WF_ITEMS] = slots;
    }
    if constexpr (IsBatch<X>::value) {
        if (blockIdx.x == 0 && threadIdx.x < B.n) {
            const uint32_t r = threadIdx.x;
            W.items[r] = B.slot_end[r] - slot_begin(B, r);
            *reinterpret_cast<Consts*>(static_cast<char*>(W.consts) + (size_t)r * WF_CONSTS_BYTES) =
                make_consts(B.a[r]);
        }
    }
}

// Extend, persistent over its queue: every lane advances its path by one
// free-flight step per iteration; a lane whose flight ended (a vertex, an
// escape, or the bounce limits) hands the path on and takes the next queued
// path, so lanes with long empty-space flights do not hold up the others.
// ff_step is the loop body of free_flight (pt.comp:307-332). Only what the
// flight needs stays in registers. Vertices go to shade; escapes and paths at
// the bounce limits go to this wave's scatter kernel, which finishes them, so
// this kernel carries none of the escape, accumulation or path-start code.
#ifndef VV_EXTEND_MIN_BLOCKS
#define VV_EXTEND_MIN_BLOCKS 8
#endif
enum { EXT_END = 3 };
// FIRST: the first-flight queue (bounce 0: cubic B-spline density along the
// flight), otherwise later flights (trilinear); each kernel carries only its
// sampler. Every wave launches both; with all of a pass's frames in flight
// first flights occur in the first wave only (and with several samples per
// pixel), so the other launch finds its queue empty.
template <bool FIRST, class X>
__global__ void __launch_bounds__(128, VV_EXTEND_MIN_BLOCKS)
    k_wf_extend(const __grid_constant__ X B, const WfArgs W, int cur, uint32_t tail) {
    if (W.counts[WF_STOP] != 0u) return;
    if (FIRST) {
        // The wave's first launch decides whether the waves go on: with at most
        // `tail` live paths left, the finishing launch takes queue `cur` over.
        // Every block reads the same counts (nothing changes them before this
        // launch ends), so all blocks decide alike.
        uint32_t live = W.counts[WF_FIRST0 + cur] + W.counts[cur];
        if (live <= tail) {
            if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[WF_STOP] = (uint32_t)cur + 1u;
            return;
        }
    }
    const uint32_t n = W.counts[FIRST ? WF_FIRST0 + cur : cur];
    const uint32_t* queue = FIRST ? W.first[cur] : n < W.bin_min ? W.ext[cur] : W.sorted;
    uint32_t* taken = &W.counts[FIRST ? WF_TAKE_FIRST : WF_TAKE_EXT];
    const Consts C0 = kernel_consts(B);
    uint32_t slot = 0, r = 0;
    f3 origin, dir, spectral;
    Rng rng;
    uint32_t word = 0;  // P2.w: volumes, sample, hero
    Flight F;
    Vertex V;
    bool active = false, drained = false;
    for (;;) {
        int done = 0;
        bool need = !active && !drained;
        if (__any_sync(0xffffffffu, need)) {
            uint32_t k = take_item(taken, n, need);
            if (need && k != ~0u) {
                slot = queue[k];
                r = request_of(B, slot);
                const PtArgs& A = args_of(B, r);
                const Consts& C = consts_of(B, W, r, C0);
                const float4* q = rec(W.path, slot, PATH_N);
                float4 a = q[0], b = q[1], c = q[2];
                origin = xyz(a);
                rng.s = ubits(a.w);
                dir = xyz(b);
                spectral = xyz(c);
                word = ubits(c.w);
                uint32_t surfaces = ubits(b.w) >> 16, volumes = word & 1023u;
                if (!(surfaces <= C.max_bounces && volumes <= C.volume_limit)) {
                    done = EXT_END;
                } else {
                    count(A, COUNT_VERTEX);
                    ff_begin(A, origin, dir, F);
                    active = true;
                }
            }
            drained = __any_sync(0xffffffffu, need && k == ~0u);
        }
        if (active) {
            int res = ff_step(args_of(B, r), origin, dir, FIRST, (int)(word >> 30), spectral, F, V.idx, V.s,
                              V.cap_plane, V.cut, rng);
            if (res != FF_CONTINUE) {
                active = false;
                done = res;
            }
        }
        if (__any_sync(0xffffffffu, done != 0)) {
            if (done != 0) {
                if (done != EXT_END) {  // free flight changed the spectral ratios
                    float4* q = rec(W.path, slot, PATH_N);
                    float4 d = q[3];
                    q[2] = f4(spectral, fbits(word));
                    q[3] = d;
                }
                float4* v = rec(W.vtx, slot, VTX_N);
                if (done == FF_HIT) {
                    store_vertex(W, slot, V, rng.s);
                } else {
                    // Escapes and paths at the bounce limits: the random state
                    // and whether the scatter kernel runs the escape (pt.comp:431-447).
                    v[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    v[3] = make_float4(0.0f, 0.0f, fbits(rng.s), fbits(done == FF_ESCAPE ? 1u : 0u));
                }
            }
            push(W.shade, &W.counts[WF_SHADE], slot, done == FF_HIT);
            push(W.esc[cur], &W.counts[WF_ESC0 + cur], slot, done != 0 && done != FF_HIT);
        }
        if (drained && !__any_sync(0xffffffffu, active)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[WF_SCATTER] = 0;
}

#ifndef VV_SHADE_MIN_BLOCKS
#define VV_SHADE_MIN_BLOCKS 4
#endif
template <class X>
__global__ void __launch_bounds__(128, VV_SHADE_MIN_BLOCKS) k_wf_shade(const __grid_constant__ X B, const WfArgs W,
                                                                      int cur) {
    if (W.counts[WF_STOP] != 0u) return;
    uint32_t n = W.counts[WF_SHADE];
    const Consts C0 = kernel_consts(B);
    WF_FOR_EACH(n) {
        uint32_t i = base_ + (threadIdx.x & 31u);
        bool valid = i < n;
        uint32_t slot = valid ? W.shade[i] : 0u;
        if (valid) {
            const uint32_t r = request_of(B, slot);
            Path P;
            float4 b = rec(W.path, slot, PATH_N)[1];
            P.dir = xyz(b);
            P.bounce = ubits(b.w) & 0xffffu;
            Vertex V;
            load_vertex(W, slot, V, P.rng.s);
            PixelSums S;
            if (P.bounce == 0u) load_acc_guides(W, slot, S);
            stage_shade(args_of(B, r), consts_of(B, W, r, C0), P, S, V);
            store_shaded(W, slot, V, P.rng.s);
            if (P.bounce == 0u) store_acc_guides(W, slot, S);
        }
        push(W.shadow, &W.counts[WF_SHADOW], slot, valid);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counts[cur] = 0;
        W.counts[WF_FIRST0 + cur] = 0;
        W.counts[WF_TAKE_EXT] = 0;
        W.counts[WF_TAKE_FIRST] = 0;
        W.counts[WF_ESC0 + (cur ^ 1)] = 0;  // finished by the previous wave's scatter
    }
}

// Shadow rays, persistent over their queue like extend: one ratio-tracking
// step (tr_step, the loop body of transmittance, pt.comp:344-369) per
// iteration, lanes refilled as their rays finish. With a light map, a lane
// whose key-light ray finished draws the light map's sample (pt.comp:466-476,
// in the reference's order of random numbers) and queues the slot for
// k_wf_shadow_map, which traces the sample's ray: a lane here traces one kind
// of ray, and the random state travels in the shadow record between them.
#ifndef VV_SHADOW_MIN_BLOCKS
#define VV_SHADOW_MIN_BLOCKS 8
#endif
// MAP: the frame has a light map (lighting.w == 2); the kernel without it is
// the key light's shadow rays alone. In a batched pass MAP is set when any
// request has a light map, and each lane follows its own request's lighting.
template <bool MAP, class X>
__global__ void __launch_bounds__(128, VV_SHADOW_MIN_BLOCKS) k_wf_shadow(const __grid_constant__ X B, const WfArgs W) {
    if (W.counts[WF_STOP] != 0u) return;
    const uint32_t n = W.counts[WF_SHADOW];
    uint32_t slot = 0, r = 0;
    f3 origin;
    Rng rng;
    Shadow T;
    bool active = false, drained = false;
    for (;;) {
        bool need = !active && !drained;
        if (__any_sync(0xffffffffu, need)) {
            uint32_t k = take_item(&W.counts[WF_TAKE_SHADOW], n, need);
            if (need && k != ~0u) {
                slot = W.shadow[k];
                r = request_of(B, slot);
                const float4* q = rec(W.shd, slot, SHD_N);
                float4 a = q[0], b = q[1];
                origin = xyz(a);
                rng.s = ubits(a.w);
                tr_begin(args_of(B, r), origin, xyz(b), T);
                active = true;
            }
            drained = __any_sync(0xffffffffu, need && k == ~0u);
        }
        bool done = false, to_map = false;
        if (active && !tr_step(args_of(B, r), origin, T, rng)) {
            const PtArgs& A = args_of(B, r);
            const bool map = MAP && (!IsBatch<X>::value || A.u.lighting[3] == 2u);
            float4* h = rec(W.sh, slot, SH_N);
            if (!map) {
                h[0] = f4(T.result, fbits(rng.s));
                h[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                done = true;
            } else {
                Vertex V;
                sample_map_light(A, rng, V);
                h[0] = f4(T.result, fbits(rng.s));
                h[1] = f4(V.map_light, V.map_pdf);
                W.mapdir[slot] = f4(V.map_dir, 0.0f);
                to_map = V.map_pdf > 0.0f;
                done = !to_map;
            }
            active = false;
        }
        if (MAP) push(W.map, &W.counts[WF_MAP], slot, to_map);
        if (__any_sync(0xffffffffu, done)) push(W.scatter, &W.counts[WF_SCATTER], slot, done);
        if (drained && !__any_sync(0xffffffffu, active)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[WF_SHADE] = 0;
}

// The light map sample's shadow rays (after k_wf_shadow<true>): the ray from
// the vertex along the sample's direction, continuing the slot's random
// stream from the key light's ray and the sample; its transmittance scales
// the sample's radiance for scatter.
template <class X>
__global__ void __launch_bounds__(128, VV_SHADOW_MIN_BLOCKS) k_wf_shadow_map(const __grid_constant__ X B,
                                                                            const WfArgs W) {
    if (W.counts[WF_STOP] != 0u) return;
    const uint32_t n = W.counts[WF_MAP];
    uint32_t slot = 0, r = 0;
    f3 origin;
    Rng rng;
    Shadow T;
    bool active = false, drained = false;
    for (;;) {
        bool need = !active && !drained;
        if (__any_sync(0xffffffffu, need)) {
            uint32_t k = take_item(&W.counts[WF_TAKE_MAP], n, need);
            if (need && k != ~0u) {
                slot = W.map[k];
                r = request_of(B, slot);
                origin = xyz(rec(W.shd, slot, SHD_N)[0]);
                rng.s = ubits(rec(W.sh, slot, SH_N)[0].w);
                tr_begin(args_of(B, r), origin, xyz(W.mapdir[slot]), T);
                active = true;
            }
            drained = __any_sync(0xffffffffu, need && k == ~0u);
        }
        bool done = false;
        if (active && !tr_step(args_of(B, r), origin, T, rng)) {
            float4* h = rec(W.sh, slot, SH_N);
            float4 h0 = h[0], h1 = h[1];
            h[0] = make_float4(h0.x, h0.y, h0.z, fbits(rng.s));
            h[1] = f4(xyz(h1) * T.result, h1.w);
            done = true;
            active = false;
        }
        if (__any_sync(0xffffffffu, done)) push(W.scatter, &W.counts[WF_SCATTER], slot, done);
        if (drained && !__any_sync(0xffffffffu, active)) break;
    }
}

// Scatter, and the end of the flights that left the volume or hit the bounce
// limits in this wave's extend (queued after the scatter entries).
#ifndef VV_SCATTER_MIN_BLOCKS
#define VV_SCATTER_MIN_BLOCKS 6
#endif
template <class X>
__global__ void __launch_bounds__(128, VV_SCATTER_MIN_BLOCKS) k_wf_scatter(const __grid_constant__ X B,
                                                                          const WfArgs W, int cur) {
    if (W.counts[WF_STOP] != 0u) return;
    uint32_t n_scatter = W.counts[WF_SCATTER], n = n_scatter + W.counts[WF_ESC0 + cur];
    int nxt = cur ^ 1;
    const Consts C0 = kernel_consts(B);
    WF_FOR_EACH(n) {
        uint32_t i = base_ + (threadIdx.x & 31u);
        bool valid = i < n;
        bool ended = i >= n_scatter;
        uint32_t slot = valid ? (ended ? W.esc[cur][i - n_scatter] : W.scatter[i]) : 0u;
        const uint32_t r = request_of(B, slot);
        const PtArgs& A = args_of(B, r);
        const Consts& C = consts_of(B, W, r, C0);
        bool to_ext = false, to_first = false, done = false;
        uint32_t item = 0, key = 0;
        PixelSums S;
        if (valid) {
            Path P;
            uint32_t sample;
            load_path(W, slot, P, sample);
            load_acc_head(W, slot, P, item, S);
            bool escaped = false;
            if (!ended) {
                Vertex V;
                load_shaded(W, slot, V);
                const float4* h = rec(W.sh, slot, SH_N);
                float4 h0 = h[0], h1 = h[1];
                V.light_t = xyz(h0);
                P.rng.s = ubits(h0.w);
                V.map_light = xyz(h1);
                V.map_pdf = h1.w;
                V.map_dir = A.u.lighting[3] == 2u ? xyz(W.mapdir[slot]) : mk(0.0f);
                to_ext = stage_scatter(A, C, P, V);
                if (to_ext) key = flight_bin(W, P.origin, P.dir);
            } else {
                float4 v3 = rec(W.vtx, slot, VTX_N)[3];
                P.rng.s = ubits(v3.z);
                escaped = ubits(v3.w) != 0u;
            }
            if (!to_ext) {
                load_acc_guides(W, slot, S);
                if (escaped) stage_escape(A, C, P, S);
                to_first = end_sample(A, C, P, S, item, sample);
                done = !to_first;
                if (to_first) store_acc_guides(W, slot, S);
            }
            if (!done) {
                store_path(W, slot, P, sample);
                store_acc_head(W, slot, P, item, S);
            }
        }
        accumulate_items<IsBatch<X>::value>(A, done, item, S, r);
        if (refill(B, W, r, C, slot, done)) to_first = true;
        push_key(W.ext[nxt], W.ext_key[nxt], &W.counts[nxt], slot, key, to_ext);
        push(W.first[nxt], &W.counts[WF_FIRST0 + nxt], slot, to_first);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counts[WF_SHADOW] = 0;
        W.counts[WF_TAKE_SHADOW] = 0;
        W.counts[WF_MAP] = 0;
        W.counts[WF_TAKE_MAP] = 0;
    }
}

// Counting sort of the next wave's later-flight queue by bin: counts, an
// exclusive scan (one block), then placement. Order within a bin is free.
// Queues shorter than W.bin_min (the late waves' few long walks, where a
// warp's lanes rarely share a region anyway) skip the three launches' work,
// which would otherwise add to every wave's chain of dependent launches.
__global__ void __launch_bounds__(256) k_wf_bin_count(const WfArgs W, const uint32_t* keys, int count) {
    if (W.counts[WF_STOP] != 0u) return;
    const uint32_t n = W.counts[count];
    if (n < W.bin_min) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&W.bin_count[keys[i]], 1u);
}
__global__ void __launch_bounds__(1024) k_wf_bin_scan(const WfArgs W, int count) {
    if (W.counts[WF_STOP] != 0u || W.counts[count] < W.bin_min) return;
    __shared__ uint32_t part[1024];
    const uint32_t per = (W.nbins + 1023u) / 1024u, lo = threadIdx.x * per;
    const uint32_t hi = min(lo + per, W.nbins);
    uint32_t sum = 0;
    for (uint32_t b = lo; b < hi; b++) sum += W.bin_count[b];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive scan of the 1024 partial sums
        uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t b = lo; b < hi; b++) {
        uint32_t c = W.bin_count[b];
        W.bin_next[b] = run;
        run += c;
        W.bin_count[b] = 0u;
    }
}
__global__ void __launch_bounds__(256) k_wf_bin_place(const WfArgs W, const uint32_t* queue, const uint32_t* keys,
                                                      int count) {
    if (W.counts[WF_STOP] != 0u) return;
    const uint32_t n = W.counts[count];
    if (n < W.bin_min) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t at = atomicAdd(&W.bin_next[keys[i]], 1u);
        if (at < W.capacity) W.sorted[at] = queue[i];  // always below n when the counts started at zero
    }
}

// The paths still alive, run to completion one thread each (the reference's
// loop), including their pixels' remaining samples and frames (a batched
// pass's from each path's own request).
template <class X>
__global__ void __launch_bounds__(128, 4) k_wf_finish(const __grid_constant__ X B, const WfArgs W, int cur) {
    uint32_t stop = W.counts[WF_STOP];
    if (stop != 0u) cur = (int)stop - 1;  // else the waves ran out first: `cur` is the next wave's queue
    uint32_t n_first = W.counts[WF_FIRST0 + cur], n = n_first + W.counts[cur];
    const Consts C0 = kernel_consts(B);
    // With no more paths than warps (the usual tail: at most 1024 paths), each
    // path runs alone in its warp, on every SM, instead of 32 to a warp on a
    // few SMs, where the lanes would take turns through each other's divergent
    // random walks. More paths (the waves ran out first) take a lane each.
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, threads = gridDim.x * blockDim.x;
    const bool alone = n <= (threads >> 5);
    if (alone && (threadIdx.x & 31u) != 0u) return;
    const uint32_t first = alone ? tid >> 5 : tid, stride = alone ? threads >> 5 : threads;
    for (uint32_t i = first; i < n; i += stride) {
        uint32_t slot = i < n_first ? W.first[cur][i] : W.ext[cur][i - n_first];
        const uint32_t r = request_of(B, slot);
        const PtArgs& A = args_of(B, r);
        const Consts& C = consts_of(B, W, r, C0);
        const bool multi = IsBatch<X>::value || A.frames > 1u;
        const float n_total = (float)(A.u.path[0] + A.u.path[2]);
        uint32_t* counter = IsBatch<X>::value ? &W.items[r] : &W.counts[WF_ITEMS];
        Path P;
        PixelSums S;
        uint32_t sample, item;
        load_path(W, slot, P, sample);
        load_acc_head(W, slot, P, item, S);
        load_acc_guides(W, slot, S);
        uint32_t total = A.frames * A.width * A.height;
        for (;;) {
            do {
                while (bounce_step(A, C, P, S)) {
                }
            } while (end_sample(A, C, P, S, item, sample));
            uint32_t pixel = item / A.frames;
            accumulate(A, pixel % A.width, pixel / A.width, S, multi, !multi && A.write_hdr != 0, n_total);
            item = atomicAdd(counter, 1u);
            if (item >= total) break;
            sample = 0u;
            start_item(A, C, item, P, S);
        }
    }
}

template <class K> static int blocks_per_sm(K kernel, int threads) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess || n < 1) n = 1;
    return n;
}

// The waves of a pass over `slots` paths in flight and `items` work items
// (the largest count of one request's items per slot sets the rounds): waves
// of the four stages until few paths are left, then one finishing launch.
template <class X>
static cudaError_t run_waves(const X& a, const WfArgs& w, int sms, cudaStream_t s, int* launches, uint32_t slots,
                             uint32_t rounds, bool map) {
    static int g_ext = 0, g_shade = 0, g_shadow = 0, g_scatter = 0, g_finish = 0;
    if (!g_ext) {
        g_ext = sms * blocks_per_sm(k_wf_extend<false, X>, 128);
        g_shade = sms * blocks_per_sm(k_wf_shade<X>, 128);
        g_shadow = sms * blocks_per_sm(k_wf_shadow<false, X>, 128);
        g_scatter = sms * blocks_per_sm(k_wf_scatter<X>, 128);
        g_finish = sms * blocks_per_sm(k_wf_finish<X>, 128);
    }
    const char* env = std::getenv("VV_WF_TAIL");
    uint32_t tail = env ? (uint32_t)std::atoi(env) : 1024u;
    k_wf_init<X><<<(slots + 255) / 256 < (uint32_t)(sms * 8) ? (slots + 255) / 256 : sms * 8, 256, 0, s>>>(a, w, slots);
    *launches += 1;
    // All waves are queued at once, with no host round trip: the first launch
    // of each wave stops the waves on the device once at most `tail` paths
    // are left, the rest of the queued waves then return at once, and the
    // finishing launch runs the remaining paths to completion. Enough waves
    // for the pass: about 10 per round of slots plus 16 for the tail of long
    // random walks (a path has at most 4 surface and 80 volume events at
    // g = 0.6); if they still run out, the finishing launch takes what is
    // left. The head/neck workload's 16-frame passes stop after about 21
    // waves; every wave queued beyond that returns at once but still costs a
    // launch (16 instead of 24 queued: 389.7 -> 391.9 M path samples/s, a
    // third fewer launches).
    const char* base = std::getenv("VV_WF_WAVES");  // the waves beside the rounds' share (16 by default)
    const uint32_t first = base ? (uint32_t)std::max(1, std::atoi(base)) : 16u;
    int waves = (int)std::min<uint32_t>(first + 10u * rounds, 4096u);
    int cur = 0;
    for (int wave = 0; wave < waves; wave++) {
        k_wf_extend<true, X><<<g_ext, 128, 0, s>>>(a, w, cur, tail);
        k_wf_extend<false, X><<<g_ext, 128, 0, s>>>(a, w, cur, tail);
        k_wf_shade<X><<<g_shade, 128, 0, s>>>(a, w, cur);
        if (map) {
            k_wf_shadow<true, X><<<g_shadow, 128, 0, s>>>(a, w);
            k_wf_shadow_map<X><<<g_shadow, 128, 0, s>>>(a, w);
            *launches += 1;
        } else {
            k_wf_shadow<false, X><<<g_shadow, 128, 0, s>>>(a, w);
        }
        k_wf_scatter<X><<<g_scatter, 128, 0, s>>>(a, w, cur);
        *launches += 5;
        // The next wave's later flights, ordered by bin.
        k_wf_bin_count<<<sms * 4, 256, 0, s>>>(w, w.ext_key[cur ^ 1], cur ^ 1);
        k_wf_bin_scan<<<1, 1024, 0, s>>>(w, cur ^ 1);
        k_wf_bin_place<<<sms * 4, 256, 0, s>>>(w, w.ext[cur ^ 1], w.ext_key[cur ^ 1], cur ^ 1);
        *launches += 3;
        cur ^= 1;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_wf_finish<X><<<g_finish, 128, 0, s>>>(a, w, cur);
    *launches += 1;
    return cudaGetLastError();
}

// Host side: one request's pass.
cudaError_t launch_pt_wavefront(const PtArgs& a, const WfArgs& w, int sms, cudaStream_t s, int* launches) {
    if (a.u.path[2] >= (uint32_t)WF_MAX_SAMPLES) return cudaErrorInvalidValue;  // the host routes these elsewhere
    uint32_t pixels = a.width * a.height;
    uint32_t items = a.frames * pixels;
    uint32_t slots = items < w.capacity ? items : w.capacity;  // paths in flight
    uint32_t rounds = (items + slots - 1) / slots;
    return run_waves(a, w, sms, s, launches, slots, rounds, a.u.lighting[3] == 2u);
}

#if VV_DFMT == 0
// A batched pass: request r's items start in its own slots and refill them
// from its own counter. The host has checked the batch (at most VV_BATCH_MAX
// requests, each with at least one slot and fewer than 2^28 pixels).
cudaError_t launch_pt_wavefront_batch(const PtBatch& b, const WfArgs& w, int sms, cudaStream_t s, int* launches) {
    if (b.n == 0 || b.n > (uint32_t)VV_BATCH_MAX || !w.items || !w.consts) return cudaErrorInvalidValue;
    uint32_t rounds = 1, begin = 0;
    bool map = false;
    for (uint32_t r = 0; r < b.n; r++) {
        const PtArgs& a = b.a[r];
        if (a.u.path[2] >= (uint32_t)WF_MAX_SAMPLES) return cudaErrorInvalidValue;
        uint32_t slots = b.slot_end[r] - begin, items = a.frames * a.width * a.height;
        if (b.slot_end[r] <= begin || slots > items) return cudaErrorInvalidValue;
        rounds = std::max(rounds, (items + slots - 1) / slots);
        map = map || a.u.lighting[3] == 2u;
        begin = b.slot_end[r];
    }
    if (begin > w.capacity) return cudaErrorInvalidValue;
    return run_waves(b, w, sms, s, launches, begin, rounds, map);
}
#endif

}  // namespace VV_FMT_NS
}  // namespace vv
