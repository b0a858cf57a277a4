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

// Slot layout: 16 x float4 = 256 bytes per pixel (WF_SLOT_BYTES); the light
// map's sample, when there is a light map, in a parallel array of 2 x float4.
enum {
    Q_ORIGIN = 0,   // origin.xyz, last_pdf
    Q_DIR = 1,      // dir.xyz, rng
    Q_THRU = 2,     // throughput.xyz, pixel
    Q_SPEC = 3,     // spectral.xyz, bounce | surfaces << 16
    Q_RAD = 4,      // radiance.xyz, volumes
    Q_SUM = 5,      // sum.xyz, background
    Q_ALB = 6,      // albedo sum
    Q_NOR = 7,      // normal sum
    Q_IDX = 8,      // vertex idx.xyz, cut
    Q_SA = 9,       // sample albedo.xyz, extinction
    Q_SB = 10,      // roughness, metalness, density, subsurface
    Q_SC = 11,      // coat, label, ghost | surface_event << 1, cap_plane
    Q_N = 12,       // shading normal
    Q_LD = 13,      // light direction
    Q_LT = 14,      // light transmittance
    Q_CTL = 15,     // frame, sample, hero, escape flag (extend -> scatter)
    Q_COUNT = 16
};
// W.map entries per slot: light map sample direction.xyz and pdf (0: none);
// its radiance / pdf x transmittance.
enum { M_DIR = 0, M_LIGHT = 1, M_COUNT = 2 };
static_assert(Q_COUNT * 16 == WF_SLOT_BYTES, "slot layout");

__device__ __forceinline__ float4* slot_of(const WfArgs& W, uint32_t s) { return W.slots + (size_t)s * Q_COUNT; }
__device__ __forceinline__ float4* map_of(const WfArgs& W, uint32_t s) { return W.map + (size_t)s * M_COUNT; }
__device__ __forceinline__ float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ f3 xyz(float4 q) { return mk(q.x, q.y, q.z); }
__device__ __forceinline__ uint32_t ubits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float fbits(uint32_t u) { return __uint_as_float(u); }

struct Ctl {
    uint32_t pixel, frame, sample;
};

__device__ void load_path(const float4* q, Path& P, Ctl& c) {
    float4 a = q[Q_ORIGIN], b = q[Q_DIR], t = q[Q_THRU], s = q[Q_SPEC], r = q[Q_RAD], k = q[Q_CTL];
    P.origin = xyz(a);
    P.last_pdf = a.w;
    P.dir = xyz(b);
    P.rng.s = ubits(b.w);
    P.throughput = xyz(t);
    c.pixel = ubits(t.w);
    P.spectral = xyz(s);
    P.bounce = ubits(s.w) & 0xffffu;
    P.surfaces = ubits(s.w) >> 16;
    P.radiance = xyz(r);
    P.volumes = ubits(r.w);
    c.frame = ubits(k.x);
    c.sample = ubits(k.y);
    P.hero = (int)ubits(k.z);
}
__device__ void store_path(float4* q, const Path& P, const Ctl& c) {
    q[Q_ORIGIN] = f4(P.origin, P.last_pdf);
    q[Q_DIR] = f4(P.dir, fbits(P.rng.s));
    q[Q_THRU] = f4(P.throughput, fbits(c.pixel));
    q[Q_SPEC] = f4(P.spectral, fbits(P.bounce | (P.surfaces << 16)));
    q[Q_RAD] = f4(P.radiance, fbits(P.volumes));
    q[Q_CTL] = make_float4(fbits(c.frame), fbits(c.sample), fbits((uint32_t)P.hero), 0.0f);
}
__device__ void load_sums(const float4* q, PixelSums& S) {
    float4 a = q[Q_SUM];
    S.sum = xyz(a);
    S.background = a.w;
    S.albedo = q[Q_ALB];
    S.normal = q[Q_NOR];
}
__device__ void store_sums(float4* q, const PixelSums& S) {
    q[Q_SUM] = f4(S.sum, S.background);
    q[Q_ALB] = S.albedo;
    q[Q_NOR] = S.normal;
}
__device__ void load_vertex(const float4* q, Vertex& V) {
    float4 a = q[Q_IDX], b = q[Q_SA], c = q[Q_SB], d = q[Q_SC];
    V.idx = xyz(a);
    V.cut = a.w;
    V.s.albedo = xyz(b);
    V.s.extinction = b.w;
    V.s.roughness = c.x;
    V.s.metalness = c.y;
    V.s.density = c.z;
    V.s.subsurface = c.w;
    V.s.coat = d.x;
    V.s.label = ubits(d.y);
    uint32_t fl = ubits(d.z);
    V.s.ghost = (fl & 1u) != 0u;
    V.surface_event = (fl & 2u) != 0u;
    V.cap_plane = (int)ubits(d.w);
}
__device__ void store_vertex(float4* q, const Vertex& V) {
    q[Q_IDX] = f4(V.idx, V.cut);
    q[Q_SA] = f4(V.s.albedo, V.s.extinction);
    q[Q_SB] = make_float4(V.s.roughness, V.s.metalness, V.s.density, V.s.subsurface);
    q[Q_SC] = make_float4(V.s.coat, fbits(V.s.label), fbits((V.s.ghost ? 1u : 0u) | (V.surface_event ? 2u : 0u)),
                          fbits((uint32_t)V.cap_plane));
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

// Ends a sample path: firefly clamp and sums, then the pixel's next sample
// (pt.comp:403, 546-560). Returns true when the slot has a new path; false when
// the work item (one pixel of one frame) is done and accumulated.
__device__ bool end_path(const PtArgs& A, const Consts& C, Path& P, PixelSums& S, Ctl& c) {
    finish_path(P, S);
    uint32_t spf = A.u.path[2];
    uint32_t px = c.pixel % A.width, py = c.pixel / A.width;
    if (++c.sample < spf) {
        start_path(A, C, P, px, py);
        return true;
    }
    // One frame per launch: this slot owns the pixel; several: frames of one
    // pixel may finish concurrently in different slots.
    bool multi = A.frames > 1;
    accumulate(A, px, py, S, multi, !multi && A.write_hdr != 0, (float)(A.u.path[0] + spf));
    return false;
}

// Starts work item `item` (frame item % frames, pixel item / frames) in a slot.
__device__ void start_item(const PtArgs& A, const Consts& C, uint32_t item, Path& P, PixelSums& S, Ctl& c) {
    // Frames vary fastest: the frames of one pixel are neighbouring items, so a
    // warp traces two pixels' nearly identical primary rays (measured at 16
    // frames per pass: 239 -> 267 M path samples/s against pixels fastest).
    c.frame = item % A.frames;
    c.pixel = item / A.frames;
    c.sample = 0u;
    uint32_t px = c.pixel % A.width, py = c.pixel / A.width;
    P.rng.s = seed_of(px, py, A.u.path[0] + c.frame * A.u.path[2]);
    P.rng.pcg();
    S = {mk(0.0f), 0.0f, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
    start_path(A, C, P, px, py);
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

// A lane whose item ended takes the next one and starts it in its slot.
__device__ __forceinline__ bool refill(const PtArgs& A, const WfArgs& W, const Consts& C, uint32_t slot, bool need) {
    uint32_t item = take_item(&W.counts[WF_ITEMS], A.frames * A.width * A.height, need);
    if (item == ~0u) return false;
    Path P;
    PixelSums S;
    Ctl c;
    start_item(A, C, item, P, S, c);
    float4* q = slot_of(W, slot);
    store_path(q, P, c);
    store_sums(q, S);
    return true;
}

// Grid-stride loop over a queue with a warp-uniform bound, so that `push` sees
// all 32 lanes.
#define WF_FOR_EACH(n)                                                                          \
    for (uint32_t base_ = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base_ < (n);          \
         base_ += gridDim.x * blockDim.x)

__global__ void __launch_bounds__(256) k_wf_init(const __grid_constant__ PtArgs A, const WfArgs W, uint32_t slots) {
    Consts C = make_consts(A);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
        Path P;
        PixelSums S;
        Ctl c;
        start_item(A, C, i, P, S, c);
        float4* q = slot_of(W, i);
        store_path(q, P, c);
        store_sums(q, S);
        W.first[0][i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k < WF_COUNTERS; k++) W.counts[k] = 0;
        W.counts[WF_FIRST0] = slots;
        W.counts[WF_ITEMS] = slots;
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
template <bool FIRST>
__global__ void __launch_bounds__(128, VV_EXTEND_MIN_BLOCKS)
    k_wf_extend(const __grid_constant__ PtArgs A, const WfArgs W, int cur, uint32_t tail) {
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
    const uint32_t* queue = FIRST ? W.first[cur] : W.ext[cur];
    uint32_t* taken = &W.counts[FIRST ? WF_TAKE_FIRST : WF_TAKE_EXT];
    const Consts C = make_consts(A);
    uint32_t slot = 0;
    f3 origin, dir, spectral;
    Rng rng;
    uint32_t hero = 0, bounce = 0;
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
                const float4* q = slot_of(W, slot);
                float4 a = q[Q_ORIGIN], b = q[Q_DIR], s = q[Q_SPEC];
                origin = xyz(a);
                dir = xyz(b);
                rng.s = ubits(b.w);
                spectral = xyz(s);
                bounce = ubits(s.w) & 0xffffu;
                uint32_t surfaces = ubits(s.w) >> 16, volumes = ubits(q[Q_RAD].w);
                hero = ubits(q[Q_CTL].z);
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
            int r = ff_step(A, origin, dir, FIRST, (int)hero, spectral, F, V.idx, V.s, V.cap_plane, V.cut, rng);
            if (r != FF_CONTINUE) {
                active = false;
                done = r;
            }
        }
        if (__any_sync(0xffffffffu, done != 0)) {
            if (done != 0) {
                float4* q = slot_of(W, slot);
                if (done == FF_HIT) store_vertex(q, V);
                q[Q_DIR] = f4(dir, fbits(rng.s));
                float4 s = q[Q_SPEC];
                q[Q_SPEC] = f4(spectral, s.w);
                // Q_CTL.w: whether the scatter kernel runs the escape (pt.comp:431-447).
                if (done != FF_HIT) ((float*)(q + Q_CTL))[3] = fbits(done == FF_ESCAPE ? 1u : 0u);
            }
            push(W.shade, &W.counts[WF_SHADE], slot, done == FF_HIT);
            push(W.esc[cur], &W.counts[WF_ESC0 + cur], slot, done != 0 && done != FF_HIT);
        }
        if (drained && !__any_sync(0xffffffffu, active)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[WF_SCATTER] = 0;
}

__global__ void __launch_bounds__(128, 4) k_wf_shade(const __grid_constant__ PtArgs A, const WfArgs W, int cur) {
    if (W.counts[WF_STOP] != 0u) return;
    uint32_t n = W.counts[WF_SHADE];
    Consts C = make_consts(A);
    WF_FOR_EACH(n) {
        uint32_t i = base_ + (threadIdx.x & 31u);
        bool valid = i < n;
        uint32_t slot = valid ? W.shade[i] : 0u;
        if (valid) {
            float4* q = slot_of(W, slot);
            Path P;
            float4 d = q[Q_DIR];
            P.dir = xyz(d);
            P.rng.s = ubits(d.w);
            P.bounce = ubits(q[Q_SPEC].w) & 0xffffu;
            PixelSums S;
            if (P.bounce == 0u) load_sums(q, S);
            Vertex V;
            load_vertex(q, V);
            stage_shade(A, C, P, S, V);
            q[Q_DIR] = f4(P.dir, fbits(P.rng.s));
            store_vertex(q, V);
            q[Q_N] = f4(V.n, 0.0f);
            q[Q_LD] = f4(V.light_dir, 0.0f);
            if (P.bounce == 0u) store_sums(q, S);
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
// whose key-light ray finished draws the light map's sample and traces its
// ray next (pt.comp:466-476, in the reference's order of random numbers).
#ifndef VV_SHADOW_MIN_BLOCKS
#define VV_SHADOW_MIN_BLOCKS 8
#endif
// MAP: the frame has a light map (lighting.w == 2); the kernel without it is
// the key light's shadow rays alone.
template <bool MAP>
__global__ void __launch_bounds__(128, VV_SHADOW_MIN_BLOCKS) k_wf_shadow(const __grid_constant__ PtArgs A, const WfArgs W) {
    if (W.counts[WF_STOP] != 0u) return;
    const uint32_t n = W.counts[WF_SHADOW];
    uint32_t slot = 0;
    f3 origin;
    Rng rng;
    Shadow T;
    bool active = false, drained = false, map_ray = false;
    for (;;) {
        bool need = !active && !drained;
        if (__any_sync(0xffffffffu, need)) {
            uint32_t k = take_item(&W.counts[WF_TAKE_SHADOW], n, need);
            if (need && k != ~0u) {
                slot = W.shadow[k];
                const float4* q = slot_of(W, slot);
                rng.s = ubits(q[Q_DIR].w);
                origin = xyz(q[Q_IDX]);
                tr_begin(A, origin, xyz(q[Q_LD]), T);
                active = true;
                map_ray = false;
            }
            drained = __any_sync(0xffffffffu, need && k == ~0u);
        }
        bool done = false;
        if (active && !tr_step(A, origin, T, rng)) {
            if (!MAP) {
                done = true;
            } else {
                float4* q = slot_of(W, slot);
                float4* m = map_of(W, slot);
                if (map_ray) {
                    float4 ml = m[M_LIGHT];
                    m[M_LIGHT] = f4(xyz(ml) * T.result, 0.0f);
                    done = true;
                } else {
                    q[Q_LT] = f4(T.result, 0.0f);
                    Vertex V;
                    sample_map_light(A, rng, V);
                    m[M_DIR] = f4(V.map_dir, V.map_pdf);
                    m[M_LIGHT] = f4(V.map_light, 0.0f);
                    if (V.map_pdf > 0.0f) {
                        tr_begin(A, origin, V.map_dir, T);
                        map_ray = true;
                    } else {
                        done = true;
                    }
                }
            }
            if (done) active = false;
        }
        if (__any_sync(0xffffffffu, done)) {
            if (done) {
                float4* q = slot_of(W, slot);
                float4 d = q[Q_DIR];
                q[Q_DIR] = make_float4(d.x, d.y, d.z, fbits(rng.s));
                if (!MAP) q[Q_LT] = f4(T.result, 0.0f);
            }
            push(W.scatter, &W.counts[WF_SCATTER], slot, done);
        }
        if (drained && !__any_sync(0xffffffffu, active)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counts[WF_SHADE] = 0;
}

// Scatter, and the end of the flights that left the volume or hit the bounce
// limits in this wave's extend (queued after the scatter entries).
__global__ void __launch_bounds__(128, 6) k_wf_scatter(const __grid_constant__ PtArgs A, const WfArgs W, int cur) {
    if (W.counts[WF_STOP] != 0u) return;
    uint32_t n_scatter = W.counts[WF_SCATTER], n = n_scatter + W.counts[WF_ESC0 + cur];
    int nxt = cur ^ 1;
    Consts C = make_consts(A);
    WF_FOR_EACH(n) {
        uint32_t i = base_ + (threadIdx.x & 31u);
        bool valid = i < n;
        bool ended = i >= n_scatter;
        uint32_t slot = valid ? (ended ? W.esc[cur][i - n_scatter] : W.scatter[i]) : 0u;
        bool to_ext = false, to_first = false, need = false;
        if (valid) {
            float4* q = slot_of(W, slot);
            Path P;
            Ctl c;
            load_path(q, P, c);
            bool escaped = ended && ubits(q[Q_CTL].w) != 0u;
            if (!ended) {
                Vertex V;
                load_vertex(q, V);
                V.n = xyz(q[Q_N]);
                V.light_dir = xyz(q[Q_LD]);
                V.light_t = xyz(q[Q_LT]);
                V.map_pdf = 0.0f;
                if (A.u.lighting[3] == 2u) {
                    const float4* m = map_of(W, slot);
                    float4 md = m[M_DIR];
                    V.map_dir = xyz(md);
                    V.map_pdf = md.w;
                    V.map_light = xyz(m[M_LIGHT]);
                }
                to_ext = stage_scatter(A, C, P, V);
            }
            if (!to_ext) {
                PixelSums S;
                load_sums(q, S);
                if (escaped) stage_escape(A, C, P, S);
                to_first = end_path(A, C, P, S, c);
                need = !to_first;
                store_sums(q, S);
            }
            store_path(q, P, c);
        }
        if (refill(A, W, C, slot, need)) to_first = true;
        push(W.ext[nxt], &W.counts[nxt], slot, to_ext);
        push(W.first[nxt], &W.counts[WF_FIRST0 + nxt], slot, to_first);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counts[WF_SHADOW] = 0;
        W.counts[WF_TAKE_SHADOW] = 0;
    }
}

// The paths still alive, run to completion one thread each (the reference's
// loop), including their pixels' remaining samples and frames.
__global__ void __launch_bounds__(128, 4) k_wf_finish(const __grid_constant__ PtArgs A, const WfArgs W, int cur) {
    uint32_t stop = W.counts[WF_STOP];
    if (stop != 0u) cur = (int)stop - 1;  // else the waves ran out first: `cur` is the next wave's queue
    uint32_t n_first = W.counts[WF_FIRST0 + cur], n = n_first + W.counts[cur];
    Consts C = make_consts(A);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t slot = i < n_first ? W.first[cur][i] : W.ext[cur][i - n_first];
        float4* q = slot_of(W, slot);
        Path P;
        Ctl c;
        PixelSums S;
        load_path(q, P, c);
        load_sums(q, S);
        uint32_t total = A.frames * A.width * A.height;
        for (;;) {
            do {
                while (bounce_step(A, C, P, S)) {
                }
            } while (end_path(A, C, P, S, c));
            uint32_t item = atomicAdd(&W.counts[WF_ITEMS], 1u);
            if (item >= total) break;
            start_item(A, C, item, P, S, c);
        }
    }
}

template <class K> static int blocks_per_sm(K kernel, int threads) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess || n < 1) n = 1;
    return n;
}

// Host side: waves of the four stages until few paths are left, then one
// finishing launch. Checks the live count every `check` waves (one 4-byte read).
cudaError_t launch_pt_wavefront(const PtArgs& a, const WfArgs& w, int sms, cudaStream_t s, int* launches) {
    static int g_ext = 0, g_shade = 0, g_shadow = 0, g_scatter = 0, g_finish = 0;
    if (!g_ext) {
        g_ext = sms * blocks_per_sm(k_wf_extend<false>, 128);
        g_shade = sms * blocks_per_sm(k_wf_shade, 128);
        g_shadow = sms * blocks_per_sm(k_wf_shadow<false>, 128);
        g_scatter = sms * blocks_per_sm(k_wf_scatter, 128);
        g_finish = sms * blocks_per_sm(k_wf_finish, 128);
    }
    const char* env = std::getenv("VV_WF_TAIL");
    uint32_t tail = env ? (uint32_t)std::atoi(env) : 1024u;
    uint32_t pixels = a.width * a.height;
    uint32_t items = a.frames * pixels;
    uint32_t slots = items < w.capacity ? items : w.capacity;  // paths in flight
    const bool map = a.u.lighting[3] == 2u;
    k_wf_init<<<(slots + 255) / 256 < (uint32_t)(sms * 8) ? (slots + 255) / 256 : sms * 8, 256, 0, s>>>(a, w, slots);
    *launches += 1;
    // All waves are queued at once, with no host round trip: the first launch
    // of each wave stops the waves on the device once at most `tail` paths
    // are left, the rest of the queued waves then return at once, and the
    // finishing launch runs the remaining paths to completion. Enough waves
    // for the pass: about 10 per round of slots plus the tail of long random
    // walks (a path has at most 4 surface and 80 volume events at g = 0.6);
    // if they still run out, the finishing launch takes what is left.
    uint32_t rounds = (items + slots - 1) / slots;
    int waves = (int)std::min<uint32_t>(24u + 10u * rounds, 4096u);
    int cur = 0;
    for (int wave = 0; wave < waves; wave++) {
        k_wf_extend<true><<<g_ext, 128, 0, s>>>(a, w, cur, tail);
        k_wf_extend<false><<<g_ext, 128, 0, s>>>(a, w, cur, tail);
        k_wf_shade<<<g_shade, 128, 0, s>>>(a, w, cur);
        if (map) k_wf_shadow<true><<<g_shadow, 128, 0, s>>>(a, w);
        else k_wf_shadow<false><<<g_shadow, 128, 0, s>>>(a, w);
        k_wf_scatter<<<g_scatter, 128, 0, s>>>(a, w, cur);
        *launches += 5;
        cur ^= 1;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_wf_finish<<<g_finish, 128, 0, s>>>(a, w, cur);
    *launches += 1;
    return cudaGetLastError();
}

}  // namespace VV_FMT_NS
}  // namespace vv
