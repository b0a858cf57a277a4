/*
 * volpt_probe.h — test hooks of libvolpt.so.
 *
 * These entry points have no counterpart in the reference: they run single
 * device functions of the path tracer on a renderer's current state so that the
 * parity tests can compare them with the CPU oracle one sample at a time.
 */
#ifndef VOLPT_PROBE_H
#define VOLPT_PROBE_H

#include "volpt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Cubic B-spline density and its gradient (per index unit) at n continuous
 * voxel indices idx[3n] (common.glsl:124-136): out[4n] = value, gx, gy, gz.
 * Runs record's preparation (masks, majorants) for `params` first. */
vv_status vv_probe_bspline(vv_renderer* r, const vv_frame_params* params, const float* idx, size_t n,
                           float* out);

/* pt.comp's per-pixel result for n pixels (x, y pairs) at accumulation count
 * `accumulated`: out[12n] = radiance sum (rgb), background, albedo sum (rgb,
 * luminance^2), normal sum (rgb, depth). */
vv_status vv_probe_paths(vv_renderer* r, const vv_frame_params* params, uint32_t accumulated,
                         const int* pixels, size_t n, float* out);

/* vv_probe_paths run by the parity build of the same device code: samplers in
 * the texture-unit arithmetic the CPU oracle models (texel coordinates through
 * index_to_tex, texels decoded before filtering, the reference's 8 folded
 * B-spline fetches, the LUT at (d * 4095 + 0.5) / 4096) and no fused
 * multiply-adds (--fmad=false), so that a replay differs from the oracle's only
 * where CUDA's transcendental functions and the C library's differ. */
vv_status vv_probe_paths_exact(vv_renderer* r, const vv_frame_params* params, uint32_t accumulated,
                               const int* pixels, size_t n, float* out);

/* The extinction a free flight samples at n continuous voxel indices idx[3n]
 * (extinction_at, pt.comp:277-292, then path_sigma, pt.comp:143-145) with
 * direction dir[3] (index space) and, with smooth = 1, the first flight's
 * B-spline density; and the flight majorant of the brick there (pt.comp:157-163):
 * out[4n] = sigma (rgb), majorant. Runs record's preparation first. */
vv_status vv_probe_extinction(vv_renderer* r, const vv_frame_params* params, const float* idx, size_t n,
                              const float dir[3], int smooth, float* out);

/* Event counting for the roofline's algorithmic-byte model: enable = 1 starts
 * counting the path tracer's memory events over the following records (at
 * some cost in speed); enable = 0 stops and copies up to n totals to out, in
 * the order: majorant lookups, cubic densities, trilinear densities, mask
 * lookups, label fetches, normal lookups, cubic gradients, pixel
 * accumulations, paths, path vertices. */
vv_status vv_count_events(vv_renderer* r, int enable, uint64_t* out, size_t n);

/* Device time of the path-tracing launches: enable = 1 starts recording CUDA
 * events around each launch on the stream it runs on; enable = 0 stops, waits,
 * and returns the summed milliseconds and the number of launches. */
vv_status vv_time_pt(vv_renderer* r, int enable, double* ms, uint64_t* launches);

/* Light map importance sampling (pt.comp:204-233) from n random-stream states
 * seeds[n]: out[6n] = texel column, texel row, pdf, direction (xyz). Needs a
 * light map (vv_set_environment_map). */
vv_status vv_probe_light_samples(vv_renderer* r, const vv_frame_params* params, const uint32_t* seeds, size_t n,
                                 float* out);

#ifdef __cplusplus
}
#endif

#endif /* VOLPT_PROBE_H */
