/*
 * volpt.h — C ABI of the GB300 progressive volume path tracer.
 *
 * A drop-in for the path-tracing compute path of volview's `render` crate
 * (crates/render/src/lib.rs:14-23): volume, label, transfer-function and light
 * map upload, camera, clip planes, label visibility, accumulate-frame and
 * tone-mapped readback. Every type here is plain C (fixed-size integers, floats,
 * pointers and sizes), so a Rust `extern "C"` block binds it directly.
 *
 * Conventions
 *  - Every call returns vv_status; on failure vv_last_error() describes why.
 *  - The renderer owns its device memory; inputs are borrowed and copied.
 *  - One renderer per host thread; calls on one renderer are serialised. Device
 *    work is ordered on the context's CUDA stream: path-tracing passes run on
 *    the renderer's own streams (six passes in turn), and the context stream waits for each
 *    record's display, so work queued on it afterwards (readbacks, the caller's
 *    own kernels) sees the frame; consecutive records overlap on the device.
 *  - There is no CPU fallback: without a CUDA device every call that needs one
 *    returns VV_ERR_CUDA.
 */
#ifndef VOLPT_H
#define VOLPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VV_LABEL_COUNT 256

typedef enum vv_status {
    VV_OK = 0,
    VV_ERR_ARG = 1,     /* invalid argument (null pointer, size mismatch, bad enum) */
    VV_ERR_OOM = 2,     /* device allocation failed */
    VV_ERR_CUDA = 3,    /* CUDA runtime error or no device */
    VV_ERR_TIMEOUT = 4, /* a bounded device-side wait ran out (reserved: no kernel
                           of this library waits on another) */
    VV_ERR_STATE = 5,   /* call out of order (e.g. record before resize) */
    VV_ERR_LIMIT = 6    /* size above a documented maximum */
} vv_status;

typedef struct vv_context vv_context;
typedef struct vv_renderer vv_renderer;
typedef struct vv_batch vv_batch;

/* ------------------------------------------------------------------ inputs */

/* A scalar CT volume in Hounsfield units (volio::Volume,
 * crates/volio/src/volume.rs:9-19): voxel (i, j, k) at hu[i + dims[0] * (j +
 * dims[1] * k)]; `direction` is column-major, its columns the unit patient-space
 * (LPS, mm) directions of the i, j, k axes. */
typedef struct vv_volume {
    uint32_t dims[3];
    double spacing[3];
    double origin[3];
    double direction[9];
    const int16_t* hu;
} vv_volume;

/* A transfer-function control point (crates/render/src/transfer.rs:8-14). */
typedef struct vv_control_point {
    float hu;
    float color[3];   /* linear RGB albedo */
    float extinction; /* 1/mm */
} vv_control_point;

/* A piecewise-linear transfer function over HU (transfer.rs:26-29). */
typedef struct vv_transfer_function {
    uint32_t count;
    const vv_control_point* points;
} vv_transfer_function;

/* The segmentation model's decision margins on its own grid
 * (renderer.rs:104-114): per node, grid axis 0 fastest, 4 bytes: best label,
 * runner-up label, margin x 16, and 1 where finer labels replaced them. */
typedef struct vv_soft_label_grid {
    uint32_t dims[3];
    uint32_t src_axis[3]; /* volume axis each grid axis runs along */
    uint32_t flip[3];     /* 1 = that grid axis runs reversed */
    const uint8_t* data;
} vv_soft_label_grid;

/* Equirectangular linear-RGB light map, rows from the zenith down
 * (crates/render/src/environment.rs:13-17). */
typedef struct vv_environment_map {
    uint32_t width, height;
    const float* rgb;
} vv_environment_map;

/* ------------------------------------------------------- per-frame settings */

/* Orbit camera in patient space (crates/render/src/camera.rs:9-23). */
typedef struct vv_orbit_camera {
    float target[3];
    float distance;
    float yaw;
    float pitch;
    float fov_y;
} vv_orbit_camera;

enum { VV_LABEL_OFF = 0, VV_LABEL_TINT = 1, VV_LABEL_ISOLATE = 2, VV_LABEL_HYBRID = 3 };

/* LabelParams (renderer.rs:129-183). */
typedef struct vv_label_params {
    int32_t mode;
    float tint;
    float extinction;
    float ghost_opacity;
    float cut_margin_mm;
    uint32_t smoothing;
    float colors[VV_LABEL_COUNT][4];    /* rgb albedo, a visibility (0 hidden) */
    float materials[VV_LABEL_COUNT][4]; /* roughness, metalness, subsurface, coat */
    uint8_t ghost[VV_LABEL_COUNT];      /* 1 = drawn translucently */
    float density[VV_LABEL_COUNT][4];   /* hybrid ramp start/end, median, IQR */
    float surface[VV_LABEL_COUNT][4];   /* pattern, colour variation, relief, size */
    float optics[VV_LABEL_COUNT][4];    /* measured mu_s' rgb, w = 1 if measured */
} vv_label_params;

enum { VV_ENV_DOME = 0, VV_ENV_STUDIO = 1, VV_ENV_MAP = 2 };
enum { VV_TONE_NONE = 0, VV_TONE_ACES = 1, VV_TONE_AGX = 2 };

/* Lighting (renderer.rs:206-307). */
typedef struct vv_lighting {
    float azimuth;
    float elevation;
    float intensity;
    float ambient;
    int32_t environment;
    float light_size;
    float env_rotation;
    float anisotropy;
    float chromatic;
    int32_t shadows;
    int32_t ambient_occlusion;
    float exposure;
    int32_t auto_exposure;
    float bloom;
    float vignette;
    float grain;
    int32_t tone_mapper;
    float roughness;
    float metalness;
    float subsurface;
    float scattering_distance;
    float subsurface_strength;
    float surface_detail;
} vv_lighting;

enum { VV_PLANE_SAGITTAL = 0, VV_PLANE_CORONAL = 1, VV_PLANE_AXIAL = 2 };

/* ClipPlane / Clipping (renderer.rs:400-429). */
typedef struct vv_clip_plane {
    int32_t enabled;
    int32_t plane;
    int32_t cut_positive;
    float position;
} vv_clip_plane;

typedef struct vv_clipping {
    vv_clip_plane planes[3];
    int32_t all;
} vv_clipping;

/* VV_DENOISE_LEARNED (no counterpart in the reference): the U-Net whose
 * weights vv_set_denoiser_weights loaded, run on the accumulation before the
 * display passes. */
enum { VV_DENOISE_OFF = 0, VV_DENOISE_ATROUS = 1, VV_DENOISE_OIDN = 2, VV_DENOISE_LEARNED = 3 };

/* Option<PathTracing> (renderer.rs:333-373); enabled = 0 is None. */
typedef struct vv_path_tracing {
    int32_t enabled;
    uint32_t bounces;
    uint32_t samples_per_frame;
    int32_t denoiser;
    float aperture;
    int32_t has_focus;
    float focus[3];
} vv_path_tracing;

/* FrameParams (renderer.rs:309-331). */
typedef struct vv_frame_params {
    vv_orbit_camera camera;
    float step_mm;
    int32_t srgb_encode;
    vv_label_params labels;
    vv_lighting lighting;
    int32_t preintegrate;
    int32_t skip_empty_space;
    vv_clipping clipping;
    vv_path_tracing path_tracing;
    int32_t smooth_sampling;
} vv_frame_params;

/* Geometry of an uploaded volume (renderer.rs:546-551, 944-946). */
typedef struct vv_renderer_info {
    float bounds_lo[3];
    float bounds_hi[3];
    float min_spacing;
    float center[3];
    float diagonal;
    uint32_t dims[3];
} vv_renderer_info;

/* Size in bytes of the uniform block (the reference's std140 `Uniforms`,
 * renderer.rs:43-74 = shaders/common.glsl:4-33). */
#define VV_UNIFORMS_BYTES 21200

/* ---------------------------------------------------------------- defaults */

/* Lighting::default (renderer.rs:264-292). */
void vv_lighting_default(vv_lighting* out);
/* LabelParams::default (renderer.rs:166-182). */
void vv_label_params_default(vv_label_params* out);
/* PathTracing::default (renderer.rs:359-373), enabled; denoiser a-trous. */
void vv_path_tracing_default(vv_path_tracing* out);
/* Clipping::default (renderer.rs:418-429). */
void vv_clipping_default(vv_clipping* out);
/* OrbitCamera::framing (camera.rs:25-34). */
void vv_orbit_camera_framing(const float center[3], float diagonal, vv_orbit_camera* out);

/* ----------------------------------------------------------------- context */

/* Replaces ash/Vulkan `Context::new` (crates/render/src/context.rs:37): a CUDA
 * device and a stream owned by the context. */
vv_status vv_context_create(int device, vv_context** out);
/* As vv_context_create, but on the caller's stream (a cudaStream_t, or NULL for
 * the legacy default stream); the caller keeps ownership of the stream. */
vv_status vv_context_create_on_stream(int device, void* stream, vv_context** out);
vv_status vv_context_destroy(vv_context* ctx);

/* ---------------------------------------------------------------- renderer */

/* Renderer::new (renderer.rs:555): converts HU to normalised density on the
 * device, uploads the transfer function and computes the normal volume. */
vv_status vv_renderer_create(vv_context* ctx, const vv_volume* volume,
                             const vv_transfer_function* tf, vv_renderer** out);

/* Storage and running-sum precision: an extension beyond the reference
 * (whose density is R16_UNORM and whose sums are FP32), for the precision
 * variant of the workload. vv_renderer_create uses the reference's
 * {VV_DENSITY_UNORM16, VV_SUMS_FP32, 0, VV_MAJORANTS_REFERENCE, VV_MASK_UNORM16}. */
enum {
    VV_DENSITY_UNORM16 = 0, /* round(t * 65535), t = normalised density (the reference) */
    VV_DENSITY_FP16 = 1,    /* t as binary16, rounded to nearest even */
    VV_DENSITY_BF16 = 2,    /* t as bfloat16, rounded to nearest even */
    VV_DENSITY_FP32 = 3     /* t as binary32 */
};
enum {
    VV_SUMS_FP32 = 0,       /* accumulation images are plain FP32 running sums */
    VV_SUMS_KAHAN = 1       /* FP32 running sums with Kahan compensation per merge */
};
/* The transfer function's 64 bucket maxima, from which the brick majorants
 * come. The reference takes them from the FP32 LUT (renderer.rs:2164-2174)
 * while the tracer samples the LUT rounded to FP16 (renderer.rs:2177-2195), so
 * where an entry rounds up a sampled extinction can exceed its brick's
 * majorant by up to an FP16 half-ulp (measured 2.4e-4 relative for some
 * transfer functions). VV_MAJORANTS_BOUND takes the maxima of the FP16 LUT
 * the tracer samples, then rounds them up by 2^-20 relative (past the
 * rounding of the linear interpolation), so every sampled extinction is at or
 * below its majorant. */
enum {
    VV_MAJORANTS_REFERENCE = 0, /* bucket maxima of the FP32 LUT (the reference) */
    VV_MAJORANTS_BOUND = 1      /* of the FP16 LUT, rounded up: true bounds */
};
/* The two label-mask volumes (the binary and the blurred mask; RG16_UNORM in
 * the reference, renderer.rs:1455-1470). VV_MASK_FP16 / VV_MASK_BF16 store
 * the mask values as binary16 / bfloat16 (rounded to nearest even) and need
 * the density in the same format. */
enum {
    VV_MASK_UNORM16 = 0,    /* round(m * 65535) (the reference) */
    VV_MASK_FP16 = 1,       /* m as binary16; density_format VV_DENSITY_FP16 */
    VV_MASK_BF16 = 2        /* m as bfloat16; density_format VV_DENSITY_BF16 */
};
typedef struct vv_precision {
    uint32_t density_format; /* VV_DENSITY_* */
    uint32_t sums;           /* VV_SUMS_* */
    uint32_t fp64_after;     /* 0: never; else the running sums continue in FP64
                                once they hold this many samples per pixel */
    uint32_t majorants;      /* VV_MAJORANTS_* */
    uint32_t mask_format;    /* VV_MASK_* */
} vv_precision;
/* vv_renderer_create with a storage and running-sum precision. Frames
 * accumulated by the wavefront passes are summed per pass (FP32, atomically
 * for several frames per pass), then merged into the running sums. */
vv_status vv_renderer_create_ex(vv_context* ctx, const vv_volume* volume, const vv_transfer_function* tf,
                                const vv_precision* precision, vv_renderer** out);
/* Renderer::destroy (renderer.rs:2072). VV_ERR_STATE (nothing freed) while
 * views of the renderer's volume exist. */
vv_status vv_renderer_destroy(vv_renderer* r);
/* A view of `base`'s volume: a renderer on context `ctx` (same device) that
 * reads base's device volumes (density, normals, labels, soft label grid),
 * transfer function and light map instead of holding copies, with label
 * masks, majorants, images and path-tracing passes of its own. An extension
 * beyond the reference, for serving several views of one resident volume at
 * once. A view of a view is a view of its base. While views exist the base's
 * vv_set_transfer_function, vv_set_labels, vv_set_environment_map and
 * vv_renderer_destroy return VV_ERR_STATE, as do those calls on a view. */
vv_status vv_renderer_create_view(vv_context* ctx, vv_renderer* base, vv_renderer** out);
/* The renderer's public fields bounds, min_spacing, center and diagonal
 * (renderer.rs:545-551), and the volume's dimensions. */
vv_status vv_renderer_get_info(const vv_renderer* r, vv_renderer_info* out);
/* Renderer::default_camera (renderer.rs:944-946). */
vv_status vv_default_camera(const vv_renderer* r, vv_orbit_camera* out);

/* Renderer::set_transfer_function (renderer.rs:1226). */
vv_status vv_set_transfer_function(vv_renderer* r, const vv_transfer_function* tf);
/* Renderer::set_labels (renderer.rs:1241): n must equal the voxel count;
 * `soft` may be NULL. */
vv_status vv_set_labels(vv_renderer* r, const uint8_t* labels, size_t n,
                        const vv_soft_label_grid* soft);
/* Renderer::set_environment_map (renderer.rs:1283); NULL removes the map.
 * Prepares the importance-sampling tables (environment.rs:57-130) and restarts
 * the accumulation; Environment::Map renders with the studio until a map is
 * set, as the reference does. Maps above 16384 texels per axis: VV_ERR_LIMIT. */
vv_status vv_set_environment_map(vv_renderer* r, const vv_environment_map* map);
/* Renderer::resize (renderer.rs:1313): (re)allocates the output images. */
vv_status vv_resize(vv_renderer* r, uint32_t width, uint32_t height);

/* Renderer::record (renderer.rs:1499): one accumulate-frame (samples_per_frame
 * paths per pixel), then the denoiser and the display passes. Returns
 * VV_ERR_STATE where the reference panics (record before resize). Asynchronous:
 * returns once the work is queued; the context stream waits for the display. */
vv_status vv_record(vv_renderer* r, uint64_t frame, const vv_frame_params* params);
/* `frames` consecutive accumulate-frames with the same params in path-tracing
 * passes of up to 64 frames (all of a pass's frames in flight at once,
 * consecutive passes overlapping); the denoiser and display passes run once,
 * after the last.
 * Equivalent to `frames` calls of vv_record except that intermediate displays
 * are skipped. A pass holds at most 2^31 (frame, pixel) pairs; longer calls
 * take more passes.
 * No counterpart in the reference. */
vv_status vv_record_frames(vv_renderer* r, uint64_t first_frame, uint32_t frames,
                           const vv_frame_params* params);
/* Renderer::accumulated_samples (renderer.rs:1217). */
uint32_t vv_accumulated_samples(const vv_renderer* r);
/* Waits for the renderer's work on its stream. */
vv_status vv_synchronize(vv_renderer* r);

/* Tone-mapped RGBA8 output (the image render_to_rgba reads back), width*height*4 bytes. */
vv_status vv_read_output(vv_renderer* r, uint8_t* rgba, size_t capacity);
/* The RGBA16F HDR image as raw half bits, width*height*4 values. */
vv_status vv_read_hdr(vv_renderer* r, uint16_t* rgba_half, size_t capacity);
/* The RGBA32F accumulation images (radiance+background, albedo+lum^2,
 * normal+depth), width*height*4 floats each; any pointer may be NULL. */
vv_status vv_read_accumulation(vv_renderer* r, float* accum, float* albedo, float* normal,
                               size_t capacity_floats);

/* render_to_rgba (crates/render/src/offscreen.rs:11): resize, `frames`
 * accumulate-frames, display passes, read back width*height*4 bytes. */
vv_status vv_render_to_rgba(vv_renderer* r, const vv_frame_params* params, uint32_t width,
                            uint32_t height, uint32_t frames, uint8_t* out, size_t capacity);

/* ------------------------------------------------------------ introspection */

/* The uniform block `record` would upload for `params` at the current
 * accumulation count (the reference's std140 layout, VV_UNIFORMS_BYTES). */
vv_status vv_pack_uniforms(vv_renderer* r, const vv_frame_params* params, uint64_t frame,
                           void* out, size_t capacity);

enum {
    VV_VOLUME_DENSITY = 0,  /* uint16 per voxel (R16_UNORM; FP16 / BF16 bits, or float, per vv_precision) */
    VV_VOLUME_NORMALS = 1,  /* 4 x int8 per voxel (RGBA8_SNORM) */
    VV_VOLUME_MASK = 2,     /* 2 x 16-bit codes per voxel: RG16_UNORM, or binary16 /
                               bfloat16 under VV_MASK_FP16 / VV_MASK_BF16 */
    VV_VOLUME_LABELS = 3,   /* uint8 per voxel */
    VV_VOLUME_MAJORANT = 4, /* float per brick, brick grid x-fastest */
    VV_VOLUME_SHADOW = 5,   /* ray marcher's shadow volume: RGBA16F, ceil(dims / 2), x-fastest */
    VV_VOLUME_AO = 6        /* ray marcher's occlusion volume: R16F, ceil(dims / 4), x-fastest */
};
/* Copies a device volume out in x-fastest voxel order (whatever its layout on
 * the device). */
vv_status vv_read_volume(vv_renderer* r, int which, void* out, size_t capacity);

/* Kernel launches this renderer has issued since creation (for accounting). */
uint64_t vv_kernel_launches(const vv_renderer* r);

/* Weights of the learned denoiser (VV_DENOISE_LEARNED): `count` floats, its 19
 * convolutions in order (e0a e0b e1a .. e4b, d3a d3b .. d0a d0b, head; see
 * volview_gb300/learned_denoiser.py), each as weights [cout][3][3][cin] then
 * biases [cout]. NULL unloads them. Waits for the renderer's work. */
vv_status vv_set_denoiser_weights(vv_renderer* r, const float* params, size_t count);

/* ------------------------------------------------------------------ serving */
/* Extensions for a render-request loop over several renderers (no
 * counterpart in the reference). */

/* *idle = 1 when every call made on the renderer has finished on the device,
 * 0 while its work is in flight. Never blocks. */
vv_status vv_query(vv_renderer* r, int* idle);
/* Device bytes the renderer holds now: its volumes, images, lighting volumes
 * and path-tracing pass state (which grows with the frames per pass and the
 * image on first use). */
vv_status vv_renderer_memory(const vv_renderer* r, uint64_t* bytes);
/* Starts a new view: the accumulation restarts and auto exposure meters
 * afresh, as in a renderer just created, so a reused renderer's next image
 * does not depend on the ones before it. */
vv_status vv_reset_view(vv_renderer* r);
/* The renderer's path-tracing pass state: `passes` passes in flight (1 to 6;
 * 6 by default), each holding up to `slot_frames` frames' worth of path slots
 * (1 to 16; 16 by default). Fewer passes and frames take less device memory
 * (a pass at 1024^2 and 16 frames holds 5.7 GB) at some throughput when the
 * renderer runs alone; several renderers serving at once keep the device busy
 * between them. Waits for the renderer's work and frees the state of the
 * passes it drops. VV_ERR_ARG outside the ranges. */
vv_status vv_set_pass_budget(vv_renderer* r, uint32_t passes, uint32_t slot_frames);

/* ------------------------------------------------------------ batched passes */

/* A batch engine on context `ctx`: `passes` batched passes in flight (1 to 6)
 * on streams of its own, each holding the path state that its requests share,
 * up to `slot_frames` frames' worth of slots per request (1 to 16) and 2^24
 * slots in all unless one frame of each request needs more. An extension
 * beyond the reference (whose Renderer::record serves one view per call,
 * renderer.rs:1499): the serving loop's one wavefront over several requests. */
vv_status vv_batch_create(vv_context* ctx, uint32_t passes, uint32_t slot_frames, vv_batch** out);
vv_status vv_batch_destroy(vv_batch* b);
/* One request of a batched pass: `frames` accumulate-frames (1 to 64) of
 * `params` from frame index `first_frame`, as vv_record_frames(r,
 * first_frame, frames, params) adds them; display != 0 runs the denoiser and
 * the display after them (a request's last pass). */
typedef struct vv_batch_request {
    const vv_frame_params* params;
    uint64_t first_frame;
    uint32_t frames;
    uint32_t display;
} vv_batch_request;
/* Queues one pass whose waves trace the frames of every request at once:
 * request i accumulates into renderers[i] with the same paths, random streams
 * and sums as vv_record_frames (summed in a different order: equal to within
 * FP32 rounding). 1 to 8 distinct renderers, of any volumes (bases and
 * views), created with the reference's storage formats, resized, path
 * tracing enabled. Each renderer's context stream waits for its share, so
 * vv_query and vv_synchronize on it see the pass. VV_ERR_ARG / VV_ERR_LIMIT
 * for a batch outside these bounds (below 2^28 pixels and 2^20 samples per
 * frame per request). */
vv_status vv_batch_record(vv_batch* b, uint32_t n, vv_renderer* const* renderers,
                          const vv_batch_request* requests);
/* Device bytes of the engine's shared path state, and a wait for its passes. */
vv_status vv_batch_memory(const vv_batch* b, uint64_t* bytes);
vv_status vv_batch_synchronize(vv_batch* b);
/* Kernel launches of the engine's path tracing so far. */
uint64_t vv_batch_launches(const vv_batch* b);
/* Batched passes queued and not yet finished, without blocking (at most the
 * engine's passes in flight: each pass stream's latest pass). */
vv_status vv_batch_in_flight(vv_batch* b, uint32_t* passes);

/* --------------------------------------------------- allocation-free denoise */

/* The a-trous denoiser (the passes `record` runs after a frame) on device
 * buffers the caller owns, for callers that cannot allocate device memory when
 * they need the image: e.g. a per-frame callback running under a device-memory
 * budget fixed at start-up, or a process where another runtime owns every
 * device allocation. No counterpart in the reference.
 *
 * accum, albedo, normal: the RGBA32F accumulation images (width*height*4
 * floats each, as vv_read_accumulation lays them out, 16-byte aligned) on the
 * current device; hdr: the RGBA16F output (width*height*4 half values, 8-byte
 * aligned); samples: the paths per pixel accumulated in them. Misaligned
 * buffers return VV_ERR_ARG. Work is queued on `stream` (a cudaStream_t, NULL
 * for the legacy default stream) and the call returns without waiting. A CUDA
 * error already pending on the calling thread is returned (VV_ERR_CUDA, "pending
 * CUDA error before the call") and cleared, before anything is queued.
 *
 * Allocates nothing: its four scratch images live in a fixed device array of
 * 512 x 512 pixels each (16 MiB, held by every device that loads the library
 * until the process exits); larger images return VV_ERR_LIMIT. The first call
 * with a given CUDA context current looks the array's device address up in
 * that context (make it before any stream capture); resetting the device while
 * the library is loaded is not supported. All calls share the array: calls
 * that overlap on the GPU race on it. Each call overwrites the scratch before
 * reading it. */
vv_status vv_denoise_atrous_noalloc(const float* accum, const float* albedo, const float* normal, uint16_t* hdr,
                                    uint32_t width, uint32_t height, uint32_t samples, void* stream);

/* Description of the last error on this thread ("" if none). */
const char* vv_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* VOLPT_H */
