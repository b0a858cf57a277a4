// vv_host.cpp — the renderer behind include/volpt.h.
//
// Restates the host side of volview's `render` crate for the path-tracing
// path: Renderer::new / set_transfer_function / set_labels / resize / record
// (crates/render/src/renderer.rs), render_to_rgba (offscreen.rs), the transfer
// function (transfer.rs) and the orbit camera (camera.rs). Vulkan images become
// device buffers on one CUDA stream; descriptor sets become kernel arguments.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/volpt.h"
#include "../../include/volpt_nn.h"
#include "vv_device.cuh"
#include "vv_kernels.h"

using namespace vv;

// ------------------------------------------------------------------ errors
static thread_local std::string g_error;

static vv_status fail(vv_status s, const std::string& msg) {
    g_error = msg;
    return s;
}
static vv_status cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? VV_ERR_OOM : VV_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                               \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
    } while (0)

extern "C" const char* vv_last_error(void) { return g_error.c_str(); }

namespace vv {
// Error reporting for entry points defined in other translation units.
vv_status internal_fail(vv_status s, const std::string& msg) { return fail(s, msg); }
}  // namespace vv

// ---------------------------------------------------------------- defaults
static float to_radians(float deg) { return deg * (3.14159265358979323846f / 180.0f); }

extern "C" void vv_lighting_default(vv_lighting* L) {
    std::memset(L, 0, sizeof(*L));
    L->azimuth = to_radians(-60.0f);
    L->elevation = to_radians(40.0f);
    L->intensity = 3.0f;
    L->ambient = 0.3f;
    L->environment = VV_ENV_STUDIO;
    L->light_size = to_radians(12.0f);
    L->env_rotation = 0.0f;
    L->anisotropy = 0.0f;
    L->chromatic = 1.0f;
    L->shadows = 1;
    L->ambient_occlusion = 1;
    L->exposure = 0.0f;
    L->auto_exposure = 1;
    L->bloom = 0.04f;
    L->vignette = 0.25f;
    L->grain = 0.012f;
    L->tone_mapper = VV_TONE_ACES;
    L->roughness = 0.5f;
    L->metalness = 0.0f;
    L->subsurface = 0.3f;
    L->scattering_distance = 4.0f;
    L->subsurface_strength = 1.0f;
    L->surface_detail = 1.0f;
}

extern "C" void vv_label_params_default(vv_label_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->mode = VV_LABEL_OFF;
    p->tint = 0.7f;
    p->extinction = 0.5f;
    p->ghost_opacity = 0.08f;
    p->cut_margin_mm = 2.0f;
    p->smoothing = 1;
    for (int i = 0; i < VV_LABEL_COUNT; i++) {
        for (int c = 0; c < 4; c++) p->colors[i][c] = 1.0f;
        p->materials[i][0] = 0.5f; p->materials[i][1] = 0.0f; p->materials[i][2] = 0.3f; p->materials[i][3] = 0.0f;
        p->density[i][0] = 0.0f; p->density[i][1] = 1e-3f; p->density[i][2] = 0.5f; p->density[i][3] = 1.0f;
    }
}

extern "C" void vv_path_tracing_default(vv_path_tracing* pt) {
    std::memset(pt, 0, sizeof(*pt));
    pt->enabled = 1;
    pt->bounces = 4;
    pt->samples_per_frame = 1;
    pt->denoiser = VV_DENOISE_ATROUS;
}

extern "C" void vv_clipping_default(vv_clipping* c) {
    std::memset(c, 0, sizeof(*c));
    for (int i = 0; i < 3; i++) c->planes[i].plane = i;
}

extern "C" void vv_orbit_camera_framing(const float center[3], float diagonal, vv_orbit_camera* out) {
    float fov = to_radians(30.0f);
    for (int i = 0; i < 3; i++) out->target[i] = center[i];
    out->distance = 0.55f * diagonal / std::tan(fov / 2.0f);
    out->yaw = 0.0f;
    out->pitch = 0.0f;
    out->fov_y = fov;
}

// ----------------------------------------------------------------- context
struct vv_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool owns_stream = false;
    int sms = 0;
};

extern "C" vv_status vv_context_create_on_stream(int device, void* stream, vv_context** out) {
    if (!out) return fail(VV_ERR_ARG, "null output pointer");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(VV_ERR_CUDA, "no CUDA device");
    if (device < 0 || device >= n) return fail(VV_ERR_ARG, "device index out of range");
    CK(cudaSetDevice(device));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    vv_context* c = new vv_context();
    c->device = device;
    c->sms = sms;
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return cuda_fail(e, "cudaStreamCreate");
        }
        c->owns_stream = true;
    }
    *out = c;
    return VV_OK;
}

extern "C" vv_status vv_context_create(int device, vv_context** out) {
    return vv_context_create_on_stream(device, nullptr, out);
}

extern "C" vv_status vv_context_destroy(vv_context* c) {
    if (!c) return VV_OK;
    cudaSetDevice(c->device);
    if (c->owns_stream) cudaStreamDestroy(c->stream);
    delete c;
    return VV_OK;
}

// ---------------------------------------------------------- device buffers
struct DBuf {
    void* p = nullptr;
    size_t n = 0;
    bool borrowed = false;  // another renderer's buffer (a view's shared volume): never freed or resized here
    cudaError_t alloc(size_t bytes) {
        if (p && n == bytes && !borrowed) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) n = bytes;
        else p = nullptr;
        return e;
    }
    void release() {
        if (p && !borrowed) cudaFree(p);
        p = nullptr;
        n = 0;
        borrowed = false;
    }
    void borrow(const DBuf& owner) {
        release();
        p = owner.p;
        n = owner.n;
        borrowed = p != nullptr;
    }
    size_t owned_bytes() const { return borrowed ? 0 : n; }
    template <class T> T* as() const { return (T*)p; }
};

// Everything that decides which voxels are opaque (renderer.rs:436-449).
struct OpacityKey {
    uint64_t generation;
    int mode;
    uint32_t extinction_bits;
    uint64_t visible[4], ghost[4];
    uint32_t ghost_opacity_bits;
    int margin;
    uint32_t smoothing;
    bool operator==(const OpacityKey& o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};

// Path-tracing passes in flight at once (each on its own stream, with its own
// path state: up to 2^24 slots, 5.4 GB at 1024^2 with 16 frames per pass).
// Measured at 1024^2 with 16 frames per call: 306, 316, 323, 325 and 323 M path
// samples/s with 2, 3, 4, 6 and 8 passes; one frame per call: 11.8, 10.7, 9.2,
// 8.2 and 7.8 ms per frame.
#ifndef VV_PASSES
#define VV_PASSES 6
#endif
// Frames per pass of a long vv_record_frames call.
#ifndef VV_SUBPASS_FRAMES
#define VV_SUBPASS_FRAMES 64
#endif

struct vv_renderer {
    vv_context* ctx;
    // A view (vv_renderer_create_view) reads the volume, transfer function,
    // labels and light map of `base` (never a view itself), which counts its
    // live views and keeps those unchanged while any exist.
    vv_renderer* base = nullptr;
    int views = 0;
    Vol vol;
    double spacing[3];
    // geometry
    float w2i[16], i2w[16];
    float dims[3];
    float bounds_lo[3], bounds_hi[3];
    float min_spacing, max_spacing;
    float center[3];
    float diagonal;
    // transfer function
    float bucket[64];
    uint32_t majorants = VV_MAJORANTS_REFERENCE;  // VV_MAJORANTS_*: which bucket maxima
    // device volumes
    DBuf density, normals, mask_a, mask_b, labels, majorant, lut, bucket_dev, tables, soft, work, exposure;
    int soft_dims[3] = {1, 1, 1};
    int soft_push[4] = {0, 0, 0, 0};
    bool has_labels = false;
    uint64_t generation = 0;
    bool have_mask_key = false, have_majorant_key = false;
    OpacityKey mask_key, majorant_key;
    // outputs
    uint32_t width = 0, height = 0;
    DBuf accum, albedo, normal, ping, pong, guide_nd, guide_alb, hdr, out, bloom[4];
    int bw[4], bh[4];
    // pre-integrated transfer function (RGBA32F, 4096), ray-marcher lighting volumes
    DBuf preint, shadow_vol, ao_vol;
    // the lighting volumes as the image loop reads them: 3D textures with a
    // white border, written from shadow_vol / ao_vol after each rebuild
    struct TexVol {
        cudaArray_t arr = nullptr;
        cudaTextureObject_t tex = 0;
        cudaSurfaceObject_t surf = 0;
    } shadow_tex, ao_tex;
    int shadow_dims[3] = {0, 0, 0}, ao_dims[3] = {0, 0, 0};
    std::vector<uint8_t> ao_key, shadow_key;
    // light map (Environment::Map): RGBA16F radiance, RG32F sampling table,
    // RGBA16F diffuse convolution (32 x 16, the ray marcher's ambient light)
    DBuf env_rad, env_table, env_diffuse, env_guide;
    int env_w = 0, env_h = 0, env_gm = 0, env_gr = 0;
    bool has_env = false;
    float env_peak_u = 0.0f;
    // wavefront tracer: path slots, stage queues, counters
    // Path-tracing passes, VV_PASSES in flight: each has its own stream, wavefront
    // state and sums of its frames; a pass's sums are merged into the
    // accumulation (and displayed) after the previous call's display, so a
    // call's pass overlaps the tail of the previous one.
    struct Pass {
        DBuf slots, map, queues, counts, accum, albedo, normal, binq, bins;
        uint32_t nbins = 0;  // the bin count `bins` is laid out for (counts, then insertion points)
        cudaStream_t stream = nullptr;
        cudaEvent_t shown = nullptr;  // after the pass's merge and display
    } pass[VV_PASSES];
    int next_pass = 0;
    int passes = VV_PASSES;  // passes in use (vv_set_pass_budget)
    int slot_frames = 16;    // frames' worth of path slots per pass (vv_set_pass_budget)
    bool prep_work = false;  // set-up queued on the context stream since prep_done was last recorded
    cudaEvent_t prep_done = nullptr;  // the latest set-up's end, which every pass waits for
    // accumulation
    uint32_t accumulated = 0;
    bool have_params = false;
    // running-sum precision (vv_precision): Kahan compensation of the three
    // accumulation images, and FP64 running sums once past fp64_after samples
    uint32_t sums = VV_SUMS_FP32, fp64_after = 0;
    DBuf comp[3], wide[3];
    bool wide_active = false;
    // the learned denoiser (VV_DENOISE_LEARNED): its weights (FP16) and biases
    // per convolution, and its tensors for the padded image size
    struct UNet {
        bool loaded = false;
        DBuf w[19], b[19];
        int wp = 0, hp = 0;
        DBuf in, ea[5], eb[5], pool[5], up[4], cat[4], da[4], db[4], head;
    } unet;
    vv_frame_params accumulated_params;
    // host staging for the label tables
    LabelTables* tables_host = nullptr;
    bool tables_valid = false;
    uint64_t launches = 0;
    unsigned long long* counters = nullptr;  // set while counting events
    // CUDA events around each path-tracing launch while timing is on.
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pt_events;
};

// The path tracer's and the ray marcher's launchers of one density storage
// format (compiled once per format, vv::fmt0 .. vv::fmt3).
struct FormatLaunchers {
    decltype(&fmt0::launch_pt) pt;
    decltype(&fmt0::launch_pt_wavefront) pt_wavefront;
    decltype(&fmt0::launch_ao) ao;
    decltype(&fmt0::launch_shadow_sweep) shadow_sweep;
    decltype(&fmt0::launch_pad_lighting) pad_lighting;
    decltype(&fmt0::launch_dvr) dvr;
    decltype(&fmt0::launch_bspline_probe) bspline_probe;
    decltype(&fmt0::launch_light_sample_probe) light_sample_probe;
    decltype(&fmt0::launch_pt_pixels) pt_pixels;
    decltype(&fmt0::launch_extinction_probe) extinction_probe;
};
#define VV_FORMAT_TABLE(ns)                                                                                   \
    {ns::launch_pt, ns::launch_pt_wavefront, ns::launch_ao, ns::launch_shadow_sweep, ns::launch_pad_lighting, \
     ns::launch_dvr, ns::launch_bspline_probe, ns::launch_light_sample_probe, ns::launch_pt_pixels,          \
     ns::launch_extinction_probe}
static const FormatLaunchers FORMAT_LAUNCHERS[6] = {VV_FORMAT_TABLE(fmt0), VV_FORMAT_TABLE(fmt1),
                                                    VV_FORMAT_TABLE(fmt2), VV_FORMAT_TABLE(fmt3),
                                                    VV_FORMAT_TABLE(fmt4), VV_FORMAT_TABLE(fmt5)};
// The build of the renderer's storage: the density format's, or 4 / 5 for
// FP16 / BF16 density with the mask in the same format.
static int build_of(const Vol& v) {
    if (v.mfmt == MF_FP16) return 4;
    if (v.mfmt == MF_BF16) return 5;
    return v.dfmt & 3;
}
static const FormatLaunchers& kernels_of(const vv_renderer* r) { return FORMAT_LAUNCHERS[build_of(r->vol)]; }

static void free_tex_vol(vv_renderer::TexVol& t) {
    if (t.tex) cudaDestroyTextureObject(t.tex);
    if (t.surf) cudaDestroySurfaceObject(t.surf);
    if (t.arr) cudaFreeArray(t.arr);
    t = vv_renderer::TexVol();
}

// Records the start event of a timed path-tracing launch (if timing is on).
static void pt_timer_start(vv_renderer* r, cudaStream_t s) {
    if (!r->timing) return;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    r->pt_events.push_back({a, b});
}
static void pt_timer_stop(vv_renderer* r, cudaStream_t s) {
    if (r->timing && !r->pt_events.empty()) cudaEventRecord(r->pt_events.back().second, s);
}

// ------------------------------------------------------------ host math
// Vector arithmetic follows glam (normalize multiplies by the reciprocal length).
struct h3 {
    float x, y, z;
};
static h3 add(h3 a, h3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static h3 sub(h3 a, h3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static h3 scl(h3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static float hdot(h3 a, h3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
static h3 hcross(h3 a, h3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
static h3 hnorm(h3 a) { return scl(a, 1.0f / std::sqrt(hdot(a, a))); }

// camera.rs:34-48
static h3 cam_forward(const vv_orbit_camera& c) {
    float sy = std::sin(c.yaw), cy = std::cos(c.yaw), sp = std::sin(c.pitch), cp = std::cos(c.pitch);
    return {cp * sy, cp * cy, -sp};
}

// transfer.rs:72-86
static void tf_eval(const vv_transfer_function* tf, float hu, float out[4]) {
    const vv_control_point* p = tf->points;
    auto put = [&](const vv_control_point& c) {
        out[0] = c.color[0]; out[1] = c.color[1]; out[2] = c.color[2]; out[3] = c.extinction;
    };
    if (hu <= p[0].hu) { put(p[0]); return; }
    for (uint32_t k = 0; k + 1 < tf->count; k++) {
        if (hu <= p[k + 1].hu) {
            float t = (hu - p[k].hu) / std::fmax(p[k + 1].hu - p[k].hu, 1e-6f);
            float a[4] = {p[k].color[0], p[k].color[1], p[k].color[2], p[k].extinction};
            float b[4] = {p[k + 1].color[0], p[k + 1].color[1], p[k + 1].color[2], p[k + 1].extinction};
            for (int i = 0; i < 4; i++) out[i] = a[i] + (b[i] - a[i]) * t;
            return;
        }
    }
    put(p[tf->count - 1]);
}

// Uploads the LUT (transfer.rs:90-97, f16-rounded as upload_tf does,
// renderer.rs:2177-2182) and computes the bucket maxima (renderer.rs:2164-2174).
static vv_status upload_tf(vv_renderer* r, const vv_transfer_function* tf) {
    if (!tf || tf->count == 0 || !tf->points) return fail(VV_ERR_ARG, "empty transfer function");
    std::vector<float> lut(4 * 4096);
    for (int i = 0; i < 4096; i++) {
        float t = (float)i / 4095.0f;
        tf_eval(tf, -1024.0f + t * (3071.0f - -1024.0f), &lut[4 * i]);
    }
    std::vector<float> lut_half(4 * 4096);
    for (int i = 0; i < 4 * 4096; i++) lut_half[i] = (float)(_Float16)lut[i];
    // VV_MAJORANTS_BOUND: the maxima of the FP16 entries the tracer samples,
    // rounded up past the interpolation's rounding; else the reference's.
    const bool bound = r->majorants == VV_MAJORANTS_BOUND;
    const std::vector<float>& from = bound ? lut_half : lut;
    for (int b = 0; b < 64; b++) {
        int end = std::min((b + 1) * 64 + 1, 4096);
        float m = 0.0f;
        for (int i = b * 64; i < end; i++) m = std::fmax(m, from[4 * i + 3]);
        if (bound && m > 0.0f) m = std::nextafter(m * (1.0f + 0x1p-20f), INFINITY);
        r->bucket[b] = m;
    }
    CK(r->lut.alloc(lut_half.size() * sizeof(float)));
    CK(cudaMemcpyAsync(r->lut.p, lut_half.data(), lut_half.size() * sizeof(float), cudaMemcpyHostToDevice,
                       r->ctx->stream));
    // transfer.rs:103-117: cumulative integrals of (albedo x extinction,
    // extinction) over density, trapezoid rule in f64, for pre-integration.
    std::vector<float> preint(4 * 4096, 0.0f);
    double sum[4] = {0.0, 0.0, 0.0, 0.0};
    const double dx = 1.0 / 4095.0;
    for (int i = 1; i < 4096; i++) {
        const float* e0 = &lut[4 * (i - 1)];
        const float* e1 = &lut[4 * i];
        double a[4] = {(double)(e0[0] * e0[3]), (double)(e0[1] * e0[3]), (double)(e0[2] * e0[3]), (double)e0[3]};
        double b[4] = {(double)(e1[0] * e1[3]), (double)(e1[1] * e1[3]), (double)(e1[2] * e1[3]), (double)e1[3]};
        for (int c = 0; c < 4; c++) {
            sum[c] += 0.5 * (a[c] + b[c]) * dx;
            preint[4 * i + c] = (float)sum[c];
        }
    }
    CK(r->preint.alloc(preint.size() * sizeof(float)));
    CK(cudaMemcpyAsync(r->preint.p, preint.data(), preint.size() * sizeof(float), cudaMemcpyHostToDevice,
                       r->ctx->stream));
    CK(r->bucket_dev.alloc(64 * sizeof(float)));
    CK(cudaMemcpyAsync(r->bucket_dev.p, r->bucket, sizeof(r->bucket), cudaMemcpyHostToDevice, r->ctx->stream));
    CK(cudaStreamSynchronize(r->ctx->stream));
    return VV_OK;
}

// volio Volume::index_to_world / world_to_index (volume.rs:22-35) in f64, cast to
// f32; bounds, centre and diagonal as in Renderer::new (renderer.rs:819-834).
static void set_geometry(vv_renderer* r, const vv_volume* v) {
    double m[9];
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) m[3 * c + k] = v->direction[3 * c + k] * v->spacing[c];
    double a = m[0], b = m[3], c = m[6], d = m[1], e = m[4], f = m[7], g = m[2], h = m[5], k = m[8];
    double A = e * k - f * h, B = -(d * k - f * g), C = d * h - e * g;
    double det = a * A + b * B + c * C;
    double inv[9] = {A / det, -(b * k - c * h) / det, (b * f - c * e) / det,
                     B / det, (a * k - c * g) / det, -(a * f - c * d) / det,
                     C / det, -(a * h - b * g) / det, (a * e - b * d) / det};  // column-major
    for (int col = 0; col < 3; col++) {
        for (int row = 0; row < 3; row++) {
            r->w2i[4 * col + row] = (float)inv[3 * col + row];
            r->i2w[4 * col + row] = (float)m[3 * col + row];
        }
        r->w2i[4 * col + 3] = 0.0f;
        r->i2w[4 * col + 3] = 0.0f;
    }
    for (int row = 0; row < 3; row++) {
        double t = -(inv[row] * v->origin[0] + inv[3 + row] * v->origin[1] + inv[6 + row] * v->origin[2]);
        r->w2i[12 + row] = (float)t;
        r->i2w[12 + row] = (float)v->origin[row];
    }
    r->w2i[15] = 1.0f;
    r->i2w[15] = 1.0f;
    auto world = [&](double x, double y, double z, double* o) {
        for (int q = 0; q < 3; q++) o[q] = m[q] * x + m[3 + q] * y + m[6 + q] * z + v->origin[q];
    };
    double cw[3];
    world((v->dims[0] - 1.0) * 0.5, (v->dims[1] - 1.0) * 0.5, (v->dims[2] - 1.0) * 0.5, cw);
    for (int q = 0; q < 3; q++) {
        r->center[q] = (float)cw[q];
        r->dims[q] = (float)v->dims[q];
        r->bounds_lo[q] = 3.4028235e38f;
        r->bounds_hi[q] = -3.4028235e38f;
        r->spacing[q] = v->spacing[q];
    }
    for (int i = 0; i < 8; i++) {
        double w[3];
        world((i & 1) ? v->dims[0] - 0.5 : -0.5, (i & 2) ? v->dims[1] - 0.5 : -0.5, (i & 4) ? v->dims[2] - 0.5 : -0.5, w);
        for (int q = 0; q < 3; q++) {
            r->bounds_lo[q] = std::fmin(r->bounds_lo[q], (float)w[q]);
            r->bounds_hi[q] = std::fmax(r->bounds_hi[q], (float)w[q]);
        }
    }
    r->min_spacing = (float)std::fmin(v->spacing[0], std::fmin(v->spacing[1], v->spacing[2]));
    r->max_spacing = (float)std::fmax(v->spacing[0], std::fmax(v->spacing[1], v->spacing[2]));
    double ext = 0.0;
    for (int q = 0; q < 3; q++) {
        double x = std::fmax((double)v->dims[q] - 1.0, 0.0) * v->spacing[q];
        ext += x * x;
    }
    r->diagonal = (float)std::sqrt(ext);
}

// renderer.rs:80-87
static float tissue_majorant(const vv_label_params& l, float anisotropy, float limit) {
    float g = std::fmin(std::fmax(anisotropy, 0.0f), 0.95f);
    float largest = 0.0f;
    for (int i = 0; i < 256; i++)
        if (l.colors[i][3] > 0.5f && !l.ghost[i] && l.optics[i][3] > 0.0f) {
            float m = 0.0f;
            for (int c = 0; c < 3; c++) m = std::fmax(m, l.optics[i][c]);
            largest = std::fmax(largest, m);
        }
    return std::fmin(largest / (1.0f - g), limit);
}

// The uniform block `record` writes (renderer.rs:1516-1660) and the clip planes
// of clip_uniforms (renderer.rs:1449-1466), std140.
static void pack(const vv_renderer* r, const vv_frame_params& p, uint32_t accumulated, uint64_t frame,
                 UHead& u, LabelTables& t) {
    std::memset(&u, 0, sizeof(u));
    const vv_orbit_camera& cam = p.camera;
    h3 f = cam_forward(cam);
    h3 right = hnorm(hcross(f, {0.0f, 0.0f, 1.0f}));
    h3 up = hcross(right, f);
    h3 eye = sub({cam.target[0], cam.target[1], cam.target[2]}, scl(f, cam.distance));
    float tan_half = std::tan(cam.fov_y / 2.0f);
    float aspect = (float)r->width / (float)r->height;
    const vv_lighting& L = p.lighting;
    float se = std::sin(L.elevation), ce = std::cos(L.elevation), sa = std::sin(L.azimuth), ca = std::cos(L.azimuth);
    h3 ld = hnorm(add(add(scl(scl(scl(f, -1.0f), ce), ca), scl(scl(right, ce), sa)), scl(up, se)));
    // Environment::Map without a light map falls back to the studio (renderer.rs:1524-1535);
    // the map's brightest column turns to the key light's azimuth.
    int environment = L.environment == VV_ENV_MAP && !r->has_env ? VV_ENV_STUDIO : L.environment;
    float env_rotation = 0.0f;
    if (r->has_env) {
        float key_phi = std::atan2(std::sin(L.azimuth), -std::cos(L.azimuth));
        env_rotation = (r->env_peak_u - 0.5f) * 6.28318530717958647692f - key_phi + L.env_rotation;
    }
    const vv_label_params& lab = p.labels;
    std::memcpy(u.w2i, r->w2i, sizeof(u.w2i));
    auto put3 = [](float* d, h3 v, float w) { d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = w; };
    put3(u.eye, eye, 1.0f);
    put3(u.forward, f, 0.0f);
    put3(u.right, scl(scl(right, tan_half), aspect), 0.0f);
    put3(u.up, scl(up, tan_half), 0.0f);
    u.dims[0] = r->dims[0]; u.dims[1] = r->dims[1]; u.dims[2] = r->dims[2]; u.dims[3] = p.step_mm;
    u.flags[0] = (uint32_t)frame; u.flags[1] = p.srgb_encode ? 1u : 0u; u.flags[2] = r->width; u.flags[3] = r->height;
    u.labels[0] = r->has_labels ? (float)lab.mode : 0.0f;
    u.labels[1] = lab.tint; u.labels[2] = lab.extinction; u.labels[3] = lab.ghost_opacity;
    put3(u.light_dir, ld, L.intensity);
    float amb = environment == VV_ENV_STUDIO ? 0.5f * L.ambient : L.ambient;
    u.ambient[0] = amb; u.ambient[1] = amb; u.ambient[2] = amb; u.ambient[3] = std::exp2(L.exposure);
    u.material[0] = L.roughness; u.material[1] = L.metalness; u.material[2] = (float)L.tone_mapper;
    u.material[3] = L.light_size;
    u.lighting[0] = L.shadows ? 1u : 0u; u.lighting[1] = L.ambient_occlusion ? 1u : 0u;
    u.lighting[2] = p.preintegrate ? 1u : 0u; u.lighting[3] = (uint32_t)environment;
    u.light_cells[0] = 2.0f * r->max_spacing; u.light_cells[1] = 4.0f * r->max_spacing;
    {
        h3 col[3] = {{r->i2w[0], r->i2w[1], r->i2w[2]}, {r->i2w[4], r->i2w[5], r->i2w[6]}, {r->i2w[8], r->i2w[9], r->i2w[10]}};
        h3 b = {r->i2w[12], r->i2w[13], r->i2w[14]};
        uint32_t n = 0;
        for (int i = 0; i < 3; i++) {
            const vv_clip_plane& cp = p.clipping.planes[i];
            if (!cp.enabled) continue;
            float sign = cp.cut_positive ? 1.0f : -1.0f;
            h3 normal = {0.0f, 0.0f, 0.0f};
            int axis = cp.plane < 0 ? 0 : (cp.plane > 2 ? 2 : cp.plane);
            (&normal.x)[axis] = 1.0f;
            normal = scl(normal, sign);
            h3 an = {hdot(col[0], normal), hdot(col[1], normal), hdot(col[2], normal)};
            put3(u.clip_planes + 4 * n, an, sign * cp.position - hdot(normal, b));
            put3(u.clip_normals + 4 * n, normal, 0.0f);
            n++;
        }
        u.clip[0] = n; u.clip[1] = p.clipping.all ? 1u : 0u;
    }
    uint32_t skip = p.skip_empty_space ? 1u : 0u;
    const vv_path_tracing& pt = p.path_tracing;
    if (pt.enabled) {
        u.path[0] = accumulated; u.path[1] = pt.bounces; u.path[2] = std::max(pt.samples_per_frame, 1u); u.path[3] = skip;
        float focus = cam.distance;
        if (pt.has_focus) focus = hdot(sub({pt.focus[0], pt.focus[1], pt.focus[2]}, eye), f);
        u.lens[0] = pt.aperture; u.lens[1] = std::fmax(focus, 1.0f);
    } else {
        u.path[3] = skip;
    }
    u.env[0] = env_rotation; u.env[1] = p.smooth_sampling ? 1.0f : 0.0f; u.env[2] = L.anisotropy; u.env[3] = L.chromatic;
    u.finish[0] = L.bloom; u.finish[1] = L.vignette; u.finish[2] = L.grain; u.finish[3] = L.auto_exposure ? 1.0f : 0.0f;
    std::memcpy(u.tf_bucket_max, r->bucket, sizeof(r->bucket));
    u.subsurface[0] = L.subsurface * L.subsurface_strength;
    u.subsurface[1] = 10.0f / std::fmax(L.scattering_distance, 0.1f);
    u.subsurface[2] = 0.7f;
    u.subsurface[3] = 2.0f * r->max_spacing;
    for (int i = 0; i < 256; i++) {
        const float* c = lab.colors[i];
        t.colors[i] = make_float4(c[0], c[1], c[2], (c[3] > 0.5f && lab.ghost[i]) ? 2.0f : c[3]);
        const float* m = lab.materials[i];
        t.materials[i] = make_float4(m[0], m[1], m[3], m[2] * L.subsurface_strength);
        const float* d = lab.density[i];
        t.density[i] = make_float4(d[0], d[1], d[2], d[3]);
        const float* s = lab.surface[i];
        t.surface[i] = make_float4(s[0], s[1] * L.surface_detail, s[2] * L.surface_detail, s[3]);
        const float* o = lab.optics[i];
        t.optics[i] = make_float4(o[0], o[1], o[2], o[3]);
    }
    float limit = 1.0f / (2.0f * r->max_spacing);
    u.tissue[0] = tissue_majorant(lab, L.anisotropy, limit);
    u.tissue[1] = limit;
}

static OpacityKey opacity_key(const vv_renderer* r, const vv_label_params& l) {
    OpacityKey k;
    std::memset(&k, 0, sizeof(k));
    k.generation = r->generation;
    k.mode = r->has_labels ? l.mode : VV_LABEL_OFF;
    std::memcpy(&k.extinction_bits, &l.extinction, 4);
    for (int i = 0; i < 256; i++) {
        if (l.colors[i][3] > 0.5f) k.visible[i / 64] |= 1ull << (i % 64);
        if (l.ghost[i]) k.ghost[i / 64] |= 1ull << (i % 64);
    }
    std::memcpy(&k.ghost_opacity_bits, &l.ghost_opacity, 4);
    float m = std::round(l.cut_margin_mm / r->min_spacing);
    k.margin = (int)std::fmin(std::fmax(m, 0.0f), 3.0f);
    k.smoothing = std::min(l.smoothing, 8u);
    return k;
}

// FrameParams equality except the denoiser (renderer.rs:1537-1544), with f32
// comparisons as Rust's PartialEq makes them (-0 == 0, NaN != NaN).
static bool feq(const float* a, const float* b, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!(a[i] == b[i])) return false;
    return true;
}
static bool same_accumulation(const vv_frame_params& a, const vv_frame_params& b) {
#define F(x) feq(&a.x, &b.x, 1)
#define I(x) (a.x == b.x)
    const vv_label_params &la = a.labels, &lb = b.labels;
    const vv_lighting &A = a.lighting, &B = b.lighting;
    bool cam = feq(a.camera.target, b.camera.target, 3) && F(camera.distance) && F(camera.yaw) && F(camera.pitch) &&
               F(camera.fov_y);
    bool labels = la.mode == lb.mode && la.tint == lb.tint && la.extinction == lb.extinction &&
                  la.ghost_opacity == lb.ghost_opacity && la.cut_margin_mm == lb.cut_margin_mm &&
                  la.smoothing == lb.smoothing && feq(&la.colors[0][0], &lb.colors[0][0], 1024) &&
                  feq(&la.materials[0][0], &lb.materials[0][0], 1024) && !std::memcmp(la.ghost, lb.ghost, 256) &&
                  feq(&la.density[0][0], &lb.density[0][0], 1024) && feq(&la.surface[0][0], &lb.surface[0][0], 1024) &&
                  feq(&la.optics[0][0], &lb.optics[0][0], 1024);
    bool light = A.azimuth == B.azimuth && A.elevation == B.elevation && A.intensity == B.intensity &&
                 A.ambient == B.ambient && A.environment == B.environment && A.light_size == B.light_size &&
                 A.env_rotation == B.env_rotation && A.anisotropy == B.anisotropy && A.chromatic == B.chromatic &&
                 A.shadows == B.shadows && A.ambient_occlusion == B.ambient_occlusion && A.exposure == B.exposure &&
                 A.auto_exposure == B.auto_exposure && A.bloom == B.bloom && A.vignette == B.vignette &&
                 A.grain == B.grain && A.tone_mapper == B.tone_mapper && A.roughness == B.roughness &&
                 A.metalness == B.metalness && A.subsurface == B.subsurface &&
                 A.scattering_distance == B.scattering_distance && A.subsurface_strength == B.subsurface_strength &&
                 A.surface_detail == B.surface_detail;
    bool clip = I(clipping.all);
    for (int i = 0; i < 3; i++)
        clip = clip && I(clipping.planes[i].enabled) && I(clipping.planes[i].plane) &&
               I(clipping.planes[i].cut_positive) && F(clipping.planes[i].position);
    bool pt = I(path_tracing.enabled);
    if (pt && a.path_tracing.enabled)
        pt = I(path_tracing.bounces) && I(path_tracing.samples_per_frame) && F(path_tracing.aperture) &&
             I(path_tracing.has_focus) && (!a.path_tracing.has_focus || feq(a.path_tracing.focus, b.path_tracing.focus, 3));
    return cam && F(step_mm) && I(srgb_encode) && labels && light && I(preintegrate) && I(skip_empty_space) && clip &&
           pt && I(smooth_sampling);
#undef F
#undef I
}

// ---------------------------------------------------------------- renderer
// The volume, transfer function, labels and light map of a renderer change
// only while no view shares them (and never through a view).
static vv_status check_unshared(const vv_renderer* r) {
    if (r->base) return fail(VV_ERR_STATE, "a view shares its base's volume, transfer function, labels and light map");
    if (r->views > 0) return fail(VV_ERR_STATE, "the renderer's volume has live views: destroy them first");
    return VV_OK;
}

static vv_status use_device(const vv_renderer* r) {
    CK(cudaSetDevice(r->ctx->device));
    return VV_OK;
}

static m3 w2i_m3(const vv_renderer* r) {
    const float* m = r->w2i;
    return {mk(m[0], m[1], m[2]), mk(m[4], m[5], m[6]), mk(m[8], m[9], m[10])};
}

extern "C" vv_status vv_renderer_create(vv_context* ctx, const vv_volume* volume, const vv_transfer_function* tf,
                                        vv_renderer** out) {
    vv_precision p = {VV_DENSITY_UNORM16, VV_SUMS_FP32, 0, VV_MAJORANTS_REFERENCE, VV_MASK_UNORM16};
    return vv_renderer_create_ex(ctx, volume, tf, &p, out);
}

extern "C" vv_status vv_renderer_create_ex(vv_context* ctx, const vv_volume* volume, const vv_transfer_function* tf,
                                           const vv_precision* precision, vv_renderer** out) {
    if (!ctx || !volume || !tf || !out || !precision) return fail(VV_ERR_ARG, "null argument");
    if (precision->density_format > VV_DENSITY_FP32) return fail(VV_ERR_ARG, "unknown density format");
    if (precision->sums > VV_SUMS_KAHAN) return fail(VV_ERR_ARG, "unknown running-sum mode");
    if (precision->majorants > VV_MAJORANTS_BOUND) return fail(VV_ERR_ARG, "unknown majorant mode");
    if (precision->mask_format > VV_MASK_BF16) return fail(VV_ERR_ARG, "unknown mask format");
    if ((precision->mask_format == VV_MASK_FP16 && precision->density_format != VV_DENSITY_FP16) ||
        (precision->mask_format == VV_MASK_BF16 && precision->density_format != VV_DENSITY_BF16))
        return fail(VV_ERR_ARG, "an FP16 / BF16 mask needs the density in the same format");
    if (!volume->hu) return fail(VV_ERR_ARG, "volume has no voxels");
    for (int i = 0; i < 3; i++)
        if (volume->dims[i] == 0) return fail(VV_ERR_ARG, "volume has a zero dimension");
    Vol v = make_vol((int)volume->dims[0], (int)volume->dims[1], (int)volume->dims[2]);
    if ((double)v.bx * v.by * v.bz * 512.0 > 2147483647.0 || volume->dims[0] > 16384 || volume->dims[1] > 16384 ||
        volume->dims[2] > 16384)
        return fail(VV_ERR_LIMIT, "volume exceeds 2^31 bricked voxels or 16384 per axis");
    CK(cudaSetDevice(ctx->device));
    v.dfmt = (int)precision->density_format;
    v.mfmt = precision->mask_format == VV_MASK_FP16 ? MF_FP16 : precision->mask_format == VV_MASK_BF16 ? MF_BF16
                                                                                                      : MF_UNORM16;
    vv_renderer* r = new vv_renderer();
    r->ctx = ctx;
    r->vol = v;
    r->sums = precision->sums;
    r->fp64_after = precision->fp64_after;
    r->majorants = precision->majorants;
    set_geometry(r, volume);
    r->tables_host = nullptr;
    cudaError_t e = cudaMallocHost((void**)&r->tables_host, sizeof(LabelTables));
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(e, "cudaMallocHost");
    }
    auto bail = [&](vv_status s) {
        vv_renderer_destroy(r);
        return s;
    };
    vv_status s = upload_tf(r, tf);
    if (s != VV_OK) return bail(s);
    long n = (long)volume->dims[0] * volume->dims[1] * volume->dims[2];
    long elems = vol_elems(v);
    DBuf hu;
    if ((e = hu.alloc(n * sizeof(int16_t))) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc"));
    if ((e = r->density.alloc(elems * density_bytes(v.dfmt))) != cudaSuccess ||
        (e = r->normals.alloc(elems * sizeof(uint32_t))) != cudaSuccess ||
        (e = r->majorant.alloc((size_t)v.bx * v.by * v.bz * sizeof(float))) != cudaSuccess ||
        (e = r->tables.alloc(sizeof(LabelTables))) != cudaSuccess ||
        (e = r->work.alloc(256)) != cudaSuccess || (e = r->exposure.alloc(sizeof(float))) != cudaSuccess) {
        hu.release();
        return bail(cuda_fail(e, "cudaMalloc"));
    }
    cudaStream_t st = ctx->stream;
    e = cudaMemcpyAsync(hu.p, volume->hu, n * sizeof(int16_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_density(hu.as<int16_t>(), r->density.p, v, st);
    if (e == cudaSuccess) e = launch_normals(r->density.p, r->normals.as<uint32_t>(), v, w2i_m3(r), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->exposure.p, 0, sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->work.p, 0, 256, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    hu.release();
    if (e != cudaSuccess) return bail(cuda_fail(e, "volume upload"));
    r->launches += 2;
    *out = r;
    return VV_OK;
}

// A renderer that reads `base`'s device volume (density, normals, labels,
// soft label grid), transfer function and light map instead of holding its
// own copies: the per-request state of several requests on one resident
// volume. Its label masks, majorants, label tables, images and passes are its
// own, so each view renders with its own frame parameters.
extern "C" vv_status vv_renderer_create_view(vv_context* ctx, vv_renderer* base, vv_renderer** out) {
    if (!ctx || !base || !out) return fail(VV_ERR_ARG, "null argument");
    vv_renderer* root = base->base ? base->base : base;
    if (ctx->device != root->ctx->device) return fail(VV_ERR_ARG, "a view must be on its volume's device");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(root->ctx->stream));  // the volume's uploads have finished
    vv_renderer* r = new vv_renderer();
    r->ctx = ctx;
    r->base = root;
    r->vol = root->vol;
    std::memcpy(r->spacing, root->spacing, sizeof(r->spacing));
    std::memcpy(r->w2i, root->w2i, sizeof(r->w2i));
    std::memcpy(r->i2w, root->i2w, sizeof(r->i2w));
    std::memcpy(r->dims, root->dims, sizeof(r->dims));
    std::memcpy(r->bounds_lo, root->bounds_lo, sizeof(r->bounds_lo));
    std::memcpy(r->bounds_hi, root->bounds_hi, sizeof(r->bounds_hi));
    std::memcpy(r->center, root->center, sizeof(r->center));
    r->min_spacing = root->min_spacing;
    r->max_spacing = root->max_spacing;
    r->diagonal = root->diagonal;
    std::memcpy(r->bucket, root->bucket, sizeof(r->bucket));
    r->majorants = root->majorants;
    std::memcpy(r->soft_dims, root->soft_dims, sizeof(r->soft_dims));
    std::memcpy(r->soft_push, root->soft_push, sizeof(r->soft_push));
    r->has_labels = root->has_labels;
    r->generation = root->generation;
    r->env_w = root->env_w;
    r->env_h = root->env_h;
    r->env_gm = root->env_gm;
    r->env_gr = root->env_gr;
    r->has_env = root->has_env;
    r->env_peak_u = root->env_peak_u;
    r->sums = root->sums;
    r->fp64_after = root->fp64_after;
    DBuf* shared[][2] = {{&r->density, &root->density}, {&r->normals, &root->normals}, {&r->labels, &root->labels},
                         {&r->soft, &root->soft}, {&r->lut, &root->lut}, {&r->bucket_dev, &root->bucket_dev},
                         {&r->preint, &root->preint}, {&r->env_rad, &root->env_rad},
                         {&r->env_table, &root->env_table}, {&r->env_diffuse, &root->env_diffuse},
                         {&r->env_guide, &root->env_guide}};
    for (auto& b : shared) b[0]->borrow(*b[1]);
    r->tables_host = nullptr;
    cudaError_t e = cudaMallocHost((void**)&r->tables_host, sizeof(LabelTables));
    if (e != cudaSuccess) {
        delete r;
        return cuda_fail(e, "cudaMallocHost");
    }
    root->views++;
    const long elems = vol_elems(r->vol);
    if ((e = r->majorant.alloc((size_t)r->vol.bx * r->vol.by * r->vol.bz * sizeof(float))) != cudaSuccess ||
        (e = r->tables.alloc(sizeof(LabelTables))) != cudaSuccess || (e = r->work.alloc(256)) != cudaSuccess ||
        (e = r->exposure.alloc(sizeof(float))) != cudaSuccess ||
        (r->has_labels && ((e = r->mask_a.alloc(elems * sizeof(uint32_t))) != cudaSuccess ||
                           (e = r->mask_b.alloc(elems * sizeof(uint32_t))) != cudaSuccess))) {
        vv_renderer_destroy(r);
        return cuda_fail(e, "cudaMalloc");
    }
    e = cudaMemsetAsync(r->exposure.p, 0, sizeof(float), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->work.p, 0, 256, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        vv_renderer_destroy(r);
        return cuda_fail(e, "view set-up");
    }
    *out = r;
    return VV_OK;
}

extern "C" vv_status vv_renderer_destroy(vv_renderer* r) {
    if (!r) return VV_OK;
    if (r->views > 0) return fail(VV_ERR_STATE, "the renderer's volume has live views: destroy them first");
    cudaSetDevice(r->ctx->device);
    if (r->base) r->base->views--;
    cudaStreamSynchronize(r->ctx->stream);
    for (auto& P : r->pass) {
        if (P.stream) cudaStreamSynchronize(P.stream);
        DBuf* pb[] = {&P.slots, &P.map, &P.queues, &P.counts, &P.accum, &P.albedo, &P.normal, &P.binq, &P.bins};
        for (DBuf* b : pb) b->release();
        if (P.shown) cudaEventDestroy(P.shown);
        if (P.stream) cudaStreamDestroy(P.stream);
    }
    if (r->prep_done) cudaEventDestroy(r->prep_done);
    DBuf* all[] = {&r->density, &r->normals, &r->mask_a, &r->mask_b, &r->labels, &r->majorant, &r->env_rad,
                   &r->env_table, &r->env_diffuse, &r->env_guide, &r->preint, &r->shadow_vol, &r->ao_vol, &r->lut,
                   &r->bucket_dev, &r->tables, &r->soft, &r->work, &r->exposure, &r->accum, &r->albedo,
                   &r->normal, &r->ping, &r->pong, &r->guide_nd, &r->guide_alb, &r->hdr, &r->out, &r->bloom[0], &r->bloom[1], &r->bloom[2],
                   &r->bloom[3], &r->comp[0], &r->comp[1], &r->comp[2], &r->wide[0], &r->wide[1],
                   &r->wide[2]};
    for (DBuf* b : all) b->release();
    free_tex_vol(r->shadow_tex);
    free_tex_vol(r->ao_tex);
    {
        auto& U = r->unet;
        for (int k = 0; k < 19; k++) {
            U.w[k].release();
            U.b[k].release();
        }
        DBuf* t[] = {&U.in, &U.head};
        for (DBuf* b : t) b->release();
        for (int l = 0; l < 5; l++) {
            U.ea[l].release();
            U.eb[l].release();
            U.pool[l].release();
        }
        for (int l = 0; l < 4; l++) {
            U.up[l].release();
            U.cat[l].release();
            U.da[l].release();
            U.db[l].release();
        }
    }
    if (r->tables_host) cudaFreeHost(r->tables_host);
    if (r->counters) cudaFree(r->counters);
    delete r;
    return VV_OK;
}

extern "C" vv_status vv_renderer_get_info(const vv_renderer* r, vv_renderer_info* out) {
    if (!r || !out) return fail(VV_ERR_ARG, "null argument");
    for (int i = 0; i < 3; i++) {
        out->bounds_lo[i] = r->bounds_lo[i];
        out->bounds_hi[i] = r->bounds_hi[i];
        out->center[i] = r->center[i];
    }
    out->min_spacing = r->min_spacing;
    out->diagonal = r->diagonal;
    out->dims[0] = r->vol.nx; out->dims[1] = r->vol.ny; out->dims[2] = r->vol.nz;
    return VV_OK;
}

extern "C" vv_status vv_default_camera(const vv_renderer* r, vv_orbit_camera* out) {
    if (!r || !out) return fail(VV_ERR_ARG, "null argument");
    vv_orbit_camera_framing(r->center, r->diagonal, out);
    return VV_OK;
}

extern "C" vv_status vv_set_transfer_function(vv_renderer* r, const vv_transfer_function* tf) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    if (check_unshared(r) != VV_OK) return VV_ERR_STATE;
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    CK(cudaStreamSynchronize(r->ctx->stream));
    s = upload_tf(r, tf);
    if (s != VV_OK) return s;
    r->generation++;
    return VV_OK;
}

extern "C" vv_status vv_set_labels(vv_renderer* r, const uint8_t* labels, size_t n, const vv_soft_label_grid* soft) {
    if (!r || !labels) return fail(VV_ERR_ARG, "null argument");
    size_t voxels = (size_t)r->vol.nx * r->vol.ny * r->vol.nz;
    if (n != voxels)
        return fail(VV_ERR_ARG, "label volume has " + std::to_string(n) + " voxels, expected " + std::to_string(voxels));
    if (soft) {
        if (!soft->data) return fail(VV_ERR_ARG, "soft label grid has no data");
        for (int a = 0; a < 3; a++) {
            if (soft->dims[a] == 0) return fail(VV_ERR_ARG, "soft label grid has a zero dimension");
            if (soft->src_axis[a] > 2) return fail(VV_ERR_ARG, "soft label grid axis out of range");
        }
    }
    if (check_unshared(r) != VV_OK) return VV_ERR_STATE;
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    cudaStream_t st = r->ctx->stream;
    CK(cudaStreamSynchronize(st));
    long elems = vol_elems(r->vol);
    CK(r->labels.alloc(elems));
    CK(r->mask_a.alloc(elems * sizeof(uint32_t)));
    CK(r->mask_b.alloc(elems * sizeof(uint32_t)));
    DBuf lin;
    CK(lin.alloc(voxels));
    cudaError_t e = cudaMemcpyAsync(lin.p, labels, voxels, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_brick_u8(lin.as<uint8_t>(), r->labels.as<uint8_t>(), r->vol, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    lin.release();
    if (e != cudaSuccess) return cuda_fail(e, "label upload");
    r->launches += 1;
    if (soft) {
        size_t nodes = (size_t)soft->dims[0] * soft->dims[1] * soft->dims[2];
        CK(r->soft.alloc(nodes * 4));
        CK(cudaMemcpyAsync(r->soft.p, soft->data, nodes * 4, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        for (int a = 0; a < 3; a++) r->soft_dims[a] = (int)soft->dims[a];
        int flips = 0;
        for (int a = 0; a < 3; a++) flips |= (soft->flip[a] ? 1 : 0) << a;
        r->soft_push[0] = (int)soft->src_axis[0];
        r->soft_push[1] = (int)soft->src_axis[1];
        r->soft_push[2] = (int)soft->src_axis[2];
        r->soft_push[3] = flips | 8;
    } else {
        r->soft.release();
        r->soft_dims[0] = r->soft_dims[1] = r->soft_dims[2] = 1;
        r->soft_push[0] = r->soft_push[1] = r->soft_push[2] = r->soft_push[3] = 0;
    }
    r->has_labels = true;
    r->generation++;
    return VV_OK;
}

// EnvironmentMap::prepare (environment.rs:57-130) without the diffuse
// convolution (only the ray marcher reads it), and the upload of
// renderer.rs:2224-2290: radiance normalised to a mean luminance of 1 over the
// sphere, min(60000), to RGBA16F; the importance-sampling table as RG32F,
// (w + 1) x h: per row the conditional CDF and each texel's probability, in
// the last column the marginal CDF and the row's probability. Sums in f64 in
// the Rust's order, per-texel arithmetic in f32 (this file is compiled
// without floating-point contraction, as Rust compiles).
static float env_lum(const float* c) { return 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2]; }

// environment.rs:133-175: the normalised radiance box-filtered to at most
// 128 x 64, convolved with a clamped cosine lobe into 32 x 16 texels, as RGBA16F.
static void light_map_diffuse(int w, int h, const std::vector<float>& rad, std::vector<uint16_t>& out) {
    const float PI_F = 3.14159265358979323846f;
    auto direction = [&](float uu, float vv, float d[3]) {
        float phi = (uu - 0.5f) * 2.0f * PI_F, theta = vv * PI_F;
        d[0] = std::sin(theta) * std::sin(phi);
        d[1] = std::cos(theta);
        d[2] = std::sin(theta) * std::cos(phi);
    };
    auto half_bits = [](float v) {
        _Float16 hv = (_Float16)v;
        uint16_t b;
        std::memcpy(&b, &hv, 2);
        return b;
    };
    int sw = std::min(128, w), sh = std::max(sw / 2, 1);
    std::vector<float> small(6 * (size_t)sw * sh);
    for (int i = 0; i < sw * sh; i++) {
        int sx = i % sw, sy = i / sw;
        int x0 = sx * w / sw, x1 = std::max((sx + 1) * w / sw, sx * w / sw + 1);
        int y0 = sy * h / sh, y1 = std::max((sy + 1) * h / sh, sy * h / sh + 1);
        float c[3] = {0.0f, 0.0f, 0.0f};
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++)
                for (int k = 0; k < 3; k++) c[k] = c[k] + rad[4 * ((size_t)y * w + x) + k];
        float n = (float)((y1 - y0) * (x1 - x0));
        float uu = ((float)sx + 0.5f) / (float)sw, vv = ((float)sy + 0.5f) / (float)sh;
        float solid = (2.0f * PI_F / (float)sw) * (PI_F / (float)sh) * std::sin(PI_F * vv);
        float* e = small.data() + 6 * (size_t)i;
        for (int k = 0; k < 3; k++) e[k] = c[k] / n * solid;
        direction(uu, vv, e + 3);
    }
    const int dw = 32, dh = 16;
    out.assign(4 * dw * dh, 0);
    for (int i = 0; i < dw * dh; i++) {
        float nrm[3];
        direction(((float)(i % dw) + 0.5f) / (float)dw, ((float)(i / dw) + 0.5f) / (float)dh, nrm);
        float c[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < sw * sh; j++) {
            const float* e = small.data() + 6 * (size_t)j;
            float cs = nrm[0] * e[3] + nrm[1] * e[4] + nrm[2] * e[5];
            if (cs > 0.0f)
                for (int k = 0; k < 3; k++) c[k] = c[k] + e[k] * cs;
        }
        for (int k = 0; k < 3; k++) out[4 * i + k] = half_bits(std::min(c[k] / PI_F, 60000.0f));
        out[4 * i + 3] = half_bits(1.0f);
    }
}

static float prepare_light_map(int w, int h, const float* px, std::vector<uint16_t>& rad, std::vector<float>& table,
                               std::vector<uint16_t>& diffuse) {
    const float PI_F = 3.14159265358979323846f;
    auto sin_theta = [&](int y) { return std::sin(PI_F * ((float)y + 0.5f) / (float)h); };
    double sum[3] = {0.0, 0.0, 0.0}, weight = 0.0;
    for (int y = 0; y < h; y++) {
        float st = sin_theta(y);
        double row[3] = {0.0, 0.0, 0.0};
        for (int x = 0; x < w; x++)
            for (int c = 0; c < 3; c++) row[c] = row[c] + (double)px[3 * ((size_t)y * w + x) + c];
        for (int c = 0; c < 3; c++) sum[c] = sum[c] + row[c] * (double)st;
        weight = weight + (double)st * (double)w;
    }
    float mean_rgb[3] = {(float)(sum[0] / weight), (float)(sum[1] / weight), (float)(sum[2] / weight)};
    float mean = std::max(env_lum(mean_rgb), 1e-6f);
    size_t n = (size_t)w * h;
    rad.resize(4 * n);
    auto half_bits = [](float v) {
        _Float16 hv = (_Float16)v;
        uint16_t b;
        std::memcpy(&b, &hv, 2);
        return b;
    };
    std::vector<float> rad_f(4 * n);
    for (size_t i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) {
            rad_f[4 * i + c] = px[3 * i + c] / mean;
            rad[4 * i + c] = half_bits(std::min(rad_f[4 * i + c], 60000.0f));
        }
        rad_f[4 * i + 3] = 1.0f;
        rad[4 * i + 3] = half_bits(1.0f);
    }
    light_map_diffuse(w, h, rad_f, diffuse);
    std::vector<float> f(n);
    for (size_t i = 0; i < n; i++) f[i] = env_lum(px + 3 * i) * sin_theta((int)(i / (size_t)w));
    std::vector<double> row_sums(h);
    double total = 0.0;
    for (int y = 0; y < h; y++) {
        double a = 0.0;
        for (int x = 0; x < w; x++) a = a + (double)f[(size_t)y * w + x];
        row_sums[y] = a;
    }
    for (int y = 0; y < h; y++) total = total + row_sums[y];
    total = std::max(total, 1e-12);
    table.assign(2 * (size_t)(w + 1) * h, 0.0f);
    double marginal = 0.0;
    for (int y = 0; y < h; y++) {
        float* row = table.data() + 2 * (size_t)y * (w + 1);
        double acc = 0.0;
        for (int x = 0; x < w; x++) {
            double fx = (double)f[(size_t)y * w + x];
            acc = acc + fx;
            row[2 * x] = row_sums[y] > 0.0 ? (float)(acc / row_sums[y]) : (float)(x + 1) / (float)w;
            row[2 * x + 1] = (float)(fx / total);
        }
        row[2 * (w - 1)] = 1.0f;
        marginal = marginal + row_sums[y];
        row[2 * w] = (float)(marginal / total);
        row[2 * w + 1] = (float)(row_sums[y] / total);
    }
    table[2 * ((size_t)(h - 1) * (w + 1) + w)] = 1.0f;
    double pxs = 0.0, pzs = 0.0;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            double l = (double)f[(size_t)y * w + x];
            float uu = ((float)x + 0.5f) / (float)w, vv = ((float)y + 0.5f) / (float)h;
            float phi = (uu - 0.5f) * 2.0f * PI_F, theta = vv * PI_F;
            pxs = pxs + l * l * (double)(std::sin(theta) * std::sin(phi));
            pzs = pzs + l * l * (double)(std::sin(theta) * std::cos(phi));
        }
    return 0.5f + (float)(std::atan2(pxs, pzs) / (2.0 * 3.14159265358979323846));
}

// Guides for the inverse-CDF searches of the sampling table (Chen and Asau's
// guide table): bucket k of g covers u in [k / g, (k + 1) / g), and the first
// index whose CDF reaches u lies between the first indices for k / g and
// (k + 1) / g, so a search within them returns what the search over the whole
// CDF returns, with the same comparisons in f32. g is a power of two, so k / g
// and the device's bucket floor(u * g) are exact.
static void guide_of(const float* cdf, size_t stride, int n, int g, uint16_t* out) {
    int i = 0;
    for (int k = 0; k <= g; k++) {
        float u = (float)k / (float)g;
        while (i < n - 1 && !(cdf[stride * (size_t)i] >= u)) i++;
        out[k] = (uint16_t)i;
    }
}
static void search_guides(int w, int h, const std::vector<float>& table, int& gm, int& gr,
                          std::vector<uint16_t>& guide) {
    gm = 1;
    while (gm < h && gm < 16384) gm *= 2;  // about one row per bucket
    gr = 1;
    while (gr < (w + 3) / 4 && gr < 4096) gr *= 2;  // about four columns per bucket
    guide.assign((size_t)(gm + 1) + (size_t)h * (gr + 1), 0);
    const size_t row = 2 * (size_t)(w + 1);
    guide_of(table.data() + 2 * (size_t)w, row, h, gm, guide.data());
    for (int y = 0; y < h; y++)
        guide_of(table.data() + row * y, 2, w, gr, guide.data() + (gm + 1) + (size_t)y * (gr + 1));
}

extern "C" vv_status vv_set_environment_map(vv_renderer* r, const vv_environment_map* map) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    if (check_unshared(r) != VV_OK) return VV_ERR_STATE;
    vv_status st = use_device(r);
    if (st != VV_OK) return st;
    CK(cudaStreamSynchronize(r->ctx->stream));  // the reference waits for the device to go idle
    if (!map) {
        r->env_rad.release();
        r->env_table.release();
        r->env_diffuse.release();
        r->env_guide.release();
        r->has_env = false;
        r->env_w = r->env_h = r->env_gm = r->env_gr = 0;
        r->env_peak_u = 0.0f;
        r->have_params = false;
        return VV_OK;
    }
    if (!map->rgb) return fail(VV_ERR_ARG, "null light map pixels");
    if (map->width == 0 || map->height == 0) return fail(VV_ERR_ARG, "empty light map");
    if (map->width > 16384 || map->height > 16384) return fail(VV_ERR_LIMIT, "light map above 16384 texels per axis");
    int w = (int)map->width, h = (int)map->height;
    std::vector<uint16_t> rad, diffuse;
    std::vector<float> table;
    float peak = prepare_light_map(w, h, map->rgb, rad, table, diffuse);
    int gm = 1, gr = 1;
    std::vector<uint16_t> guide;
    search_guides(w, h, table, gm, gr, guide);
    CK(r->env_guide.alloc(guide.size() * sizeof(uint16_t)));
    CK(cudaMemcpy(r->env_guide.p, guide.data(), guide.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    CK(r->env_rad.alloc(rad.size() * sizeof(uint16_t)));
    CK(r->env_table.alloc(table.size() * sizeof(float)));
    CK(r->env_diffuse.alloc(diffuse.size() * sizeof(uint16_t)));
    CK(cudaMemcpy(r->env_diffuse.p, diffuse.data(), diffuse.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(r->env_rad.p, rad.data(), rad.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(r->env_table.p, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice));
    r->env_w = w;
    r->env_h = h;
    r->env_gm = gm;
    r->env_gr = gr;
    r->env_peak_u = peak;
    r->has_env = true;
    r->have_params = false;  // accumulated_params = None
    return VV_OK;
}

extern "C" vv_status vv_resize(vv_renderer* r, uint32_t width, uint32_t height) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(VV_ERR_ARG, "image size must be 1..16384 per axis");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    CK(cudaStreamSynchronize(r->ctx->stream));  // the context stream follows every pass's display
    size_t px = (size_t)width * height;
    for (int k = 0; k < VV_PASSES; k++) {
        vv_renderer::Pass& P = r->pass[k];
        if (!P.stream) {
            CK(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&P.shown, cudaEventDisableTiming));
        }
        CK(P.counts.alloc(WF_COUNTERS * sizeof(uint32_t)));
        if (k >= r->passes) {  // passes beyond the budget hold no sums
            P.accum.release();
            P.albedo.release();
            P.normal.release();
            continue;
        }
        CK(P.accum.alloc(px * 16));
        CK(P.albedo.alloc(px * 16));
        CK(P.normal.alloc(px * 16));
    }
    if (!r->prep_done) CK(cudaEventCreateWithFlags(&r->prep_done, cudaEventDisableTiming));
    CK(r->accum.alloc(px * 16));
    CK(r->albedo.alloc(px * 16));
    CK(r->normal.alloc(px * 16));
    for (int k = 0; k < 3; k++) {
        if (r->sums == VV_SUMS_KAHAN) CK(r->comp[k].alloc(px * 16));
        if (r->fp64_after) CK(r->wide[k].alloc(px * 32));
    }
    CK(r->ping.alloc(px * 16));
    CK(r->pong.alloc(px * 16));
    CK(r->guide_nd.alloc(px * 16));
    CK(r->guide_alb.alloc(px * 16));
    CK(r->hdr.alloc(px * 8));
    CK(r->out.alloc(px * 4));
    uint32_t qw = (width + 3) / 4, qh = (height + 3) / 4;
    uint32_t ew = (qw + 1) / 2, eh = (qh + 1) / 2;
    uint32_t ws[4] = {qw, qw, ew, ew}, hs[4] = {qh, qh, eh, eh};
    for (int i = 0; i < 4; i++) {
        CK(r->bloom[i].alloc((size_t)ws[i] * hs[i] * 8));
        r->bw[i] = (int)ws[i];
        r->bh[i] = (int)hs[i];
    }
    r->width = width;
    r->height = height;
    r->have_params = false;
    return VV_OK;
}

extern "C" uint32_t vv_accumulated_samples(const vv_renderer* r) { return r ? r->accumulated : 0; }
extern "C" uint64_t vv_kernel_launches(const vv_renderer* r) { return r ? r->launches : 0; }

extern "C" vv_status vv_query(vv_renderer* r, int* idle) {
    if (!r || !idle) return fail(VV_ERR_ARG, "null argument");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    // The context stream waits for every pass's display, so it is idle when
    // all of the renderer's work is.
    cudaError_t e = cudaStreamQuery(r->ctx->stream);
    if (e == cudaErrorNotReady) {
        *idle = 0;
        return VV_OK;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamQuery");
    *idle = 1;
    return VV_OK;
}

extern "C" vv_status vv_renderer_memory(const vv_renderer* r, uint64_t* bytes) {
    if (!r || !bytes) return fail(VV_ERR_ARG, "null argument");
    const DBuf* all[] = {&r->density, &r->normals, &r->mask_a, &r->mask_b, &r->labels, &r->majorant, &r->lut,
                         &r->bucket_dev, &r->tables, &r->soft, &r->work, &r->exposure, &r->accum, &r->albedo,
                         &r->normal, &r->ping, &r->pong, &r->guide_nd, &r->guide_alb, &r->hdr, &r->out,
                         &r->bloom[0], &r->bloom[1], &r->bloom[2], &r->bloom[3], &r->preint, &r->shadow_vol,
                         &r->ao_vol, &r->env_rad, &r->env_table, &r->env_diffuse, &r->env_guide, &r->comp[0],
                         &r->comp[1], &r->comp[2], &r->wide[0], &r->wide[1], &r->wide[2]};
    uint64_t n = 0;
    for (const DBuf* b : all) n += b->owned_bytes();  // a view's shared volumes count for its base
    for (const auto& P : r->pass) {
        const DBuf* pb[] = {&P.slots, &P.map, &P.queues, &P.counts, &P.accum, &P.albedo, &P.normal, &P.binq, &P.bins};
        for (const DBuf* b : pb) n += b->n;
    }
    if (r->shadow_tex.arr) n += (uint64_t)(r->shadow_dims[0] + 2) * (r->shadow_dims[1] + 2) * (r->shadow_dims[2] + 2) * 8;
    if (r->ao_tex.arr) n += (uint64_t)(r->ao_dims[0] + 2) * (r->ao_dims[1] + 2) * (r->ao_dims[2] + 2) * 2;
    *bytes = n;
    return VV_OK;
}

extern "C" vv_status vv_reset_view(vv_renderer* r) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    // Exposure 0 = not yet metered (the state of a new renderer's texel).
    CK(cudaMemsetAsync(r->exposure.p, 0, sizeof(float), r->ctx->stream));
    r->prep_work = true;     // the next pass starts after it
    r->have_params = false;  // the next record restarts the accumulation
    return VV_OK;
}

extern "C" vv_status vv_set_pass_budget(vv_renderer* r, uint32_t passes, uint32_t slot_frames) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    if (passes < 1 || passes > VV_PASSES || slot_frames < 1 || slot_frames > 16)
        return fail(VV_ERR_ARG, "passes must be 1..6 and slot_frames 1..16");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    CK(cudaStreamSynchronize(r->ctx->stream));
    for (auto& P : r->pass)
        if (P.stream) CK(cudaStreamSynchronize(P.stream));
    for (int k = (int)passes; k < VV_PASSES; k++) {
        vv_renderer::Pass& P = r->pass[k];
        DBuf* pb[] = {&P.slots, &P.map, &P.queues, &P.accum, &P.albedo, &P.normal, &P.binq, &P.bins};
        for (DBuf* b : pb) b->release();
    }
    if ((int)slot_frames < r->slot_frames)  // smaller slots: the next pass allocates anew
        for (auto& P : r->pass) {
            P.slots.release();
            P.map.release();
            P.queues.release();
            P.binq.release();
        }
    r->passes = (int)passes;
    r->slot_frames = (int)slot_frames;
    r->next_pass = 0;
    const size_t px = (size_t)r->width * r->height;
    for (int k = 0; k < r->passes && px > 0; k++) {  // sums of passes now in use, at the image's size
        vv_renderer::Pass& P = r->pass[k];
        CK(P.accum.alloc(px * 16));
        CK(P.albedo.alloc(px * 16));
        CK(P.normal.alloc(px * 16));
    }
    return VV_OK;
}

extern "C" vv_status vv_synchronize(vv_renderer* r) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    CK(cudaStreamSynchronize(r->ctx->stream));
    int32_t status = 0;
    CK(cudaMemcpy(&status, r->work.as<uint8_t>() + 4, 4, cudaMemcpyDeviceToHost));
    if (status != 0) return fail(VV_ERR_TIMEOUT, "a device-side bounded wait ran out");
    return VV_OK;
}

// The accumulated count `record` would use for `p` (0 after a reset).
static uint32_t accumulated_for(const vv_renderer* r, const vv_frame_params& p) {
    if (!r->have_params || !same_accumulation(r->accumulated_params, p)) return 0;
    return r->accumulated;
}

static PtArgs pt_args(vv_renderer* r, const UHead& u) {
    PtArgs a;
    std::memset(&a, 0, sizeof(a));
    a.u = u;
    a.density = r->density.p;
    a.mask = r->mask_a.as<uint32_t>();
    a.normals = r->normals.as<uint32_t>();
    a.labels = r->labels.as<uint8_t>();
    a.majorant = r->majorant.as<float>();
    a.env_rad = r->env_rad.as<ushort4>();
    a.env_diffuse = r->env_diffuse.as<ushort4>();
    a.preint = r->preint.as<float4>();
    a.env_table = r->env_table.as<float2>();
    a.env_guide = r->env_guide.as<uint16_t>();
    a.env_w = r->env_w;
    a.env_h = r->env_h;
    a.env_gm = r->env_gm;
    a.env_gr = r->env_gr;
    a.lut = r->lut.as<float4>();
    a.tab = r->tables.as<LabelTables>();
    a.vol = r->vol;
    a.accum = r->accum.as<float4>();
    a.albedo = r->albedo.as<float4>();
    a.normal = r->normal.as<float4>();
    a.hdr = r->hdr.as<ushort4>();
    a.width = r->width;
    a.height = r->height;
    a.frames = 1;
    a.tiles_x = (r->width + 7) / 8;
    a.tiles_y = (r->height + 3) / 4;
    a.counter = r->work.as<uint32_t>();
    a.status = r->work.as<int32_t>() + 1;
    a.counters = r->counters;
    a.write_hdr = 1;
    const char* k = std::getenv("VV_PT_KERNEL");
    a.persistent = !(k && std::strcmp(k, "frame") == 0);
    return a;
}

// The wavefront state of pass `P` for `cap` paths in flight on stream `s`:
// its records, queues, counters and later-flight bins over volume `v`
// (allocated when the pass needs more than it has).
static cudaError_t wf_state(vv_renderer::Pass& P, size_t cap, const Vol& v, cudaStream_t s, WfArgs& w) {
    if (P.slots.n < cap * WF_SLOT_BYTES) {
        cudaError_t ce = cudaStreamSynchronize(s);  // the pass's previous use of its state has ended
        if (ce == cudaSuccess) ce = P.slots.alloc(cap * WF_SLOT_BYTES);
        if (ce == cudaSuccess) ce = P.map.alloc(cap * WF_MAP_BYTES);
        if (ce == cudaSuccess) ce = P.queues.alloc(cap * 10 * sizeof(uint32_t));
        if (ce != cudaSuccess) return ce;
    }
    cap = P.slots.n / WF_SLOT_BYTES;
    w = WfArgs();
    w.capacity = (uint32_t)cap;
    // The records of vv_wavefront.cu, each an array over the slots.
    float4* rec = P.slots.as<float4>();
    w.path = rec;
    w.acc = rec + 4 * cap;
    w.vtx = rec + 8 * cap;
    w.shd = rec + 12 * cap;
    w.sh = rec + 16 * cap;
    w.mapdir = P.map.as<float4>();
    uint32_t* q = P.queues.as<uint32_t>();
    w.ext[0] = q;
    w.ext[1] = q + cap;
    w.shade = q + 2 * cap;
    w.shadow = q + 3 * cap;
    w.scatter = q + 4 * cap;
    w.esc[0] = q + 5 * cap;
    w.esc[1] = q + 6 * cap;
    w.first[0] = q + 7 * cap;
    w.first[1] = q + 8 * cap;
    w.map = q + 9 * cap;
    w.counts = P.counts.as<uint32_t>();
    // Later flights binned by the 32-voxel cell of their origin (coarser cells
    // while there would be more than 2^16 bins) and the octant of their
    // direction, so that a warp's lanes fly through the same region in the
    // same direction (measured on the head/neck workload: 379.4 -> 392.4 M path
    // samples/s; 16- and 64-voxel cells 386.0 and 390.3, no octant 388.0).
    {
        int shift = 5, cx, cy, cz;
        for (;; shift++) {
            cx = (v.nx + (1 << shift) - 1) >> shift;
            cy = (v.ny + (1 << shift) - 1) >> shift;
            cz = (v.nz + (1 << shift) - 1) >> shift;
            if ((size_t)cx * cy * cz * 8 <= 65536) break;
        }
        const uint32_t nbins = (uint32_t)(cx * cy * cz * 8);
        cudaError_t ce = cudaSuccess;
        if (P.binq.n < cap * 3 * sizeof(uint32_t)) {
            ce = cudaStreamSynchronize(s);  // the pass's previous use of its state has ended
            if (ce == cudaSuccess) ce = P.binq.alloc(cap * 3 * sizeof(uint32_t));
        }
        if (ce == cudaSuccess && P.bins.n < (size_t)nbins * 2 * sizeof(uint32_t)) {
            ce = cudaStreamSynchronize(s);
            if (ce == cudaSuccess) ce = P.bins.alloc((size_t)nbins * 2 * sizeof(uint32_t));
            P.nbins = 0;
        }
        // The counts start at zero and every wave's scan leaves them at zero,
        // but only for the layout of the volume they were last used with: the
        // insertion points follow the counts, so a pass over another volume
        // (a batch engine's passes change volumes) zeroes the buffer first.
        if (ce == cudaSuccess && P.nbins != nbins) {
            ce = cudaMemsetAsync(P.bins.p, 0, P.bins.n, s);
            P.nbins = nbins;
        }
        if (ce != cudaSuccess) return ce;
        uint32_t* bq = P.binq.as<uint32_t>();
        w.ext_key[0] = bq;
        w.ext_key[1] = bq + cap;
        w.sorted = bq + 2 * cap;
        w.bin_count = P.bins.as<uint32_t>();
        w.bin_next = w.bin_count + nbins;
        w.nbins = nbins;
        w.cell_shift = shift;
        w.cells_x = cx;
        w.cells_y = cy;
        w.cells_z = cz;
        // Queues of fewer than 16384 later flights go unordered (the late
        // waves, whose chains of launches the ordering lengthened): 392.7 ->
        // 394.2 M path samples/s, one vv_record per frame 7.08 -> 6.90 ms
        // (65536: 393.0 and 7.07; 262144: 392.2 and 7.03).
        const char* e = std::getenv("VV_WF_BIN_MIN");
        w.bin_min = e ? (uint32_t)std::max(0, std::atoi(e)) : 16384u;
    }
    return cudaSuccess;
}

// The path-tracing launches of one pass on stream `s`: the wavefront tracer,
// or with VV_PT_KERNEL=persistent / frame the single-kernel tracers
// (persistent warps with path regeneration / one thread per pixel, the
// reference's shape).
static cudaError_t run_pt(vv_renderer* r, vv_renderer::Pass& P, PtArgs& a, cudaStream_t s, int* launches) {
    const char* k = std::getenv("VV_PT_KERNEL");
    if (k && (std::strcmp(k, "persistent") == 0 || std::strcmp(k, "frame") == 0)) {
        a.persistent = std::strcmp(k, "persistent") == 0 || a.frames > 1;
        return kernels_of(r).pt(a, r->ctx->sms, s, launches);
    }
    // A wavefront slot counts its pixel's samples in 20 bits; 2^20 or more
    // samples per frame run on the persistent single-kernel tracer.
    if (a.u.path[2] >= WF_MAX_SAMPLES) {
        a.persistent = 1;
        return kernels_of(r).pt(a, r->ctx->sms, s, launches);
    }
    // Paths in flight: with several frames per pass, up to 16 frames' worth
    // (VV_WF_SLOTS overrides), at most 2^24 slots (4.6 GB of path state) unless
    // one frame needs more. Every frame of a 16-frame pass then runs in the
    // same waves: fewer, fuller waves and no refills (measured at 1024^2:
    // 171 M path samples/s with one frame's worth, 217 with 4, 238 with 16).
    size_t px = (size_t)r->width * r->height;
    const char* e = std::getenv("VV_WF_SLOTS");
    size_t per_pixel = e ? (size_t)std::max(1, std::atoi(e)) : (size_t)r->slot_frames;
    size_t cap = std::min(px * std::min<size_t>(per_pixel, a.frames), std::max(px, (size_t)1 << 24));
    WfArgs w;
    cudaError_t ce = wf_state(P, cap, r->vol, s, w);
    if (ce != cudaSuccess) return ce;
    return kernels_of(r).pt_wavefront(a, w, r->ctx->sms, s, launches);
}

static PostArgs post_args(vv_renderer* r, const UHead& u) {
    PostArgs a;
    std::memset(&a, 0, sizeof(a));
    a.u = u;
    a.width = r->width;
    a.height = r->height;
    a.accum = r->accum.as<float4>();
    a.albedo = r->albedo.as<float4>();
    a.normal = r->normal.as<float4>();
    a.ping = r->ping.as<float4>();
    a.pong = r->pong.as<float4>();
    a.guide_nd = r->guide_nd.as<float4>();
    a.guide_alb = r->guide_alb.as<float4>();
    a.hdr = r->hdr.as<ushort4>();
    for (int i = 0; i < 4; i++) {
        a.bloom[i] = r->bloom[i].as<ushort4>();
        a.bw[i] = r->bw[i];
        a.bh[i] = r->bh[i];
    }
    a.exposure = r->exposure.as<float>();
    a.out = r->out.as<uchar4>();
    return a;
}

// Uniform upload, masks and majorants when their inputs changed
// (renderer.rs:1554-1706); returns the packed head.
static vv_status prepare_frame(vv_renderer* r, const vv_frame_params& p, uint64_t frame, UHead& u) {
    if (!r->accum.p) return fail(VV_ERR_STATE, "resize() must be called before record()");
    if (p.labels.mode < 0 || p.labels.mode > 3) return fail(VV_ERR_ARG, "label mode out of range");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    cudaStream_t st = r->ctx->stream;
    if (p.path_tracing.enabled && (!r->have_params || !same_accumulation(r->accumulated_params, p))) {
        r->accumulated = 0;
        r->accumulated_params = p;
        r->have_params = true;
    }
    LabelTables* t = new LabelTables();
    pack(r, p, r->accumulated, frame, u, *t);
    // The tables go to the device through pinned staging, only when they
    // changed; the previous copy must have finished before the staging buffer
    // is overwritten.
    if (!r->tables_valid || std::memcmp(t, r->tables_host, sizeof(LabelTables)) != 0) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) {
            std::memcpy(r->tables_host, t, sizeof(LabelTables));
            e = cudaMemcpyAsync(r->tables.p, r->tables_host, sizeof(LabelTables), cudaMemcpyHostToDevice, st);
        }
        if (e != cudaSuccess) {
            delete t;
            return cuda_fail(e, "label table upload");
        }
        r->tables_valid = true;
        r->prep_work = true;
    }
    delete t;
    OpacityKey key = opacity_key(r, p.labels);
    if (key.mode != VV_LABEL_OFF && !(r->have_mask_key && r->mask_key == key)) {
        MaskLaunch L;
        L.v = r->vol;
        L.density = r->density.p;
        L.labels = r->labels.as<uint8_t>();
        static const uint8_t* none = nullptr;
        L.soft = r->soft.p ? r->soft.as<uint8_t>() : none;
        for (int a = 0; a < 3; a++) L.soft_dims[a] = r->soft_dims[a];
        for (int a = 0; a < 4; a++) L.soft_push[a] = r->soft.p ? r->soft_push[a] : 0;
        L.margin = key.margin;
        L.radius = (int)key.smoothing;
        L.mode = key.mode;
        L.colors = r->tables.as<LabelTables>()->colors;
        L.scratch = r->mask_b.as<uint32_t>();
        L.out = r->mask_a.as<uint32_t>();
        CK(launch_masks(L, st));
        r->prep_work = true;
        r->launches += 4;
        r->mask_key = key;
        r->have_mask_key = true;
    }
    if (!(r->have_majorant_key && r->majorant_key == key)) {
        r->prep_work = true;
        CK(launch_majorant(r->density.p, r->mask_a.as<uint32_t>(), r->vol, key.mode, p.labels.extinction,
                           r->bucket_dev.as<float>(), r->majorant.as<float>(), st));
        r->launches += 1;
        r->majorant_key = key;
        r->have_majorant_key = true;
    }
    if (p.path_tracing.enabled && r->accumulated == 0) {
        size_t bytes = (size_t)r->width * r->height * 16;
        CK(cudaMemsetAsync(r->accum.p, 0, bytes, st));
        CK(cudaMemsetAsync(r->albedo.p, 0, bytes, st));
        CK(cudaMemsetAsync(r->normal.p, 0, bytes, st));
        for (int k = 0; k < 3; k++)
            if (r->comp[k].p) CK(cudaMemsetAsync(r->comp[k].p, 0, bytes, st));
        r->wide_active = false;
        r->prep_work = true;
    }
    return VV_OK;
}

// Denoiser and display passes after the frame(s) (renderer.rs:1793-1803).
// The ray marcher's frame (renderer.rs:1707-1790): the occlusion volume when
// the opacity or the clipping changed, the shadow volume when the light or the
// tint changed as well, then dvr.comp into the HDR image and the display.
static void append_key(std::vector<uint8_t>& k, const void* p, size_t n) {
    const uint8_t* b = (const uint8_t*)p;
    k.insert(k.end(), b, b + n);
}
static cudaError_t make_tex_vol(vv_renderer::TexVol& t, int w, int h, int d, bool rgba) {
    cudaChannelFormatDesc f = rgba ? cudaCreateChannelDescHalf4() : cudaCreateChannelDescHalf();
    cudaError_t e = cudaMalloc3DArray(&t.arr, &f, make_cudaExtent(w + 2, h + 2, d + 2), cudaArraySurfaceLoadStore);
    if (e != cudaSuccess) return e;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = t.arr;
    if ((e = cudaCreateSurfaceObject(&t.surf, &rd)) != cudaSuccess) return e;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    for (int k = 0; k < 3; k++) td.addressMode[k] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    return cudaCreateTextureObject(&t.tex, &rd, &td, nullptr);
}

static vv_status record_ray_march(vv_renderer* r, const vv_frame_params& p, const UHead& u) {
    cudaStream_t st = r->ctx->stream;
    const int dims[3] = {(int)r->vol.nx, (int)r->vol.ny, (int)r->vol.nz};
    if (!r->shadow_vol.p) {
        for (int a = 0; a < 3; a++) {
            r->shadow_dims[a] = (dims[a] + 1) / 2;  // SHADOW_DOWNSAMPLE (renderer.rs:35)
            r->ao_dims[a] = (dims[a] + 3) / 4;      // AO_DOWNSAMPLE (renderer.rs:39)
        }
        CK(r->shadow_vol.alloc((size_t)r->shadow_dims[0] * r->shadow_dims[1] * r->shadow_dims[2] * 8));
        CK(r->ao_vol.alloc((size_t)r->ao_dims[0] * r->ao_dims[1] * r->ao_dims[2] * 2));
        CK(cudaMemsetAsync(r->shadow_vol.p, 0, r->shadow_vol.n, st));
        CK(cudaMemsetAsync(r->ao_vol.p, 0, r->ao_vol.n, st));
        CK(make_tex_vol(r->shadow_tex, r->shadow_dims[0], r->shadow_dims[1], r->shadow_dims[2], true));
        CK(make_tex_vol(r->ao_tex, r->ao_dims[0], r->ao_dims[1], r->ao_dims[2], false));
        CK(kernels_of(r).pad_lighting(r->shadow_vol.as<uint16_t>(), 4, r->shadow_dims[0], r->shadow_dims[1],
                               r->shadow_dims[2], r->shadow_tex.surf, st));
        CK(kernels_of(r).pad_lighting(r->ao_vol.as<uint16_t>(), 1, r->ao_dims[0], r->ao_dims[1], r->ao_dims[2],
                               r->ao_tex.surf, st));
        r->launches += 2;
    }
    PtArgs a = pt_args(r, u);
    int launches = 0;
    OpacityKey opacity = opacity_key(r, p.labels);
    std::vector<uint8_t> ao_key;  // (opacity, clip key: renderer.rs:1663-1667)
    append_key(ao_key, &opacity, sizeof(opacity));
    append_key(ao_key, u.clip, 2 * sizeof(uint32_t));
    append_key(ao_key, u.clip_planes, 12 * sizeof(float));
    if (p.lighting.ambient_occlusion && r->ao_key != ao_key) {
        CK(kernels_of(r).ao(a, r->ao_vol.as<uint16_t>(), r->ao_dims[0], r->ao_dims[1], r->ao_dims[2], st));
        CK(kernels_of(r).pad_lighting(r->ao_vol.as<uint16_t>(), 1, r->ao_dims[0], r->ao_dims[1], r->ao_dims[2],
                               r->ao_tex.surf, st));
        launches += 2;
        r->ao_key = ao_key;
    }
    std::vector<uint8_t> shadow_key = ao_key;  // + light direction bits and the tint (renderer.rs:1730-1748)
    append_key(shadow_key, u.light_dir, 3 * sizeof(float));
    append_key(shadow_key, p.labels.colors, sizeof(p.labels.colors));
    append_key(shadow_key, &p.lighting.scattering_distance, sizeof(float));
    if (p.lighting.shadows && r->shadow_key != shadow_key) {
        // record_shadow_sweep (renderer.rs:1907-1928): sweep away from the light
        // along its dominant axis in shadow-volume units.
        const float* m = u.w2i;
        float ld[3] = {u.light_dir[0], u.light_dir[1], u.light_dir[2]};
        float l_idx[3];
        for (int k = 0; k < 3; k++) {
            float v = m[k] * ld[0];
            v = m[4 + k] * ld[1] + v;
            v = m[8 + k] * ld[2] + v;
            l_idx[k] = v * ((float)r->shadow_dims[k] / r->dims[k]);
        }
        float ax = std::fabs(l_idx[0]), ay = std::fabs(l_idx[1]), az = std::fabs(l_idx[2]);
        int axis = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
        int sign = l_idx[axis] >= 0.0f ? 1 : -1;
        CK(kernels_of(r).shadow_sweep(a, r->shadow_vol.as<ushort4>(), r->shadow_dims[0], r->shadow_dims[1],
                               r->shadow_dims[2], axis, sign, st, &launches));
        CK(kernels_of(r).pad_lighting(r->shadow_vol.as<uint16_t>(), 4, r->shadow_dims[0], r->shadow_dims[1],
                               r->shadow_dims[2], r->shadow_tex.surf, st));
        launches += 1;
        r->shadow_key = shadow_key;
    }
    LightTex sv{r->shadow_tex.tex, r->shadow_dims[0], r->shadow_dims[1], r->shadow_dims[2], 1};
    LightTex av{r->ao_tex.tex, r->ao_dims[0], r->ao_dims[1], r->ao_dims[2], 0};
    CK(kernels_of(r).dvr(a, sv, av, st));
    launches += 1;
    PostArgs pa = post_args(r, u);
    CK(launch_post(pa, st, &launches));
    r->launches += launches;
    return VV_OK;
}

// ------------------------------------------------------ learned denoiser
// The U-Net of volview_gb300/learned_denoiser.py: levels of 32..96 channels,
// two 3x3 convolutions (ReLU) per level, average pooling down, nearest
// upsampling and concatenated skips up, a 16-channel head. Its 19
// convolutions in order: e0a e0b e1a e1b e2a e2b e3a e3b e4a e4b, d3a d3b
// d2a d2b d1a d1b d0a d0b, head.
static const int UNET_LEVELS[5] = {32, 48, 64, 80, 96};
static void unet_conv_shape(int k, int& cin, int& cout) {
    if (k < 10) {  // encoder: level k / 2
        int l = k / 2;
        cout = UNET_LEVELS[l];
        cin = (k % 2) ? cout : (l == 0 ? 16 : UNET_LEVELS[l - 1]);
    } else if (k < 18) {  // decoder: level 3 - (k - 10) / 2
        int l = 3 - (k - 10) / 2;
        cout = UNET_LEVELS[l];
        cin = ((k - 10) % 2) ? cout : UNET_LEVELS[l + 1] + UNET_LEVELS[l];
    } else {
        cin = UNET_LEVELS[0];
        cout = 16;
    }
}

extern "C" vv_status vv_set_denoiser_weights(vv_renderer* r, const float* params, size_t count) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    vv_status st = use_device(r);
    if (st != VV_OK) return st;
    CK(cudaStreamSynchronize(r->ctx->stream));  // no display may be using the weights
    if (!params) {
        r->unet.loaded = false;
        return VV_OK;
    }
    size_t expect = 0;
    for (int k = 0; k < 19; k++) {
        int cin, cout;
        unet_conv_shape(k, cin, cout);
        expect += (size_t)cout * 9 * cin + cout;
    }
    if (count != expect)
        return fail(VV_ERR_ARG, "denoiser weights: " + std::to_string(count) + " floats, expected " + std::to_string(expect));
    const float* p = params;
    std::vector<uint16_t> w16;
    for (int k = 0; k < 19; k++) {
        int cin, cout;
        unet_conv_shape(k, cin, cout);
        size_t nw = (size_t)cout * 9 * cin;
        w16.resize(nw);
        for (size_t i = 0; i < nw; i++) {
            _Float16 v = (_Float16)p[i];
            std::memcpy(&w16[i], &v, 2);
        }
        CK(r->unet.w[k].alloc(nw * 2));
        CK(r->unet.b[k].alloc((size_t)cout * 4));
        CK(cudaMemcpy(r->unet.w[k].p, w16.data(), nw * 2, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(r->unet.b[k].p, p + nw, (size_t)cout * 4, cudaMemcpyHostToDevice));
        p += nw + cout;
    }
    r->unet.loaded = true;
    return VV_OK;
}

// The network on the accumulation (n paths per pixel) into the HDR image, on
// stream s, over the image padded to multiples of 256 pixels per axis.
static vv_status run_unet(vv_renderer* r, float n, cudaStream_t s, int* launches) {
    auto& U = r->unet;
    const int W = (int)r->width, H = (int)r->height;
    const int wp = (W + 255) / 256 * 256, hp = (H + 255) / 256 * 256;
    if (U.wp != wp || U.hp != hp) {
        CK(cudaStreamSynchronize(s));  // the buffers' previous use has ended
        CK(U.in.alloc((size_t)wp * hp * 16 * 2));
        CK(U.head.alloc((size_t)wp * hp * 16 * 2));
        for (int l = 0; l < 5; l++) {
            size_t px = (size_t)(wp >> l) * (hp >> l);
            CK(U.ea[l].alloc(px * UNET_LEVELS[l] * 2));
            CK(U.eb[l].alloc(px * UNET_LEVELS[l] * 2));
            if (l) CK(U.pool[l].alloc(px * UNET_LEVELS[l - 1] * 2));
            if (l < 4) {
                CK(U.cat[l].alloc(px * (UNET_LEVELS[l + 1] + UNET_LEVELS[l]) * 2));
                CK(U.da[l].alloc(px * UNET_LEVELS[l] * 2));
                CK(U.db[l].alloc(px * UNET_LEVELS[l] * 2));
            }
        }
        U.wp = wp;
        U.hp = hp;
    }
    void* st = (void*)s;
    auto ok = [](vv_status v, const char* what) { return v == VV_OK ? VV_OK : fail(v, std::string("denoiser: ") + what); };
    auto conv = [&](const DBuf& x, int l, int k, DBuf& y, int relu) {
        int cin, cout;
        unet_conv_shape(k, cin, cout);
        *launches += 1;
        return ok(vv_nn_conv3x3(x.p, 1, hp >> l, wp >> l, cin, U.w[k].p, U.b[k].as<float>(), cout, relu, y.p, st),
                  "convolution");
    };
    vv_status v = ok(vv_nn_features_image(r->accum.as<float>(), r->albedo.as<float>(), r->normal.as<float>(), n, W, H,
                                          wp, hp, U.in.p, st), "features");
    *launches += 1;
    const DBuf* x = &U.in;
    for (int l = 0; l < 5 && v == VV_OK; l++) {
        if (l) {
            v = ok(vv_nn_avgpool2(U.eb[l - 1].p, 1, hp >> (l - 1), wp >> (l - 1), UNET_LEVELS[l - 1], U.pool[l].p, 0,
                                  st), "pooling");
            *launches += 1;
            x = &U.pool[l];
        }
        if (v == VV_OK) v = conv(*x, l, 2 * l, U.ea[l], 1);
        if (v == VV_OK) v = conv(U.ea[l], l, 2 * l + 1, U.eb[l], 1);
    }
    const DBuf* y = &U.eb[4];
    int cy = UNET_LEVELS[4];
    for (int l = 3; l >= 0 && v == VV_OK; l--) {
        // The level's channel counts are multiples of 8 and the buffers are
        // cudaMalloc'd: the upsampling and the concat in one pass.
        v = ok(vv_nn_upsample_concat(y->p, 1, hp >> (l + 1), wp >> (l + 1), cy, U.eb[l].p, UNET_LEVELS[l],
                                     U.cat[l].p, st),
               "upsampling and concat");
        *launches += 1;
        int k = 10 + 2 * (3 - l);
        if (v == VV_OK) v = conv(U.cat[l], l, k, U.da[l], 1);
        if (v == VV_OK) v = conv(U.da[l], l, k + 1, U.db[l], 1);
        y = &U.db[l];
        cy = UNET_LEVELS[l];
    }
    if (v == VV_OK) v = conv(*y, 0, 18, U.head, 0);
    if (v == VV_OK)
        v = ok(vv_nn_prediction_to_hdr(U.head.p, 16, wp, W, H, r->accum.as<float>(), n, r->hdr.p, st), "HDR store");
    *launches += 1;
    return v;
}

// One path-tracing pass of `frames` accumulate-frames and its display
// (record, renderer.rs:1770-1797). The pass runs on its own stream into its own
// sums, starting after this call's set-up work (if it queued any) and after
// the previous use of its stream; then, after the previous call's display, its
// sums are merged into the accumulation, the HDR image is stored, denoised and
// displayed, and the context stream waits for that display. So a call returns
// at once, and consecutive calls overlap: one pass's last, nearly empty waves
// run beside the next pass's first ones.
static cudaError_t pass_args(vv_renderer* r, vv_renderer::Pass& P, const UHead& u, uint32_t frames, cudaStream_t s,
                             PtArgs& a);
static vv_status end_pass(vv_renderer* r, vv_renderer::Pass& P, vv_renderer::Pass& prev, const vv_frame_params& p,
                          UHead& u, uint32_t frames, bool display, cudaStream_t s, int launches);

// Every pass waits for the renderer's latest set-up on its context stream
// (masks, majorants, label tables, zeroed running sums): passes run on
// several streams, so the one right after the set-up is not the only one
// that may read what it writes.
static cudaError_t wait_for_set_up(vv_renderer* r, cudaStream_t s) {
    if (r->prep_work) {
        cudaError_t e = cudaEventRecord(r->prep_done, r->ctx->stream);
        if (e != cudaSuccess) return e;
        r->prep_work = false;
    }
    return cudaStreamWaitEvent(s, r->prep_done, 0);
}

static vv_status record_pass(vv_renderer* r, const vv_frame_params& p, UHead& u, uint32_t frames,
                             bool display = true) {
    vv_renderer::Pass& P = r->pass[r->next_pass % r->passes];
    vv_renderer::Pass& prev = r->pass[(r->next_pass + r->passes - 1) % r->passes];
    r->next_pass = (r->next_pass + 1) % r->passes;
    cudaStream_t s = P.stream;
    CK(wait_for_set_up(r, s));
    const char* single = std::getenv("VV_PT_KERNEL");
    if (single) CK(cudaStreamWaitEvent(s, prev.shown, 0));  // the single-kernel tracers share one work counter
    PtArgs a;
    CK(pass_args(r, P, u, frames, s, a));
    int launches = 0;
    pt_timer_start(r, s);
    CK(run_pt(r, P, a, s, &launches));
    pt_timer_stop(r, s);
    return end_pass(r, P, prev, p, u, frames, display, s, launches);
}

// A pass's arguments with its own sums (zeroed on stream `s` once their last
// use, possibly a batched pass on another stream, has ended).
static cudaError_t pass_args(vv_renderer* r, vv_renderer::Pass& P, const UHead& u, uint32_t frames, cudaStream_t s,
                             PtArgs& a) {
    cudaError_t e = cudaStreamWaitEvent(s, P.shown, 0);
    size_t bytes = (size_t)r->width * r->height * 16;
    if (e == cudaSuccess) e = cudaMemsetAsync(P.accum.p, 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(P.albedo.p, 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(P.normal.p, 0, bytes, s);
    a = pt_args(r, u);
    a.frames = frames;
    a.accum = P.accum.as<float4>();
    a.albedo = P.albedo.as<float4>();
    a.normal = P.normal.as<float4>();
    a.write_hdr = 0;
    return e;
}

// The end of a pass whose path tracing is queued on stream `s`: its sums (P)
// merged into the running sums after the previous pass's display (prev), the
// denoiser and the display, then P.shown, which the context stream waits for.
static vv_status end_pass(vv_renderer* r, vv_renderer::Pass& P, vv_renderer::Pass& prev, const vv_frame_params& p,
                          UHead& u, uint32_t frames, bool display, cudaStream_t s, int launches) {
    uint32_t spf = std::max(p.path_tracing.samples_per_frame, 1u);
    // The last frame's view of the counts: accumulated before it, spf after.
    r->accumulated += (frames - 1) * spf;
    u.path[0] = r->accumulated;
    PostArgs pa = post_args(r, u);
    CK(cudaStreamWaitEvent(s, prev.shown, 0));
    if (r->sums == VV_SUMS_FP32 && !r->fp64_after) {
        CK(launch_merge(pa, P.accum.as<float4>(), P.albedo.as<float4>(), P.normal.as<float4>(),
                        (float)(r->accumulated + spf), s));
    } else {
        // The running sums hold the samples before this pass's first frame;
        // past fp64_after of them they continue in FP64.
        uint32_t before = r->accumulated - (frames - 1) * spf;
        PreciseSums ps;
        for (int k = 0; k < 3; k++) {
            ps.comp[k] = r->comp[k].as<float4>();
            ps.wide[k] = r->wide[k].as<double>();
        }
        ps.kahan = r->sums == VV_SUMS_KAHAN;
        ps.wide_mode = 0;
        if (r->fp64_after && (r->wide_active || before >= r->fp64_after)) {
            ps.wide_mode = r->wide_active ? 2 : 1;
            r->wide_active = true;
        }
        CK(launch_merge_precise(pa, P.accum.as<float4>(), P.albedo.as<float4>(), P.normal.as<float4>(), ps,
                                (double)(r->accumulated + spf), s));
    }
    launches += 1;
    if (display && p.path_tracing.denoiser == VV_DENOISE_ATROUS) CK(launch_denoise(pa, s, &launches));
    if (display && p.path_tracing.denoiser == VV_DENOISE_LEARNED) {
        vv_status v = run_unet(r, (float)(r->accumulated + spf), s, &launches);
        if (v != VV_OK) return v;
    }
    r->accumulated += spf;
    if (display && p.path_tracing.denoiser != VV_DENOISE_OIDN) CK(launch_post(pa, s, &launches));
    CK(cudaEventRecord(P.shown, s));
    CK(cudaStreamWaitEvent(r->ctx->stream, P.shown, 0));
    r->launches += launches;
    return VV_OK;
}

static vv_status check_denoiser(const vv_renderer* r, const vv_frame_params* params) {
    if (params->path_tracing.enabled && params->path_tracing.denoiser == VV_DENOISE_LEARNED && !r->unet.loaded)
        return fail(VV_ERR_STATE, "the learned denoiser has no weights (vv_set_denoiser_weights)");
    return VV_OK;
}

extern "C" vv_status vv_record(vv_renderer* r, uint64_t frame, const vv_frame_params* params) {
    if (!r || !params) return fail(VV_ERR_ARG, "null argument");
    if (check_denoiser(r, params) != VV_OK) return VV_ERR_STATE;
    UHead u;
    vv_status s = prepare_frame(r, *params, frame, u);
    if (s != VV_OK) return s;
    if (!params->path_tracing.enabled) return record_ray_march(r, *params, u);
    return record_pass(r, *params, u, 1);
}

extern "C" vv_status vv_record_frames(vv_renderer* r, uint64_t first_frame, uint32_t frames,
                                      const vv_frame_params* params) {
    if (!r || !params) return fail(VV_ERR_ARG, "null argument");
    if (!params->path_tracing.enabled)
        return fail(VV_ERR_ARG, "vv_record_frames accumulates path-traced frames (path_tracing.enabled = 0)");
    if (frames == 0) return VV_OK;
    if (!r->accum.p) return fail(VV_ERR_STATE, "resize() must be called before record()");
    if (check_denoiser(r, params) != VV_OK) return VV_ERR_STATE;
    // Long calls run as passes of at most VV_SUBPASS_FRAMES frames on the pass
    // streams in turn, so that each pass's last waves overlap the next one's
    // first (one long pass refilling its slots ran at 327 M path samples/s
    // at 1024^2, 64-frame passes in turn at 339); only the last one displays.
    // A pass's work items, (frame, pixel) pairs, are counted in 32 bits on the
    // device with room for the counter's overshoot: at most 2^31 per pass.
    const uint64_t px = (uint64_t)r->width * r->height;
    const uint32_t per_pass = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(VV_SUBPASS_FRAMES, (1ull << 31) / px));
    uint32_t done = 0;
    while (done < frames) {
        uint32_t n = std::min<uint32_t>(frames - done, per_pass);
        UHead u;
        vv_status s = prepare_frame(r, *params, first_frame + done + n - 1, u);
        if (s != VV_OK) return s;
        s = record_pass(r, *params, u, n, done + n == frames);
        if (s != VV_OK) return s;
        done += n;
    }
    return VV_OK;
}

// ------------------------------------------------------------ batched passes
// A batch engine: passes in flight on streams of its own, each with the
// wavefront state (slots, queues, bins) that the requests of one batched
// pass share, and each request's item counter and constants.
struct vv_batch {
    vv_context* ctx;
    struct BatchPass {
        vv_renderer::Pass p;  // its sums stay empty: each request's go to its renderer's pass sums
        DBuf items, consts;
    } pass[VV_PASSES];
    int passes = 2;
    int next = 0;
    int slot_frames = 16;
    uint64_t launches = 0;
};

extern "C" vv_status vv_batch_create(vv_context* ctx, uint32_t passes, uint32_t slot_frames, vv_batch** out) {
    if (!ctx || !out) return fail(VV_ERR_ARG, "null argument");
    if (passes < 1 || passes > VV_PASSES || slot_frames < 1 || slot_frames > 16)
        return fail(VV_ERR_ARG, "passes must be 1..6 and slot_frames 1..16");
    CK(cudaSetDevice(ctx->device));
    vv_batch* b = new vv_batch();
    b->ctx = ctx;
    b->passes = (int)passes;
    b->slot_frames = (int)slot_frames;
    for (int k = 0; k < b->passes; k++) {
        auto& B = b->pass[k];
        cudaError_t e = cudaStreamCreateWithFlags(&B.p.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.p.shown, cudaEventDisableTiming);
        if (e == cudaSuccess) e = B.p.counts.alloc(WF_COUNTERS * sizeof(uint32_t));
        if (e == cudaSuccess) e = B.items.alloc(VV_BATCH_MAX * sizeof(uint32_t));
        if (e == cudaSuccess) e = B.consts.alloc(VV_BATCH_MAX * WF_CONSTS_BYTES);
        if (e != cudaSuccess) {
            vv_batch_destroy(b);
            return cuda_fail(e, "batch engine");
        }
    }
    *out = b;
    return VV_OK;
}

extern "C" vv_status vv_batch_destroy(vv_batch* b) {
    if (!b) return VV_OK;
    cudaSetDevice(b->ctx->device);
    for (auto& B : b->pass) {
        if (B.p.stream) cudaStreamSynchronize(B.p.stream);
        DBuf* pb[] = {&B.p.slots, &B.p.map, &B.p.queues, &B.p.counts, &B.p.binq, &B.p.bins, &B.items, &B.consts};
        for (DBuf* d : pb) d->release();
        if (B.p.shown) cudaEventDestroy(B.p.shown);
        if (B.p.stream) cudaStreamDestroy(B.p.stream);
    }
    delete b;
    return VV_OK;
}

extern "C" vv_status vv_batch_memory(const vv_batch* b, uint64_t* bytes) {
    if (!b || !bytes) return fail(VV_ERR_ARG, "null argument");
    uint64_t n = 0;
    for (const auto& B : b->pass) {
        const DBuf* pb[] = {&B.p.slots, &B.p.map, &B.p.queues, &B.p.counts, &B.p.binq, &B.p.bins, &B.items,
                            &B.consts};
        for (const DBuf* d : pb) n += d->n;
    }
    *bytes = n;
    return VV_OK;
}

extern "C" vv_status vv_batch_synchronize(vv_batch* b) {
    if (!b) return fail(VV_ERR_ARG, "null batch engine");
    CK(cudaSetDevice(b->ctx->device));
    for (auto& B : b->pass)
        if (B.p.stream) CK(cudaStreamSynchronize(B.p.stream));
    return VV_OK;
}

extern "C" uint64_t vv_batch_launches(const vv_batch* b) { return b ? b->launches : 0; }

extern "C" vv_status vv_batch_in_flight(vv_batch* b, uint32_t* passes) {
    if (!b || !passes) return fail(VV_ERR_ARG, "null argument");
    CK(cudaSetDevice(b->ctx->device));
    uint32_t n = 0;
    for (int k = 0; k < b->passes; k++) {
        cudaError_t e = cudaEventQuery(b->pass[k].p.shown);
        if (e == cudaErrorNotReady) n++;
        else if (e != cudaSuccess) return cuda_fail(e, "cudaEventQuery");
    }
    *passes = n;
    return VV_OK;
}

// One batched pass: request i adds requests[i].frames accumulate-frames to
// renderer i, exactly as vv_record_frames would for a call of that many
// frames (the same paths, random streams and sums), with the work items of
// every request in the same waves. The renderers (of any resident volumes)
// use the reference's storage formats. Each renderer's merge,
// denoiser and display follow on the engine's stream, and its context stream
// waits for them, so vv_query / vv_synchronize on the renderer see the pass.
extern "C" vv_status vv_batch_record(vv_batch* b, uint32_t n, vv_renderer* const* renderers,
                                     const vv_batch_request* requests) {
    if (!b || !renderers || !requests) return fail(VV_ERR_ARG, "null argument");
    if (n == 0) return VV_OK;
    if (n > (uint32_t)VV_BATCH_MAX) return fail(VV_ERR_LIMIT, "at most 8 requests per batched pass");
    // The bin grid of the later flights spans the largest volume of the batch
    // (each request's own volume, geometry and transfer function are in its
    // arguments; the grid only orders the flights).
    Vol grid = make_vol(1, 1, 1);
    for (uint32_t i = 0; i < n; i++) {
        vv_renderer* r = renderers[i];
        const vv_batch_request& q = requests[i];
        if (!r || !q.params) return fail(VV_ERR_ARG, "null renderer or frame parameters");
        for (uint32_t j = 0; j < i; j++)
            if (renderers[j] == r) return fail(VV_ERR_ARG, "a renderer appears twice in one batched pass");
        grid.nx = std::max(grid.nx, r->vol.nx);
        grid.ny = std::max(grid.ny, r->vol.ny);
        grid.nz = std::max(grid.nz, r->vol.nz);
        if (r->ctx->device != b->ctx->device) return fail(VV_ERR_ARG, "renderer and batch engine on different devices");
        if (build_of(r->vol) != 0)
            return fail(VV_ERR_ARG, "batched passes take the reference's storage (R16_UNORM density, RG16_UNORM mask)");
        if (!q.params->path_tracing.enabled) return fail(VV_ERR_ARG, "a batched pass path-traces (path_tracing.enabled = 0)");
        if (q.frames == 0 || q.frames > VV_SUBPASS_FRAMES) return fail(VV_ERR_ARG, "frames per request must be 1..64");
        if (!r->accum.p) return fail(VV_ERR_STATE, "resize() must be called before record()");
        if (check_denoiser(r, q.params) != VV_OK) return VV_ERR_STATE;
        const uint64_t px = (uint64_t)r->width * r->height;
        if (px >= (1ull << 28) || px * q.frames >= (1ull << 31))
            return fail(VV_ERR_LIMIT, "a batched request has fewer than 2^28 pixels and 2^31 work items");
        if (std::max(q.params->path_tracing.samples_per_frame, 1u) >= WF_MAX_SAMPLES)
            return fail(VV_ERR_LIMIT, "a batched request takes fewer than 2^20 samples per frame");
    }
    CK(cudaSetDevice(b->ctx->device));
    auto& E = b->pass[b->next % b->passes];
    b->next = (b->next + 1) % b->passes;
    cudaStream_t s = E.p.stream;
    PtBatch B;
    std::memset(&B, 0, sizeof(B));
    B.n = n;
    std::vector<UHead> heads(n);
    std::vector<vv_renderer::Pass*> own(n), prev(n);
    std::vector<size_t> cap(n);
    size_t total = 0, budget = (size_t)1 << 24;
    for (uint32_t i = 0; i < n; i++) {
        vv_renderer* r = renderers[i];
        const vv_batch_request& q = requests[i];
        vv_status st = prepare_frame(r, *q.params, q.first_frame + q.frames - 1, heads[i]);
        if (st != VV_OK) return st;
        own[i] = &r->pass[r->next_pass % r->passes];
        prev[i] = &r->pass[(r->next_pass + r->passes - 1) % r->passes];
        r->next_pass = (r->next_pass + 1) % r->passes;
        CK(wait_for_set_up(r, s));
        CK(pass_args(r, *own[i], heads[i], q.frames, s, B.a[i]));
        const size_t px = (size_t)r->width * r->height;
        const size_t items = px * q.frames;
        cap[i] = std::min(items, px * (size_t)std::min(b->slot_frames, r->slot_frames));
        total += cap[i];
        budget = std::max(budget, px);
    }
    // Paths in flight: each request's share of at most 2^24 slots (4.8 GB of
    // path state), and at least one frame's worth (or all its items).
    size_t end = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (total > budget) {
            const size_t px = (size_t)renderers[i]->width * renderers[i]->height;
            const size_t floor_i = std::min(px * requests[i].frames, px);
            cap[i] = std::max(floor_i, (size_t)((double)cap[i] * (double)budget / (double)total));
        }
        end += cap[i];
        B.slot_end[i] = (uint32_t)end;
    }
    WfArgs w;
    CK(wf_state(E.p, end, grid, s, w));
    w.items = E.items.as<uint32_t>();
    w.consts = E.consts.p;
    int launches = 0;
    CK(fmt0::launch_pt_wavefront_batch(B, w, b->ctx->sms, s, &launches));
    b->launches += launches;
    for (uint32_t i = 0; i < n; i++) {
        vv_status st = end_pass(renderers[i], *own[i], *prev[i], *requests[i].params, heads[i], requests[i].frames,
                                requests[i].display != 0, s, 0);
        if (st != VV_OK) return st;
    }
    CK(cudaEventRecord(E.p.shown, s));
    return VV_OK;
}

static vv_status read_dev(vv_renderer* r, void* dst, const DBuf& src, size_t bytes, size_t capacity) {
    if (!r || !dst) return fail(VV_ERR_ARG, "null argument");
    if (!src.p) return fail(VV_ERR_STATE, "resize() must be called first");
    if (capacity < bytes) return fail(VV_ERR_ARG, "output buffer too small");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    CK(cudaMemcpyAsync(dst, src.p, bytes, cudaMemcpyDeviceToHost, r->ctx->stream));
    CK(cudaStreamSynchronize(r->ctx->stream));
    return VV_OK;
}

extern "C" vv_status vv_read_output(vv_renderer* r, uint8_t* rgba, size_t capacity) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    return read_dev(r, rgba, r->out, (size_t)r->width * r->height * 4, capacity);
}

extern "C" vv_status vv_read_hdr(vv_renderer* r, uint16_t* rgba, size_t capacity) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    return read_dev(r, rgba, r->hdr, (size_t)r->width * r->height * 8, capacity * 2);
}

extern "C" vv_status vv_read_accumulation(vv_renderer* r, float* accum, float* albedo, float* normal,
                                          size_t capacity_floats) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    size_t bytes = (size_t)r->width * r->height * 16;
    vv_status s;
    if (accum && (s = read_dev(r, accum, r->accum, bytes, capacity_floats * 4)) != VV_OK) return s;
    if (albedo && (s = read_dev(r, albedo, r->albedo, bytes, capacity_floats * 4)) != VV_OK) return s;
    if (normal && (s = read_dev(r, normal, r->normal, bytes, capacity_floats * 4)) != VV_OK) return s;
    return VV_OK;
}

extern "C" vv_status vv_render_to_rgba(vv_renderer* r, const vv_frame_params* params, uint32_t width,
                                       uint32_t height, uint32_t frames, uint8_t* out, size_t capacity) {
    if (!r || !params || !out) return fail(VV_ERR_ARG, "null argument");
    if (capacity < (size_t)width * height * 4) return fail(VV_ERR_ARG, "output buffer too small");
    vv_status s = vv_resize(r, width, height);
    if (s != VV_OK) return s;
    // offscreen.rs:30-51: with OIDN requested but unavailable, `frames` frames are
    // traced without display and one more with the a-trous filter.
    bool oidn = params->path_tracing.denoiser == VV_DENOISE_OIDN;
    uint32_t last = oidn ? frames + 1 : frames;
    for (uint32_t f = 1; f < last; f++)
        if ((s = vv_record(r, f, params)) != VV_OK) return s;
    vv_frame_params p = *params;
    if (oidn) p.path_tracing.denoiser = VV_DENOISE_ATROUS;
    if ((s = vv_record(r, frames, &p)) != VV_OK) return s;
    return vv_read_output(r, out, capacity);
}

extern "C" vv_status vv_pack_uniforms(vv_renderer* r, const vv_frame_params* params, uint64_t frame, void* out,
                                      size_t capacity) {
    if (!r || !params || !out) return fail(VV_ERR_ARG, "null argument");
    if (capacity < VV_UNIFORMS_BYTES) return fail(VV_ERR_ARG, "output buffer too small");
    if (!r->width) return fail(VV_ERR_STATE, "resize() must be called first");
    UHead u;
    LabelTables* t = new LabelTables();
    pack(r, *params, accumulated_for(r, *params), frame, u, *t);
    std::memcpy(out, &u, sizeof(u));
    std::memcpy((uint8_t*)out + sizeof(u), t, sizeof(*t));
    delete t;
    return VV_OK;
}

extern "C" vv_status vv_read_volume(vv_renderer* r, int which, void* out, size_t capacity) {
    if (!r || !out) return fail(VV_ERR_ARG, "null argument");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    cudaStream_t st = r->ctx->stream;
    size_t voxels = (size_t)r->vol.nx * r->vol.ny * r->vol.nz;
    if (which == VV_VOLUME_MAJORANT || which == VV_VOLUME_SHADOW || which == VV_VOLUME_AO) {
        const DBuf& b = which == VV_VOLUME_MAJORANT ? r->majorant : (which == VV_VOLUME_SHADOW ? r->shadow_vol : r->ao_vol);
        if (!b.p) return fail(VV_ERR_STATE, "that volume has not been computed");
        if (capacity < b.n) return fail(VV_ERR_ARG, "output buffer too small");
        CK(cudaMemcpyAsync(out, b.p, b.n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return VV_OK;
    }
    const DBuf* src = nullptr;
    int elem = 0;
    switch (which) {
        case VV_VOLUME_DENSITY: src = &r->density; elem = density_bytes(r->vol.dfmt); break;
        case VV_VOLUME_NORMALS: src = &r->normals; elem = 4; break;
        case VV_VOLUME_MASK: src = &r->mask_a; elem = 4; break;
        case VV_VOLUME_LABELS: src = &r->labels; elem = 1; break;
        default: return fail(VV_ERR_ARG, "unknown volume");
    }
    if (!src->p) return fail(VV_ERR_STATE, "that volume has not been computed");
    if (capacity < voxels * elem) return fail(VV_ERR_ARG, "output buffer too small");
    DBuf tmp;
    CK(tmp.alloc(voxels * elem));
    cudaError_t e = launch_unbrick(src->p, tmp.p, r->vol, elem, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp.p, voxels * elem, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    tmp.release();
    if (e != cudaSuccess) return cuda_fail(e, "volume readback");
    return VV_OK;
}

// ------------------------------------------------------------ event counts
// Counts the path tracer's memory events (COUNT_* in vv_kernels.h) over the
// next records until vv_count_events(r, 0, out) returns the totals.
extern "C" vv_status vv_count_events(vv_renderer* r, int enable, uint64_t* out, size_t n) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    if (enable) {
        if (!r->counters) CK(cudaMalloc((void**)&r->counters, COUNT_N * sizeof(unsigned long long)));
        CK(cudaMemsetAsync(r->counters, 0, COUNT_N * sizeof(unsigned long long), r->ctx->stream));
        return VV_OK;
    }
    if (!r->counters) return fail(VV_ERR_STATE, "counting was not enabled");
    unsigned long long c[COUNT_N];
    CK(cudaStreamSynchronize(r->ctx->stream));
    CK(cudaMemcpy(c, r->counters, sizeof(c), cudaMemcpyDeviceToHost));
    cudaFree(r->counters);
    r->counters = nullptr;
    for (size_t i = 0; i < n && i < (size_t)COUNT_N; i++) out[i] = c[i];
    return VV_OK;
}

// Device time of the path-tracing launches: enable = 1 starts recording CUDA
// events around each launch on the renderer's stream; enable = 0 stops, waits,
// and returns the summed milliseconds and the number of launches.
extern "C" vv_status vv_time_pt(vv_renderer* r, int enable, double* ms, uint64_t* launches) {
    if (!r) return fail(VV_ERR_ARG, "null renderer");
    vv_status s = use_device(r);
    if (s != VV_OK) return s;
    if (enable) {
        r->timing = true;
        return VV_OK;
    }
    r->timing = false;
    CK(cudaStreamSynchronize(r->ctx->stream));
    double total = 0.0;
    for (auto& ev : r->pt_events) {
        float t = 0.0f;
        cudaError_t e = cudaEventElapsedTime(&t, ev.first, ev.second);
        if (e == cudaSuccess) total += t;
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
    }
    if (ms) *ms = total;
    if (launches) *launches = r->pt_events.size();
    r->pt_events.clear();
    return VV_OK;
}

// ---------------------------------------------------------- parity probes
// Not part of the reference's interface: entry points the parity tests use to
// run single device functions on the renderer's current state.
extern "C" vv_status vv_probe_bspline(vv_renderer* r, const vv_frame_params* params, const float* idx, size_t n,
                                      float* out) {
    if (!r || !params || !idx || !out) return fail(VV_ERR_ARG, "null argument");
    UHead u;
    vv_status s = prepare_frame(r, *params, 1, u);
    if (s != VV_OK) return s;
    DBuf di, dout;
    CK(di.alloc(n * 12));
    CK(dout.alloc(n * 16));
    cudaStream_t st = r->ctx->stream;
    PtArgs a = pt_args(r, u);
    cudaError_t e = cudaMemcpyAsync(di.p, idx, n * 12, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = kernels_of(r).bspline_probe(a, di.as<float>(), dout.as<float>(), (int)n, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, n * 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    di.release();
    dout.release();
    if (e != cudaSuccess) return cuda_fail(e, "bspline probe");
    return VV_OK;
}

extern "C" vv_status vv_probe_extinction(vv_renderer* r, const vv_frame_params* params, const float* idx, size_t n,
                                         const float dir[3], int smooth, float* out) {
    if (!r || !params || !idx || !dir || !out) return fail(VV_ERR_ARG, "null argument");
    if (n == 0) return VV_OK;
    if (n > (size_t)INT32_MAX / 4) return fail(VV_ERR_LIMIT, "too many points for one probe");
    UHead u;
    vv_status s = prepare_frame(r, *params, 1, u);
    if (s != VV_OK) return s;
    DBuf di, dout;
    CK(di.alloc(n * 12));
    CK(dout.alloc(n * 16));
    cudaStream_t st = r->ctx->stream;
    PtArgs a = pt_args(r, u);
    cudaError_t e = cudaMemcpyAsync(di.p, idx, n * 12, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = kernels_of(r).extinction_probe(a, di.as<float>(), dout.as<float>(), (int)n, dir, smooth, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, n * 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    di.release();
    dout.release();
    if (e != cudaSuccess) return cuda_fail(e, "extinction probe");
    return VV_OK;
}

extern "C" vv_status vv_probe_light_samples(vv_renderer* r, const vv_frame_params* params, const uint32_t* seeds,
                                             size_t n, float* out) {
    if (!r || !params || !seeds || !out) return fail(VV_ERR_ARG, "null argument");
    if (!r->has_env) return fail(VV_ERR_STATE, "no light map");
    UHead u;
    vv_status s = prepare_frame(r, *params, 1, u);
    if (s != VV_OK) return s;
    DBuf ds, dout;
    CK(ds.alloc(n * 4));
    CK(dout.alloc(n * 24));
    cudaStream_t st = r->ctx->stream;
    PtArgs a = pt_args(r, u);
    cudaError_t e = cudaMemcpyAsync(ds.p, seeds, n * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = kernels_of(r).light_sample_probe(a, ds.as<uint32_t>(), dout.as<float>(), (int)n, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, n * 24, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ds.release();
    dout.release();
    if (e != cudaSuccess) return cuda_fail(e, "light sample probe");
    return VV_OK;
}

static decltype(&exact0::launch_pt_pixels) const EXACT_PT_PIXELS[6] = {
    exact0::launch_pt_pixels, exact1::launch_pt_pixels, exact2::launch_pt_pixels, exact3::launch_pt_pixels,
    exact4::launch_pt_pixels, exact5::launch_pt_pixels};

static vv_status probe_paths(vv_renderer* r, const vv_frame_params* params, uint32_t accumulated, const int* pixels,
                             size_t n, float* out, bool exact) {
    if (!r || !params || !pixels || !out) return fail(VV_ERR_ARG, "null argument");
    if (n == 0) return VV_OK;
    if (n > (size_t)INT32_MAX / 12) return fail(VV_ERR_LIMIT, "too many pixels for one probe");
    UHead u;
    vv_status s = prepare_frame(r, *params, 1, u);
    if (s != VV_OK) return s;
    u.path[0] = accumulated;
    DBuf dp, dout;
    CK(dp.alloc(n * 8));
    CK(dout.alloc(n * 48));
    cudaStream_t st = r->ctx->stream;
    PtArgs a = pt_args(r, u);
    cudaError_t e = cudaMemcpyAsync(dp.p, pixels, n * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = (exact ? EXACT_PT_PIXELS[build_of(r->vol)] : kernels_of(r).pt_pixels)(a, dp.as<int>(), dout.as<float>(),
                                                                               (int)n, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.p, n * 48, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dp.release();
    dout.release();
    if (e != cudaSuccess) return cuda_fail(e, "path probe");
    return VV_OK;
}

extern "C" vv_status vv_probe_paths(vv_renderer* r, const vv_frame_params* params, uint32_t accumulated,
                                    const int* pixels, size_t n, float* out) {
    return probe_paths(r, params, accumulated, pixels, n, out, false);
}

extern "C" vv_status vv_probe_paths_exact(vv_renderer* r, const vv_frame_params* params, uint32_t accumulated,
                                          const int* pixels, size_t n, float* out) {
    return probe_paths(r, params, accumulated, pixels, n, out, true);
}
