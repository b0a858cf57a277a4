"""Python mirror of volview's `render` crate API over libvolpt.so (include/volpt.h).

`Context`, `Renderer` and `render_to_rgba` follow crates/render/src/lib.rs:14-23:
Renderer(ctx, volume, tf) ~ Renderer::new (renderer.rs:555), set_transfer_function
(:1226), set_labels (:1241), set_environment_map (:1283), resize (:1313), record
(:1499), accumulated_samples (:1217), destroy (:2072), render_to_rgba
(offscreen.rs:11). Errors raise VolptError where the Rust returns Err; `record`
raises where the Rust panics (record before resize).

There is no CPU fallback: importing works anywhere, but every call needs the CUDA
library and a device, and fails loudly without them.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvolpt.so")
P = C.c_void_p

# Every entry point include/volpt.h declares: (name, restype, argtypes).
EXPORTS = [
    ("vv_last_error", C.c_char_p, []),
    ("vv_lighting_default", None, [P]),
    ("vv_label_params_default", None, [P]),
    ("vv_path_tracing_default", None, [P]),
    ("vv_clipping_default", None, [P]),
    ("vv_orbit_camera_framing", None, [P, C.c_float, P]),
    ("vv_context_create", C.c_int, [C.c_int, P]),
    ("vv_context_create_on_stream", C.c_int, [C.c_int, P, P]),
    ("vv_context_destroy", C.c_int, [P]),
    ("vv_renderer_create", C.c_int, [P, P, P, P]),
    ("vv_renderer_create_ex", C.c_int, [P, P, P, P, P]),
    ("vv_renderer_destroy", C.c_int, [P]),
    ("vv_renderer_create_view", C.c_int, [P, P, P]),
    ("vv_batch_create", C.c_int, [P, C.c_uint32, C.c_uint32, P]),
    ("vv_batch_destroy", C.c_int, [P]),
    ("vv_batch_record", C.c_int, [P, C.c_uint32, P, P]),
    ("vv_batch_memory", C.c_int, [P, P]),
    ("vv_batch_synchronize", C.c_int, [P]),
    ("vv_batch_launches", C.c_uint64, [P]),
    ("vv_batch_in_flight", C.c_int, [P, P]),
    ("vv_renderer_get_info", C.c_int, [P, P]),
    ("vv_default_camera", C.c_int, [P, P]),
    ("vv_set_transfer_function", C.c_int, [P, P]),
    ("vv_set_labels", C.c_int, [P, P, C.c_size_t, P]),
    ("vv_set_environment_map", C.c_int, [P, P]),
    ("vv_resize", C.c_int, [P, C.c_uint32, C.c_uint32]),
    ("vv_record", C.c_int, [P, C.c_uint64, P]),
    ("vv_record_frames", C.c_int, [P, C.c_uint64, C.c_uint32, P]),
    ("vv_accumulated_samples", C.c_uint32, [P]),
    ("vv_synchronize", C.c_int, [P]),
    ("vv_read_output", C.c_int, [P, P, C.c_size_t]),
    ("vv_read_hdr", C.c_int, [P, P, C.c_size_t]),
    ("vv_read_accumulation", C.c_int, [P, P, P, P, C.c_size_t]),
    ("vv_render_to_rgba", C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, C.c_size_t]),
    ("vv_pack_uniforms", C.c_int, [P, P, C.c_uint64, P, C.c_size_t]),
    ("vv_read_volume", C.c_int, [P, C.c_int, P, C.c_size_t]),
    ("vv_kernel_launches", C.c_uint64, [P]),
    ("vv_query", C.c_int, [P, P]),
    ("vv_renderer_memory", C.c_int, [P, P]),
    ("vv_reset_view", C.c_int, [P]),
    ("vv_set_pass_budget", C.c_int, [P, C.c_uint32, C.c_uint32]),
    ("vv_set_denoiser_weights", C.c_int, [P, P, C.c_size_t]),
    ("vv_denoise_atrous_noalloc", C.c_int, [P, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P]),
]
# Test hooks (include/volpt_probe.h).
PROBES = [
    ("vv_probe_bspline", C.c_int, [P, P, P, C.c_size_t, P]),
    ("vv_probe_paths", C.c_int, [P, P, C.c_uint32, P, C.c_size_t, P]),
    ("vv_probe_paths_exact", C.c_int, [P, P, C.c_uint32, P, C.c_size_t, P]),
    ("vv_probe_light_samples", C.c_int, [P, P, P, C.c_size_t, P]),
    ("vv_probe_extinction", C.c_int, [P, P, P, C.c_size_t, P, C.c_int, P]),
    ("vv_count_events", C.c_int, [P, C.c_int, P, C.c_size_t]),
    ("vv_time_pt", C.c_int, [P, C.c_int, P, P]),
]

# The learned denoiser's operators (include/volpt_nn.h).
I, L, F = C.c_int, C.c_long, C.c_float
NN = [
    ("vv_nn_conv3x3", I, [P, I, I, I, I, P, P, I, I, P, P]),
    ("vv_nn_flip_weights", I, [P, I, I, P, P]),
    ("vv_nn_conv3x3_wgrad", I, [P, P, I, I, I, I, I, P, P]),
    ("vv_nn_bias_grad", I, [P, L, I, P, P]),
    ("vv_nn_relu_backward", I, [P, P, L, P]),
    ("vv_nn_avgpool2", I, [P, I, I, I, I, P, I, P]),
    ("vv_nn_upsample2", I, [P, I, I, I, I, P, I, P]),
    ("vv_nn_concat", I, [P, I, P, I, L, P, P]),
    ("vv_nn_upsample_concat", I, [P, I, I, I, I, P, I, P, P]),
    ("vv_nn_split", I, [P, I, I, L, P, P, P]),
    ("vv_nn_features", I, [P, P, P, F, L, P, P]),
    ("vv_nn_l1_loss", I, [P, I, P, L, F, P, P, P]),
    ("vv_nn_adam", I, [P, P, P, P, P, L, F, F, F, F, F, I, P]),
    ("vv_nn_add", I, [P, P, L, P]),
    ("vv_nn_radiance", I, [P, I, L, P, P]),
    ("vv_nn_features_image", I, [P, P, P, F, I, I, I, I, P, P]),
    ("vv_nn_prediction_to_hdr", I, [P, I, I, I, I, P, F, P, P]),
    ("vv_nn_conv3x3_tc", I, [P, I, I, I, I, P, P, I, I, P, P]),
    ("vv_nn_tc_status", I, [P, I]),
]

COUNT_NAMES = ["majorant", "cubic", "trilinear", "mask", "label", "normal", "gradient", "pixel", "path", "vertex"]
# Unique element bytes each event must read (and write, for pixels).
COUNT_BYTES = [4, 128, 16, 32, 1, 32, 128, 104, 0, 0]

_lib = None


class VolptError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"volpt status {status}: {message}")
        self.status = status


def load():
    """Loads libvolpt.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build()
        lib = C.CDLL(LIB_PATH)
        for name, res, args in EXPORTS + PROBES + NN:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status):
    if status != abi.VV_OK:
        raise VolptError(status, load().vv_last_error().decode())


def _ref(x):
    return C.byref(x) if x is not None else None


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class Context:
    """CUDA device + stream (replaces the Vulkan Context, context.rs:37)."""

    def __init__(self, device=0, stream=None):
        self.handle = C.c_void_p()
        if stream is None:
            check(load().vv_context_create(device, C.byref(self.handle)))
        else:
            check(load().vv_context_create_on_stream(device, C.c_void_p(stream), C.byref(self.handle)))

    def destroy(self):
        if self.handle:
            load().vv_context_destroy(self.handle)
            self.handle = C.c_void_p()


class Renderer:
    def __init__(self, ctx, volume, tf, precision=None, view_of=None):
        """`precision` (abi.Precision) selects the density storage and running sums;
        None is the reference's (R16_UNORM, FP32 sums). With `view_of` (a
        Renderer) the renderer is a view of that renderer's volume
        (vv_renderer_create_view): `volume`, `tf` and `precision` are unused."""
        self.ctx = ctx
        self.handle = C.c_void_p()
        if view_of is not None:
            self.precision = view_of.precision
            check(load().vv_renderer_create_view(ctx.handle, view_of.handle, C.byref(self.handle)))
        else:
            self.precision = precision if precision is not None else abi.precision()
            check(load().vv_renderer_create_ex(ctx.handle, C.byref(volume), C.byref(tf), C.byref(self.precision),
                                               C.byref(self.handle)))
        info = abi.RendererInfo()
        check(load().vv_renderer_get_info(self.handle, C.byref(info)))
        self.info = info
        self.bounds = (tuple(info.bounds_lo), tuple(info.bounds_hi))
        self.min_spacing = info.min_spacing
        self.center = tuple(info.center)
        self.diagonal = info.diagonal
        self.dims = tuple(info.dims)
        self.width = self.height = 0

    def default_camera(self):
        cam = abi.OrbitCamera()
        check(load().vv_default_camera(self.handle, C.byref(cam)))
        return cam

    def set_transfer_function(self, tf):
        check(load().vv_set_transfer_function(self.handle, C.byref(tf)))

    def set_labels(self, labels, soft=None):
        labels = np.ascontiguousarray(labels, np.uint8)
        check(load().vv_set_labels(self.handle, _ptr(labels), labels.size, _ref(soft)))

    def set_environment_map(self, env):
        """`env`: an abi.EnvironmentMap (abi.env_struct), or None to remove the map."""
        check(load().vv_set_environment_map(self.handle, _ref(env)))

    def resize(self, width, height):
        check(load().vv_resize(self.handle, width, height))
        self.width, self.height = width, height

    def record(self, frame, params):
        check(load().vv_record(self.handle, frame, C.byref(params)))

    def record_frames(self, first_frame, frames, params):
        check(load().vv_record_frames(self.handle, first_frame, frames, C.byref(params)))

    def accumulated_samples(self):
        return load().vv_accumulated_samples(self.handle)

    def synchronize(self):
        check(load().vv_synchronize(self.handle))

    def idle(self):
        """True once every call made on this renderer has finished on the device (never blocks)."""
        v = C.c_int(0)
        check(load().vv_query(self.handle, C.byref(v)))
        return bool(v.value)

    def device_bytes(self):
        """Device memory this renderer holds now."""
        v = C.c_uint64(0)
        check(load().vv_renderer_memory(self.handle, C.byref(v)))
        return int(v.value)

    def set_denoiser_weights(self, params):
        """Loads the learned denoiser's weights (a flat float32 array, see
        learned_denoiser.UNet.weights_blob) for DENOISE_LEARNED; None unloads."""
        if params is None:
            check(load().vv_set_denoiser_weights(self.handle, None, 0))
            return
        blob = np.ascontiguousarray(params, np.float32).ravel()
        check(load().vv_set_denoiser_weights(self.handle, _ptr(blob), blob.size))

    def set_pass_budget(self, passes, slot_frames):
        """vv_set_pass_budget: passes in flight (1..6) and frames' worth of path
        slots per pass (1..16)."""
        check(load().vv_set_pass_budget(self.handle, passes, slot_frames))

    def reset_view(self):
        """A new view: the accumulation restarts and auto exposure meters afresh."""
        check(load().vv_reset_view(self.handle))

    def read_output(self, out=None):
        out = np.empty((self.height, self.width, 4), np.uint8) if out is None else out
        check(load().vv_read_output(self.handle, _ptr(out), out.nbytes))
        return out

    def read_hdr(self):
        out = np.empty((self.height, self.width, 4), np.uint16)
        check(load().vv_read_hdr(self.handle, _ptr(out), out.size))
        return out

    def read_accumulation(self, normal=True):
        """(radiance sums, albedo sums, normal sums or None) as (h, w, 4) float32."""
        shape = (self.height, self.width, 4)
        a, b = np.empty(shape, np.float32), np.empty(shape, np.float32)
        c = np.empty(shape, np.float32) if normal else None
        check(load().vv_read_accumulation(self.handle, _ptr(a), _ptr(b), _ptr(c) if normal else None, a.size))
        return a, b, c

    def pack_uniforms(self, params, frame=1):
        out = np.zeros(abi.VV_UNIFORMS_BYTES, np.uint8)
        check(load().vv_pack_uniforms(self.handle, C.byref(params), frame, _ptr(out), out.nbytes))
        return out

    def read_volume(self, which):
        nx, ny, nz = self.dims
        if which == abi.VOLUME_MAJORANT:
            shape, dt = ((nz + 7) // 8, (ny + 7) // 8, (nx + 7) // 8), np.float32
        elif which == abi.VOLUME_SHADOW:
            shape, dt = ((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2, 4), np.uint16
        elif which == abi.VOLUME_AO:
            shape, dt = ((nz + 3) // 4, (ny + 3) // 4, (nx + 3) // 4), np.uint16
        else:
            density_dt = np.float32 if self.precision.density_format == abi.DENSITY_FP32 else np.uint16
            shape, dt = {abi.VOLUME_DENSITY: ((nz, ny, nx), density_dt),
                         abi.VOLUME_NORMALS: ((nz, ny, nx, 4), np.int8),
                         abi.VOLUME_MASK: ((nz, ny, nx, 2), np.uint16),
                         abi.VOLUME_LABELS: ((nz, ny, nx), np.uint8)}[which]
        out = np.empty(shape, dt)
        check(load().vv_read_volume(self.handle, which, _ptr(out), out.nbytes))
        return out

    def kernel_launches(self):
        return load().vv_kernel_launches(self.handle)

    def probe_bspline(self, params, idx):
        idx = np.ascontiguousarray(idx, np.float32).reshape(-1, 3)
        out = np.zeros((idx.shape[0], 4), np.float32)
        check(load().vv_probe_bspline(self.handle, C.byref(params), _ptr(idx), idx.shape[0], _ptr(out)))
        return out

    def probe_light_samples(self, params, seeds):
        """(n, 6): texel column, row, pdf, direction xyz of light map samples from `seeds`."""
        seeds = np.ascontiguousarray(seeds, np.uint32).ravel()
        out = np.zeros((seeds.size, 6), np.float32)
        check(load().vv_probe_light_samples(self.handle, C.byref(params), _ptr(seeds), seeds.size, _ptr(out)))
        return out

    def probe_extinction(self, params, idx, direction=(0.0, 0.0, 1.0), smooth=True):
        """(n, 4): sampled extinction (rgb) at continuous indices idx and the
        flight majorant of the brick there (vv_probe_extinction)."""
        idx = np.ascontiguousarray(idx, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(direction, np.float32)
        out = np.zeros((idx.shape[0], 4), np.float32)
        check(load().vv_probe_extinction(self.handle, C.byref(params), _ptr(idx), idx.shape[0], _ptr(d), int(smooth),
                                         _ptr(out)))
        return out

    def probe_paths(self, params, accumulated, pixels, exact=False):
        """One path per listed (x, y) pixel at accumulation count `accumulated`
        (12 floats each); `exact` runs the parity build (vv_probe_paths_exact)."""
        pix = np.ascontiguousarray(pixels, np.int32).reshape(-1, 2)
        out = np.zeros((pix.shape[0], 12), np.float32)
        fn = load().vv_probe_paths_exact if exact else load().vv_probe_paths
        check(fn(self.handle, C.byref(params), accumulated, _ptr(pix), pix.shape[0], _ptr(out)))
        return out

    def time_pt(self, enable):
        """Starts (True) or stops (False -> (ms, launches)) timing the path-tracing launches."""
        ms, n = C.c_double(0.0), C.c_uint64(0)
        check(load().vv_time_pt(self.handle, int(enable), C.byref(ms), C.byref(n)))
        return None if enable else (ms.value, n.value)

    def count_events(self, enable):
        out = np.zeros(len(COUNT_NAMES), np.uint64)
        check(load().vv_count_events(self.handle, int(enable), _ptr(out), out.size))
        return None if enable else dict(zip(COUNT_NAMES, (int(v) for v in out)))

    @classmethod
    def view(cls, ctx, base):
        """A view of `base`'s resident volume on context `ctx`."""
        return cls(ctx, None, None, view_of=base)

    def destroy(self):
        if self.handle:
            check(load().vv_renderer_destroy(self.handle))
            self.handle = C.c_void_p()


class BatchEngine:
    """vv_batch: batched passes over several renderers of one volume."""

    def __init__(self, ctx, passes=2, slot_frames=16):
        self.ctx = ctx
        self.handle = C.c_void_p()
        check(load().vv_batch_create(ctx.handle, passes, slot_frames, C.byref(self.handle)))

    def record(self, items):
        """One batched pass over `items`: (renderer, params, first_frame,
        frames, display) tuples."""
        n = len(items)
        handles = (C.c_void_p * max(n, 1))(*[r.handle for r, *_ in items])
        reqs = (abi.BatchRequest * max(n, 1))()
        keep = []
        for k, (r, params, first, frames, display) in enumerate(items):
            keep.append(params)
            reqs[k].params = C.cast(C.pointer(params), C.c_void_p)
            reqs[k].first_frame = first
            reqs[k].frames = frames
            reqs[k].display = 1 if display else 0
        check(load().vv_batch_record(self.handle, n, handles, reqs))

    def device_bytes(self):
        n = C.c_uint64()
        check(load().vv_batch_memory(self.handle, C.byref(n)))
        return int(n.value)

    def synchronize(self):
        check(load().vv_batch_synchronize(self.handle))

    def kernel_launches(self):
        return int(load().vv_batch_launches(self.handle))

    def in_flight(self):
        n = C.c_uint32()
        check(load().vv_batch_in_flight(self.handle, C.byref(n)))
        return int(n.value)

    def destroy(self):
        if self.handle:
            check(load().vv_batch_destroy(self.handle))
            self.handle = C.c_void_p()


def render_to_rgba(renderer, params, width, height, frames):
    """offscreen.rs:11: resize, `frames` accumulate-frames, tone-mapped RGBA8."""
    out = np.empty((height, width, 4), np.uint8)
    check(load().vv_render_to_rgba(renderer.handle, C.byref(params), width, height, frames, _ptr(out), out.nbytes))
    renderer.width, renderer.height = width, height
    return out
