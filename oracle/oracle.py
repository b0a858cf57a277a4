"""Python driver of the CPU oracle (test infrastructure only).

Runs the reference's path on the CPU — density conversion, transfer-function
LUT, normals, masks, majorants, path-traced accumulate-frames, a-trous denoise —
from the restatement in liboracle.so, and (where it was built) from the
reference's own shaders compiled as CPU code (oracle/_ref, see build_ref.py).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
P = C.c_void_p


class Scene(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("density", P), ("normals", P), ("mask", P), ("labels", P),
                ("label_dims", C.c_int * 3), ("majorant", P), ("brick_dims", C.c_int * 3), ("tf_lut", P),
                ("preint", P), ("env_rad", P), ("env_table", P), ("env_dims", C.c_int * 2),
                ("density_format", C.c_int), ("mask_format", C.c_int)]


class Geometry(C.Structure):
    _fields_ = [("world_to_index", C.c_float * 16), ("index_to_world", C.c_float * 16), ("dims", C.c_float * 3),
                ("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3), ("min_spacing", C.c_float),
                ("max_spacing", C.c_float), ("center", C.c_float * 3), ("diagonal", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        from . import build_oracle
        path = build_oracle.build()
        _lib = C.CDLL(path)
        _lib.vvo_uniform_size.restype = C.c_long
        _lib.vvo_mask_margin.restype = C.c_int
        _lib.vvo_tf_evaluate.argtypes = [P, C.c_float, P]
        _lib.vvo_pack_uniforms.argtypes = [P, P, C.c_int, C.c_int, C.c_float, P, C.c_uint32, C.c_uint64,
                                           C.c_uint32, C.c_uint32, P]
        _lib.vvo_env_prepare.restype = C.c_float
        _lib.vvo_env_prepare.argtypes = [C.c_int, C.c_int, P, P, P, P]
    return _lib


_lib64 = None


def lib64():
    """The FP64 instance of the path tracer's restatement (oracle_api64.cpp)."""
    global _lib64
    if _lib64 is None:
        from . import build_oracle
        build_oracle.build()
        _lib64 = C.CDLL(build_oracle.LIB64)
        _lib64.vvo64_real_bytes.restype = C.c_long
        _lib64.vvo64_pt_pixel_sums.argtypes = [P, P, P, C.c_long, C.c_uint32, C.c_uint32, P, C.c_int]
        assert _lib64.vvo64_real_bytes() == 8
    return _lib64


def ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def tf_evaluate(tf, hu):
    out = np.zeros(4, np.float32)
    lib().vvo_tf_evaluate(C.byref(tf), hu, ptr(out))
    return out


def tf_lut(tf):
    out = np.zeros((4096, 4), np.float32)
    lib().vvo_tf_lut(C.byref(tf), ptr(out))
    return out


def tf_lut_half(tf):
    out = np.zeros((4096, 4), np.uint16)
    lib().vvo_tf_lut_half(C.byref(tf), ptr(out))
    return out


def tf_cumulative(tf):
    out = np.zeros((4096, 4), np.float32)
    lib().vvo_tf_cumulative(C.byref(tf), ptr(out))
    return out


def bucket_max(tf):
    out = np.zeros(64, np.float32)
    lib().vvo_bucket_max(C.byref(tf), ptr(out))
    return out


# vv_precision.majorants: the reference's bucket maxima (of the FP32 LUT), or
# true bounds of the FP16 LUT the tracer samples.
MAJORANTS_REFERENCE, MAJORANTS_BOUND = 0, 1


def bucket_bound(tf):
    """Bucket maxima of the FP16-rounded LUT (the values pt.comp samples), each
    multiplied by 1 + 2^-20 and rounded up to the next float32."""
    lut = tf_lut_half(tf).view(np.float16).astype(np.float32)
    out = np.zeros(64, np.float32)
    for k in range(64):
        m = np.float32(lut[64 * k:min(64 * k + 65, 4096), 3].max())
        if m > 0:
            m = np.nextafter(np.float32(m * np.float32(1.0 + 2.0 ** -20)), np.float32(np.inf), dtype=np.float32)
        out[k] = m
    return out


def hu_to_unorm16(hu):
    hu = np.ascontiguousarray(hu, np.int16)
    out = np.zeros(hu.shape, np.uint16)
    lib().vvo_hu_to_unorm16(ptr(hu), C.c_long(hu.size), ptr(out))
    return out


# Density storage formats of the precision variant (vv_precision.density_format).
DENSITY_UNORM16, DENSITY_FP16, DENSITY_BF16, DENSITY_FP32 = 0, 1, 2, 3
# Label-mask storage formats (vv_precision.mask_format): RG16_UNORM, or two
# binary16 / bfloat16 channels.
MASK_UNORM16, MASK_FP16, MASK_BF16 = 0, 1, 2


def normalised_density(hu):
    """t = clamp((hu + 1024) / 4095, 0, 1) in float32 (transfer.rs:121-124 before quantisation)."""
    h = np.ascontiguousarray(hu, np.int16).astype(np.float32)
    t = (h - np.float32(-1024.0)) / np.float32(3071.0 - -1024.0)
    return np.clip(t, np.float32(0.0), np.float32(1.0)).astype(np.float32)


def density_encode(hu, fmt=DENSITY_UNORM16):
    """The stored density volume: R16_UNORM codes, or t as FP16 / BF16 bits
    (round to nearest even) or float32."""
    if fmt == DENSITY_UNORM16:
        return hu_to_unorm16(hu)
    t = normalised_density(hu)
    if fmt == DENSITY_FP16:
        return t.astype(np.float16).view(np.uint16)
    if fmt == DENSITY_BF16:
        w = t.view(np.uint32).astype(np.uint64)
        return ((w + 0x7FFF + ((w >> 16) & 1)) >> 16).astype(np.uint16)
    if fmt == DENSITY_FP32:
        return t
    raise ValueError(f"unknown density format {fmt}")


def env_prepare(rgb, diffuse=False):
    """EnvironmentMap::prepare + upload (environment.rs:57-175, renderer.rs:2224-2290) of an
    (h, w, 3) linear-RGB light map: (RGBA16F radiance (h, w, 4) uint16, RG32F table
    (h, w + 1, 2), peak_u), and with `diffuse` the RGBA16F diffuse convolution (16, 32, 4)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    rad = np.zeros((h, w, 4), np.uint16)
    table = np.zeros((h, w + 1, 2), np.float32)
    dif = np.zeros((16, 32, 4), np.uint16) if diffuse else None
    peak = lib().vvo_env_prepare(w, h, ptr(rgb), ptr(rad), ptr(table), ptr(dif))
    return (rad, table, float(peak)) + ((dif,) if diffuse else ())


def geometry(volume):
    g = Geometry()
    lib().vvo_geometry_of(C.byref(volume), C.byref(g))
    return g


def pack_uniforms(volume, bucket, params, accumulated, frame, width, height, has_labels=True,
                  has_env_map=False, env_peak_u=0.0):
    out = np.zeros(21200, np.uint8)
    lib().vvo_pack_uniforms(C.byref(volume), ptr(np.ascontiguousarray(bucket, np.float32)), int(has_labels),
                            int(has_env_map), env_peak_u, C.byref(params), accumulated, frame, width, height,
                            ptr(out))
    return out


def mask_margin(volume, label_params):
    return lib().vvo_mask_margin(C.byref(volume), C.byref(label_params))


def threads():
    return max(1, min(os.cpu_count() or 1, 64))


class CpuRenderer:
    """The reference's Renderer flow on the CPU: upload, then accumulate-frames.

    Mirrors Renderer::new / set_labels / record (renderer.rs:555, 1241, 1499) with
    every pass run by the oracle. Arrays are x-fastest, shaped (z, y, x, ...).
    """

    def __init__(self, volume, tf, hu, density_format=DENSITY_UNORM16, majorants=MAJORANTS_REFERENCE,
                 mask_format=MASK_UNORM16):
        self.volume = volume
        self.hu = np.ascontiguousarray(hu, np.int16)
        self.dims = tuple(volume.dims)
        self.geo = geometry(volume)
        self.density_format = density_format
        self.mask_format = mask_format
        self.majorants = majorants
        self.density = density_encode(self.hu, density_format)
        self.set_transfer_function(tf)
        self.labels = np.zeros((1, 1, 1), np.uint8)
        self.soft = None
        self.soft_push = [0, 0, 0, 0]
        self.has_labels = False
        self.mask = None
        self.mask_key = None
        self.accumulated = 0
        self.accum_key = None
        self.env_rad = self.env_table = self.env_diffuse = None
        self.env_peak_u = 0.0
        zero = self._uniforms_geometry_only()
        self.normals = np.zeros(self.density.shape + (4,), np.int8)
        lib().vvo_normals(ptr(zero), C.byref(self.scene()), ptr(self.normals), threads())

    def _uniforms_geometry_only(self):
        """Uniforms::zeroed_with (renderer.rs:2119-2126): geometry only."""
        u = np.zeros(21200, np.uint8)
        f = u.view(np.float32)
        w2i = np.array(self.geo.world_to_index, np.float32)
        f[0:16] = w2i
        f[16 + 4 * 4: 16 + 4 * 4 + 3] = np.array(self.geo.dims, np.float32)  # dims.xyz, w = 0
        return u

    def set_transfer_function(self, tf):
        self.tf = tf
        self.lut = tf_lut_half(tf)
        self.preint = tf_cumulative(tf)
        self.bucket = bucket_bound(tf) if self.majorants == MAJORANTS_BOUND else bucket_max(tf)
        self.mask_key = None

    def set_labels(self, labels, soft=None, src_axis=(0, 1, 2), flip=(0, 0, 0)):
        self.labels = np.ascontiguousarray(labels, np.uint8)
        if soft is not None:
            self.soft = np.ascontiguousarray(soft, np.uint8)
            flips = sum(int(f) << a for a, f in enumerate(flip))
            self.soft_push = [src_axis[0], src_axis[1], src_axis[2], flips | 8]
        else:
            self.soft = None
            self.soft_push = [0, 0, 0, 0]
        self.has_labels = True
        self.mask_key = None

    def set_environment_map(self, rgb=None):
        """Renderer::set_environment_map (renderer.rs:1283): (h, w, 3) linear RGB, or None."""
        if rgb is None:
            self.env_rad = self.env_table = self.env_diffuse = None
            self.env_peak_u = 0.0
        else:
            self.env_rad, self.env_table, self.env_peak_u, self.env_diffuse = env_prepare(rgb, diffuse=True)
        self.accum_key = None

    def brick_dims(self):
        return tuple((d + 7) // 8 for d in self.dims)

    def scene(self):
        s = Scene()
        s.dims[:] = self.dims
        s.density = ptr(self.density)
        s.density_format = self.density_format
        s.mask_format = self.mask_format
        s.normals = ptr(getattr(self, "normals", None))
        s.mask = ptr(self.mask)
        s.labels = ptr(self.labels)
        s.label_dims[:] = self.labels.shape[::-1]
        s.majorant = ptr(getattr(self, "majorant", None))
        s.brick_dims[:] = self.brick_dims()
        s.tf_lut = ptr(self.lut)
        s.preint = ptr(self.preint)
        if self.env_rad is not None:
            s.env_rad = ptr(self.env_rad)
            s.env_table = ptr(self.env_table)
            s.env_dims[:] = (self.env_rad.shape[1], self.env_rad.shape[0])
        else:
            s.env_dims[:] = (1, 1)
        s._keep = self
        return s

    def uniforms(self, params, frame, width, height):
        return pack_uniforms(self.volume, self.bucket, params, self.accumulated, frame, width, height,
                             has_labels=self.has_labels, has_env_map=self.env_rad is not None,
                             env_peak_u=self.env_peak_u)

    def adopt(self, mask=None, majorant=None, normals=None):
        """Takes the pre-pass volumes from elsewhere (e.g. the device), so that a
        later stage is compared on identical inputs; `prepare` then keeps them."""
        if normals is not None:
            self.normals = np.ascontiguousarray(normals, np.int8)
        if mask is not None:
            self.mask = np.ascontiguousarray(mask, np.uint16)
        if majorant is not None:
            self.majorant = np.ascontiguousarray(majorant, np.float32)
        self.mask_key = "adopted"

    def prepare(self, params, width, height):
        """The mask and majorant passes `record` runs when the opacity key changed."""
        if self.mask_key == "adopted":
            return
        u = self.uniforms(params, 0, width, height)
        mode = int(params.labels.mode) if self.has_labels else 0
        lp = params.labels
        key = (mode, bytes(lp.colors), bytes(lp.ghost), float(lp.extinction), float(lp.ghost_opacity),
               mask_margin(self.volume, lp), min(int(lp.smoothing), 8))
        if key != self.mask_key:
            if mode != 0:
                self.mask = np.zeros(self.density.shape + (2,), np.uint16)
                scratch = np.zeros_like(self.mask)
                soft = self.soft
                sd = (C.c_int * 3)(*(soft.shape[2::-1] if soft is not None else (1, 1, 1)))
                push = (C.c_int * 4)(*self.soft_push)
                lib().vvo_mask(ptr(u), C.byref(self.scene()), ptr(soft), sd, push, mask_margin(self.volume, lp),
                               min(int(lp.smoothing), 8), ptr(self.mask), ptr(scratch), threads())
            self.majorant = np.zeros(self.brick_dims()[::-1], np.float32)
            lib().vvo_majorant(ptr(u), C.byref(self.scene()), ptr(self.majorant))
            self.mask_key = key

    def resize(self, width, height):
        self.width, self.height = width, height
        self.accum = np.zeros((height, width, 4), np.float32)
        self.albedo = np.zeros_like(self.accum)
        self.normal = np.zeros_like(self.accum)
        self.hdr = np.zeros((height, width, 4), np.uint16)
        self.accum_key = None

    def record(self, params, frame=1, rows=None):
        """One accumulate-frame (pt.comp) over all rows or rows [y0, y1)."""
        key = _params_key(params)
        if key != self.accum_key:
            self.accumulated = 0
            self.accum_key = key
        self.prepare(params, self.width, self.height)
        u = self.uniforms(params, frame, self.width, self.height)
        y0, y1 = rows if rows is not None else (0, self.height)
        lib().vvo_pt_frame(ptr(u), C.byref(self.scene()), ptr(self.accum), ptr(self.albedo), ptr(self.normal),
                           ptr(self.hdr), y0, y1, threads())
        self.accumulated += max(int(params.path_tracing.samples_per_frame), 1)
        return u

    def trace_pixel(self, params, x, y, accumulated=0):
        """pt.comp's result for one pixel at accumulation count `accumulated`."""
        self.prepare(params, self.width, self.height)
        saved = self.accumulated
        self.accumulated = accumulated
        u = self.uniforms(params, 1, self.width, self.height)
        self.accumulated = saved
        out = np.zeros(12, np.float32)
        lib().vvo_pt_pixel(ptr(u), C.byref(self.scene()), x, y, ptr(out))
        return out

    def trace_pixels(self, params, pixels, accumulated=0, threads=None):
        """trace_pixel for every (x, y) row of `pixels`, on `threads` host threads: (n, 12)."""
        self.prepare(params, self.width, self.height)
        saved = self.accumulated
        self.accumulated = accumulated
        u = self.uniforms(params, 1, self.width, self.height)
        self.accumulated = saved
        pix = np.ascontiguousarray(pixels, np.int32).reshape(-1, 2)
        out = np.zeros((pix.shape[0], 12), np.float32)
        lib().vvo_pt_pixels(ptr(u), C.byref(self.scene()), ptr(pix), C.c_long(pix.shape[0]), ptr(out),
                            threads or globals()["threads"]())
        return out

    def pixel_sums_fp64(self, params, pixels, first, count, threads=None):
        """The FP64 oracle: for each (x, y) row of `pixels`, the double-precision
        sums of `count` paths at accumulation indices first .. first + count - 1
        (one path per frame, the per-pixel streams of pt.comp), traced by the
        restatement compiled in double precision over this renderer's inputs:
        (n, 12) float64 (radiance sum, background, albedo sums and
        luminance^2, normal sums and depth)."""
        self.prepare(params, self.width, self.height)
        saved = self.accumulated
        self.accumulated = 0
        u = self.uniforms(params, 1, self.width, self.height)
        self.accumulated = saved
        pix = np.ascontiguousarray(pixels, np.int32).reshape(-1, 2)
        out = np.zeros((pix.shape[0], 12), np.float64)
        lib64().vvo64_pt_pixel_sums(ptr(u), C.byref(self.scene()), ptr(pix), C.c_long(pix.shape[0]),
                                    C.c_uint32(first), C.c_uint32(count), ptr(out),
                                    threads or globals()["threads"]())
        return out

    def denoise(self, params):
        """record_denoise over the current accumulation (uses the last frame's counts)."""
        saved = self.accumulated
        spf = max(int(params.path_tracing.samples_per_frame), 1)
        self.accumulated -= spf  # u.path.x is the count before the last frame
        u = self.uniforms(params, 1, self.width, self.height)
        self.accumulated = saved
        hdr = np.zeros((self.height, self.width, 4), np.uint16)
        ping = np.zeros((self.height, self.width, 4), np.float32)
        pong = np.zeros_like(ping)
        lib().vvo_denoise(ptr(u), ptr(self.accum), ptr(self.albedo), ptr(self.normal), ptr(hdr), ptr(ping),
                          ptr(pong), threads())
        return hdr

    def post(self, params, hdr, exposure, frame=1):
        """record_post: bloom, auto exposure (updates `exposure`, a 1-float array) and tone mapping."""
        saved = self.accumulated
        spf = max(int(params.path_tracing.samples_per_frame), 1)
        self.accumulated -= spf
        u = self.uniforms(params, frame, self.width, self.height)
        self.accumulated = saved
        out = np.zeros((self.height, self.width, 4), np.uint8)
        lib().vvo_post(ptr(u), ptr(np.ascontiguousarray(hdr, np.uint16)), ptr(exposure), ptr(out))
        return out

    def light_samples(self, params, seeds):
        """(n, 6): texel column and row (linear scans of the CDFs), pdf and
        direction of the light map samples that pt.comp draws from `seeds`."""
        seeds = np.ascontiguousarray(seeds, np.uint32).ravel()
        out = np.zeros((seeds.size, 6), np.float32)
        u = self.uniforms(params, 1, self.width, self.height)
        lib().vvo_light_samples(ptr(u), C.byref(self.scene()), ptr(seeds), C.c_long(seeds.size), ptr(out))
        return out

    def extinction(self, params, idx, direction=(0.0, 0.0, 1.0), smooth=True):
        """(n, 4): the flight's sampled extinction (path_sigma, rgb) at continuous
        indices idx and the flight majorant of the brick there."""
        self.prepare(params, self.width, self.height)
        idx = np.ascontiguousarray(idx, np.float32).reshape(-1, 3)
        out = np.zeros((idx.shape[0], 4), np.float32)
        u = self.uniforms(params, 1, self.width, self.height)
        d = np.ascontiguousarray(direction, np.float32)
        lib().vvo_extinction(ptr(u), C.byref(self.scene()), ptr(idx), C.c_long(idx.shape[0]), ptr(d), int(smooth),
                             ptr(out), threads())
        return out

    def bspline(self, params, idx):
        idx = np.ascontiguousarray(idx, np.float32).reshape(-1, 3)
        out = np.zeros((idx.shape[0], 4), np.float32)
        u = self.uniforms(params, 1, 16, 16)
        lib().vvo_bspline(ptr(u), C.byref(self.scene()), ptr(idx), C.c_long(idx.shape[0]), ptr(out))
        return out


def _params_key(params):
    """Accumulation key: every FrameParams field except the denoiser (renderer.rs:1537-1544)."""
    saved = params.path_tracing.denoiser
    params.path_tracing.denoiser = 0
    key = bytes(params)
    params.path_tracing.denoiser = saved
    return key
