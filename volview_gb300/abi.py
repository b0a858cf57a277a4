"""ctypes mirror of include/volpt.h: struct layouts, enums and defaults.

The defaults restate the reference's `Default` impls and CLI defaults
(crates/render/src/renderer.rs, crates/app/src/main.rs); the C library exports
the same defaults (vv_*_default) and a test checks that both agree.
"""
import ctypes as C
import math

import numpy as np

VV_LABEL_COUNT = 256
VV_UNIFORMS_BYTES = 21200

VV_OK, VV_ERR_ARG, VV_ERR_OOM, VV_ERR_CUDA, VV_ERR_TIMEOUT, VV_ERR_STATE, VV_ERR_LIMIT = range(7)
LABEL_OFF, LABEL_TINT, LABEL_ISOLATE, LABEL_HYBRID = range(4)
ENV_DOME, ENV_STUDIO, ENV_MAP = range(3)
TONE_NONE, TONE_ACES, TONE_AGX = range(3)
PLANE_SAGITTAL, PLANE_CORONAL, PLANE_AXIAL = range(3)
DENOISE_OFF, DENOISE_ATROUS, DENOISE_OIDN, DENOISE_LEARNED = range(4)
VOLUME_DENSITY, VOLUME_NORMALS, VOLUME_MASK, VOLUME_LABELS, VOLUME_MAJORANT, VOLUME_SHADOW, VOLUME_AO = range(7)
DENSITY_UNORM16, DENSITY_FP16, DENSITY_BF16, DENSITY_FP32 = range(4)
SUMS_FP32, SUMS_KAHAN = range(2)
MAJORANTS_REFERENCE, MAJORANTS_BOUND = range(2)
MASK_UNORM16, MASK_FP16, MASK_BF16 = range(3)


class Precision(C.Structure):
    """vv_precision: density storage format, running-sum mode, FP64 threshold,
    bucket maxima of the majorants, label-mask storage format."""
    _fields_ = [("density_format", C.c_uint32), ("sums", C.c_uint32), ("fp64_after", C.c_uint32),
                ("majorants", C.c_uint32), ("mask_format", C.c_uint32)]


def precision(density_format=DENSITY_UNORM16, sums=SUMS_FP32, fp64_after=0, majorants=MAJORANTS_REFERENCE,
              mask_format=MASK_UNORM16):
    return Precision(density_format, sums, fp64_after, majorants, mask_format)

F4x256 = (C.c_float * 4) * VV_LABEL_COUNT


class BatchRequest(C.Structure):
    """vv_batch_request: one request's frames in a batched pass."""
    _fields_ = [("params", C.c_void_p), ("first_frame", C.c_uint64), ("frames", C.c_uint32),
                ("display", C.c_uint32)]


class Volume(C.Structure):
    _fields_ = [("dims", C.c_uint32 * 3), ("spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("direction", C.c_double * 9), ("hu", C.POINTER(C.c_int16))]


class ControlPoint(C.Structure):
    _fields_ = [("hu", C.c_float), ("color", C.c_float * 3), ("extinction", C.c_float)]


class TransferFunction(C.Structure):
    _fields_ = [("count", C.c_uint32), ("points", C.POINTER(ControlPoint))]


class SoftLabelGrid(C.Structure):
    _fields_ = [("dims", C.c_uint32 * 3), ("src_axis", C.c_uint32 * 3), ("flip", C.c_uint32 * 3),
                ("data", C.POINTER(C.c_uint8))]


class EnvironmentMap(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.POINTER(C.c_float))]


class OrbitCamera(C.Structure):
    _fields_ = [("target", C.c_float * 3), ("distance", C.c_float), ("yaw", C.c_float),
                ("pitch", C.c_float), ("fov_y", C.c_float)]


class LabelParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("tint", C.c_float), ("extinction", C.c_float),
                ("ghost_opacity", C.c_float), ("cut_margin_mm", C.c_float), ("smoothing", C.c_uint32),
                ("colors", F4x256), ("materials", F4x256), ("ghost", C.c_uint8 * VV_LABEL_COUNT),
                ("density", F4x256), ("surface", F4x256), ("optics", F4x256)]


class Lighting(C.Structure):
    _fields_ = [("azimuth", C.c_float), ("elevation", C.c_float), ("intensity", C.c_float),
                ("ambient", C.c_float), ("environment", C.c_int32), ("light_size", C.c_float),
                ("env_rotation", C.c_float), ("anisotropy", C.c_float), ("chromatic", C.c_float),
                ("shadows", C.c_int32), ("ambient_occlusion", C.c_int32), ("exposure", C.c_float),
                ("auto_exposure", C.c_int32), ("bloom", C.c_float), ("vignette", C.c_float),
                ("grain", C.c_float), ("tone_mapper", C.c_int32), ("roughness", C.c_float),
                ("metalness", C.c_float), ("subsurface", C.c_float), ("scattering_distance", C.c_float),
                ("subsurface_strength", C.c_float), ("surface_detail", C.c_float)]


class ClipPlane(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("plane", C.c_int32), ("cut_positive", C.c_int32),
                ("position", C.c_float)]


class Clipping(C.Structure):
    _fields_ = [("planes", ClipPlane * 3), ("all", C.c_int32)]


class PathTracing(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("bounces", C.c_uint32), ("samples_per_frame", C.c_uint32),
                ("denoiser", C.c_int32), ("aperture", C.c_float), ("has_focus", C.c_int32),
                ("focus", C.c_float * 3)]


class FrameParams(C.Structure):
    _fields_ = [("camera", OrbitCamera), ("step_mm", C.c_float), ("srgb_encode", C.c_int32),
                ("labels", LabelParams), ("lighting", Lighting), ("preintegrate", C.c_int32),
                ("skip_empty_space", C.c_int32), ("clipping", Clipping), ("path_tracing", PathTracing),
                ("smooth_sampling", C.c_int32)]


class RendererInfo(C.Structure):
    _fields_ = [("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3), ("min_spacing", C.c_float),
                ("center", C.c_float * 3), ("diagonal", C.c_float), ("dims", C.c_uint32 * 3)]


def f32(x):
    """Rounds a Python float to the nearest f32."""
    return float(np.float32(x))


def to_radians(deg):
    """Rust's f32::to_radians: deg * (PI / 180) in f32."""
    return float(np.float32(deg) * np.float32(np.float32(math.pi) / np.float32(180.0)))


def lighting_default():
    """Lighting::default (renderer.rs:264-292)."""
    L = Lighting()
    L.azimuth = to_radians(-60.0)
    L.elevation = to_radians(40.0)
    L.intensity = 3.0
    L.ambient = 0.3
    L.environment = ENV_STUDIO
    L.light_size = to_radians(12.0)
    L.env_rotation = 0.0
    L.anisotropy = 0.0
    L.chromatic = 1.0
    L.shadows = 1
    L.ambient_occlusion = 1
    L.exposure = 0.0
    L.auto_exposure = 1
    L.bloom = 0.04
    L.vignette = 0.25
    L.grain = 0.012
    L.tone_mapper = TONE_ACES
    L.roughness = 0.5
    L.metalness = 0.0
    L.subsurface = 0.3
    L.scattering_distance = 4.0
    L.subsurface_strength = 1.0
    L.surface_detail = 1.0
    return L


def label_params_default():
    """LabelParams::default (renderer.rs:166-182)."""
    p = LabelParams()
    p.mode = LABEL_OFF
    p.tint = 0.7
    p.extinction = 0.5
    p.ghost_opacity = 0.08
    p.cut_margin_mm = 2.0
    p.smoothing = 1
    a = np.ctypeslib.as_array(p.colors)
    a[:] = 1.0
    np.ctypeslib.as_array(p.materials)[:] = [0.5, 0.0, 0.3, 0.0]
    np.ctypeslib.as_array(p.density)[:] = [0.0, 1e-3, 0.5, 1.0]
    return p


def path_tracing_default():
    """PathTracing::default (renderer.rs:359-373) without OIDN: a-trous denoiser."""
    pt = PathTracing()
    pt.enabled = 1
    pt.bounces = 4
    pt.samples_per_frame = 1
    pt.denoiser = DENOISE_ATROUS
    pt.aperture = 0.0
    pt.has_focus = 0
    return pt


def clipping_default():
    c = Clipping()
    for i in range(3):
        c.planes[i].enabled = 0
        c.planes[i].plane = i
        c.planes[i].cut_positive = 0
        c.planes[i].position = 0.0
    c.all = 0
    return c


_libm = None


def tanf(x):
    """The C library's single-precision tangent (what Rust's f32::tan calls)."""
    global _libm
    if _libm is None:
        import ctypes.util
        _libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        _libm.tanf.restype = C.c_float
        _libm.tanf.argtypes = [C.c_float]
    return _libm.tanf(x)


def camera_framing(center, diagonal):
    """OrbitCamera::framing (camera.rs:25-34)."""
    cam = OrbitCamera()
    fov = to_radians(30.0)
    for i in range(3):
        cam.target[i] = center[i]
    cam.distance = f32(np.float32(np.float32(0.55) * np.float32(diagonal)) /
                       np.float32(tanf(f32(np.float32(fov) / np.float32(2.0)))))
    cam.yaw = 0.0
    cam.pitch = 0.0
    cam.fov_y = fov
    return cam


def tf_struct(points):
    """A TransferFunction over [(hu, (r, g, b), extinction), ...]; keeps its array alive."""
    arr = (ControlPoint * len(points))()
    for i, (hu, col, ext) in enumerate(points):
        arr[i].hu = hu
        arr[i].color[:] = col
        arr[i].extinction = ext
    tf = TransferFunction(len(points), arr)
    tf._keep = arr
    return tf


# TransferFunction::presets (crates/render/src/transfer.rs:32-70).
PRESETS = {
    "bone": [(-1024.0, (0.0, 0.0, 0.0), 0.0), (180.0, (0.9, 0.6, 0.45), 0.0),
             (300.0, (0.95, 0.85, 0.7), 0.6), (1200.0, (1.0, 0.97, 0.9), 3.0),
             (3071.0, (1.0, 1.0, 1.0), 4.0)],
    "angio": [(-1024.0, (0.0, 0.0, 0.0), 0.0), (120.0, (0.7, 0.1, 0.08), 0.0),
              (200.0, (0.85, 0.15, 0.1), 0.5), (450.0, (0.95, 0.3, 0.2), 1.5),
              (600.0, (0.95, 0.88, 0.75), 2.5), (3071.0, (1.0, 1.0, 1.0), 4.0)],
    "soft tissue": [(-1024.0, (0.0, 0.0, 0.0), 0.0), (-200.0, (0.9, 0.75, 0.5), 0.0),
                    (-80.0, (0.95, 0.8, 0.5), 0.004), (-20.0, (0.8, 0.5, 0.4), 0.004),
                    (40.0, (0.75, 0.3, 0.25), 0.03), (150.0, (0.85, 0.2, 0.15), 0.15),
                    (300.0, (0.95, 0.3, 0.2), 0.8), (500.0, (0.95, 0.88, 0.75), 2.0),
                    (3071.0, (1.0, 1.0, 1.0), 4.0)],
}


def volume_struct(hu, spacing, origin=(0.0, 0.0, 0.0), direction=None):
    """A Volume over int16 array `hu` shaped (z, y, x); keeps the array alive."""
    hu = np.ascontiguousarray(hu, dtype=np.int16)
    v = Volume()
    v.dims[:] = [hu.shape[2], hu.shape[1], hu.shape[0]]
    v.spacing[:] = list(spacing)
    v.origin[:] = list(origin)
    v.direction[:] = list(direction) if direction is not None else [1, 0, 0, 0, 1, 0, 0, 0, 1]
    v.hu = hu.ctypes.data_as(C.POINTER(C.c_int16))
    v._keep = hu
    return v


def env_struct(rgb):
    """An EnvironmentMap over float32 linear RGB `rgb` shaped (height, width, 3), rows from the zenith."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    e = EnvironmentMap()
    e.width, e.height = rgb.shape[1], rgb.shape[0]
    e.rgb = rgb.ctypes.data_as(C.POINTER(C.c_float))
    e._keep = rgb
    return e


def soft_struct(data, src_axis=(0, 1, 2), flip=(0, 0, 0)):
    """A SoftLabelGrid over uint8 array `data` shaped (gz, gy, gx, 4)."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    g = SoftLabelGrid()
    g.dims[:] = [data.shape[2], data.shape[1], data.shape[0]]
    g.src_axis[:] = list(src_axis)
    g.flip[:] = list(flip)
    g.data = data.ctypes.data_as(C.POINTER(C.c_uint8))
    g._keep = data
    return g


def frame_params(camera, step_mm, labels=None, lighting=None, path_tracing=None, clipping=None,
                 smooth_sampling=True, skip_empty_space=True, srgb_encode=True):
    p = FrameParams()
    p.camera = camera
    p.step_mm = step_mm
    p.srgb_encode = int(srgb_encode)
    p.labels = labels if labels is not None else label_params_default()
    p.lighting = lighting if lighting is not None else lighting_default()
    p.preintegrate = 0
    p.skip_empty_space = int(skip_empty_space)
    p.clipping = clipping if clipping is not None else clipping_default()
    p.path_tracing = path_tracing if path_tracing is not None else path_tracing_default()
    p.smooth_sampling = int(smooth_sampling)
    return p
