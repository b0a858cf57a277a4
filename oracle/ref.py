"""Drives the reference's own shaders compiled as CPU code (test infrastructure).

oracle/build_ref.py compiles shaders/{pt,majorant,normals,mask,denoise,tonemap,
bloom}.comp into oracle/_ref/libref_<shader>.so. This module binds the same
buffers the reference's Renderer binds (crates/render/src/renderer.rs:1938-1971:
linear CLAMP_TO_EDGE for density, transfer function, normals and mask; nearest
for labels, majorants, pre-integration, soft labels and the mask's blur partner)
and runs the shaders' invocations over the same grids the reference dispatches.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
P = C.c_void_p

# glsl::Format
R16_UNORM, RG16_UNORM, RGBA8_SNORM, RGBA8_UNORM, R32F, RG32F, RGBA32F, RGBA16F, R16F, R8_UINT, RGBA8_UINT = range(11)
NEAREST, LINEAR = 0, 1

_libs = {}


def available():
    return all(os.path.exists(os.path.join(REF_DIR, f"libref_{n}.so")) for n in ("pt", "majorant", "normals", "mask",
                                                                                  "denoise"))


def shader(name):
    if name not in _libs:
        l = C.CDLL(os.path.join(REF_DIR, f"libref_{name}.so"))
        l.ref_bind_texture.argtypes = [C.c_char_p, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        l.ref_bind_image.argtypes = [C.c_char_p, P, C.c_int, C.c_int, C.c_int, C.c_int]
        l.ref_set_uniforms.argtypes = [P, C.c_long]
        l.ref_run.argtypes = [C.c_int] * 7
        if hasattr(l, "ref_set_push"):
            l.ref_set_push.argtypes = [P, C.c_long]
        _libs[name] = l
    return _libs[name]


def _p(a):
    return C.c_void_p(a.ctypes.data)


def bind_common(l, r, dummy):
    """Binds the renderer's textures the way write_descriptors does."""
    w, h, d = r.dims
    l.ref_bind_texture(b"density_tex", _p(r.density), R16_UNORM, w, h, d, LINEAR, 0)
    l.ref_bind_texture(b"tf_tex", _p(r.lut), RGBA16F, 4096, 1, 1, LINEAR, 0)
    lw, lh, ld = r.labels.shape[::-1]
    l.ref_bind_texture(b"label_tex", _p(r.labels), R8_UINT, lw, lh, ld, NEAREST, 0)
    l.ref_bind_texture(b"normal_tex", _p(r.normals), RGBA8_SNORM, w, h, d, LINEAR, 0)
    l.ref_bind_texture(b"preint_tex", _p(r.preint), RGBA32F, 4096, 1, 1, NEAREST, 0)
    if r.mask is not None:
        l.ref_bind_texture(b"mask_tex", _p(r.mask), RG16_UNORM, w, h, d, LINEAR, 0)
    else:
        l.ref_bind_texture(b"mask_tex", _p(dummy), RG16_UNORM, 1, 1, 1, LINEAR, 0)
    if getattr(r, "majorant", None) is not None:
        bw, bh, bd = r.majorant.shape[::-1]
        l.ref_bind_texture(b"majorant_tex", _p(r.majorant), R32F, bw, bh, bd, NEAREST, 0)
    if getattr(r, "env_rad", None) is not None:
        eh, ew = r.env_rad.shape[:2]
        l.ref_bind_texture(b"env_tex", _p(r.env_rad), RGBA16F, ew, eh, 1, LINEAR, 0)
        l.ref_bind_texture(b"env_table_tex", _p(r.env_table), RG32F, ew + 1, eh, 1, NEAREST, 0)


def normals(r, uniforms):
    l = shader("normals")
    dummy = np.zeros(16, np.uint8)
    out = np.zeros(r.density.shape + (4,), np.int8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    w, h, d = r.dims
    l.ref_bind_image(b"normal_image", _p(out), RGBA8_SNORM, w, h, d)
    l.ref_run(0, w, 0, h, 0, d, _threads())
    return out


def mask(r, uniforms, margin, radius):
    """mask.comp passes 0-3 (renderer.rs:1671-1694)."""
    l = shader("mask")
    dummy = np.zeros(16, np.uint8)
    w, h, d = r.dims
    a = np.zeros(r.density.shape + (2,), np.uint16)
    b = np.zeros_like(a)
    l.ref_set_uniforms(_p(uniforms), 21200)
    saved = r.mask
    r.mask = a
    bind_common(l, r, dummy)
    r.mask = saved
    soft = r.soft if r.soft is not None else np.zeros((1, 1, 1, 4), np.uint8)
    sw, sh, sd = soft.shape[2::-1]
    l.ref_bind_texture(b"soft_tex", _p(soft), RGBA8_UINT, sw, sh, sd, NEAREST, 0)
    l.ref_bind_texture(b"mask_b_tex", _p(b), RG16_UNORM, w, h, d, NEAREST, 0)
    l.ref_bind_image(b"mask_image", _p(a), RG16_UNORM, w, h, d)
    l.ref_bind_image(b"mask_b_image", _p(b), RG16_UNORM, w, h, d)
    for pas in range(4):
        push = np.array([w, h, d, 0, margin, pas, radius, 0] + list(r.soft_push), np.int32)
        l.ref_set_push(_p(push), push.nbytes)
        l.ref_run(0, w, 0, h, 0, d, _threads())
    return a


def majorant(r, uniforms):
    l = shader("majorant")
    dummy = np.zeros(16, np.uint8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    bw, bh, bd = r.brick_dims()
    out = np.zeros((bd, bh, bw), np.float32)
    l.ref_bind_image(b"majorant_image", _p(out), R32F, bw, bh, bd)
    l.ref_run(0, bw, 0, bh, 0, bd, _threads())
    return out


def pt_frame(r, uniforms, accum, albedo, normal, hdr, rows=None):
    """pt.comp over the image (or rows [y0, y1)), updating the images in place."""
    l = shader("pt")
    dummy = np.zeros(16, np.uint8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    H, W = accum.shape[:2]
    l.ref_bind_image(b"accum_image", _p(accum), RGBA32F, W, H, 1)
    l.ref_bind_image(b"guide_albedo_image", _p(albedo), RGBA32F, W, H, 1)
    l.ref_bind_image(b"guide_normal_image", _p(normal), RGBA32F, W, H, 1)
    l.ref_bind_image(b"hdr_image", _p(hdr), RGBA16F, W, H, 1)
    y0, y1 = rows if rows is not None else (0, H)
    l.ref_run(0, W, y0, y1, 0, 1, _threads())


def denoise(uniforms, accum, albedo, normal):
    """record_denoise's 7 passes (renderer.rs:1868-1904); returns the HDR image."""
    l = shader("denoise")
    H, W = accum.shape[:2]
    ping = np.zeros((H, W, 4), np.float32)
    pong = np.zeros_like(ping)
    hdr = np.zeros((H, W, 4), np.uint16)
    l.ref_set_uniforms(_p(uniforms), 21200)
    for name, img in ((b"accum_image", accum), (b"guide_albedo_image", albedo), (b"guide_normal_image", normal),
                      (b"ping_image", ping), (b"pong_image", pong)):
        l.ref_bind_image(name, _p(img), RGBA32F, W, H, 1)
    l.ref_bind_image(b"hdr_image", _p(hdr), RGBA16F, W, H, 1)
    passes = [[0, 0, 0, 0]] + [[1 + k, 1 << k, k % 2, 0] for k in range(5)] + [[-1, 0, 1, 0]]
    for sweep in passes:
        push = np.array([W, H, 1, 0] + sweep, np.int32)
        l.ref_set_push(_p(push), push.nbytes)
        l.ref_run(0, W, 0, H, 0, 1, _threads())
    return hdr


def post(uniforms, hdr, exposure):
    """record_post (renderer.rs:1817-1866): bloom passes 0-6, then tonemap.comp."""
    H, W = hdr.shape[:2]
    qw, qh = (W + 3) // 4, (H + 3) // 4
    ew, eh = (qw + 1) // 2, (qh + 1) // 2
    imgs = [np.zeros((qh, qw, 4), np.uint16), np.zeros((qh, qw, 4), np.uint16),
            np.zeros((eh, ew, 4), np.uint16), np.zeros((eh, ew, 4), np.uint16)]
    exp_img = np.ascontiguousarray(exposure, np.float32)
    l = shader("bloom")
    l.ref_set_uniforms(_p(uniforms), 21200)
    l.ref_bind_image(b"hdr_image", _p(hdr), RGBA16F, W, H, 1)
    for name, img in zip((b"bloom_a", b"bloom_b", b"bloom_c", b"bloom_d"), imgs):
        l.ref_bind_image(name, _p(img), RGBA16F, img.shape[1], img.shape[0], 1)
    l.ref_bind_image(b"exposure_image", _p(exp_img), R32F, 1, 1, 1)
    for pas in range(7):
        e = 1 if pas >= 4 else 0
        w, h = imgs[2 * e].shape[1], imgs[2 * e].shape[0]
        push = np.array([w, h, 1, 0, pas, 0, 0, 0, 0, 0, 0, 0], np.int32)
        l.ref_set_push(_p(push), push.nbytes)
        if pas == 1:
            l.ref_run_workgroup64()
        else:
            l.ref_run(0, w, 0, h, 0, 1, _threads())
    t = shader("tonemap")
    out = np.zeros((H, W, 4), np.uint8)
    t.ref_set_uniforms(_p(uniforms), 21200)
    t.ref_bind_image(b"hdr_image", _p(hdr), RGBA16F, W, H, 1)
    t.ref_bind_texture(b"bloom_narrow", _p(imgs[0]), RGBA16F, qw, qh, 1, LINEAR, 0)
    t.ref_bind_texture(b"bloom_wide", _p(imgs[2]), RGBA16F, ew, eh, 1, LINEAR, 0)
    t.ref_bind_image(b"exposure_image", _p(exp_img), R32F, 1, 1, 1)
    t.ref_bind_image(b"out_image", _p(out), RGBA8_UNORM, W, H, 1)
    t.ref_run(0, W, 0, H, 0, 1, _threads())
    exposure[...] = exp_img
    return out


def _threads():
    return max(1, min(os.cpu_count() or 1, 64))


SHADOW_DOWNSAMPLE, AO_DOWNSAMPLE = 2, 4  # renderer.rs:35-40
CLAMP_TO_BORDER_WHITE = 1


def _downsampled(dims, k):
    """renderer.rs:2139-2145: (nx, ny, nz) divided by k, rounded up."""
    return tuple((d + k - 1) // k for d in dims)


def ao_volume(r, uniforms):
    """ao.comp over the occlusion volume (renderer.rs:1709-1728): R16F, (z, y, x)."""
    l = shader("ao")
    dummy = np.zeros(16, np.uint8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    ad = _downsampled(r.dims, AO_DOWNSAMPLE)
    out = np.zeros(ad[::-1], np.uint16)
    l.ref_bind_image(b"ao_image", _p(out), R16F, *ad)
    push = np.array([ad[0], ad[1], ad[2], 0, 0, 0, 0, 0], np.int32)
    l.ref_set_push(_p(push), push.nbytes)
    l.ref_run(0, ad[0], 0, ad[1], 0, ad[2], _threads())
    return out


def shadow_volume(r, uniforms):
    """record_shadow_sweep (renderer.rs:1907-1950) with shadow.comp: slices swept
    away from the key light along its dominant axis; RGBA16F, (z, y, x, 4),
    starting from zeros."""
    l = shader("shadow")
    dummy = np.zeros(16, np.uint8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    sd = _downsampled(r.dims, SHADOW_DOWNSAMPLE)
    vol = np.zeros(sd[::-1] + (4,), np.uint16)
    l.ref_bind_texture(b"shadow_tex", _p(vol), RGBA16F, *sd, LINEAR, CLAMP_TO_BORDER_WHITE)
    l.ref_bind_image(b"shadow_image", _p(vol), RGBA16F, *sd)
    return l, sd, vol


def _shadow_axis(w2i_cols, light_dir, sd, dims):
    """renderer.rs:1915-1928 in f32: the light's dominant axis in shadow-volume units and its sign."""
    f32 = np.float32
    m = [np.array(w2i_cols[c][:3], f32) for c in range(3)]
    v = np.array(light_dir, f32)
    l_idx = m[0] * v[0]
    l_idx = m[1] * v[1] + l_idx
    l_idx = m[2] * v[2] + l_idx
    l_idx = l_idx * (np.array(sd, f32) / np.array(dims, f32))
    a = np.abs(l_idx)
    axis = 0 if (a[0] >= a[1] and a[0] >= a[2]) else (1 if a[1] >= a[2] else 2)
    return axis, (1 if l_idx[axis] >= 0 else -1)


def shadow_sweep(r, uniforms, light_dir):
    """The shadow volume of `light_dir` (the packed uniform's light_dir.xyz)."""
    l, sd, vol = shadow_volume(r, uniforms)
    cols = uniforms.view(np.float32)[0:16].reshape(4, 4)
    axis, sign = _shadow_axis(cols, light_dir, sd, r.dims)
    u_axis, v_axis = (axis + 1) % 3, (axis + 2) % 3
    n = sd[axis]
    for i in range(n):
        sl = n - 1 - i if sign > 0 else i
        push = np.array([sd[0], sd[1], sd[2], 0, axis, sl, sign, 0], np.int32)
        l.ref_set_push(_p(push), push.nbytes)
        l.ref_run(0, sd[u_axis], 0, sd[v_axis], 0, 1, _threads())
    return vol


def dvr(r, uniforms, width, height, shadow=None, ao=None):
    """dvr.comp over the image: RGBA16F (radiance, transmittance), (height, width, 4)."""
    l = shader("dvr")
    dummy = np.zeros(16, np.uint8)
    l.ref_set_uniforms(_p(uniforms), 21200)
    bind_common(l, r, dummy)
    if shadow is not None:
        sz, sy, sx = shadow.shape[:3]
        l.ref_bind_texture(b"shadow_tex", _p(shadow), RGBA16F, sx, sy, sz, LINEAR, CLAMP_TO_BORDER_WHITE)
    if ao is not None:
        az, ay, ax = ao.shape
        l.ref_bind_texture(b"ao_tex", _p(ao), R16F, ax, ay, az, LINEAR, CLAMP_TO_BORDER_WHITE)
    if getattr(r, "env_diffuse", None) is not None:
        dh, dw = r.env_diffuse.shape[:2]
        l.ref_bind_texture(b"env_diffuse_tex", _p(r.env_diffuse), RGBA16F, dw, dh, 1, LINEAR, 0)
    hdr = np.zeros((height, width, 4), np.uint16)
    l.ref_bind_image(b"hdr_image", _p(hdr), RGBA16F, width, height, 1)
    l.ref_run(0, width, 0, height, 0, 1, _threads())
    return hdr
