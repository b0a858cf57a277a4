"""The oracle against the reference's own known answers (CPU only).

transfer.rs:130-149 holds the reference's only tests on this path; they pin the
density normalisation and the transfer-function LUT. The shader restatement is
pinned by golden vectors produced by the reference's shaders compiled as CPU
code (tests/golden/make_golden.py), and live against those shaders when
oracle/_ref was built here.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from volview_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_scene.npz")


def test_interpolates_between_points():
    # transfer.rs:130-139
    tf = abi.tf_struct([(0.0, (0.0, 0.0, 0.0), 0.0), (100.0, (1.0, 1.0, 1.0), 2.0)])
    assert list(O.tf_evaluate(tf, -50.0)) == [0.0, 0.0, 0.0, 0.0]
    assert list(O.tf_evaluate(tf, 50.0)) == [0.5, 0.5, 0.5, 1.0]
    assert list(O.tf_evaluate(tf, 500.0)) == [1.0, 1.0, 1.0, 2.0]


def test_lut_matches_density_normalisation():
    # transfer.rs:141-149
    assert O.hu_to_unorm16(np.array([-1024, 3071, -2000], np.int16)).tolist() == [0, 65535, 0]
    tf = abi.tf_struct(abi.PRESETS["bone"])
    lut = O.tf_lut(tf)
    assert np.array_equal(lut[1024 + 300], O.tf_evaluate(tf, 300.0))


def test_bucket_max_covers_the_next_entry():
    tf = abi.tf_struct(abi.PRESETS["bone"])
    lut = O.tf_lut(tf)
    b = O.bucket_max(tf)
    for k in range(64):
        assert b[k] == lut[64 * k:min(64 * k + 65, 4096), 3].max()


def _golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("golden fixtures not generated")
    return np.load(GOLDEN)


def _scene_from_golden(g):
    from volview_gb300 import scene
    vol = abi.volume_struct(g["hu"], tuple(g["spacing"]))
    tf = abi.tf_struct(abi.PRESETS["bone"])
    r = O.CpuRenderer(vol, tf, g["hu"])
    r.set_labels(g["labels"], g["soft"])
    params = abi.FrameParams.from_buffer_copy(g["params"].tobytes())
    r.resize(int(g["width"]), int(g["height"]))
    return r, params


def test_oracle_matches_reference_golden_volumes():
    g = _golden()
    r, params = _scene_from_golden(g)
    u = r.record(params, 1)
    assert np.array_equal(r.density, g["density"])
    assert np.array_equal(r.normals, g["normals"])
    assert np.array_equal(r.mask, g["mask"])
    assert np.array_equal(r.majorant, g["majorant"])
    assert np.array_equal(u, g["uniforms_frame1"])


def test_oracle_matches_reference_golden_frames():
    g = _golden()
    r, params = _scene_from_golden(g)
    for f in range(1, int(g["frames"]) + 1):
        r.record(params, f)
    # Same arithmetic, same order: bit-exact.
    assert np.array_equal(r.accum, g["accum"])
    assert np.array_equal(r.albedo, g["albedo"])
    assert np.array_equal(r.normal, g["normal"])
    assert np.array_equal(r.hdr, g["hdr"])
    assert np.array_equal(r.denoise(params), g["denoised"])
    exposure = np.zeros(1, np.float32)
    assert np.array_equal(r.post(params, g["denoised"], exposure, int(g["frames"])), g["post1"])
    assert np.array_equal(r.post(params, g["denoised"], exposure, int(g["frames"])), g["post2"])
    assert np.array_equal(exposure, g["exposure"])


def test_oracle_matches_reference_shaders_live(small_cfg):
    from oracle import ref as R
    if not R.available():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    cfg = small_cfg
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    r.set_labels(cfg["labels_vol"], cfg["soft"])
    g = r.geo
    from volview_gb300 import scene
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True)
    r.resize(48, 48)
    assert np.array_equal(R.normals(r, r._uniforms_geometry_only()), r.normals)
    u = r.record(params, 1)
    assert np.array_equal(R.mask(r, u, O.mask_margin(cfg["volume"], params.labels), 1), r.mask)
    assert np.array_equal(R.majorant(r, u), r.majorant)
    acc = np.zeros((48, 48, 4), np.float32)
    alb, nor = np.zeros_like(acc), np.zeros_like(acc)
    hdr = np.zeros((48, 48, 4), np.uint16)
    R.pt_frame(r, u, acc, alb, nor, hdr)
    assert np.array_equal(acc, r.accum) and np.array_equal(alb, r.albedo) and np.array_equal(nor, r.normal)


def _light_map_golden():
    path = os.path.join(os.path.dirname(GOLDEN), "small_light_map.npz")
    if not os.path.exists(path):
        pytest.skip("light map fixture not generated")
    return np.load(path)


def test_oracle_matches_reference_golden_light_map_frames():
    """pt.comp with Environment::Map (env_uv, env_pdf, sample_env, the light
    map's next-event estimate and MIS) against the reference's shader."""
    g = _light_map_golden()
    vol = abi.volume_struct(g["hu"], tuple(g["spacing"]))
    tf = abi.tf_struct(abi.PRESETS["bone"])
    r = O.CpuRenderer(vol, tf, g["hu"])
    r.set_labels(g["labels"], g["soft"])
    r.set_environment_map(g["light_map"])
    # The preparation is the oracle's restatement (environment.rs has no tests):
    # these are regression values, the frames below are the reference's.
    assert np.array_equal(r.env_rad, g["env_rad"]) and np.array_equal(r.env_table, g["env_table"])
    assert r.env_peak_u == float(g["env_peak_u"])
    params = abi.FrameParams.from_buffer_copy(g["params"].tobytes())
    assert params.lighting.environment == abi.ENV_MAP
    r.resize(int(g["width"]), int(g["height"]))
    u = r.record(params, 1)
    assert np.array_equal(u, g["uniforms_frame1"])
    for f in range(2, int(g["frames"]) + 1):
        r.record(params, f)
    assert np.array_equal(r.accum, g["accum"])
    assert np.array_equal(r.albedo, g["albedo"])
    assert np.array_equal(r.normal, g["normal"])
    assert np.array_equal(r.hdr, g["hdr"])


def test_light_map_tables():
    """The sampling table's invariants (environment.rs:81-108): rows' conditional
    CDFs end at 1, the marginal CDF ends at 1, probabilities sum to 1."""
    from volview_gb300 import scene
    rad, table, peak = O.env_prepare(scene.synthetic_light_map(48, 24, seed=9))
    assert rad.shape == (24, 48, 4) and table.shape == (24, 49, 2)
    assert np.all(table[:, 47, 0] == 1.0) and table[-1, 48, 0] == 1.0
    assert np.all(np.diff(table[:, :48, 0], axis=1) >= 0)
    assert np.all(np.diff(table[:, 48, 0]) >= 0)
    assert abs(float(table[:, :48, 1].astype(np.float64).sum()) - 1.0) < 1e-5
    assert abs(float(table[:, 48, 1].astype(np.float64).sum()) - 1.0) < 1e-5
    assert 0.0 <= peak <= 1.0
    # Radiance is normalised to a mean luminance of 1 over the sphere.
    h = rad.shape[0]
    f = rad[..., :3].view(np.float16).astype(np.float64)
    s = np.sin(np.pi * (np.arange(h) + 0.5) / h)[:, None]
    mean = (f * s[..., None]).sum((0, 1)) / (s.sum() * rad.shape[1])
    assert abs(float(mean @ np.array([0.2126, 0.7152, 0.0722])) - 1.0) < 2e-3


def test_density_formats():
    """The precision variant's stored density: t = clamp((hu + 1024) / 4095, 0, 1)
    in float32, as binary16 and bfloat16 rounded to nearest even (checked here
    against rounding the significand with numpy's half-to-even rint), or float32."""
    hu = np.arange(-1100, 3200, dtype=np.int16)
    t = O.normalised_density(hu)
    assert t.dtype == np.float32 and t.min() == 0.0 and t.max() == 1.0
    assert np.array_equal(t, np.clip((hu.astype(np.float32) + np.float32(1024)) / np.float32(4095), 0, 1))
    half = O.density_encode(hu, O.DENSITY_FP16).view(np.float16).astype(np.float64)
    assert np.array_equal(half, t.astype(np.float16).astype(np.float64))
    m, e = np.frexp(t.astype(np.float64))
    expect = np.ldexp(np.rint(m * 256.0) / 256.0, e)
    bf = (O.density_encode(hu, O.DENSITY_BF16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    assert np.array_equal(bf, expect)
    assert np.array_equal(O.density_encode(hu, O.DENSITY_FP32), t)
    assert np.array_equal(O.density_encode(hu), O.hu_to_unorm16(hu))


def test_mask_formats(small_cfg):
    """The label mask stored as two binary16 / bfloat16 channels: each stored
    value is the format's round-to-nearest-even encoding (monotone codes), and
    the decoded mask stays within the format's rounding, compounded over the
    binary pass and three blur passes, of the RG16_UNORM mask."""
    from volview_gb300 import scene
    cfg = small_cfg
    masks = {}
    for dfmt, mfmt in ((O.DENSITY_UNORM16, O.MASK_UNORM16), (O.DENSITY_FP16, O.MASK_FP16),
                       (O.DENSITY_BF16, O.MASK_BF16)):
        cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"], density_format=dfmt, mask_format=mfmt)
        cpu.set_labels(cfg["labels_vol"], cfg["soft"])
        p = scene.frame_params_for(cfg, [0.0, 0.0, 0.0], 100.0)
        cpu.prepare(p, 16, 16)
        masks[mfmt] = cpu.mask
    ref = masks[O.MASK_UNORM16].astype(np.float64) / 65535.0
    half = masks[O.MASK_FP16].view(np.float16).astype(np.float64)
    bf = (masks[O.MASK_BF16].astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    for got, bits in ((half, 11), (bf, 8)):
        assert got.min() >= 0.0 and got.max() <= 1.0
        assert np.all(np.abs(got - ref) <= 4 * 2.0 ** -bits * ref + 2.0 / 65535)
    assert np.array_equal(half.astype(np.float16).view(np.uint16), masks[O.MASK_FP16])
    assert (ref > 0).sum() > 0 and ((ref > 0) & (ref < 1)).sum() > 0  # a blurred edge to compare on


def test_light_map_samples_follow_luminance(small_cfg):
    """The oracle's light map samples (pt.comp:204-233) land on texels in
    proportion to luminance x sin(theta), with the pdf of the texel they land on."""
    from volview_gb300 import abi, scene
    m = scene.synthetic_light_map()
    cpu = O.CpuRenderer(small_cfg["volume"], small_cfg["tf"], small_cfg["hu"])
    cpu.set_environment_map(m)
    cpu.resize(16, 16)
    p = scene.frame_params_for(small_cfg, [0.0, 0.0, 0.0], 100.0)
    p.lighting.environment = abi.ENV_MAP
    seeds = np.random.default_rng(5).integers(0, 2 ** 32, 1 << 16, dtype=np.uint64).astype(np.uint32)
    b = cpu.light_samples(p, seeds)
    h, w = m.shape[:2]
    lum = (m.astype(np.float64) @ np.array([0.2126, 0.7152, 0.0722])) * np.sin(np.pi * (np.arange(h) + 0.5) / h)[:, None]
    prob = lum / lum.sum()
    x, y = b[:, 0].astype(int), b[:, 1].astype(int)
    freq = np.bincount(y * w + x, minlength=h * w).reshape(h, w) / len(seeds)
    assert np.abs(freq - prob).max() < 4 * np.sqrt(prob.max() / len(seeds))
    # pdf = p(texel) w h / (2 pi^2 sin(theta)), theta within the texel's row
    s0, s1 = np.sin(np.pi * y / h), np.sin(np.pi * (y + 1) / h)
    scale = prob[y, x] * w * h / (2 * np.pi ** 2)
    assert np.all(b[:, 2] >= scale / np.maximum(s0, s1) * (1 - 1e-4))
    assert np.all(b[:, 2] <= scale / np.maximum(np.minimum(s0, s1), 1e-6) * (1 + 1e-4))
    assert np.all(np.abs(np.linalg.norm(b[:, 3:], axis=1) - 1) < 1e-5)


def test_oracle_matches_reference_shaders_live_light_map(small_cfg):
    from oracle import ref as R
    if not R.available():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    from volview_gb300 import scene
    cfg = small_cfg
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    r.set_labels(cfg["labels_vol"], cfg["soft"])
    r.set_environment_map(scene.synthetic_light_map())
    g = r.geo
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True)
    params.lighting.environment = abi.ENV_MAP
    r.resize(48, 48)
    acc = np.zeros((48, 48, 4), np.float32)
    alb, nor = np.zeros_like(acc), np.zeros_like(acc)
    hdr = np.zeros((48, 48, 4), np.uint16)
    for f in range(1, 4):
        u = r.record(params, f)
        R.pt_frame(r, u, acc, alb, nor, hdr)
    assert np.array_equal(acc, r.accum) and np.array_equal(alb, r.albedo) and np.array_equal(nor, r.normal)
    assert np.array_equal(hdr, r.hdr)


def _modes_golden():
    path = os.path.join(os.path.dirname(GOLDEN), "small_modes.npz")
    if not os.path.exists(path):
        pytest.skip("mode fixtures not generated")
    return np.load(path)


def _mode_case_params():
    from volview_gb300 import scene
    return scene.MODE_CASES


@pytest.mark.parametrize("case", _mode_case_params())
def test_oracle_matches_reference_golden_modes(case):
    """The reference's other rendering modes (label modes Off, Tint and Isolate
    with hidden labels, ghosted labels and shells, binary masks, the Dome
    environment, the thin lens): the oracle's masks, majorants, uniforms and two
    accumulate-frames against mask.comp, majorant.comp and pt.comp compiled as
    CPU code, bit for bit."""
    g = _modes_golden()
    vol = abi.volume_struct(g["hu"], tuple(g["spacing"]))
    tf = abi.tf_struct(abi.PRESETS["bone"])
    r = O.CpuRenderer(vol, tf, g["hu"])
    r.set_labels(g["labels"], g["soft"] if int(g[f"{case}_soft"]) else None)
    params = abi.FrameParams.from_buffer_copy(g[f"{case}_params"].tobytes())
    r.resize(int(g["width"]), int(g["height"]))
    u = r.record(params, 1)
    assert np.array_equal(u, g[f"{case}_uniforms"])
    if int(params.labels.mode) != abi.LABEL_OFF:
        assert np.array_equal(r.mask, g[f"{case}_mask"])
    assert np.array_equal(r.majorant, g[f"{case}_majorant"])
    for f in range(2, int(g["frames"]) + 1):
        r.record(params, f)
    assert np.array_equal(r.accum, g[f"{case}_accum"])
    assert np.array_equal(r.albedo, g[f"{case}_albedo"])
    assert np.array_equal(r.normal, g[f"{case}_normal"])


@pytest.mark.parametrize("case", _mode_case_params())
def test_oracle_matches_reference_shaders_live_modes(small_cfg, case):
    """The same modes at 48^3 / 48x48 against the reference's shaders, live."""
    from oracle import ref as R
    if not R.available():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    from volview_gb300 import scene
    cfg = small_cfg
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    g = r.geo
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True)
    params.camera.distance = abi.f32(params.camera.distance * 0.45)
    soft = scene.mode_case(case, params, list(g.center))
    r.set_labels(cfg["labels_vol"], cfg["soft"] if soft else None)
    r.resize(48, 48)
    u = r.record(params, 1)
    if int(params.labels.mode) != abi.LABEL_OFF:
        margin = O.mask_margin(cfg["volume"], params.labels)
        assert np.array_equal(R.mask(r, u, margin, int(params.labels.smoothing)), r.mask)
    assert np.array_equal(R.majorant(r, u), r.majorant)
    acc = np.zeros((48, 48, 4), np.float32)
    alb, nor = np.zeros_like(acc), np.zeros_like(acc)
    hdr = np.zeros((48, 48, 4), np.uint16)
    R.pt_frame(r, u, acc, alb, nor, hdr)
    assert np.array_equal(acc, r.accum) and np.array_equal(alb, r.albedo) and np.array_equal(nor, r.normal)
