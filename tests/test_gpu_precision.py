"""The precision variant (GPU): density stored as FP16, BF16 or FP32 instead of
R16_UNORM, the label mask as FP16 or BF16 beside density of the same format,
and running sums with Kahan compensation or in FP64 past a sample count
(vv_renderer_create_ex / vv_precision).

Tolerances (written here, checked below):
* stored density, normals and majorant: bit-exact against the oracle run on
  the same format (round-to-nearest-even encodings of the same normalised
  density t = clamp((hu + 1024) / 4095, 0, 1));
* stored mask: every code within one step of the oracle's in the same format
  (the bar of the RG16_UNORM mask), 99.9 % of them equal;
* single-path replays: the bars of tests/parity_util.py, for the parity build
  of the probe and the product build, on each format;
* running sums over 300 single-frame passes: with Kahan compensation, and with
  FP64 from the 100th sample on, every non-negative sum (radiance, coverage,
  albedo, squared luminance, depth) within 3 ulp (float32) of the FP64 running
  sum (Kahan's bound 2 eps sum|x| plus the final rounding), the signed normal
  sums within 1e-4; plain FP32 sums drift further on average.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parity_util import adopt_device_inputs, all_pixels, check_replays
from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu

FORMATS = [abi.DENSITY_FP16, abi.DENSITY_BF16, abi.DENSITY_FP32]
# (density format, mask format): the density formats with the RG16_UNORM mask,
# then FP16 / BF16 density with the mask in the same format.
STORAGE = [(f, abi.MASK_UNORM16) for f in FORMATS] + [(abi.DENSITY_FP16, abi.MASK_FP16),
                                                      (abi.DENSITY_BF16, abi.MASK_BF16)]
STORAGE_IDS = ["fp16", "bf16", "fp32", "fp16-mask", "bf16-mask"]


def _params(cfg, gpu):
    p = scene.frame_params_for(cfg, list(gpu.center), gpu.diagonal, clip_sagittal=True)
    p.camera.distance = abi.f32(p.camera.distance * 0.45)
    return p


@pytest.fixture(scope="module", params=STORAGE, ids=STORAGE_IDS)
def fmt_pair(request, small_cfg, gpu_ctx):
    cfg, (fmt, mfmt) = small_cfg, request.param
    gpu = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"], abi.precision(density_format=fmt, mask_format=mfmt))
    gpu.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"], density_format=fmt, mask_format=mfmt)
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    params = _params(cfg, gpu)
    gpu.resize(48, 48)
    cpu.resize(48, 48)
    yield cfg, gpu, cpu, params
    gpu.destroy()


def test_stored_density_bit_exact(fmt_pair):
    cfg, gpu, cpu, params = fmt_pair
    got = gpu.read_volume(abi.VOLUME_DENSITY)
    assert got.dtype == cpu.density.dtype and np.array_equal(got, cpu.density)
    t = O.normalised_density(cfg["hu"])
    dec = {abi.DENSITY_FP16: lambda d: d.view(np.float16).astype(np.float32),
           abi.DENSITY_BF16: lambda d: (d.astype(np.uint32) << 16).view(np.float32),
           abi.DENSITY_FP32: lambda d: d}[gpu.precision.density_format](got)
    ulp = {abi.DENSITY_FP16: 2.0 ** -11, abi.DENSITY_BF16: 2.0 ** -8, abi.DENSITY_FP32: 0.0}
    assert np.all(np.abs(dec - t) <= ulp[gpu.precision.density_format] * np.maximum(t, 2.0 ** -14) + 1e-30)


def test_normals_bit_exact(fmt_pair):
    cfg, gpu, cpu, params = fmt_pair
    assert np.array_equal(gpu.read_volume(abi.VOLUME_NORMALS), cpu.normals)


def test_mask_in_storage_format(fmt_pair):
    """The binary and blur passes (mask.comp) store the mask in the renderer's
    mask format: codes within one step of the oracle's in that format (codes of
    non-negative FP16 / BF16 values are monotone, like UNORM16 codes)."""
    cfg, gpu, cpu, params = fmt_pair
    gpu.probe_bspline(params, np.zeros((1, 3), np.float32))  # runs record's mask and majorant passes
    ref = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"], density_format=gpu.precision.density_format,
                        mask_format=gpu.precision.mask_format)
    ref.set_labels(cfg["labels_vol"], cfg["soft"])
    ref.prepare(params, 48, 48)
    got = gpu.read_volume(abi.VOLUME_MASK)
    d = np.abs(got.astype(np.int32) - ref.mask.astype(np.int32))
    assert d.max() <= 1
    assert (d == 0).mean() >= 0.999
    assert ((ref.mask != 0) & (ref.mask != ref.mask.max())).any()  # a blurred edge was compared


def test_majorant_bit_exact(fmt_pair):
    """The majorant from the stored values (majorant.comp:26-71): min/max of the
    decoded densities, so it bounds every interpolated sample of the format."""
    cfg, gpu, cpu, params = fmt_pair
    gpu.probe_bspline(params, np.zeros((1, 3), np.float32))  # runs record's mask and majorant passes
    cpu_mask = cpu.mask
    cpu.mask = gpu.read_volume(abi.VOLUME_MASK)
    u = cpu.uniforms(params, 1, 48, 48)
    maj = np.zeros(cpu.brick_dims()[::-1], np.float32)
    O.lib().vvo_majorant(O.ptr(u), O.C.byref(cpu.scene()), O.ptr(maj))
    cpu.mask = cpu_mask
    assert np.array_equal(gpu.read_volume(abi.VOLUME_MAJORANT), maj)


def test_single_path_replays(fmt_pair):
    cfg, gpu, cpu, params = fmt_pair
    adopt_device_inputs(gpu, cpu, params)
    check_replays(gpu, cpu, params, all_pixels(48, 48),
                  label=f"density format {gpu.precision.density_format}, mask {gpu.precision.mask_format}")


def test_bspline_matches_oracle(fmt_pair):
    cfg, gpu, cpu, params = fmt_pair
    rng = np.random.default_rng(3)
    idx = rng.uniform(-0.5, 47.5, size=(4096, 3)).astype(np.float32)
    a, b = gpu.probe_bspline(params, idx), cpu.bspline(params, idx)
    assert np.abs(a[:, 0] - b[:, 0]).max() <= 1e-4 * max(float(np.abs(b[:, 0]).max()), 1e-6)
    assert np.abs(a[:, 1:] - b[:, 1:]).max() <= 1e-4 * max(float(np.abs(b[:, 1:]).max()), 1e-6)


def _sums(cfg, gpu_ctx, precision, frames):
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"], precision)
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = _params(cfg, r)
    p.path_tracing.denoiser = abi.DENOISE_OFF
    r.resize(24, 24)
    for f in range(1, frames + 1):
        r.record(f, p)
    assert r.accumulated_samples() == frames
    acc, alb, nor = r.read_accumulation()
    hdr = r.read_hdr()
    r.destroy()
    return acc, alb, nor, hdr


def test_running_sums(small_cfg, gpu_ctx):
    """Single-frame passes give every renderer the same per-frame sums, so the
    accumulations differ only by how they are summed."""
    cfg, n = small_cfg, 300
    plain = _sums(cfg, gpu_ctx, abi.precision(), n)
    kahan = _sums(cfg, gpu_ctx, abi.precision(sums=abi.SUMS_KAHAN), n)
    wide = _sums(cfg, gpu_ctx, abi.precision(fp64_after=1), n)
    late = _sums(cfg, gpu_ctx, abi.precision(sums=abi.SUMS_KAHAN, fp64_after=100), n)
    for k in range(3):  # radiance, albedo guide, normal guide
        ref = wide[k].astype(np.float64)
        ulp = np.spacing(np.abs(wide[k])).astype(np.float64)
        tol = 3 * ulp + 1e-30
        if k == 2:
            tol[..., :3] = 1e-4  # signed normal components: Kahan's bound is relative to sum |x|
        assert np.all(np.abs(kahan[k] - ref) <= tol)
        assert np.all(np.abs(late[k] - ref) <= tol)
        assert np.abs(plain[k] - ref).mean() >= np.abs(kahan[k] - ref).mean()
    # The HDR store is the running sum over the sample count, in FP64 when the sums are.
    d = np.abs(wide[3].view(np.float16).astype(np.float32) - plain[3].view(np.float16).astype(np.float32))
    assert d.max() <= 2e-3 * max(float(np.abs(plain[3].view(np.float16).astype(np.float32)).max()), 1e-6)


def test_create_rejects_unknown_precision(small_cfg, gpu_ctx):
    cfg = small_cfg
    for bad in (abi.precision(density_format=7), abi.precision(sums=5), abi.precision(mask_format=3),
                abi.precision(mask_format=abi.MASK_FP16),
                abi.precision(density_format=abi.DENSITY_FP16, mask_format=abi.MASK_BF16),
                abi.precision(density_format=abi.DENSITY_FP32, mask_format=abi.MASK_BF16)):
        with pytest.raises(R.VolptError) as e:
            R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"], bad)
        assert e.value.status == abi.VV_ERR_ARG


@pytest.mark.parametrize("fmt,mfmt", STORAGE, ids=STORAGE_IDS)
def test_ray_marcher_and_light_map_on_each_format(small_cfg, gpu_ctx, fmt, mfmt):
    """The ray marcher (path tracing off) and light-map path tracing read the
    stored density through their format's samplers: images close to the
    R16_UNORM renderer's (mean radiance within 2 %, 99 % of the ray marcher's
    pixels within 2e-2 + 5 % of its values)."""
    cfg = small_cfg
    out = {}
    for key, precision in (("unorm", None), ("fmt", abi.precision(density_format=fmt, mask_format=mfmt))):
        r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"], precision)
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
        r.set_environment_map(abi.env_struct(scene.synthetic_light_map()))
        p = _params(cfg, r)
        r.resize(48, 48)
        march = abi.FrameParams.from_buffer_copy(bytes(p))
        march.path_tracing.enabled = 0
        r.record(1, march)
        dvr = r.read_hdr().view(np.float16).astype(np.float32)
        lit = abi.FrameParams.from_buffer_copy(bytes(p))
        lit.lighting.environment = abi.ENV_MAP
        lit.path_tracing.denoiser = abi.DENOISE_OFF
        r.record_frames(1, 64, lit)
        acc, _, _ = r.read_accumulation(normal=False)
        r.destroy()
        out[key] = (dvr, acc[..., :3] / 64.0)
    (d0, a0), (d1, a1) = out["unorm"], out["fmt"]
    assert np.isfinite(d1).all() and np.isfinite(a1).all()
    ok = np.abs(d1[..., :3] - d0[..., :3]) <= 2e-2 + 5e-2 * np.abs(d0[..., :3])
    assert ok.mean() >= 0.99
    assert abs(d1[..., :3].mean() - d0[..., :3].mean()) <= 0.02 * d0[..., :3].mean()
    assert abs(a1.mean() - a0.mean()) <= 0.02 * a0.mean()


@pytest.mark.parametrize("fmt", [abi.DENSITY_UNORM16] + FORMATS, ids=["unorm16", "fp16", "bf16", "fp32"])
def test_majorants_are_true_bounds(small_cfg, gpu_ctx, fmt):
    """Every extinction a flight samples on the device is at or below its
    brick's flight majorant with VV_MAJORANTS_BOUND, in every storage format,
    for transfer functions whose FP16 LUT exceeds the reference's FP32 bucket
    maxima; the bucket maxima (uniforms) and the majorant grid are the
    oracle's, bit for bit, in both modes. The reference's majorants are
    reported: samples above them by up to an FP16 half-ulp."""
    cfg = small_cfg
    idx = np.random.default_rng(1).uniform(-0.5, 47.5, size=(200000, 3)).astype(np.float32)
    for seed in (0, 3, 5):
        tf = scene.random_transfer_function(seed)
        for mode in (abi.MAJORANTS_REFERENCE, abi.MAJORANTS_BOUND):
            gpu = R.Renderer(gpu_ctx, cfg["volume"], tf, abi.precision(density_format=fmt, majorants=mode))
            cpu = O.CpuRenderer(cfg["volume"], tf, cfg["hu"], density_format=fmt, majorants=mode)
            p = scene.frame_params_for(cfg, list(gpu.center), gpu.diagonal)
            p.labels.mode = abi.LABEL_OFF
            gpu.resize(16, 16)
            cpu.resize(16, 16)
            assert np.array_equal(gpu.pack_uniforms(p, 1), cpu.uniforms(p, 1, 16, 16))
            counts = []
            for smooth in (True, False):
                out = gpu.probe_extinction(p, idx, smooth=smooth)
                counts.append(int((out[:, :3].max(1) > out[:, 3]).sum()))
            cpu.prepare(p, 16, 16)
            assert np.array_equal(gpu.read_volume(abi.VOLUME_MAJORANT), cpu.majorant)
            gpu.destroy()
            name = "bound" if mode == abi.MAJORANTS_BOUND else "reference"
            print(f"format {fmt}, transfer function {seed}, {name} majorants: {counts} of {len(idx)} samples "
                  f"(B-spline, trilinear) above the majorant")
            if mode == abi.MAJORANTS_BOUND:
                assert counts == [0, 0]


def test_formats_against_the_fp64_oracle(gpu_ctx):
    """Every storage format and the compensated sums, measured against the FP64 oracle
    (tests/precision_fp64_study.py) on the small scene at 256 paths per pixel,
    the same random streams: each render's luminance RMSE against the oracle's
    image is at most twice the oracle image's own Monte Carlo RMSE (what the
    paths that a rounding difference diverts contribute), and every render's
    error is nonzero only through such paths (the FP32 storage's at most the
    coarser formats' plus that noise)."""
    import precision_fp64_study as S
    cfg = scene.small_config(n=48, size=48)
    res = S.run(gpu_ctx, cfg, 256, crops=1, size=48, zoom=0.45)
    mc = res["fp64_oracle"]["mc_rmse_per_crop"][0]
    print({k: v["rmse_vs_fp64_oracle"] for k, v in res.items() if isinstance(v, dict) and "rmse_vs_fp64_oracle" in v},
          "oracle MC RMSE", mc)
    for key in ("fp32", "unorm16", "fp16", "bf16", "fp32+kahan+fp64_after_65536"):
        assert 0.0 < res[key]["rmse_vs_fp64_oracle"] <= 2.0 * mc, (key, res[key], mc)
