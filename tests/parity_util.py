"""Shared checks of the GPU parity tests: single-path replays and converged
images, the CUDA path against the CPU oracle on the same per-pixel random
streams (pt.comp:378-379).

Replay bars (the tolerance of every replay test):
* the parity build of the probe (vv_probe_paths_exact: the oracle's texture
  arithmetic, no fused multiply-adds): >= 97% of pixel-paths within 1e-4
  relative on every radiance channel, <= 2% flipped. What remains comes from
  CUDA's expf/logf/powf/sinf/cosf/atan2f/acosf differing in the last bit from
  the C library's, amplified by the null-collision weight or flipping a
  delta-tracking, roulette or event comparison;
* the product build (vv_probe_paths: fast samplers, contraction): >= 60%
  within 1e-4 and <= 15% flipped, reported beside the parity build's (its
  samplers round differently, which the null-collision weights amplify into
  drift: measured 92-99% within 1e-4 on the small scenes, 66% and 6.6%
  flipped on the head/neck phantom, against 99.3% and 0.2% for the parity
  build);
* background coverage (the first-hit guide) identical for >= 99% of pixels.

Converged image: the GPU's accumulation and the oracle's, traced from
independent random streams, within 3 sigma of the per-pixel Monte Carlo error
(sigma from the accumulated luminance^2, pt.comp:550-551) for >= 98% of
pixels, and the image means within 3 sigma of the mean's own error.
"""
import numpy as np

from volview_gb300 import abi, scene

EXACT_AGREE, EXACT_FLIPS = 0.97, 0.02
PRODUCT_AGREE, PRODUCT_FLIPS = 0.60, 0.15
LUMA = np.array([0.2126, 0.7152, 0.0722], np.float32)


def make_params(cfg, center, diagonal, zoom=0.45, **kw):
    p = scene.frame_params_for(cfg, center, diagonal, **kw)
    p.camera.distance = abi.f32(p.camera.distance * zoom)
    return p


def adopt_device_inputs(gpu, cpu, params):
    """Gives the oracle the device's masks and majorants, so that the tracer is
    compared on identical inputs (the mask pass is checked on its own: a
    one-quantum difference at the mask's zero boundary can move a brick's
    majorant between 0 and the label opacity, which changes every ray's random
    stream through that brick)."""
    gpu.probe_bspline(params, np.zeros((1, 3), np.float32))  # runs record's mask and majorant passes
    cpu.adopt(mask=gpu.read_volume(abi.VOLUME_MASK), majorant=gpu.read_volume(abi.VOLUME_MAJORANT))


def replay_stats(gpu, cpu, params, pixels, accs=(0, 5), exact=False):
    """(share within 1e-4, share flipped beyond 1e-2, worst background
    coverage agreement) of one path per pixel and accumulation index."""
    rels, cover = [], []
    for acc in accs:
        a = gpu.probe_paths(params, acc, pixels, exact=exact)
        b = cpu.trace_pixels(params, pixels, acc)
        rels.append(np.max(np.abs(a[:, :3] - b[:, :3]) / (np.abs(b[:, :3]) + 1e-5), axis=1))
        cover.append(float((a[:, 3] == b[:, 3]).mean()))
    rel = np.concatenate(rels)
    return float((rel <= 1e-4).mean()), float((rel > 1e-2).mean()), min(cover), rel.size


def check_replays(gpu, cpu, params, pixels, accs=(0, 5), label=""):
    """Both builds' replays against the oracle, at the bars above."""
    out = {}
    for exact in (True, False):
        agree, flips, cover, n = replay_stats(gpu, cpu, params, pixels, accs, exact)
        name = "parity build" if exact else "product build"
        print(f"{label} single-path replays, {name}: {agree:.2%} within 1e-4, {1 - agree - flips:.2%} drift, "
              f"{flips:.2%} flipped, of {n} pixel-paths; coverage {cover:.2%}")
        assert cover >= 0.99, f"{name}: background coverage differs ({cover:.4f})"
        if exact:
            assert agree >= EXACT_AGREE, f"{name}: only {agree:.4f} within 1e-4"
            assert flips <= EXACT_FLIPS, f"{name}: {flips:.4f} flipped"
        else:
            assert agree >= PRODUCT_AGREE, f"{name}: only {agree:.4f} within 1e-4"
            assert flips <= PRODUCT_FLIPS, f"{name}: {flips:.4f} flipped"
        out[name] = (agree, flips)
    return out


def cpu_sums(cpu, params, pixels, first_acc, frames):
    """The oracle's sums over `frames` accumulate-frames of the listed pixels,
    from accumulation index `first_acc` on: (n, 12) as vv_probe_paths lays them out."""
    spf = max(int(params.path_tracing.samples_per_frame), 1)
    total = np.zeros((len(pixels), 12), np.float64)
    for f in range(frames):
        total += cpu.trace_pixels(params, pixels, first_acc + f * spf)
    return total.astype(np.float32)


def check_converged(gpu_acc, gpu_alb, n_gpu, cpu_sum, n_cpu, label=""):
    """The per-pixel 3-sigma test. gpu_acc/gpu_alb: (n, 4) accumulation and albedo
    guide of the GPU at the compared pixels; cpu_sum: (n, 12) oracle sums."""
    def stats(acc_rgb, lum2, n):
        mean = (acc_rgb @ LUMA) / n
        var = np.maximum(lum2 / n - mean * mean, 0.0) / n
        return mean, var

    mg, vg = stats(gpu_acc[:, :3], gpu_alb[:, 3], n_gpu)
    mc, vc = stats(cpu_sum[:, :3], cpu_sum[:, 7], n_cpu)
    sigma = np.sqrt(vg + vc) + 1e-6
    inside = np.abs(mg - mc) <= 3.0 * sigma
    # The per-pixel estimates are sums of heavy-tailed path contributions, so the
    # sample variance from a few hundred paths understates the error in some
    # pixels; the whole-image mean is checked against its own error as well.
    image_sigma = np.sqrt(vg.sum() + vc.sum()) / mg.size
    print(f"{label} converged image: {inside.mean():.4%} of {mg.size} pixels within 3 sigma; image mean "
          f"{mg.mean():.5f} vs {mc.mean():.5f} (sigma {image_sigma:.5f})")
    assert inside.mean() >= 0.98
    assert abs(mg.mean() - mc.mean()) <= 3.0 * image_sigma


def converged(gpu, cpu, params, width, height, pixels=None, n_gpu=1024, n_cpu=256, label=""):
    """Accumulates n_gpu paths per pixel on the GPU (vv_record_frames) and n_cpu
    independent ones (accumulation indices past the GPU's) with the oracle, at
    `pixels` (default: every pixel), and runs the 3-sigma test."""
    p = abi.FrameParams.from_buffer_copy(bytes(params))
    p.path_tracing.denoiser = abi.DENOISE_OFF
    adopt_device_inputs(gpu, cpu, p)
    gpu.resize(width, height)
    gpu.record_frames(1, n_gpu, p)
    acc, alb, _ = gpu.read_accumulation()
    if pixels is None:
        ys, xs = np.mgrid[0:height, 0:width]
        pixels = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    pixels = np.ascontiguousarray(pixels, np.int32)
    cpu.resize(width, height)
    sums = cpu_sums(cpu, p, pixels, n_gpu, n_cpu)
    xs, ys = pixels[:, 0], pixels[:, 1]
    check_converged(acc[ys, xs], alb[ys, xs], n_gpu, sums, n_cpu, label)


def all_pixels(width, height):
    ys, xs = np.mgrid[0:height, 0:width]
    return np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
