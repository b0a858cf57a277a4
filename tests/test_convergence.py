"""The RMSE estimator behind the time-to-RMSE latencies (CPU)."""
import numpy as np

from volview_gb300 import convergence as CV


def _sums(samples):
    """Accumulation images for per-pixel radiance samples of shape (n, H, W, 3)."""
    n, h, w, _ = samples.shape
    accum = np.zeros((h, w, 4), np.float32)
    albedo = np.zeros((h, w, 4), np.float32)
    accum[..., :3] = samples.sum(0)
    lum = samples @ CV.LUMA
    albedo[..., 3] = (lum * lum).sum(0)
    return accum, albedo


def test_estimate_matches_the_error_of_the_mean():
    rng = np.random.default_rng(3)
    h, w, n = 64, 64, 48
    mean = rng.uniform(0.0, 2.0, (h, w, 3))
    scale = rng.uniform(0.1, 1.0, (h, w, 1))
    samples = mean + scale * rng.exponential(1.0, (n, h, w, 3)) - scale
    accum, albedo = _sums(samples)
    est = CV.rmse_estimate(accum, albedo, n)
    # Luminance of exponential noise: per-channel variance scale^2, channels independent.
    true_var = (scale[..., 0] ** 2) * float((CV.LUMA ** 2).sum())
    expected = np.sqrt(np.mean(true_var / n))
    assert abs(est / expected - 1.0) < 0.03
    actual = np.sqrt(np.mean(((accum[..., :3] / n - mean) @ CV.LUMA) ** 2))
    assert abs(est / actual - 1.0) < 0.05


def test_estimate_scales_as_inverse_square_root():
    rng = np.random.default_rng(4)
    samples = rng.uniform(0.0, 1.0, (256, 32, 32, 3))
    e64 = CV.rmse_estimate(*_sums(samples[:64]), 64)
    e256 = CV.rmse_estimate(*_sums(samples), 256)
    assert abs(e64 / e256 - 2.0) < 0.1
    assert CV.samples_for(e64, 64, e256) in range(230, 290)


def test_constant_image_has_no_error():
    samples = np.full((16, 8, 8, 3), 0.5)
    assert CV.rmse_estimate(*_sums(samples), 16) < 1e-3
    assert CV.rmse_estimate(*_sums(samples[:1]), 1) == float("inf")
