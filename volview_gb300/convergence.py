"""Convergence of the progressive image: the RMSE a frame's accumulation has
left, estimated from the accumulation itself.

pt.comp accumulates, per pixel, the sum of the clamped path radiance (accum.rgb)
and the sum of the squared luminance of each path (guide_albedo.a,
shaders/pt.comp:548-551). With n independent paths per pixel the sample
variance of the luminance follows, and the mean squared error of the pixel's
running mean against the tracer's own converged image is var / n. The image's
RMSE is the square root of that error averaged over pixels. This is the error
against the image the same tracer converges to (firefly clamp included), which
is what a high-spp render of the same tracer measures, without rendering one.
"""
import numpy as np

LUMA = np.array([0.2126, 0.7152, 0.0722], np.float64)


def luminance_moments(accum, albedo):
    """(sum of luminance, sum of squared luminance) per pixel, float64."""
    s1 = np.asarray(accum, np.float64)[..., :3] @ LUMA
    s2 = np.asarray(albedo, np.float64)[..., 3]
    return s1, s2


def rmse_estimate(accum, albedo, samples):
    """Estimated RMSE of the luminance of the accumulated image after `samples` paths per pixel."""
    n = float(samples)
    if n < 2:
        return float("inf")
    s1, s2 = luminance_moments(accum, albedo)
    var = np.maximum(s2 - s1 * s1 / n, 0.0) / (n - 1.0)
    return float(np.sqrt(np.mean(var / n)))


def samples_for(rmse_now, samples_now, target):
    """Paths per pixel at which the error of an image with `rmse_now` after `samples_now` reaches `target`."""
    return int(np.ceil(samples_now * (rmse_now / target) ** 2))
