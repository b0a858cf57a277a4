"""Host arithmetic of the learned denoiser's time-to-RMSE study (CPU): the
variance of a pixel's mean from the accumulation's own sums, the
inverse-variance blend of the network's image with the raw mean, and the
16-aligned training crops."""
import numpy as np

from volview_gb300 import learned_denoiser as LD


def _sums(lum):
    """Accumulation sums of per-path luminances lum[..., n] (grey radiance, so
    a pixel's luminance is its value): (acc, alb) as the renderer stores them."""
    s1 = lum.sum(axis=-1)
    s2 = (lum * lum).sum(axis=-1)
    acc = np.zeros(lum.shape[:-1] + (4,))
    acc[..., :3] = s1[..., None]
    alb = np.zeros(lum.shape[:-1] + (4,))
    alb[..., 3] = s2
    return acc, alb


def test_mean_variance_is_the_sample_variance_of_the_mean():
    rng = np.random.default_rng(1)
    n = 37
    lum = rng.gamma(2.0, 0.3, size=(5, 6, n))
    acc, alb = _sums(lum)
    expect = lum.var(axis=-1, ddof=1) / n
    assert np.allclose(LD.mean_variance(acc, alb, n), expect, rtol=1e-9, atol=1e-15)
    # Identical samples: zero variance (never negative through rounding).
    acc, alb = _sums(np.full((2, 2, n), 0.7))
    assert np.all(LD.mean_variance(acc, alb, n) >= 0.0)
    assert np.allclose(LD.mean_variance(acc, alb, n), 0.0, atol=1e-15)


def test_blend_weights_by_inverse_variance():
    rng = np.random.default_rng(2)
    n = 8
    lum = rng.gamma(2.0, 0.3, size=(4, 4, n))
    acc, alb = _sums(lum)
    net = rng.uniform(0.0, 1.0, size=(4, 4, 3))
    raw = acc[..., :3] / n
    var = LD.mean_variance(acc, alb, n)[..., None]
    for eps2 in (1e-4, 1e-2):
        w = var / (var + eps2)
        assert np.allclose(LD.blend(net, acc, alb, n, eps2), w * net + (1 - w) * raw, rtol=1e-12)
    # A network error far above the noise keeps the raw mean; far below it, the network's image.
    assert np.allclose(LD.blend(net, acc, alb, n, 1e12), raw, atol=1e-9)
    noisy = var[..., 0] > 1e-6
    assert np.allclose(LD.blend(net, acc, alb, n, 1e-14)[noisy], net[noisy], atol=1e-6)


def test_crop_pairs_are_aligned_slices_of_one_view():
    rng = np.random.default_rng(3)
    h, w, size = 96, 128, 32
    low = tuple(rng.standard_normal((h, w, 4)).astype(np.float32) for _ in range(3))
    target = rng.standard_normal((h, w, 3)).astype(np.float32)
    crops = LD.crop_pairs(low, target, 4, size, 20, np.random.default_rng(4))
    assert len(crops) == 20
    for (a, b, c), t, spp in crops:
        assert spp == 4 and a.shape == (size, size, 4) and t.shape == (size, size, 3)
        # Locate the crop in the view: its origin is a multiple of 16 and every array agrees.
        ys, xs = np.nonzero((low[0][:h - size + 1, :w - size + 1, 0] == a[0, 0, 0]))
        hits = [(y, x) for y, x in zip(ys, xs) if np.array_equal(low[0][y:y + size, x:x + size], a)]
        assert len(hits) == 1
        y, x = hits[0]
        assert y % 16 == 0 and x % 16 == 0
        sl = (slice(y, y + size), slice(x, x + size))
        assert np.array_equal(b, low[1][sl]) and np.array_equal(c, low[2][sl]) and np.array_equal(t, target[sl])


def test_luminance_rmse():
    a = np.zeros((3, 3, 3))
    b = np.ones((3, 3, 3)) * 0.5
    assert abs(LD.luminance_rmse(a, b) - 0.5) < 1e-12  # Rec. 709 weights sum to 1
    assert LD.luminance_rmse(b, b) == 0.0
