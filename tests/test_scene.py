"""Host-side scene generation: phantoms, label recipes, soft grids (CPU)."""
import numpy as np

from volview_gb300 import scene


def test_small_phantom_recipe():
    hu, lab = scene.small_phantom(1, 64)
    assert hu.shape == (64, 64, 64) and hu.dtype == np.int16
    assert set(np.unique(lab)) <= set(range(11))
    assert (hu[lab == 0] == -1000).mean() > 0.99
    assert abs(float(hu[lab == 1].mean()) - 1000) < 20
    assert abs(float(hu[lab == 2].mean()) + 800) < 20
    assert abs(float(hu[lab >= 5].mean())) < 10


def test_phantom_is_seeded():
    a, _ = scene.small_phantom(1, 32)
    b, _ = scene.small_phantom(1, 32)
    c, _ = scene.small_phantom(2, 32)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_density_stats_recipe():
    h = np.zeros(scene.BINS, np.int64)
    h[1024:1100] = 1  # HU 0..75 uniform
    s = scene.density_stats(h)
    assert s[3] > 0 and s[0] <= s[1] <= 1.0 and abs(s[2] - (1024 + 37) / 4095) < 2 / 4095
    hollow = np.zeros(scene.BINS, np.int64)
    hollow[100:200] = 1  # HU -924..-825: air
    assert scene.density_stats(hollow)[3] == -1.0


def test_soft_grid_margins():
    _, lab = scene.small_phantom(1, 32)
    g = scene.soft_grid(lab, (4.0, 4.0, 4.0))
    assert g.shape == lab.shape + (4,)
    assert np.array_equal(g[..., 0], lab)
    assert g[..., 2].max() <= 254
    inner = g[..., 2] == g[..., 2].max()
    assert (g[..., 1][~inner] != g[..., 0][~inner]).mean() > 0.9


def test_optics_recipe():
    r, g, b, w = scene.optics(scene.MUSCLES)
    assert w == 1.0 and r < g < b
    assert abs(g - 1.89 * (550 / 500) ** -1.286) < 1e-5


def test_torso_recipe_is_the_small_phantom_scaled():
    """The precision and serving workloads' torso: at 128^3 the scaled recipe
    is the small phantom voxel for voxel; scaled, its regions keep their
    proportions along each axis."""
    from volview_gb300 import scene
    hu, lab = scene.torso_phantom(1, (128, 128, 128))
    h0, l0 = scene.small_phantom(1, 128)
    assert np.array_equal(hu, h0) and np.array_equal(lab, l0)
    hu2, lab2 = scene.torso_phantom(1, (64, 64, 100))
    assert hu2.shape == (100, 64, 64) and lab2.shape == (100, 64, 64)
    assert set(np.unique(lab2)) <= set(range(11))
    frac0 = (l0 == 1).mean()
    assert abs((lab2 == 1).mean() - frac0) < 0.25 * frac0  # the skull's share of the volume
