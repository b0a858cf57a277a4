"""The FP64 oracle (CPU): the path tracer's restatement compiled in double
precision (oracle/oracle_api64.cpp), the reference of the precision variant's error figures.

It is the FP32 oracle's source with `float` defined as `double`, over the same
stored inputs, so on the same per-pixel random streams:
* background coverage (the first-hit guide) agrees for >= 99% of pixels;
* >= 60% of single paths agree within 1e-4 relative on every radiance channel
  (the rest took another branch where a double and a float comparison differ);
* the image means of 64 paths per pixel agree within 4 standard errors of the
  per-pixel differences (paired);
* sums over index ranges add up: count 8 from 0 equals count 4 from 0 plus
  count 4 from 4, within 1e-12 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O
from volview_gb300 import abi, scene


@pytest.fixture(scope="module")
def small():
    cfg = scene.small_config(n=48, size=48)
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    g = cpu.geo
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal)
    params.camera.distance = abi.f32(params.camera.distance * 0.45)
    cpu.resize(48, 48)
    ys, xs = np.mgrid[0:48, 0:48]
    pix = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    return cpu, params, pix


def test_library_computes_in_double():
    assert O.lib64().vvo64_real_bytes() == 8


def test_single_paths_against_the_fp32_oracle(small):
    cpu, params, pix = small
    for k in (0, 5):
        a32 = cpu.trace_pixels(params, pix, k).astype(np.float64)
        a64 = cpu.pixel_sums_fp64(params, pix, k, 1)
        assert (a64[:, 3] == a32[:, 3]).mean() >= 0.99
        rel = np.max(np.abs(a64[:, :3] - a32[:, :3]) / (np.abs(a64[:, :3]) + 1e-5), axis=1)
        assert (rel <= 1e-4).mean() >= 0.60, (rel <= 1e-4).mean()


def test_mean_image_against_the_fp32_oracle(small):
    cpu, params, pix = small
    n = 64
    s64 = cpu.pixel_sums_fp64(params, pix, 0, n)
    s32 = np.zeros_like(s64)
    for k in range(n):
        s32 += cpu.trace_pixels(params, pix, k)
    d = (s64[:, :3] - s32[:, :3]).mean(axis=1) / n
    assert abs(d.mean()) <= 4.0 * d.std() / np.sqrt(d.size) + 1e-9, (d.mean(), d.std())


def test_sums_over_index_ranges_add_up(small):
    cpu, params, pix = small
    sub = pix[::7]
    whole = cpu.pixel_sums_fp64(params, sub, 0, 8)
    parts = cpu.pixel_sums_fp64(params, sub, 0, 4) + cpu.pixel_sums_fp64(params, sub, 4, 4)
    assert np.allclose(whole, parts, rtol=1e-12, atol=1e-12)
