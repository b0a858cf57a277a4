"""Parity on the workloads the benchmark names, at their full sizes (GPU).

* The small phantom: 128^3 int16 HU at 1 mm, 10 labels with an FP32 soft
  margin, 256x256, the bone preset, one key light, the CLI's default view.
  Density and normals bit-exact, masks within one RG16 quantum (>= 99.9%
  exact), majorants bit-exact on the device's masks; single-path replays on a
  64x64 grid of pixels spread over the image; the converged image (1024 paths
  per pixel on the GPU, 256 independent ones from the oracle) within 3 sigma.
* The head/neck phantom the benchmark times: 512x512x400 at 0.5x0.5x1 mm,
  120 labels, the skeleton ghosted, FP16 soft margin, 1024x1024, sagittal
  clip. Density and normals bit-exact and majorants bit-exact on the device's
  masks (the mask pass is checked on the smaller scenes); single-path replays
  on 2048 pixels spread over the phantom's part of the image; a 64x64 crop of
  the converged image (1024 paths per pixel on the GPU, 256 from the oracle)
  within 3 sigma.

Bars as in tests/parity_util.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parity_util import adopt_device_inputs, all_pixels, check_replays, converged
from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu


def _pair(ctx, cfg, params_fn):
    gpu = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    gpu.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    params = params_fn(cfg, list(gpu.center), gpu.diagonal)
    gpu.resize(cfg["width"], cfg["height"])
    cpu.resize(cfg["width"], cfg["height"])
    return gpu, cpu, params


# ------------------------------------------------------------- small phantom
@pytest.fixture(scope="module")
def small_full(gpu_ctx):
    cfg = scene.small_config()  # 128^3, 256x256
    gpu, cpu, params = _pair(gpu_ctx, cfg, lambda c, ctr, diag: scene.frame_params_for(c, ctr, diag))
    yield cfg, gpu, cpu, params
    gpu.destroy()


def test_small_phantom_volumes(small_full):
    cfg, gpu, cpu, params = small_full
    assert np.array_equal(gpu.read_volume(abi.VOLUME_DENSITY), cpu.density)
    assert np.array_equal(gpu.read_volume(abi.VOLUME_NORMALS), cpu.normals)
    gpu.probe_bspline(params, np.zeros((1, 3), np.float32))  # record's mask and majorant passes
    cpu.prepare(params, cfg["width"], cfg["height"])
    m_gpu = gpu.read_volume(abi.VOLUME_MASK)
    d = np.abs(m_gpu.astype(np.int32) - cpu.mask.astype(np.int32))
    assert d.max() <= 1 and (d == 0).mean() >= 0.999
    cpu.adopt(mask=m_gpu)
    u = cpu.uniforms(params, 1, cfg["width"], cfg["height"])
    maj = np.zeros_like(cpu.majorant)
    O.lib().vvo_majorant(O.ptr(u), O.C.byref(cpu.scene()), O.ptr(maj))
    assert np.array_equal(gpu.read_volume(abi.VOLUME_MAJORANT), maj)


def test_small_phantom_replays(small_full):
    cfg, gpu, cpu, params = small_full
    adopt_device_inputs(gpu, cpu, params)
    grid = all_pixels(64, 64) * 4 + 2  # 64x64 pixels spread over the 256x256 image
    check_replays(gpu, cpu, params, grid, label="small phantom 128^3")


def test_small_phantom_converged(small_full):
    cfg, gpu, cpu, params = small_full
    converged(gpu, cpu, params, cfg["width"], cfg["height"], n_gpu=1024, n_cpu=256, label="small phantom 128^3")


# ------------------------------------------------------- head/neck phantom
@pytest.fixture(scope="module")
def head_neck(gpu_ctx):
    cfg = scene.head_neck_config()  # 512x512x400, 1024x1024
    gpu, cpu, params = _pair(gpu_ctx, cfg, lambda c, ctr, diag: scene.frame_params_for(
        c, ctr, diag, clip_sagittal=True, anisotropy=0.6, spf=1))
    yield cfg, gpu, cpu, params
    gpu.destroy()


def test_head_neck_volumes(head_neck):
    cfg, gpu, cpu, params = head_neck
    assert np.array_equal(gpu.read_volume(abi.VOLUME_DENSITY), cpu.density)
    assert np.array_equal(gpu.read_volume(abi.VOLUME_NORMALS), cpu.normals)
    adopt_device_inputs(gpu, cpu, params)
    u = cpu.uniforms(params, 1, cfg["width"], cfg["height"])
    assert np.array_equal(gpu.pack_uniforms(params, 1), u)
    maj = np.zeros_like(cpu.majorant)
    O.lib().vvo_majorant(O.ptr(u), O.C.byref(cpu.scene()), O.ptr(maj))
    assert np.array_equal(cpu.majorant, maj)


def _phantom_pixels(gpu, params, n, seed=3):
    """n pixels where the phantom is in view (primary rays that do not escape in
    a one-path probe of a coarse grid), spread over the image."""
    W, H = gpu.width, gpu.height
    grid = all_pixels(W // 8, H // 8) * 8 + 4
    first = gpu.probe_paths(params, 0, grid)
    inside = grid[first[:, 3] == 0.0]
    rng = np.random.default_rng(seed)
    pick = inside[rng.choice(len(inside), size=min(n, len(inside)), replace=False)]
    return np.ascontiguousarray(pick + rng.integers(-3, 4, size=pick.shape), np.int32)


def test_head_neck_replays(head_neck):
    cfg, gpu, cpu, params = head_neck
    adopt_device_inputs(gpu, cpu, params)
    pixels = _phantom_pixels(gpu, params, 2048)
    assert len(pixels) >= 1024
    check_replays(gpu, cpu, params, pixels, label="head/neck 512x512x400")


def test_head_neck_converged_crop(head_neck):
    cfg, gpu, cpu, params = head_neck
    W, H = cfg["width"], cfg["height"]
    x0, y0 = W // 2 - 32, H // 2 - 32
    crop = all_pixels(64, 64) + np.array([x0, y0], np.int32)
    converged(gpu, cpu, params, W, H, pixels=crop, n_gpu=1024, n_cpu=256, label="head/neck 64x64 crop")
