"""Edge cases of the CUDA path against the oracle (GPU): a volume whose
dimensions are not multiples of the 8^3 bricks (ragged bricks, anisotropic
spacing) rendered at an odd image size, labels that draw nothing, and the
size limits of the C ABI. Tolerances as in test_gpu_parity.py."""
import numpy as np
import pytest

from oracle import oracle as O
from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ragged(gpu_ctx):
    hu, lab = scene.small_phantom(seed=4, n=48)
    hu, lab = np.ascontiguousarray(hu[5:42, 9:38, 13:34]), np.ascontiguousarray(lab[5:42, 9:38, 13:34])
    spacing = (2.1, 1.3, 2.9)  # x, y, z mm: 21 x 29 x 37 voxels
    vol = abi.volume_struct(hu, spacing)
    tf = abi.tf_struct(abi.PRESETS["bone"])
    labels = scene.label_params(lab, hu, scene.SMALL_ENTRIES)
    soft = scene.soft_grid(lab, spacing, 1, 3.0, np.float32)
    cfg = dict(hu=hu, labels_vol=lab, spacing=spacing, volume=vol, tf=tf, label_params=labels, soft=soft,
               min_spacing=min(spacing))
    gpu = R.Renderer(gpu_ctx, vol, tf)
    gpu.set_labels(lab, abi.soft_struct(soft))
    cpu = O.CpuRenderer(vol, tf, hu)
    cpu.set_labels(lab, soft)
    p = scene.frame_params_for(cfg, list(gpu.center), gpu.diagonal, clip_sagittal=True)
    p.camera.distance = abi.f32(p.camera.distance * 0.5)
    gpu.resize(33, 17)
    cpu.resize(33, 17)
    yield cfg, gpu, cpu, p
    gpu.destroy()


def test_ragged_volume_passes(ragged):
    cfg, gpu, cpu, p = ragged
    assert gpu.dims == (21, 29, 37)
    assert np.array_equal(gpu.read_volume(abi.VOLUME_DENSITY), cpu.density)
    assert np.array_equal(gpu.read_volume(abi.VOLUME_NORMALS), cpu.normals)
    assert np.array_equal(gpu.pack_uniforms(p, 1), cpu.uniforms(p, 1, 33, 17))
    gpu.probe_bspline(p, np.zeros((1, 3), np.float32))  # runs the mask and majorant passes
    cpu.prepare(p, 33, 17)
    m_gpu = gpu.read_volume(abi.VOLUME_MASK)
    d = np.abs(m_gpu.astype(np.int32) - cpu.mask.astype(np.int32))
    assert d.max() <= 1 and (d == 0).mean() >= 0.999
    cpu.mask = m_gpu
    u = cpu.uniforms(p, 1, 33, 17)
    maj = np.zeros_like(cpu.majorant)
    O.lib().vvo_majorant(O.ptr(u), O.C.byref(cpu.scene()), O.ptr(maj))
    assert np.array_equal(gpu.read_volume(abi.VOLUME_MAJORANT), maj)


def test_ragged_volume_paths(ragged):
    """Replays and the accumulated image at 33 x 17 pixels over ragged bricks."""
    cfg, gpu, cpu, p = ragged
    gpu.probe_bspline(p, np.zeros((1, 3), np.float32))
    cpu.adopt(mask=gpu.read_volume(abi.VOLUME_MASK), majorant=gpu.read_volume(abi.VOLUME_MAJORANT))
    ys, xs = np.mgrid[0:17, 0:33]
    pix = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    a = gpu.probe_paths(p, 3, pix)
    b = np.stack([cpu.trace_pixel(p, int(x), int(y), 3) for x, y in pix])
    rel = np.max(np.abs(a[:, :3] - b[:, :3]) / (np.abs(b[:, :3]) + 1e-5), axis=1)
    assert (rel <= 1e-4).mean() >= 0.7 and (rel > 1e-2).mean() <= 0.15
    assert (a[:, 3] == b[:, 3]).mean() >= 0.99
    q = abi.FrameParams.from_buffer_copy(bytes(p))
    q.path_tracing.denoiser = abi.DENOISE_OFF
    gpu.record_frames(1, 512, q)
    acc = gpu.read_accumulation()[0]
    cpu.accum_key = O._params_key(q)
    cpu.accumulated = 512
    for f in range(128):
        cpu.record(q, f + 1)
    w = np.array([0.2126, 0.7152, 0.0722], np.float32)
    mg = (acc[..., :3] @ w).mean() / 512
    mc = (cpu.accum[..., :3] @ w).mean() / 128
    assert abs(mg - mc) <= 0.05 * mc + 1e-4


def test_labels_that_draw_nothing(small_cfg, gpu_ctx):
    """Hybrid mode with every label hidden: masks and majorants are zero, every
    primary ray leaves the volume (background coverage 1, no radiance), as in
    the oracle."""
    cfg = small_cfg
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
    for i in range(abi.VV_LABEL_COUNT if hasattr(abi, "VV_LABEL_COUNT") else 256):
        p.labels.colors[i][3] = 0.0
    p.path_tracing.denoiser = abi.DENOISE_OFF
    r.resize(24, 16)
    r.record(1, p)
    assert not r.read_volume(abi.VOLUME_MAJORANT).any()
    acc, alb, nor = r.read_accumulation()
    assert np.all(acc[..., 3] == 1.0) and np.all(acc[..., :3] == 0.0)
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    cpu.resize(24, 16)
    cpu.record(p, 1)
    assert np.array_equal(acc, cpu.accum) and np.array_equal(alb, cpu.albedo) and np.array_equal(nor, cpu.normal)
    r.destroy()


def test_size_limits(small_cfg, gpu_ctx):
    cfg = small_cfg
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    for w, h in ((0, 8), (8, 0), (16385, 1), (1, 16385)):
        with pytest.raises(R.VolptError) as e:
            r.resize(w, h)
        assert e.value.status == abi.VV_ERR_ARG
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
    with pytest.raises(R.VolptError) as e:
        r.record(1, p)  # no successful resize yet
    assert e.value.status == abi.VV_ERR_STATE
    r.resize(1, 1)  # the smallest image
    r.record(1, p)
    assert r.read_output().shape == (1, 1, 4)
    r.destroy()
