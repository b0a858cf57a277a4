"""The reference's other rendering modes on the GPU against the oracle (GPU).

scene.MODE_CASES: label modes Off, Tint and Isolate with hidden labels
(common.glsl:232-351), ghosted labels and their shells (pt.comp:286-289,
shading.glsl:73-144), binary label masks without a soft grid
(mask.comp:107-138), the Dome environment (pt.comp:56-82) and the thin lens
(pt.comp:406-416), each on the 48^3 phantom at 48x48 with a sagittal clip. The
oracle itself is pinned to the reference's shaders compiled as CPU code in each
of these modes (tests/test_oracle_pinned.py, tests/golden/small_modes.npz).

Tolerances: masks within one RG16 quantum and >= 99.9% exact (binary masks:
bit-exact; the soft masks call expf); majorants bit-exact on the device's
masks; single-path replays and the converged image at the bars of
tests/parity_util.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from parity_util import adopt_device_inputs, all_pixels, check_replays, converged, make_params
from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=scene.MODE_CASES)
def mode_pair(request, small_cfg, gpu_ctx):
    cfg = small_cfg
    case = request.param
    gpu = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    params = make_params(cfg, list(gpu.center), gpu.diagonal, clip_sagittal=True)
    soft = scene.mode_case(case, params, list(gpu.center))
    gpu.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]) if soft else None)
    cpu.set_labels(cfg["labels_vol"], cfg["soft"] if soft else None)
    gpu.resize(48, 48)
    cpu.resize(48, 48)
    yield case, soft, gpu, cpu, params
    gpu.destroy()


def test_mode_uniforms_bit_exact(mode_pair):
    case, soft, gpu, cpu, params = mode_pair
    a = gpu.pack_uniforms(params, 1)
    b = cpu.uniforms(params, 1, 48, 48)
    assert np.array_equal(a, b), np.nonzero(a != b)[0][:16]


def test_mode_masks_and_majorant(mode_pair, small_cfg):
    case, soft, gpu, _, params = mode_pair
    cfg = small_cfg
    gpu.probe_bspline(params, np.zeros((1, 3), np.float32))  # runs record's mask and majorant passes
    cpu = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    cpu.set_labels(cfg["labels_vol"], cfg["soft"] if soft else None)
    cpu.prepare(params, 48, 48)
    if int(params.labels.mode) != abi.LABEL_OFF:
        m_gpu = gpu.read_volume(abi.VOLUME_MASK)
        d = np.abs(m_gpu.astype(np.int32) - cpu.mask.astype(np.int32))
        assert d.max() <= 1
        if soft:
            assert (d == 0).mean() >= 0.999
        else:
            assert d.max() == 0, f"binary masks differ in {(d != 0).mean():.5f} of values"
        cpu.mask = m_gpu
    u = cpu.uniforms(params, 1, 48, 48)
    maj = np.zeros_like(cpu.majorant)
    O.lib().vvo_majorant(O.ptr(u), O.C.byref(cpu.scene()), O.ptr(maj))
    assert np.array_equal(gpu.read_volume(abi.VOLUME_MAJORANT), maj)


def test_mode_single_path_replays(mode_pair):
    case, soft, gpu, cpu, params = mode_pair
    adopt_device_inputs(gpu, cpu, params)
    check_replays(gpu, cpu, params, all_pixels(48, 48), label=case)


def test_mode_converged_image(mode_pair):
    case, soft, gpu, cpu, params = mode_pair
    converged(gpu, cpu, params, 48, 48, label=case)
