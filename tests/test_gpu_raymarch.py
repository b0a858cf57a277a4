"""The real-time ray marcher (path tracing off) against the reference's own
shaders (GPU): the occlusion volume (ao.comp), the shadow volume swept towards
the key light (shadow.comp with record_shadow_sweep) and the image (dvr.comp),
for point-sampled and pre-integrated transfer functions and a light map,
against tests/golden/small_raymarch.npz (made by tests/golden/make_golden.py
from the reference's shaders compiled as CPU code).

Tolerances: uniforms bit-exact; the half-precision volumes and image within
2e-3 absolute (plus 1e-2 relative) for >= 99 % of their values, and the whole
image's mean radiance within 1 %. The device evaluates expf/powf/sqrtf and
contracts multiply-adds, so last bits differ, and a voxel at the masks'
zero boundary may land one quantum off (see the mask parity test).
"""
import os

import numpy as np
import pytest

from volview_gb300 import abi
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_raymarch.npz")


def _half(a):
    return np.asarray(a).view(np.float16).astype(np.float32)


def _close(a, b, what):
    d = np.abs(a - b)
    ok = d <= 2e-3 + 1e-2 * np.abs(b)
    assert ok.mean() >= 0.99, f"{what}: {ok.mean():.4f} within tolerance, max diff {d.max():.4g}"


@pytest.fixture(scope="module")
def golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("ray marcher fixture not generated")
    return np.load(GOLDEN)


@pytest.mark.parametrize("case", ["point", "preint", "map"])
def test_ray_marcher_matches_reference_shaders(golden, gpu_ctx, case):
    g = golden
    vol = abi.volume_struct(g["hu"], tuple(g["spacing"]))
    tf = abi.tf_struct(abi.PRESETS["bone"])
    r = R.Renderer(gpu_ctx, vol, tf)
    r.set_labels(g["labels"], abi.soft_struct(g["soft"]))
    if case == "map":
        r.set_environment_map(abi.env_struct(g["light_map"]))
    params = abi.FrameParams.from_buffer_copy(g[f"{case}_params"].tobytes())
    assert params.path_tracing.enabled == 0
    W, H = int(g["width"]), int(g["height"])
    r.resize(W, H)
    assert np.array_equal(r.pack_uniforms(params, 1), g[f"{case}_uniforms"])
    r.record(1, params)
    assert r.accumulated_samples() == 0  # the ray marcher accumulates nothing
    ao = _half(r.read_volume(abi.VOLUME_AO))
    shadow = _half(r.read_volume(abi.VOLUME_SHADOW))
    _close(ao, _half(g[f"{case}_ao"]), "occlusion volume")
    _close(shadow, _half(g[f"{case}_shadow"]), "shadow volume")
    hdr, ref = _half(r.read_hdr()), _half(g[f"{case}_hdr"])
    _close(hdr, ref, "image")
    assert abs(hdr[..., :3].mean() - ref[..., :3].mean()) <= 0.01 * ref[..., :3].mean() + 1e-6
    out = r.read_output()
    assert out.shape == (H, W, 4) and out[..., :3].std() > 0
    r.destroy()


def test_ray_marcher_rejects_batched_frames(golden, gpu_ctx):
    g = golden
    vol = abi.volume_struct(g["hu"], tuple(g["spacing"]))
    r = R.Renderer(gpu_ctx, vol, abi.tf_struct(abi.PRESETS["bone"]))
    params = abi.FrameParams.from_buffer_copy(g["point_params"].tobytes())
    r.resize(16, 16)
    with pytest.raises(R.VolptError) as e:
        r.record_frames(1, 4, params)
    assert e.value.status == abi.VV_ERR_ARG
    r.destroy()
