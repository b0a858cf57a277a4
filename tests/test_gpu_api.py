"""Behaviour of the C ABI as the render crate defines it (GPU)."""
import numpy as np
import pytest

from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu


@pytest.fixture()
def rend(small_cfg, gpu_ctx):
    cfg = small_cfg
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
    yield cfg, r, p
    r.destroy()


def test_record_before_resize_is_a_state_error(rend):
    cfg, r, p = rend
    with pytest.raises(R.VolptError) as e:
        r.record(1, p)
    assert e.value.status == abi.VV_ERR_STATE


def test_label_size_mismatch(rend):
    cfg, r, p = rend
    with pytest.raises(R.VolptError) as e:
        r.set_labels(np.zeros(10, np.uint8))
    assert e.value.status == abi.VV_ERR_ARG


def test_ray_marcher_leaves_the_accumulation_alone(rend):
    """record with path tracing off draws with the ray marcher: the path
    tracer's accumulation neither grows nor restarts (renderer.rs:1536-1545,
    1789-1794)."""
    cfg, r, p = rend
    r.resize(16, 16)
    r.record(1, p)
    r.record(2, p)
    assert r.accumulated_samples() == 2
    q = abi.FrameParams.from_buffer_copy(bytes(p))
    q.path_tracing.enabled = 0
    r.record(3, q)
    assert r.accumulated_samples() == 2
    img = r.read_output()
    assert img[..., :3].std() > 0
    r.record(4, p)
    assert r.accumulated_samples() == 3


def test_accumulation_keys(rend):
    cfg, r, p = rend
    r.resize(32, 32)
    r.record(1, p)
    r.record(2, p)
    assert r.accumulated_samples() == 2
    p.path_tracing.denoiser = abi.DENOISE_OFF  # display only: keeps accumulating
    r.record(3, p)
    assert r.accumulated_samples() == 3
    p.camera.yaw = 0.3
    r.record(4, p)
    assert r.accumulated_samples() == 1
    p.path_tracing.samples_per_frame = 3
    r.record(5, p)
    assert r.accumulated_samples() == 3


def test_record_frames_equals_records(small_cfg, gpu_ctx):
    cfg = small_cfg
    out = []
    for batched in (False, True):
        r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
        p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
        p.path_tracing.denoiser = abi.DENOISE_OFF
        r.resize(40, 24)
        if batched:
            r.record_frames(1, 6, p)
        else:
            for f in range(1, 7):
                r.record(f, p)
        assert r.accumulated_samples() == 6
        out.append(r.read_accumulation()[0])
        r.destroy()
    a, b = out
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("kernel", ["persistent", "wavefront"])
def test_tracers_agree_with_reference_shaped_kernel(small_cfg, gpu_ctx, monkeypatch, kernel):
    """The persistent and wavefront tracers replay the one-thread-per-pixel
    kernel's paths (same random streams, same stage code)."""
    cfg = small_cfg
    out = []
    for kernel in ("frame", kernel):
        monkeypatch.setenv("VV_PT_KERNEL", kernel)
        r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
        p = scene.frame_params_for(cfg, list(r.center), r.diagonal, spf=2)
        r.resize(48, 40)
        r.record(1, p)
        r.record(2, p)
        out.append(r.read_accumulation()[0])
        r.destroy()
    ok = np.all(np.abs(out[0] - out[1]) <= 1e-4 * np.abs(out[1]) + 1e-6, axis=-1)
    assert ok.mean() >= 0.98


def test_render_to_rgba(small_cfg, gpu_ctx):
    cfg = small_cfg
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
    img = R.render_to_rgba(r, p, 64, 48, 4)
    assert img.shape == (48, 64, 4)
    assert (img[..., 3] == 255).all()
    assert r.accumulated_samples() == 4
    assert img[..., :3].std() > 0  # something was drawn
    r.destroy()


def test_record_frames_runs_long_calls_as_several_passes(rend):
    """70 frames at 2048x1024 take two passes (at most 64 frames each): all 70
    are accumulated, as 70 single-frame records would."""
    cfg, r, p = rend
    r.resize(2048, 1024)
    before = r.kernel_launches()
    r.record_frames(1, 70, p)
    r.synchronize()
    assert r.accumulated_samples() == 70
    assert r.kernel_launches() - before > 2 * 10  # two passes of waves
    acc, _, _ = r.read_accumulation(normal=False)
    assert np.isfinite(acc).all() and acc[..., 3].max() <= 70.0


def test_rmse_estimate_matches_a_converged_render(rend):
    """The RMSE the time-to-RMSE latencies use, estimated from the accumulation,
    against the error of the same image measured on a 64x longer render."""
    from volview_gb300 import convergence as CV
    cfg, r, p = rend
    p.path_tracing.denoiser = abi.DENOISE_OFF
    r.resize(64, 48)
    r.record_frames(1, 64, p)
    acc, alb, _ = r.read_accumulation()
    est = CV.rmse_estimate(acc, alb, 64)
    lum64 = acc[..., :3].astype(np.float64) @ CV.LUMA / 64
    r.record_frames(65, 4096 - 64, p)
    assert r.accumulated_samples() == 4096
    acc2, _, _ = r.read_accumulation()
    lum4096 = acc2[..., :3].astype(np.float64) @ CV.LUMA / 4096
    # The long render contains the short one: the difference's expected
    # square is (63/64)^2 (s^2/64 + s^2/4032) = 0.984 s^2/64.
    actual = np.sqrt(np.mean((lum64 - lum4096) ** 2)) / np.sqrt(0.984)
    assert est > 0
    assert abs(est / actual - 1.0) < 0.1


def test_environment_map_restarts_accumulation_and_falls_back(rend):
    """set_environment_map restarts the accumulation (renderer.rs:1299);
    Environment::Map without a map renders the studio (renderer.rs:1524-1527)."""
    cfg, r, p = rend
    r.resize(32, 24)
    p.lighting.environment = abi.ENV_MAP
    studio = abi.FrameParams.from_buffer_copy(bytes(p))
    studio.lighting.environment = abi.ENV_STUDIO
    assert np.array_equal(r.pack_uniforms(p, 1), r.pack_uniforms(studio, 1))  # no map yet
    r.record(1, p)
    r.record(2, p)
    assert r.accumulated_samples() == 2
    r.set_environment_map(abi.env_struct(scene.synthetic_light_map()))
    assert not np.array_equal(r.pack_uniforms(p, 1), r.pack_uniforms(studio, 1))
    r.record(3, p)
    assert r.accumulated_samples() == 1
    r.set_environment_map(None)
    assert np.array_equal(r.pack_uniforms(p, 1), r.pack_uniforms(studio, 1))
    big = np.zeros((4, 16385, 3), np.float32)
    with pytest.raises(R.VolptError) as e:
        r.set_environment_map(abi.env_struct(big))
    assert e.value.status == abi.VV_ERR_LIMIT
