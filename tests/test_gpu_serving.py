"""The render-request loop on the device (GPU): a request's result is the same
alone, in a mix of concurrent requests on other volumes, sizes and paths per
pixel, and on a renderer reused from another request of its volume.

Tolerance: the accumulation within 1e-5 relative (a pass of several frames
adds them with float atomics, in an order the device decides), every RGBA8
value within 1 of the lone render's and >= 99.9 % exact.
"""
import numpy as np
import pytest

from volview_gb300 import abi, scene
from volview_gb300 import serving as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def volumes():
    return {"small": scene.small_config(n=48, size=48, spp=4),
            "torso": scene.torso_config(dims=(64, 64, 100), width=64, height=48)}


def _params(cfg, yaw=0.0, clip=True, hidden=()):
    from oracle import oracle as O
    g = O.geometry(cfg["volume"])
    p = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=clip)
    p.camera.yaw = abi.f32(p.camera.yaw + yaw)
    for label in hidden:
        p.labels.colors[label][3] = 0.0
    return p


def _serve(volumes, requests, budget=60 << 30, max_active=None, **kw):
    make, base = S.renderer_factory(volumes)
    srv = S.Server(make, base, budget, max_active=max_active, keep_accumulation=True, **kw)
    try:
        for q in requests:
            srv.submit(q)
        while srv.queue or srv.active:
            srv.step()
        return requests, srv.created
    finally:
        srv.close()


def _same(a, b):
    acc_a, acc_b = a.accumulation[0], b.accumulation[0]
    assert np.all(np.abs(acc_a - acc_b) <= 1e-5 * np.abs(acc_a) + 1e-7)
    d = np.abs(a.image.astype(np.int32) - b.image.astype(np.int32))
    assert d.max() <= 1 and (d == 0).mean() >= 0.999


def test_same_alone_in_a_mix_and_on_a_reused_renderer(volumes):
    def target():
        return S.Request("small", 64, 48, 32, _params(volumes["small"], yaw=0.3, hidden=(2,)))

    alone, _ = _serve(volumes, [target()])
    mix = [S.Request("torso", 96, 64, 64, _params(volumes["torso"], yaw=-0.5)),
           S.Request("small", 40, 40, 16, _params(volumes["small"], clip=False)),
           target(),
           S.Request("torso", 32, 32, 128, _params(volumes["torso"], hidden=(1, 4)))]
    mixed, created = _serve(volumes, mix)
    assert created == 4  # all four in flight at once, each on its own renderer
    assert all(q.image is not None and q.image.shape == (q.height, q.width, 4) for q in mixed)
    reused, created = _serve(volumes, [S.Request("small", 80, 80, 48, _params(volumes["small"], yaw=-0.2)),
                                       target()], max_active=1)
    assert created == 1  # the second request ran on the first one's renderer
    _same(alone[0], mixed[2])
    _same(alone[0], reused[1])


def test_device_memory_matches_the_model(volumes):
    make, base = S.renderer_factory(volumes)
    r = make("small")
    try:
        b0 = r.device_bytes()
        assert b0 >= S.volume_bytes(volumes["small"]["volume"].dims)
        p = _params(volumes["small"])
        r.resize(64, 48)
        r.record_frames(1, 32, p)
        r.synchronize()
        assert r.idle()
        grown = r.device_bytes() - b0
        model = S.request_bytes(64, 48, 32)
        assert 0.9 * model <= grown <= 1.3 * model, (grown, model)
    finally:
        r.destroy()


def test_same_under_a_pass_budget(volumes):
    """Renderers with two passes in flight of up to 8 frames' worth of path
    slots (vv_set_pass_budget) give the same result as the default six passes
    of 16, alone and in a mix, and hold less device memory."""
    def target():
        return S.Request("small", 64, 48, 96, _params(volumes["small"], yaw=0.2))

    full, _ = _serve(volumes, [target()])
    mix = [S.Request("torso", 96, 64, 64, _params(volumes["torso"], yaw=-0.5)), target()]
    lean, _ = _serve(volumes, mix, passes=2, slot_frames=8)
    _same(full[0], lean[1])
    make, base = S.renderer_factory(volumes)
    a, b = make("small"), make("small")
    try:
        b.set_pass_budget(2, 8)
        for r in (a, b):
            r.resize(256, 256)
            r.record_frames(1, 128, _params(volumes["small"]))
            r.synchronize()
        assert b.device_bytes() < a.device_bytes()
        with pytest.raises(Exception):
            b.set_pass_budget(7, 8)
        with pytest.raises(Exception):
            b.set_pass_budget(2, 0)
    finally:
        a.destroy()
        b.destroy()
