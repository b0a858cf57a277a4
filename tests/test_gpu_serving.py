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


# ------------------------------------------------------------ batched passes
def _alone(cfg, params, w, h, spp, env=None):
    """A request rendered by a renderer of its own with vv_record_frames."""
    from volview_gb300 import renderer as R
    ctx = R.Context(0)
    r = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    try:
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]) if cfg.get("soft") is not None else None)
        if env is not None:
            r.set_environment_map(abi.env_struct(env))
        r.resize(w, h)
        r.record_frames(1, spp, params)
        r.synchronize()
        return r.read_accumulation()[0], r.read_output()
    finally:
        r.destroy()
        ctx.destroy()


class _Result:
    def __init__(self, acc, image):
        self.accumulation, self.image = (acc,), image


def test_batched_pass_matches_record_frames(volumes):
    """Two views of one volume in the same batched passes (different image
    sizes, paths per pixel, cameras, hidden labels, and one with the light map
    while the other has the studio light) give each request the result of a
    renderer of its own: the same paths, summed in another order."""
    from volview_gb300 import renderer as R
    cfg = volumes["small"]
    env = scene.synthetic_light_map()
    p1 = _params(cfg, yaw=0.3, hidden=(2,))
    p2 = _params(cfg, yaw=-0.4, clip=False)
    p2.lighting.environment = abi.ENV_MAP
    ref1 = _alone(cfg, p1, 64, 48, 40)
    ref2 = _alone(cfg, p2, 40, 40, 24, env=env)
    ctx = R.Context(0)
    base = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    base.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    base.set_environment_map(abi.env_struct(env))
    ctxs = [R.Context(0), R.Context(0)]
    views = [R.Renderer.view(c, base) for c in ctxs]
    engine = R.BatchEngine(ctx, passes=2, slot_frames=16)
    try:
        views[0].resize(64, 48)
        views[1].resize(40, 40)
        # Passes of 16 frames: request 1 takes three, request 2 two (the
        # second with 8 frames, then its display), request 1 alone last.
        engine.record([(views[0], p1, 1, 16, False), (views[1], p2, 1, 16, False)])
        engine.record([(views[0], p1, 17, 16, False), (views[1], p2, 17, 8, True)])
        engine.record([(views[0], p1, 33, 8, True)])
        for v in views:
            v.synchronize()
        assert views[0].accumulated_samples() == 40 and views[1].accumulated_samples() == 24
        _same(_Result(*ref1), _Result(views[0].read_accumulation()[0], views[0].read_output()))
        _same(_Result(*ref2), _Result(views[1].read_accumulation()[0], views[1].read_output()))
        assert engine.kernel_launches() > 0 and engine.in_flight() == 0
    finally:
        engine.destroy()
        for v in views:
            v.destroy()
        base.destroy()
        for c in ctxs + [ctx]:
            c.destroy()


def test_views_share_the_volume_and_guard_it(volumes):
    from volview_gb300 import renderer as R
    cfg = volumes["torso"]
    ctx = R.Context(0)
    base = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    base.set_labels(cfg["labels_vol"], None)
    view = R.Renderer.view(ctx, base)
    fp16 = R.Renderer(ctx, cfg["volume"], cfg["tf"], abi.precision(density_format=abi.DENSITY_FP16))
    engine = R.BatchEngine(ctx)
    try:
        assert np.array_equal(view.read_volume(abi.VOLUME_DENSITY), base.read_volume(abi.VOLUME_DENSITY))
        assert np.array_equal(view.read_volume(abi.VOLUME_LABELS), base.read_volume(abi.VOLUME_LABELS))
        shared = S.volume_bytes(cfg["volume"].dims) - S.view_volume_bytes(cfg["volume"].dims)
        assert base.device_bytes() - view.device_bytes() >= 0.9 * shared
        for call in (lambda: view.set_transfer_function(cfg["tf"]), lambda: base.set_labels(cfg["labels_vol"]),
                     lambda: view.set_environment_map(None), lambda: base.destroy()):
            with pytest.raises(R.VolptError) as e:
                call()
            assert e.value.status == abi.VV_ERR_STATE
        p = _params(cfg)
        view.resize(32, 32)
        fp16.resize(32, 32)
        for items in ([(view, p, 1, 0, True)], [(view, p, 1, 65, True)], [(view, p, 1, 4, True)] * 2,
                      [(view, p, 1, 4, True), (fp16, p, 1, 4, True)], [(fp16, p, 1, 4, True)]):
            with pytest.raises(R.VolptError) as e:
                engine.record(items)
            assert e.value.status == abi.VV_ERR_ARG
    finally:
        engine.destroy()
        fp16.destroy()
        view.destroy()
        base.destroy()
        ctx.destroy()


def test_batched_server_same_alone_and_in_a_mix(volumes):
    """The batched serving loop: a request's result equals its lone render
    through vv_record_frames, with requests of two volumes, several sizes and
    paths per pixel in flight, one view per concurrent request and one base
    per volume."""
    def target():
        return S.Request("small", 64, 48, 40, _params(volumes["small"], yaw=0.3, hidden=(2,)))

    alone, _ = _serve(volumes, [target()])
    mix = [S.Request("torso", 96, 64, 64, _params(volumes["torso"], yaw=-0.5)),
           S.Request("small", 40, 40, 16, _params(volumes["small"], clip=False)),
           target(),
           S.Request("small", 32, 32, 100, _params(volumes["small"], yaw=1.0)),
           S.Request("torso", 32, 32, 24, _params(volumes["torso"], hidden=(1, 4)))]
    make_base, make_view, engine, base, view, reserve = S.batched_factory(volumes)
    srv = S.BatchedServer(make_base, make_view, engine, 60 << 30, base, view, reserve, keep_accumulation=True,
                          frames_per_pass=16)
    try:
        for q in mix:
            srv.submit(q)
        while srv.queue or srv.active:
            srv.step()
        assert all(q.image is not None and q.image.shape == (q.height, q.width, 4) for q in mix)
        assert len(srv.bases) == 2 and srv.created == 5
        assert max(srv.batch_sizes) >= 2  # requests shared passes
        _same(alone[0], mix[2])
    finally:
        srv.close()


def test_one_engine_pass_alternates_and_mixes_volumes(volumes):
    """One engine pass (its path state and later-flight bins) serving two
    volumes of different sizes in turn, then both in the same passes: each
    request still gets its lone render's result."""
    from volview_gb300 import renderer as R
    ctx = R.Context(0)
    engine = R.BatchEngine(ctx, passes=1, slot_frames=16)
    bases, views, refs, reqs = [], [], [], []
    try:
        for name, yaw in (("small", 0.2), ("torso", -0.3), ("small", 0.5), ("torso", 0.9)):
            cfg = volumes[name]
            p = _params(cfg, yaw=yaw)
            refs.append(_alone(cfg, p, 48, 40, 32))
            base = R.Renderer(ctx, cfg["volume"], cfg["tf"])
            base.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]) if cfg.get("soft") is not None else None)
            view = R.Renderer.view(ctx, base)
            view.resize(48, 40)
            bases.append(base)
            views.append(view)
            reqs.append(p)
        engine.record([(views[0], reqs[0], 1, 16, False)])  # small alone, then torso alone
        engine.record([(views[1], reqs[1], 1, 16, False)])
        engine.record([(views[2], reqs[2], 1, 16, False), (views[3], reqs[3], 1, 16, False)])  # mixed
        engine.record([(v, p, 17, 16, True) for v, p in zip(views, reqs)])
        engine.synchronize()
        for v, ref in zip(views, refs):
            v.synchronize()
            _same(_Result(*ref), _Result(v.read_accumulation()[0], v.read_output()))
    finally:
        engine.destroy()
        for v in views:
            v.destroy()
        for b in bases:
            b.destroy()
        ctx.destroy()
