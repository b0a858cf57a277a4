"""The learned denoiser's layer plan and its numpy oracle (CPU): the plan's
channel counts are ones the tensor-core operators take, and the oracle's
U-Net gradients agree with finite differences of its loss."""
import numpy as np

from oracle import nn_ref as N
from volview_gb300 import learned_denoiser as LD

CONV_OUT = {8, 16, 32, 48, 64, 80, 96, 112, 144, 176}  # vv_nn_conv3x3's output channel counts


def test_plan_fits_the_operators():
    ch, shapes = LD.channels()
    assert shapes["e0a"] == (LD.IN_CHANNELS, LD.LEVELS[0]) and shapes["head"] == (LD.LEVELS[0], LD.OUT_CHANNELS)
    for name, (cin, cout) in shapes.items():
        assert cin % 16 == 0 and cout in CONV_OUT, name  # forward
        if name != "e0a":
            assert cout % 16 == 0 and cin in CONV_OUT, name  # input gradient: cin and cout swap
    ups = [op for op in LD.plan() if op[0] == "up_cat"]
    assert [ch[op[1]] for op in ups] == [176, 144, 112, 80]
    assert LD.PAD % (16 << (len(LD.LEVELS) - 1)) == 0  # the coarsest rows hold whole 16-pixel tiles


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    plan = LD.plan()
    _, shapes = LD.channels()
    params = {n: (rng.standard_normal((co, 3, 3, ci)) * 0.1, rng.standard_normal(co) * 0.01)
              for n, (ci, co) in shapes.items()}
    net = {"plan": plan, "params": params}
    x = rng.standard_normal((1, 256, 256, 16)) * 0.5
    ident = lambda a: np.asarray(a, np.float64)  # noqa: E731 (no FP16 rounding: exact gradients)
    y, acts = N.unet_forward(net, x, rnd=ident)
    target = rng.standard_normal(y.shape[:-1] + (3,))
    loss, dy = N.l1_loss(y, target)
    grads = N.unet_backward(net, acts, dy, rnd=ident)
    for name, idx in (("e2a", (3, 1, 2, 5)), ("d1b", (7, 0, 0, 11)), ("head", (1, 2, 1, 4))):
        w, b = params[name]
        w2 = w.copy()
        w2[idx] += 1e-4
        y2, _ = N.unet_forward({"plan": plan, "params": dict(params, **{name: (w2, b)})}, x, rnd=ident)
        fd = (N.l1_loss(y2, target)[0] - loss) / 1e-4
        assert abs(fd - grads[name][0][idx]) <= 2e-3 * max(abs(fd), 1e-3), (name, fd, grads[name][0][idx])
