"""Reference operators of the learned denoiser in numpy (float32/float64).

TEST INFRASTRUCTURE ONLY: tests/test_gpu_nn.py compares the CUDA operators of
include/volpt_nn.h (and the U-Net that volview_gb300/learned_denoiser.py
builds from them) against these. The operators have no counterpart in the
reference; they restate their definitions directly: 3x3 convolutions with
zero padding on NHWC tensors, weights [cout][3][3][cin], their input, weight
and bias gradients, 2x2 average pooling, nearest 2x upsampling, channel
concatenation, an L1 loss in log radiance and Adam (Kingma and Ba).
"""
import numpy as np


def _taps(x):
    """(N, H, W, 9, C): x shifted by each tap offset (ky - 1, kx - 1), zero padded."""
    n, h, w, c = x.shape
    p = np.zeros((n, h + 2, w + 2, c), x.dtype)
    p[:, 1:-1, 1:-1] = x
    return np.stack([p[:, ky:ky + h, kx:kx + w] for ky in range(3) for kx in range(3)], axis=3)


def conv3x3(x, w, b=None, relu=False):
    """y[p][co] = sum_tap,ci x[p + tap][ci] w[co][tap][ci] (+ b), float64 sums."""
    t = _taps(np.asarray(x, np.float64))
    y = np.einsum("nhwtc,otc->nhwo", t, np.asarray(w, np.float64).reshape(w.shape[0], 9, -1))
    if b is not None:
        y = y + np.asarray(b, np.float64)
    return np.maximum(y, 0.0) if relu else y


def conv3x3_dgrad(dy, w):
    """The gradient of conv3x3's input."""
    wf = np.asarray(w, np.float64)[:, ::-1, ::-1, :]  # flip the taps
    return conv3x3(dy, np.ascontiguousarray(wf.transpose(3, 1, 2, 0)))


def conv3x3_wgrad(x, dy):
    """dw[co][tap][ci] = sum_p dy[p][co] x[p + tap][ci], shaped (co, 3, 3, ci)."""
    t = _taps(np.asarray(x, np.float64))
    dw = np.einsum("nhwtc,nhwo->otc", t, np.asarray(dy, np.float64))
    return dw.reshape(dw.shape[0], 3, 3, -1)


def avgpool2(x):
    n, h, w, c = x.shape
    return np.asarray(x, np.float64).reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def avgpool2_backward(dy):
    return np.repeat(np.repeat(np.asarray(dy, np.float64), 2, axis=1), 2, axis=2) * 0.25


def upsample2(x):
    return np.repeat(np.repeat(np.asarray(x, np.float64), 2, axis=1), 2, axis=2)


def upsample2_backward(dy):
    n, h, w, c = dy.shape
    return np.asarray(dy, np.float64).reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def features(accum, albedo, normal, spp):
    """(..., 16): log(1 + radiance), albedo, normal means, zeros."""
    a, b, c = (np.asarray(v, np.float64) / spp for v in (accum, albedo, normal))
    z = np.zeros(a.shape[:-1] + (7,))
    return np.concatenate([np.log1p(np.maximum(a[..., :3], 0.0)), b[..., :3], c[..., :3], z], axis=-1)


def l1_loss(pred, target):
    """(loss, dpred) of mean |pred[..., :3] - target| (target: log radiance)."""
    d = np.asarray(pred, np.float64)[..., :3] - np.asarray(target, np.float64)
    g = np.zeros(pred.shape)
    g[..., :3] = np.sign(d) / d.size
    return float(np.abs(d).mean()), g


def adam(w, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    w = w - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return w, m, v


def half(x):
    """Rounds to binary16 and back (the device stores every tensor in FP16)."""
    return np.asarray(x).astype(np.float16).astype(np.float64)


def unet_forward(net, x, rnd=half):
    """The U-Net of volview_gb300.learned_denoiser on NHWC x: returns
    (prediction, activations) with the layers' weights from `net` (a dict
    with "params": name -> (w, b), and "plan"). Sums are float64; every
    stored tensor goes through `rnd` (FP16 rounding, as on the device)."""
    acts = {"input": np.asarray(x, np.float64)}
    for op in net["plan"]:
        kind = op[0]
        if kind == "conv":
            _, name, src, relu = op
            w, b = net["params"][name]
            acts[name] = rnd(conv3x3(acts[src], w, b, relu))
        elif kind == "pool":
            _, name, src = op
            acts[name] = rnd(avgpool2(acts[src]))
        elif kind == "up_cat":
            _, name, src, skip = op
            acts[name] = np.concatenate([upsample2(acts[src]), acts[skip]], axis=-1)
    return acts[net["plan"][-1][1]], acts


def unet_backward(net, acts, dpred, rnd=half):
    """Gradients {name: (dw, db)} of the U-Net for the prediction gradient,
    every stored gradient tensor through `rnd`."""
    grads, d = {}, {net["plan"][-1][1]: np.asarray(dpred, np.float64)}

    def add(name, g):
        g = rnd(g)
        d[name] = rnd(d[name] + g) if name in d else g

    for op in reversed(net["plan"]):
        kind, name = op[0], op[1]
        if name not in d:
            continue
        dy = d.pop(name)
        if kind == "conv":
            _, _, src, relu = op
            if relu:
                dy = dy * (acts[name] > 0)
            w, _ = net["params"][name]
            grads[name] = (conv3x3_wgrad(acts[src], dy), dy.sum(axis=(0, 1, 2)))
            if src != "input":
                add(src, conv3x3_dgrad(dy, w))
        elif kind == "pool":
            add(op[2], avgpool2_backward(dy))
        elif kind == "up_cat":
            _, _, src, skip = op
            cs = acts[src].shape[-1]
            add(src, upsample2_backward(dy[..., :cs]))
            add(skip, dy[..., cs:])
    return grads
