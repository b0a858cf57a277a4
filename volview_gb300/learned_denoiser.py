"""A learned denoiser: a 5-level U-Net on colour, albedo and normal, run and
trained by the tensor-core operators of include/volpt_nn.h.

Input: 16 channels from an accumulation (log(1 + radiance), albedo, normal,
zeros; vv_nn_features). Levels of 32, 48, 64, 80 and 96 channels, two 3x3
convolutions with ReLU each, 2x2 average pooling down, nearest upsampling up,
skip connections by concatenation; a 3x3 head of 16 channels whose first 3
are log(1 + radiance). (A residual connection from the input's log radiance
to the prediction, tried, trained far slower at 4 paths per pixel: the
network then has to cancel the fireflies instead of ignoring them.) FP16 weights and activations, FP32 accumulation in
every convolution, FP32 master weights for Adam, an L1 loss in log radiance
with its gradient scaled by GRAD_SCALE so that FP16 gradients stay normal.

Device memory comes from PyTorch (tensors as buffers, the current CUDA
stream); every arithmetic operation is a kernel of libvolpt.so. Images are
padded to multiples of 256 pixels per axis (the coarsest level's rows must
hold whole 16-pixel tiles).
"""
import ctypes as C

import numpy as np

from . import renderer as R

LEVELS = (32, 48, 64, 80, 96)
IN_CHANNELS, OUT_CHANNELS = 16, 16
GRAD_SCALE = 65536.0
PAD = 256


def plan():
    """The layer plan: ("conv", name, source, relu), ("pool", name, source),
    ("up_cat", name, source, skip); inputs come from the named outputs."""
    ops, src = [], "input"
    for lv, c in enumerate(LEVELS):
        if lv:
            ops.append(("pool", f"p{lv}", src))
            src = f"p{lv}"
        ops += [("conv", f"e{lv}a", src, True), ("conv", f"e{lv}b", f"e{lv}a", True)]
        src = f"e{lv}b"
    for lv in range(len(LEVELS) - 2, -1, -1):
        ops.append(("up_cat", f"u{lv}", src, f"e{lv}b"))
        ops += [("conv", f"d{lv}a", f"u{lv}", True), ("conv", f"d{lv}b", f"d{lv}a", True)]
        src = f"d{lv}b"
    ops.append(("conv", "head", src, False))
    return ops


def channels():
    """Output channels of every tensor in the plan, and each conv's (cin, cout)."""
    ch, shapes = {"input": IN_CHANNELS}, {}
    for op in plan():
        kind, name, src = op[0], op[1], op[2]
        if kind == "conv":
            if name == "head":
                cout = OUT_CHANNELS
            else:
                lv = int(name[1])
                cout = LEVELS[lv]
            shapes[name] = (ch[src], cout)
            ch[name] = cout
        elif kind == "pool":
            ch[name] = ch[src]
        else:
            ch[name] = ch[src] + ch[op[3]]
    return ch, shapes


def _check(status, what):
    if status != 0:
        raise R.VolptError(status, f"{what}: a shape the operators do not take")


class UNet:
    """The network's parameters (FP32 masters, FP16 copies, Adam moments) and
    its forward and backward passes."""

    def __init__(self, seed=0, device="cuda"):
        import torch
        self.torch, self.device = torch, device
        self.lib = R.load()
        self.plan = plan()
        self.ch, self.shapes = channels()
        rng = np.random.default_rng(seed)
        self.params = {}
        for name, (cin, cout) in self.shapes.items():
            real_in = 9 if name == "e0a" else cin  # input channels 9..15 are zeros
            std = np.sqrt(2.0 / (9 * real_in)) * (0.1 if name == "head" else 1.0)
            w = (rng.standard_normal((cout, 3, 3, cin)) * std).astype(np.float32)
            if name == "e0a":
                w[..., 9:] = 0.0
            self.params[name] = self._param(w, np.zeros(cout, np.float32))
        self.steps = 0

    def _param(self, w, b):
        t = self.torch
        p = {"w": t.tensor(w, device=self.device), "b": t.tensor(b, device=self.device)}
        p["w16"] = p["w"].half()
        for k in ("w", "b"):
            p["m" + k] = t.zeros_like(p[k])
            p["v" + k] = t.zeros_like(p[k])
            p["g" + k] = t.zeros_like(p[k])
        return p

    def numpy_params(self):
        """{name: (w, b)} as float64 arrays of the FP16 weights the kernels use."""
        return {n: (p["w16"].float().cpu().numpy().astype(np.float64), p["b"].cpu().numpy().astype(np.float64))
                for n, p in self.params.items()}

    def weights_blob(self):
        """The weights as vv_set_denoiser_weights takes them: every convolution
        in plan order, its weights [cout][3][3][cin] then its biases."""
        parts = []
        for name in self.shapes:
            p = self.params[name]
            parts += [p["w"].float().cpu().numpy().ravel(), p["b"].float().cpu().numpy().ravel()]
        return np.concatenate(parts).astype(np.float32)

    def state(self):
        return {n: (p["w"].cpu().numpy(), p["b"].cpu().numpy()) for n, p in self.params.items()}

    def load_state(self, state):
        for n, (w, b) in state.items():
            p = self.params[n]
            p["w"].copy_(self.torch.tensor(w))
            p["b"].copy_(self.torch.tensor(b))
            p["w16"].copy_(p["w"].half())

    # ------------------------------------------------------------------ passes
    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def forward(self, x):
        """x: (N, H, W, 16) FP16 on the device; returns the head's output and
        keeps the activations for backward."""
        t, s = self.torch, self._stream()
        acts = {"input": x}
        for op in self.plan:
            kind, name, src = op[0], op[1], op[2]
            a = acts[src]
            n, h, w, c = a.shape
            if kind == "conv":
                p = self.params[name]
                cout = self.shapes[name][1]
                y = t.empty((n, h, w, cout), dtype=t.float16, device=self.device)
                _check(self.lib.vv_nn_conv3x3(a.data_ptr(), n, h, w, c, p["w16"].data_ptr(), p["b"].data_ptr(), cout,
                                              int(op[3]), y.data_ptr(), s), name)
            elif kind == "pool":
                y = t.empty((n, h // 2, w // 2, c), dtype=t.float16, device=self.device)
                _check(self.lib.vv_nn_avgpool2(a.data_ptr(), n, h, w, c, y.data_ptr(), 0, s), name)
            else:
                k = acts[op[3]]
                y = t.empty((n, 2 * h, 2 * w, c + k.shape[3]), dtype=t.float16, device=self.device)
                if c % 8 == 0 and k.shape[3] % 8 == 0:  # upsampling and concat in one pass
                    _check(self.lib.vv_nn_upsample_concat(a.data_ptr(), n, h, w, c, k.data_ptr(), k.shape[3],
                                                          y.data_ptr(), s), name)
                else:
                    u = t.empty((n, 2 * h, 2 * w, c), dtype=t.float16, device=self.device)
                    _check(self.lib.vv_nn_upsample2(a.data_ptr(), n, h, w, c, u.data_ptr(), 0, s), name)
                    _check(self.lib.vv_nn_concat(u.data_ptr(), c, k.data_ptr(), k.shape[3], n * 4 * h * w,
                                                 y.data_ptr(), s), name)
            acts[name] = y
        self.acts = acts
        return acts["head"]

    def backward(self, dpred):
        """Weight and bias gradients (into each parameter's gw, gb, zeroed
        first) for the head's output gradient dpred (FP16, scaled)."""
        t, s, acts = self.torch, self._stream(), self.acts
        for p in self.params.values():
            p["gw"].zero_()
            p["gb"].zero_()
        grads = {"head": dpred}

        def add(name, g):
            if name in grads:
                _check(self.lib.vv_nn_add(grads[name].data_ptr(), g.data_ptr(), g.numel(), s), "add")
            else:
                grads[name] = g

        for op in reversed(self.plan):
            kind, name, src = op[0], op[1], op[2]
            if name not in grads:
                continue
            dy = grads.pop(name)
            a = acts[src]
            n, h, w, c = a.shape
            if kind == "conv":
                p = self.params[name]
                cout = self.shapes[name][1]
                if op[3]:
                    _check(self.lib.vv_nn_relu_backward(dy.data_ptr(), acts[name].data_ptr(), dy.numel(), s), name)
                _check(self.lib.vv_nn_conv3x3_wgrad(a.data_ptr(), dy.data_ptr(), n, h, w, c, cout,
                                                    p["gw"].data_ptr(), s), name)
                _check(self.lib.vv_nn_bias_grad(dy.data_ptr(), n * h * w, cout, p["gb"].data_ptr(), s), name)
                if src != "input":
                    wt = t.empty((c, 3, 3, cout), dtype=t.float16, device=self.device)
                    _check(self.lib.vv_nn_flip_weights(p["w16"].data_ptr(), cout, c, wt.data_ptr(), s), name)
                    dx = t.empty_like(a)
                    _check(self.lib.vv_nn_conv3x3(dy.data_ptr(), n, h, w, cout, wt.data_ptr(), None, c, 0,
                                                  dx.data_ptr(), s), name)
                    add(src, dx)
            elif kind == "pool":
                dx = t.empty_like(a)
                _check(self.lib.vv_nn_avgpool2(dy.data_ptr(), n, h, w, c, dx.data_ptr(), 1, s), name)
                add(src, dx)
            else:
                k = acts[op[3]]
                du = t.empty((n, 2 * h, 2 * w, c), dtype=t.float16, device=self.device)
                dk = t.empty_like(k)
                _check(self.lib.vv_nn_split(dy.data_ptr(), c, k.shape[3], n * 4 * h * w, du.data_ptr(),
                                            dk.data_ptr(), s), name)
                dx = t.empty_like(a)
                _check(self.lib.vv_nn_upsample2(du.data_ptr(), n, h, w, c, dx.data_ptr(), 1, s), name)
                add(src, dx)
                add(op[3], dk)

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.steps += 1
        s = self._stream()
        for name, p in self.params.items():
            for k, half in (("w", p["w16"]), ("b", None)):
                _check(self.lib.vv_nn_adam(p[k].data_ptr(), half.data_ptr() if half is not None else None,
                                           p["g" + k].data_ptr(), p["m" + k].data_ptr(), p["v" + k].data_ptr(),
                                           p[k].numel(), lr, beta1, beta2, eps, GRAD_SCALE, self.steps, s), name)

    def loss(self, pred, target):
        """L1 loss in log radiance (target: (N, H, W, 3) float32 log(1 + radiance))
        and the scaled FP16 gradient of the prediction."""
        t = self.torch
        loss = t.zeros(1, dtype=t.float32, device=self.device)
        dpred = t.empty_like(pred)
        n, h, w, c = pred.shape
        _check(self.lib.vv_nn_l1_loss(pred.data_ptr(), c, target.data_ptr(), n * h * w, GRAD_SCALE, loss.data_ptr(),
                                      dpred.data_ptr(), self._stream()), "loss")
        return loss, dpred

    def train_step(self, x, target, lr=1e-3):
        pred = self.forward(x)
        loss, dpred = self.loss(pred, target)
        self.backward(dpred)
        self.adam(lr)
        return loss

    # ---------------------------------------------------------------- helpers
    def features(self, accum, albedo, normal, spp):
        """(1, H', W', 16) FP16 input from host accumulation sums (H, W, 4), zero
        padded to multiples of PAD."""
        t = self.torch
        h, w = accum.shape[:2]
        hp, wp = -(-h // PAD) * PAD, -(-w // PAD) * PAD
        bufs = []
        for a in (accum, albedo, normal):
            b = np.zeros((hp, wp, 4), np.float32)
            b[:h, :w] = a
            bufs.append(t.tensor(b, device=self.device))
        x = t.empty((1, hp, wp, IN_CHANNELS), dtype=t.float16, device=self.device)
        _check(self.lib.vv_nn_features(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), float(spp),
                                       hp * wp, x.data_ptr(), self._stream()), "features")
        return x

    def denoise(self, accum, albedo, normal, spp):
        """The network's radiance (H, W, 3) for host accumulation sums of spp paths per pixel."""
        t = self.torch
        h, w = accum.shape[:2]
        x = self.features(accum, albedo, normal, spp)
        pred = self.forward(x)
        n, hp, wp, c = pred.shape
        rgb = t.empty((hp, wp, 3), dtype=t.float32, device=self.device)
        _check(self.lib.vv_nn_radiance(pred.data_ptr(), c, hp * wp, rgb.data_ptr(), self._stream()), "radiance")
        self.acts = None
        return rgb[:h, :w].cpu().numpy()


# ---------------------------------------------------------------- training data
def random_views(cfg, center, diagonal, count, seed):
    """`count` frame parameters around the volume: random orbit, a sagittal
    clip at a random depth half the time; denoiser off (the network sees raw
    accumulations)."""
    from . import abi, scene
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        clip = bool(rng.random() < 0.5)
        p = scene.frame_params_for(cfg, center, diagonal, clip_sagittal=clip, anisotropy=0.6, spf=1,
                                   denoiser=abi.DENOISE_OFF)
        p.camera.yaw = abi.f32(p.camera.yaw + rng.uniform(-np.pi, np.pi))
        p.camera.pitch = abi.f32(p.camera.pitch + rng.uniform(-0.4, 0.4))
        if clip:
            p.clipping.planes[0].position = abi.f32(center[0] + diagonal * rng.uniform(-0.12, 0.12))
        out.append(p)
    return out


def render_pair(renderer, params, low_spp, high_spp):
    """(low-spp accumulation sums (acc, albedo, normal), high-spp radiance (H, W, 3)):
    one accumulation, read at low_spp and continued to high_spp."""
    renderer.reset_view()
    renderer.record_frames(1, low_spp, params)
    low = renderer.read_accumulation()
    renderer.record_frames(1 + low_spp, high_spp - low_spp, params)
    acc, _, _ = renderer.read_accumulation(normal=False)
    return low, acc[..., :3] / high_spp


def atrous(renderer, params, spp):
    """The a-trous denoiser's radiance (H, W, 3) at spp paths per pixel (the
    renderer's own denoise pass; HDR read back)."""
    from . import abi
    import copy
    p = copy.deepcopy(params)
    p.path_tracing.denoiser = abi.DENOISE_ATROUS
    renderer.reset_view()
    renderer.record_frames(1, spp, p)
    return renderer.read_hdr().view(np.float16)[..., :3].astype(np.float32)


def train(net, pairs, steps, batch=4, lr=1e-3, seed=0, log_every=0):
    """Adam on random batches of `pairs` ((acc, albedo, normal) at spp, target
    radiance, spp), the learning rate rising linearly over the first fifth of
    the steps (at most 100: Adam's first steps move every weight by the full
    rate, which can blow up a deep ReLU network) and then decaying as a cosine
    to a tenth; returns the losses."""
    t = net.torch
    rng = np.random.default_rng(seed)
    feats, targets = [], []
    for (acc, alb, nor), target, spp in pairs:
        feats.append(net.features(acc, alb, nor, spp))
        targets.append(t.tensor(np.log1p(np.maximum(target, 0.0)).astype(np.float32), device=net.device))
    losses = []
    for step in range(steps):
        idx = rng.choice(len(pairs), size=batch, replace=False)
        x = t.cat([feats[i] for i in idx])
        y = t.stack([targets[i] for i in idx])
        warm = max(1, min(100, steps // 5))
        rate = lr * min(1.0, (step + 1) / warm) * (0.1 + 0.9 * 0.5 * (1 + np.cos(np.pi * step / steps)))
        losses.append(net.train_step(x, y, lr=float(rate)))
    return [float(v) for v in t.stack(losses).cpu().numpy().ravel()]


def luminance_rmse(a, b):
    w = np.array([0.2126, 0.7152, 0.0722])
    return float(np.sqrt(np.mean(((np.asarray(a, np.float64) - np.asarray(b, np.float64)) @ w) ** 2)))


def study(renderer, cfg, train_views, test_views, low_spp=4, train_spp=256, test_spp=1024, steps=400,
          batch=4, seed=0):
    """Trains a U-Net on (low_spp, train_spp) pairs of `train_views` and compares
    it with the raw accumulation and the a-trous denoiser on `test_views`
    (luminance RMSE against test_spp renders)."""
    import time
    t0 = time.perf_counter()
    pairs = [(*render_pair(renderer, p, low_spp, train_spp), low_spp) for p in train_views]
    data_s = time.perf_counter() - t0
    net = UNet(seed=seed)
    t0 = time.perf_counter()
    losses = train(net, pairs, steps, batch=batch, seed=seed)
    train_s = time.perf_counter() - t0
    rows = []
    for p in test_views:
        (acc, alb, nor), ref = render_pair(renderer, p, low_spp, test_spp)
        raw = acc[..., :3] / low_spp
        rows.append({"raw": luminance_rmse(raw, ref), "atrous": luminance_rmse(atrous(renderer, p, low_spp), ref),
                     "unet": luminance_rmse(net.denoise(acc, alb, nor, low_spp), ref)})
    mean = {k: float(np.mean([r[k] for r in rows])) for k in ("raw", "atrous", "unet")}
    return {"net": net, "losses": losses, "per_view": rows, "mean_rmse": mean, "data_s": data_s,
            "train_s": train_s, "pairs": len(pairs), "low_spp": low_spp, "train_spp": train_spp,
            "test_spp": test_spp, "steps": steps, "batch": batch}


# ------------------------------------------------------- time to a fixed RMSE
def crop_pairs(low, target, spp, size, count, rng):
    """`count` random size x size crops (aligned to 16) of one view's
    accumulation sums `low` (acc, albedo, normal) and target radiance."""
    h, w = target.shape[:2]
    out = []
    for _ in range(count):
        y = int(rng.integers(0, (h - size) // 16 + 1)) * 16
        x = int(rng.integers(0, (w - size) // 16 + 1)) * 16
        sl = (slice(y, y + size), slice(x, x + size))
        out.append((tuple(np.ascontiguousarray(a[sl]) for a in low), np.ascontiguousarray(target[sl]), spp))
    return out


def mean_variance(acc, alb, spp):
    """Per-pixel variance of the mean luminance after spp paths, from the sums of
    luminance (radiance sums) and squared luminance (albedo guide's w)."""
    w = np.array([0.2126, 0.7152, 0.0722])
    s1 = np.asarray(acc, np.float64)[..., :3] @ w
    s2 = np.asarray(alb, np.float64)[..., 3]
    return np.maximum(s2 - s1 * s1 / spp, 0.0) / (spp - 1.0) / spp


def blend(net_rgb, acc, alb, spp, eps2):
    """The network's image and the raw mean mixed per pixel by inverse variance:
    the raw mean's (estimated) against the network's error eps2 (calibrated)."""
    var = mean_variance(acc, alb, spp)[..., None]
    w = var / (var + eps2)
    return w * net_rgb + (1.0 - w) * np.asarray(acc, np.float64)[..., :3] / spp


def time_to_rmse_study(renderer, train_views, test_views, levels=(4, 8, 16, 32, 64, 128, 256, 512),
                       train_levels=(4, 16, 64, 256), train_spp=1024, plain_spp=1024, ref_spp=4096, crops=12,
                       steps=1500, seed=0):
    """Trains the U-Net on crops of full-size renders (inputs at `train_levels`
    paths/pixel, targets at train_spp), calibrates its error, then on each
    held-out view compares the plain tracer at plain_spp with the network (and
    its inverse-variance blend with the raw mean) at each of `levels`, all
    against a reference of ref_spp further, independent paths (samples
    plain_spp .. plain_spp + ref_spp - 1): the fewest paths/pixel at which the
    blend's luminance RMSE is at most the plain image's, and the wall time of
    each (render, readback, network)."""
    import time
    import torch
    from . import convergence as CV
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    pairs = []
    for p in train_views:
        renderer.reset_view()
        done, lows = 0, {}
        for lv in sorted(train_levels):
            renderer.record_frames(1 + done, lv - done, p)
            done = lv
            lows[lv] = renderer.read_accumulation()
        renderer.record_frames(1 + done, train_spp - done, p)
        acc, _, _ = renderer.read_accumulation(normal=False)
        target = acc[..., :3] / train_spp
        for lv, low in lows.items():
            pairs += crop_pairs(low, target, lv, 256, crops, rng)
    data_s = time.perf_counter() - t0
    net = UNet(seed=seed)
    t0 = time.perf_counter()
    losses = train(net, pairs, steps, batch=4, seed=seed)
    train_s = time.perf_counter() - t0
    # The network's error: its mean squared luminance error against the
    # targets on training views, less the targets' own estimated noise.
    eps = []
    for p in train_views[:4]:
        renderer.reset_view()
        cal = max(train_levels)
        renderer.record_frames(1, cal, p)
        a, b, c = renderer.read_accumulation()
        renderer.record_frames(1 + cal, train_spp - cal, p)
        acc, alb, _ = renderer.read_accumulation(normal=False)
        err2 = luminance_rmse(net.denoise(a, b, c, cal), acc[..., :3] / train_spp) ** 2
        eps.append(max(err2 - CV.rmse_estimate(acc, alb, train_spp) ** 2, 1e-9))
    eps2 = float(np.mean(eps))
    views = []
    for p in test_views:
        renderer.reset_view()
        done, lows = 0, {}
        for lv in list(levels) + [plain_spp]:
            renderer.record_frames(1 + done, lv - done, p)
            done = lv
            lows[lv] = renderer.read_accumulation()
        renderer.record_frames(1 + done, ref_spp, p)
        acc, _, _ = renderer.read_accumulation(normal=False)
        ref = (acc[..., :3] - lows[plain_spp][0][..., :3]) / ref_spp
        plain = luminance_rmse(lows[plain_spp][0][..., :3] / plain_spp, ref)
        rmse = {}
        for lv in levels:
            a, b, c = lows[lv]
            out = net.denoise(a, b, c, lv)
            rmse[lv] = {"raw": luminance_rmse(a[..., :3] / lv, ref), "unet": luminance_rmse(out, ref),
                        "blend": luminance_rmse(blend(out, a, b, lv, eps2), ref)}
        reached = [lv for lv in levels if rmse[lv]["blend"] <= plain]
        spp = reached[0] if reached else None

        def wall(n, denoise):
            renderer.reset_view()
            renderer.synchronize()
            t = time.perf_counter()
            renderer.record_frames(1, n, p)
            a2, b2, c2 = renderer.read_accumulation()
            if denoise:
                blend(net.denoise(a2, b2, c2, n), a2, b2, n, eps2)
            torch.cuda.synchronize()
            return (time.perf_counter() - t) * 1e3

        views.append({"plain_rmse": plain, "rmse": {str(k): v for k, v in rmse.items()}, "spp_to_target": spp,
                      "plain_ms": wall(plain_spp, False), "denoised_ms": wall(spp, True) if spp else None})
    return {"net": net, "losses": losses, "views": views, "data_s": data_s, "train_s": train_s, "eps": eps2 ** 0.5,
            "pairs": len(pairs), "train_levels": list(train_levels), "train_spp": train_spp, "plain_spp": plain_spp,
            "ref_spp": ref_spp, "steps": steps}
