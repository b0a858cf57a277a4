"""The learned denoiser's tensor-core operators and U-Net against the numpy
oracle (oracle/nn_ref.py) (GPU).

Tolerances (written here, checked below):
* convolution outputs and input gradients (FP16 results of FP32 sums over
  FP16 operands): within 2e-3 of the float64 reference, relative to its
  largest magnitude, plus 2e-3 relative per value;
* weight and bias gradients (FP32 sums): within 1e-3 of the reference's
  largest magnitude;
* pooling, upsampling, concatenation, ReLU masks: exact (sums of 4 values in
  FP32, rounded once);
* the whole U-Net at 256x256 against the reference run with FP16 rounding of
  every stored tensor: the prediction within 1e-2 of its largest magnitude,
  and every layer's weight gradient within 5 % (relative L2 norm);
* Adam: within 1e-6 relative of the float64 update.
"""
import numpy as np
import pytest

from oracle import nn_ref as N
from volview_gb300 import learned_denoiser as LD

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    from volview_gb300 import renderer as R
    return R.load()


def dev(a, dtype=None):
    t = torch.tensor(np.ascontiguousarray(a), device="cuda")
    return t.half() if dtype == "half" else t


def host(t):
    torch.cuda.synchronize()
    return t.float().cpu().numpy().astype(np.float64)


def close(got, ref, atol_rel, rtol=0.0):
    scale = max(float(np.abs(ref).max()), 1e-6)
    err = np.abs(got - ref)
    assert np.all(err <= atol_rel * scale + rtol * np.abs(ref)), (float(err.max()), scale)


def rand_half(rng, shape, s=1.0):
    return (rng.standard_normal(shape) * s).astype(np.float16).astype(np.float64)


S = None  # default stream


@pytest.mark.parametrize("cin,cout", [(16, 8), (16, 32), (32, 48), (48, 96), (96, 176), (176, 80), (80, 16)])
def test_conv_forward_and_gradients(lib, cin, cout):
    rng = np.random.default_rng(cin * 1000 + cout)
    n, h, w = 2, 20, 32
    x = rand_half(rng, (n, h, w, cin))
    wt = rand_half(rng, (cout, 3, 3, cin), 0.1)
    b = rng.standard_normal(cout).astype(np.float32)
    X, W, B = dev(x, "half"), dev(wt, "half"), dev(b)
    Y = torch.empty((n, h, w, cout), dtype=torch.float16, device="cuda")
    for relu in (0, 1):
        assert lib.vv_nn_conv3x3(X.data_ptr(), n, h, w, cin, W.data_ptr(), B.data_ptr(), cout, relu, Y.data_ptr(), S) == 0
        close(host(Y), N.conv3x3(x, wt, b, bool(relu)), 2e-3, 2e-3)
    # Input gradient: flipped weights through the same convolution.
    dy = rand_half(rng, (n, h, w, cout))
    DY = dev(dy, "half")
    if cout % 16 == 0:
        WT = torch.empty((cin, 3, 3, cout), dtype=torch.float16, device="cuda")
        assert lib.vv_nn_flip_weights(W.data_ptr(), cout, cin, WT.data_ptr(), S) == 0
        DX = torch.empty((n, h, w, cin), dtype=torch.float16, device="cuda")
        assert lib.vv_nn_conv3x3(DY.data_ptr(), n, h, w, cout, WT.data_ptr(), None, cin, 0, DX.data_ptr(), S) == 0
        close(host(DX), N.conv3x3_dgrad(dy, wt), 2e-3, 2e-3)
    # Weight and bias gradients.
    DW = torch.zeros((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    DB = torch.zeros(cout, dtype=torch.float32, device="cuda")
    assert lib.vv_nn_conv3x3_wgrad(X.data_ptr(), DY.data_ptr(), n, h, w, cin, cout, DW.data_ptr(), S) == 0
    assert lib.vv_nn_bias_grad(DY.data_ptr(), n * h * w, cout, DB.data_ptr(), S) == 0
    close(host(DW), N.conv3x3_wgrad(x, dy), 1e-3)
    close(host(DB), dy.sum(axis=(0, 1, 2)), 1e-3)


def test_shapes_the_operators_refuse(lib):
    X = torch.zeros((1, 16, 16, 16), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_conv3x3(X.data_ptr(), 1, 16, 20, 16, X.data_ptr(), None, 16, 0, X.data_ptr(), S) != 0  # w % 16
    assert lib.vv_nn_conv3x3(X.data_ptr(), 1, 16, 16, 8, X.data_ptr(), None, 16, 0, X.data_ptr(), S) != 0   # cin % 16
    assert lib.vv_nn_conv3x3(X.data_ptr(), 1, 16, 16, 16, X.data_ptr(), None, 24, 0, X.data_ptr(), S) != 0  # cout


def test_pool_upsample_concat_relu(lib):
    rng = np.random.default_rng(4)
    n, h, w, c = 2, 8, 16, 24
    x = rand_half(rng, (n, h, w, c))
    X = dev(x, "half")
    P = torch.empty((n, h // 2, w // 2, c), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_avgpool2(X.data_ptr(), n, h, w, c, P.data_ptr(), 0, S) == 0
    assert np.array_equal(host(P), N.half(N.avgpool2(x)))
    dp = rand_half(rng, (n, h // 2, w // 2, c))
    DX = torch.empty_like(X)
    assert lib.vv_nn_avgpool2(dev(dp, "half").data_ptr(), n, h, w, c, DX.data_ptr(), 1, S) == 0
    assert np.array_equal(host(DX), N.half(N.avgpool2_backward(dp)))
    U = torch.empty((n, 2 * h, 2 * w, c), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_upsample2(X.data_ptr(), n, h, w, c, U.data_ptr(), 0, S) == 0
    assert np.array_equal(host(U), N.upsample2(x))
    du = rand_half(rng, (n, 2 * h, 2 * w, c))
    assert lib.vv_nn_upsample2(dev(du, "half").data_ptr(), n, h, w, c, DX.data_ptr(), 1, S) == 0
    assert np.array_equal(host(DX), N.half(N.upsample2_backward(du)))
    y = rand_half(rng, (n, h, w, 16))
    Y = dev(y, "half")
    CAT = torch.empty((n, h, w, c + 16), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_concat(X.data_ptr(), c, Y.data_ptr(), 16, n * h * w, CAT.data_ptr(), S) == 0
    assert np.array_equal(host(CAT), np.concatenate([x, y], -1))
    # Upsampling and concat in one pass: the same tensor as the two passes.
    Z = dev(rand_half(rng, (n, 2 * h, 2 * w, 16)), "half")
    UC = torch.empty((n, 2 * h, 2 * w, c + 16), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_upsample_concat(X.data_ptr(), n, h, w, c, Z.data_ptr(), 16, UC.data_ptr(), S) == 0
    assert np.array_equal(host(UC), np.concatenate([N.upsample2(x), host(Z)], -1))
    assert lib.vv_nn_upsample_concat(X.data_ptr(), n, h, w, 12, Z.data_ptr(), 16, UC.data_ptr(), S) != 0  # ca % 8
    # Pooling with a channel count that is not a multiple of 8 (the per-element path).
    x6 = rand_half(rng, (n, h, w, 6))
    P6 = torch.empty((n, h // 2, w // 2, 6), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_avgpool2(dev(x6, "half").data_ptr(), n, h, w, 6, P6.data_ptr(), 0, S) == 0
    assert np.array_equal(host(P6), N.half(N.avgpool2(x6)))
    DA, DB = torch.empty_like(X), torch.empty_like(Y)
    assert lib.vv_nn_split(CAT.data_ptr(), c, 16, n * h * w, DA.data_ptr(), DB.data_ptr(), S) == 0
    assert np.array_equal(host(DA), x) and np.array_equal(host(DB), y)
    G = dev(y, "half")
    assert lib.vv_nn_relu_backward(G.data_ptr(), Y.data_ptr(), G.numel(), S) == 0
    assert np.array_equal(host(G), y * (y > 0))
    assert lib.vv_nn_add(G.data_ptr(), Y.data_ptr(), G.numel(), S) == 0
    assert np.array_equal(host(G), N.half(y * (y > 0) + y))


def test_features_loss_adam(lib):
    rng = np.random.default_rng(5)
    px, spp = 4096, 4.0
    acc, alb, nor = (rng.uniform(0, 8, (px, 4)).astype(np.float32) for _ in range(3))
    X = torch.empty((px, 16), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_features(dev(acc).data_ptr(), dev(alb).data_ptr(), dev(nor).data_ptr(), spp, px, X.data_ptr(),
                              S) == 0
    close(host(X), N.features(acc, alb, nor, spp), 1e-6, 1e-3)  # FP16 rounding (subnormals: absolute)
    pred = rand_half(rng, (px, 16))
    tgt = rng.standard_normal((px, 3)).astype(np.float32)
    loss = torch.zeros(1, device="cuda")
    D = torch.empty((px, 16), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_l1_loss(dev(pred, "half").data_ptr(), 16, dev(tgt).data_ptr(), px, 1024.0, loss.data_ptr(),
                             D.data_ptr(), S) == 0
    ref_loss, ref_g = N.l1_loss(pred, tgt)
    assert abs(float(host(loss)[0]) - ref_loss) <= 1e-5 * ref_loss
    close(host(D), N.half(ref_g * 1024.0), 0.0, 1e-3)
    w, g = rng.standard_normal(1000), rng.standard_normal(1000)
    m, v = np.zeros(1000), np.zeros(1000)
    W, G, M, V = (dev(a.astype(np.float32)) for a in (w, g * 8.0, m, v))
    for step in (1, 2, 3):
        assert lib.vv_nn_adam(W.data_ptr(), None, G.data_ptr(), M.data_ptr(), V.data_ptr(), 1000, 1e-2, 0.9, 0.999,
                              1e-8, 8.0, step, S) == 0
        w, m, v = N.adam(w, g, m, v, 1e-2, 0.9, 0.999, 1e-8, step)
    close(host(W), w, 1e-6, 1e-5)


def test_unet_matches_the_oracle():
    """Forward and backward of the full network at 256x256 against the oracle
    with the same (FP16) weights and FP16 rounding of stored tensors."""
    net = LD.UNet(seed=3)
    rng = np.random.default_rng(6)
    x = np.zeros((1, 256, 256, 16))
    x[..., :9] = rand_half(rng, (1, 256, 256, 9), 0.5)
    tgt = rng.standard_normal((1, 256, 256, 3)).astype(np.float32)
    pred = net.forward(dev(x, "half"))
    loss, dpred = net.loss(pred, dev(tgt))
    net.backward(dpred)
    ref_net = {"plan": net.plan, "params": net.numpy_params()}
    ref_pred, acts = N.unet_forward(ref_net, x)
    close(host(pred), ref_pred, 1e-2)
    ref_loss, ref_dpred = N.l1_loss(host(pred), tgt)
    assert abs(float(host(loss)[0]) - ref_loss) <= 1e-4 * ref_loss
    grads = N.unet_backward(ref_net, acts, N.half(ref_dpred * LD.GRAD_SCALE))
    for name, p in net.params.items():
        gw, gb = host(p["gw"]), host(p["gb"])
        rw, rb = grads[name]
        rel = np.linalg.norm(gw - rw) / max(np.linalg.norm(rw), 1e-12)
        assert rel <= 0.05, (name, rel)
        assert np.linalg.norm(gb - rb) <= 0.05 * max(np.linalg.norm(rb), 1e-12), name


def test_training_lowers_the_loss():
    """Thirty Adam steps (rate rising over the first ten) on one fixed pair
    lower the L1 loss."""
    net = LD.UNet(seed=1)
    rng = np.random.default_rng(7)
    x = np.zeros((2, 256, 256, 16))
    x[..., :9] = rand_half(rng, (2, 256, 256, 9), 0.3)
    tgt = np.log1p(np.abs(x[..., :3])).astype(np.float32)  # an identity-like target
    X, T = dev(x, "half"), dev(tgt)
    losses = [float(host(net.train_step(X, T, lr=1e-3 * min(1.0, (k + 1) / 10)))[0]) for k in range(30)]
    assert losses[-1] < 0.7 * losses[0], losses


def test_renderer_runs_the_network_as_its_denoiser(gpu_ctx, small_cfg):
    """DENOISE_LEARNED: the renderer runs the loaded network on its own
    accumulation before the display; its HDR image is the network's output
    for the same accumulation read back (within FP16 rounding). Without
    weights the mode is refused."""
    from volview_gb300 import abi, scene
    from volview_gb300 import renderer as R
    cfg = small_cfg
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal, denoiser=abi.DENOISE_LEARNED)
    r.resize(96, 80)
    with pytest.raises(R.VolptError) as e:
        r.record(1, p)
    assert e.value.status == abi.VV_ERR_STATE
    net = LD.UNet(seed=9)
    blob = net.weights_blob()
    with pytest.raises(R.VolptError):
        r.set_denoiser_weights(blob[:-1])
    r.set_denoiser_weights(blob)
    r.record_frames(1, 4, p)
    hdr = r.read_hdr().view(np.float16).astype(np.float32)
    acc, alb, nor = r.read_accumulation()
    ref = net.denoise(acc, alb, nor, 4)
    assert np.all(np.abs(hdr[..., :3] - ref) <= 2e-3 * np.abs(ref) + 1e-4)
    assert np.allclose(hdr[..., 3], np.float16(acc[..., 3] / 4.0).astype(np.float32), atol=1e-3)
    r.set_denoiser_weights(None)
    r.destroy()


@pytest.mark.parametrize("cin,cout,w", [(16, 32, 256), (32, 32, 128), (32, 48, 256), (48, 64, 128), (64, 64, 256),
                                        (80, 32, 128), (64, 80, 128), (32, 16, 384), (16, 8, 128)])
def test_tensor_core_convolution(lib, cin, cout, w):
    """Widths that are multiples of 128 take the tcgen05 convolution (TMA-fed
    rows, TMEM accumulators): its output against the reference at the
    convolution tolerance, the product entry point the same to the bit, and no
    bounded wait given up."""
    import ctypes as C
    rng = np.random.default_rng(cin * 1000 + cout + w)
    n, h = 2, 12
    x = rand_half(rng, (n, h, w, cin))
    wt = rand_half(rng, (cout, 3, 3, cin), 0.1)
    b = rng.standard_normal(cout).astype(np.float32)
    X, W, B = dev(x, "half"), dev(wt, "half"), dev(b)
    Y = torch.empty((n, h, w, cout), dtype=torch.float16, device="cuda")
    Y2 = torch.empty_like(Y)
    for relu in (0, 1):
        assert lib.vv_nn_conv3x3_tc(X.data_ptr(), n, h, w, cin, W.data_ptr(), B.data_ptr(), cout, relu, Y.data_ptr(),
                                    S) == 0
        close(host(Y), N.conv3x3(x, wt, b, bool(relu)), 2e-3, 2e-3)
        assert lib.vv_nn_conv3x3(X.data_ptr(), n, h, w, cin, W.data_ptr(), B.data_ptr(), cout, relu, Y2.data_ptr(),
                                 S) == 0
        assert torch.equal(Y, Y2)
    failed = C.c_int(1)
    assert lib.vv_nn_tc_status(C.byref(failed), 1) == 0 and failed.value == 0


def test_tensor_core_convolution_refuses_other_shapes(lib):
    X = torch.zeros((1, 16, 128, 176), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_conv3x3_tc(X.data_ptr(), 1, 16, 96, 16, X.data_ptr(), None, 16, 0, X.data_ptr(), S) != 0  # w
    assert lib.vv_nn_conv3x3_tc(X.data_ptr(), 1, 16, 128, 176, X.data_ptr(), None, 80, 0, X.data_ptr(), S) != 0  # smem
    assert lib.vv_nn_conv3x3_tc(X.data_ptr(), 1, 16, 128, 16, X.data_ptr(), None, 112, 0, X.data_ptr(), S) != 0  # cout


@pytest.mark.parametrize("cin,cout", [(80, 32), (32, 32)])
def test_tensor_core_convolution_long_runs(lib, cin, cout):
    """Tall images give every CTA a run of several segments, so the ring of row
    slots reloads slots as the run walks down its column: three slots for
    80 -> 32 (two CTAs per SM), four for 32 -> 32. Checked against PyTorch's
    FP32 convolution (same padding) at the convolution tolerance."""
    import ctypes as C
    torch.manual_seed(cin + cout)
    n, h, w = 1, 1536, 128
    x = (torch.randn((n, h, w, cin), device="cuda") * 0.5).half()
    wt = (torch.randn((cout, 3, 3, cin), device="cuda") * 0.1).half()
    b = torch.randn(cout, device="cuda", dtype=torch.float32)
    y = torch.empty((n, h, w, cout), dtype=torch.float16, device="cuda")
    assert lib.vv_nn_conv3x3_tc(x.data_ptr(), n, h, w, cin, wt.data_ptr(), b.data_ptr(), cout, 1, y.data_ptr(),
                                S) == 0
    ref = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), wt.float().permute(0, 3, 1, 2), b, padding=1)
    ref = torch.relu(ref).permute(0, 2, 3, 1)
    torch.cuda.synchronize()
    got, want = y.float().cpu().numpy(), ref.cpu().numpy()
    close(got.astype(np.float64), want.astype(np.float64), 2e-3, 2e-3)
    failed = C.c_int(1)
    assert lib.vv_nn_tc_status(C.byref(failed), 1) == 0 and failed.value == 0
