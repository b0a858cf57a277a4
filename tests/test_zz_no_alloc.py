"""The allocation-free a-trous entry point against the renderer's own (GPU).

vv_denoise_atrous_noalloc serves callers that cannot allocate device memory
when they need a denoised image (a per-frame callback under a device-memory
budget fixed at start-up, or a process whose device allocations belong to
another runtime): they pass their own accumulation and output buffers, and the
scratch lives in a fixed device array of 512 x 512 pixels. Its output must
match the HDR image `vv_record` produces with the a-trous denoiser, within the
FP16 ulp the denoiser parity test allows, on two calls in a row (the second one
reuses the scratch the first one left behind). This file is collected last so
that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu


def _half(a):
    return a.view(np.float16).astype(np.float32)


# Whole 16x16 tiles, partial tiles at the right and bottom edges (the kernels'
# x >= width / y >= height guards and the per-image offsets into the shared
# array), and the largest image the scratch holds (512 x 512 pixels).
SIZES = [(64, 48), (37, 23), (512, 512)]


@pytest.mark.parametrize("W,H", SIZES)
def test_noalloc_denoiser_matches_record(small_cfg, W, H):
    torch = pytest.importorskip("torch")
    cfg = small_cfg
    ctx = R.Context(0)
    r = R.Renderer(ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
    p.camera.distance = abi.f32(p.camera.distance * 0.5)
    p.path_tracing.denoiser = abi.DENOISE_ATROUS
    r.resize(W, H)
    stream = torch.cuda.current_stream()
    frame = 1
    for call in range(2):
        for _ in range(2 + call):  # different accumulations for the two calls
            r.record(frame, p)
            frame += 1
        expected = r.read_hdr()  # the renderer's a-trous output for this frame
        acc, alb, nor = (torch.from_numpy(x).cuda() for x in r.read_accumulation())
        out = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
        status = R.load().vv_denoise_atrous_noalloc(
            C.c_void_p(acc.data_ptr()), C.c_void_p(alb.data_ptr()), C.c_void_p(nor.data_ptr()),
            C.c_void_p(out.data_ptr()), W, H, r.accumulated_samples(), C.c_void_p(stream.cuda_stream))
        R.check(status)
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint16)
        a, b = _half(got), _half(expected)
        assert np.all(np.abs(a - b) <= np.abs(b) * 2.0 ** -10 + 1e-7), f"call {call + 1} differs"
    r.destroy()
    ctx.destroy()


def test_noalloc_denoiser_rejects_large_images():
    lib = R.load()
    status = lib.vv_denoise_atrous_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                           1024, 1024, 1, None)
    assert status == abi.VV_ERR_LIMIT
    assert b"512 x 512" in lib.vv_last_error()


def test_noalloc_denoiser_rejects_misaligned_buffers():
    """The images are read as float4 and the output written as 4 halves: a
    buffer that is not 16-byte (8-byte for the output) aligned is refused on the
    host, before anything is queued on the device."""
    lib = R.load()
    good, odd = C.c_void_p(4096), C.c_void_p(4096 + 20)
    for args in ((odd, good, good, good), (good, odd, good, good), (good, good, odd, good),
                 (good, good, good, C.c_void_p(4096 + 4))):
        status = lib.vv_denoise_atrous_noalloc(*args, 64, 48, 1, None)
        assert status == abi.VV_ERR_ARG
        assert b"aligned" in lib.vv_last_error()
