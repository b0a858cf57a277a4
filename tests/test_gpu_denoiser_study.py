"""The learned denoiser trained on the tracer's own renders (GPU): after a
short training on pairs of 4- and 64-path-per-pixel images of random views,
its output on held-out views is closer to 256-path renders than the raw
4-path accumulation (luminance RMSE below 0.8 of the raw image's) and than
the a-trous filter it replaces, on every held-out view."""
import numpy as np
import pytest

from volview_gb300 import abi, scene
from volview_gb300 import renderer as R

pytestmark = pytest.mark.gpu

pytest.importorskip("torch")


def test_trained_network_gains_over_the_raw_accumulation_and_atrous(gpu_ctx):
    from volview_gb300 import learned_denoiser as LD
    cfg = scene.head_neck_config(seed=4, dims=(128, 128, 100), spacing=(2.0, 2.0, 4.0), size=256)
    r = R.Renderer(gpu_ctx, cfg["volume"], cfg["tf"])
    r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
    r.resize(256, 256)
    train = LD.random_views(cfg, list(r.center), r.diagonal, 32, seed=1)
    test = LD.random_views(cfg, list(r.center), r.diagonal, 4, seed=2)
    res = LD.study(r, cfg, train, test, low_spp=4, train_spp=64, test_spp=256, steps=120, batch=4)
    r.destroy()
    m = res["mean_rmse"]
    print(f"luminance RMSE: raw {m['raw']:.4g}, a-trous {m['atrous']:.4g}, U-Net {m['unet']:.4g}; "
          f"loss {res['losses'][0]:.4g} -> {np.mean(res['losses'][-10:]):.4g}")
    assert np.mean(res["losses"][-10:]) < res["losses"][0]
    assert m["unet"] < 0.8 * m["raw"]
    assert m["unet"] < m["atrous"], "the U-Net does not beat the a-trous filter it replaces"
    for row in res["per_view"]:
        assert row["unet"] < row["atrous"], row
