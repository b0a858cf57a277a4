"""The precision variant measured against the FP64 oracle (GPU + host cores).

Renders one view to `spp` paths per pixel with the density stored as FP32,
R16_UNORM, FP16 and BF16 (and FP32 with Kahan running sums continuing in FP64),
every render on the same per-pixel random streams (accumulation indices
0 .. spp - 1). The reference image comes from the FP64 oracle: the restatement of pt.comp
compiled in double precision (arithmetic, texture filtering, sums), over the
FP32-storage renderer's stored density, normals, masks and majorants, tracing
the same paths on a few crops of the image. Each render's luminance RMSE
against it, per crop, is printed as one JSON line beside the FP64 oracle's own
Monte Carlo RMSE on those crops.

    python tests/precision_fp64_study.py --workload torso --spp 4096 --crops 3 --crop 32
    python tests/precision_fp64_study.py --workload small --spp 256 --crops 1 --crop 48

`run()` is also what tests/test_gpu_precision.py calls on the small scene.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LUMA = np.array([0.2126, 0.7152, 0.0722])
RUNS = [("fp32", "fp32", 0), ("unorm16", "fp32", 0), ("fp16", "fp32", 0), ("bf16", "fp32", 0),
        ("fp32", "kahan", 65536)]


def workload(name):
    from volview_gb300 import scene
    if name == "torso":
        return scene.torso_config()
    if name == "small":
        return scene.small_config(n=48, size=48)
    raise ValueError(name)


def crop_origins(background, size, count):
    """`count` crops of size x size on the phantom: among the blocks of a grid
    whose pixels' paths left the volume at their first bounce least often (the
    accumulation's background channel; at most 1 % of them, or the quarter of
    blocks with the least), the one nearest the candidates' centre, then each
    time the one farthest from those taken."""
    h, w = background.shape
    bh, bw = h // size, w // size
    frac = background[:bh * size, :bw * size].reshape(bh, size, bw, size).mean(axis=(1, 3)).ravel()
    cand = np.flatnonzero(frac <= 0.01)
    if cand.size < count:
        cand = np.argsort(frac, kind="stable")[:max(count, frac.size // 4)]
    pos = np.stack([cand // bw, cand % bw], 1).astype(np.float64)
    picked = [int(np.argmin(((pos - pos.mean(0)) ** 2).sum(1)))]
    while len(picked) < min(count, len(cand)):
        d = np.min([((pos - pos[k]) ** 2).sum(1) for k in picked], axis=0)
        picked.append(int(np.argmax(d)))
    return [(int(cand[k] % bw) * size, int(cand[k] // bw) * size) for k in picked]


def oracle_from_device(cfg, r):
    """The oracle's renderer over the device renderer's stored volumes."""
    from oracle import oracle as O
    from volview_gb300 import abi
    cpu = O.CpuRenderer.__new__(O.CpuRenderer)
    cpu.volume = cfg["volume"]
    cpu.hu = cfg["hu"]
    cpu.dims = tuple(cfg["volume"].dims)
    cpu.geo = O.geometry(cfg["volume"])
    cpu.density = r.read_volume(abi.VOLUME_DENSITY)
    cpu.density_format = r.precision.density_format
    cpu.mask_format = r.precision.mask_format
    cpu.majorants = r.precision.majorants
    cpu.set_transfer_function(cfg["tf"])
    cpu.normals = r.read_volume(abi.VOLUME_NORMALS)
    cpu.set_labels(cfg["labels_vol"], cfg["soft"])
    cpu.mask = r.read_volume(abi.VOLUME_MASK)
    cpu.majorant = r.read_volume(abi.VOLUME_MAJORANT)
    cpu.env_rad = cpu.env_table = None
    cpu.env_peak_u = 0.0
    cpu.accumulated = 0
    cpu.accum_key = None
    cpu.resize(r.width, r.height)
    cpu.mask_key = "device"
    return cpu


def run(ctx, cfg, spp, crops=3, size=32, zoom=None, log=None):
    from volview_gb300 import abi, scene
    from volview_gb300 import renderer as R
    W, H = cfg["width"], cfg["height"]
    out = {"paths_per_pixel": spp, "image": [W, H]}
    oracle_lum, origins = None, None
    for density, sums, fp64_after in RUNS:
        fmt = {"unorm16": abi.DENSITY_UNORM16, "fp16": abi.DENSITY_FP16, "bf16": abi.DENSITY_BF16,
               "fp32": abi.DENSITY_FP32}[density]
        prec = abi.precision(fmt, abi.SUMS_KAHAN if sums == "kahan" else abi.SUMS_FP32, fp64_after)
        r = R.Renderer(ctx, cfg["volume"], cfg["tf"], prec)
        r.set_labels(cfg["labels_vol"], abi.soft_struct(cfg["soft"]))
        p = scene.frame_params_for(cfg, list(r.center), r.diagonal)
        if zoom:
            p.camera.distance = abi.f32(p.camera.distance * zoom)
        r.resize(W, H)
        r.record(1, p)  # masks and majorants
        r.resize(W, H)  # restarts the accumulation: indices 0 .. spp - 1 below
        t0 = time.perf_counter()
        done, frame = 0, 2
        while done < spp:
            n = min(64, spp - done)
            r.record_frames(frame, n, p)
            frame, done = frame + n, done + n
        r.synchronize()
        gpu_s = time.perf_counter() - t0
        acc, _, _ = r.read_accumulation(normal=False)
        if oracle_lum is None:
            origins = crop_origins(acc[..., 3] / spp, size, crops)
            out["crops"] = [[x, y, size, size] for x, y in origins]
            t0 = time.perf_counter()
            cpu = oracle_from_device(cfg, r)
            oracle_lum, mc = [], []
            for x0, y0 in origins:
                ys, xs = np.mgrid[y0:y0 + size, x0:x0 + size]
                pix = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
                s = cpu.pixel_sums_fp64(p, pix, 0, spp)
                l1 = s[:, :3] @ LUMA
                oracle_lum.append(l1 / spp)
                var = np.maximum(s[:, 7] - l1 * l1 / spp, 0.0) / max(spp - 1.0, 1.0) / spp
                mc.append(float(np.sqrt(var.mean())))
            from oracle import oracle as O
            out["fp64_oracle"] = {"seconds": time.perf_counter() - t0, "threads": O.threads(),
                                  "mc_rmse_per_crop": mc}
        r.destroy()
        lum = np.asarray(acc[..., :3], np.float64) @ LUMA / spp
        errs = [float(np.sqrt(np.mean((lum[y0:y0 + size, x0:x0 + size].ravel() - jl) ** 2)))
                for (x0, y0), jl in zip(origins, oracle_lum)]
        key = density if sums == "fp32" else f"{density}+{sums}+fp64_after_{fp64_after}"
        out[key] = {"rmse_vs_fp64_oracle_per_crop": errs, "rmse_vs_fp64_oracle": float(np.sqrt(np.mean(np.square(errs)))),
                    "gpu_seconds": gpu_s}
        if log:
            log(key, out[key])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="torso", choices=["torso", "small"])
    ap.add_argument("--spp", type=int, default=4096)
    ap.add_argument("--crops", type=int, default=3)
    ap.add_argument("--crop", type=int, default=32)
    args = ap.parse_args()
    from volview_gb300 import renderer as R
    ctx = R.Context(0)
    cfg = workload(args.workload)
    res = run(ctx, cfg, args.spp, args.crops, args.crop, zoom=0.45 if args.workload == "small" else None,
              log=lambda k, v: print(k, v, file=sys.stderr))
    res["workload"] = args.workload
    print(json.dumps(res))
    ctx.destroy()


if __name__ == "__main__":
    main()
