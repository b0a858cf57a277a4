"""Generates tests/golden/small_scene.npz from the reference's own shaders.

Runs shaders/{normals,mask,majorant,pt,denoise}.comp — compiled as CPU code by
oracle/build_ref.py from the reference sources — on a 24^3 seeded phantom with
soft labels, hybrid label mode and a sagittal clip plane, 24x24 pixels, two
accumulate-frames of two paths each. Inputs that the reference computes on the
host (density normalisation, LUT, uniforms) come from the oracle's restatement
of the render crate; the density normalisation and LUT are themselves pinned by
the reference's unit tests (crates/render/src/transfer.rs:130-149).

light_map_fixture() writes tests/golden/small_light_map.npz: the same scene lit
by a seeded synthetic light map (Environment::Map); raymarch_fixture() writes
tests/golden/small_raymarch.npz: the real-time ray marcher's occlusion volume,
shadow volume and image (ao.comp, shadow.comp, dvr.comp); modes_fixture()
writes tests/golden/small_modes.npz: the same scene in each of the reference's
other rendering modes (scene.MODE_CASES: label modes Off, Tint and Isolate with
hidden labels, ghosted labels, binary masks, the Dome environment, the thin
lens), masks, majorants and two accumulate-frames of two paths each.

Usage (needs the reference sources): python tests/golden/make_golden.py [main|light_map|raymarch|modes ...]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402
from volview_gb300 import abi, scene  # noqa: E402


def main():
    if not R.available():
        build_ref.main([])
    n, size, frames, spf = 24, 24, 2, 2
    cfg = scene.small_config(n=n, size=size, spp=frames * spf)
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    r.set_labels(cfg["labels_vol"], cfg["soft"])
    g = r.geo
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True, spf=spf)
    r.resize(size, size)
    normals = R.normals(r, r._uniforms_geometry_only())
    r.normals = normals
    u1 = r.uniforms(params, 1, size, size)
    mask = R.mask(r, u1, O.mask_margin(cfg["volume"], params.labels), int(params.labels.smoothing))
    r.mask = mask
    majorant = R.majorant(r, u1)
    r.majorant = majorant
    acc = np.zeros((size, size, 4), np.float32)
    alb, nor = np.zeros_like(acc), np.zeros_like(acc)
    hdr = np.zeros((size, size, 4), np.uint16)
    for f in range(frames):
        r.accumulated = f * spf
        u = r.uniforms(params, f + 1, size, size)
        R.pt_frame(r, u, acc, alb, nor, hdr)
    r.accumulated = (frames - 1) * spf
    ud = r.uniforms(params, frames, size, size)
    denoised = R.denoise(ud, acc, alb, nor)
    exposure = np.zeros(1, np.float32)
    post1 = R.post(ud, denoised, exposure)
    post2 = R.post(ud, denoised, exposure)  # a second frame adapts the exposure
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_scene.npz")
    np.savez_compressed(out, hu=cfg["hu"], labels=cfg["labels_vol"], soft=cfg["soft"],
                        spacing=np.array(cfg["spacing"]), params=np.frombuffer(bytes(params), np.uint8),
                        width=size, height=size, frames=frames, density=r.density, normals=normals, mask=mask,
                        majorant=majorant, uniforms_frame1=u1, accum=acc, albedo=alb, normal=nor, hdr=hdr,
                        denoised=denoised, post1=post1, post2=post2, exposure=exposure)
    print(out, os.path.getsize(out), "bytes; background share", float(acc[..., 3].mean()) / (frames * spf))


def light_map_fixture():
    """The same scene lit by a synthetic light map (Environment::Map): the light
    map's preparation (oracle restatement of environment.rs), then two
    accumulate-frames of two paths each from the reference's pt.comp."""
    n, size, frames, spf = 24, 24, 2, 2
    cfg = scene.small_config(n=n, size=size, spp=frames * spf)
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    r.set_labels(cfg["labels_vol"], cfg["soft"])
    light_map = scene.synthetic_light_map(32, 16, seed=5)
    r.set_environment_map(light_map)
    g = r.geo
    params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True, spf=spf)
    params.lighting.environment = abi.ENV_MAP
    r.resize(size, size)
    r.normals = R.normals(r, r._uniforms_geometry_only())
    u1 = r.uniforms(params, 1, size, size)
    r.mask = R.mask(r, u1, O.mask_margin(cfg["volume"], params.labels), int(params.labels.smoothing))
    r.majorant = R.majorant(r, u1)
    acc = np.zeros((size, size, 4), np.float32)
    alb, nor = np.zeros_like(acc), np.zeros_like(acc)
    hdr = np.zeros((size, size, 4), np.uint16)
    for f in range(frames):
        r.accumulated = f * spf
        u = r.uniforms(params, f + 1, size, size)
        R.pt_frame(r, u, acc, alb, nor, hdr)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_light_map.npz")
    np.savez_compressed(out, hu=cfg["hu"], labels=cfg["labels_vol"], soft=cfg["soft"],
                        spacing=np.array(cfg["spacing"]), params=np.frombuffer(bytes(params), np.uint8),
                        width=size, height=size, frames=frames, light_map=light_map, env_rad=r.env_rad,
                        env_table=r.env_table, env_peak_u=r.env_peak_u, uniforms_frame1=u1, accum=acc,
                        albedo=alb, normal=nor, hdr=hdr)
    print(out, os.path.getsize(out), "bytes")


def raymarch_fixture():
    """The real-time ray marcher (path_tracing off) on the same scene: the
    ambient-occlusion volume (ao.comp), the shadow volume swept towards the key
    light (shadow.comp, record_shadow_sweep) and the image (dvr.comp), for
    point-sampled and pre-integrated transfer functions, studio and light map."""
    n, W, H = 24, 32, 24
    cfg = scene.small_config(n=n, size=W, spp=1)
    r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
    r.set_labels(cfg["labels_vol"], cfg["soft"])
    light_map = scene.synthetic_light_map(32, 16, seed=5)
    g = r.geo
    r.resize(W, H)
    r.normals = R.normals(r, r._uniforms_geometry_only())
    out = {"hu": cfg["hu"], "labels": cfg["labels_vol"], "soft": cfg["soft"], "spacing": np.array(cfg["spacing"]),
           "width": W, "height": H, "light_map": light_map}
    for name, pre, env in (("point", 0, False), ("preint", 1, False), ("map", 1, True)):
        params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True)
        params.camera.distance = abi.f32(params.camera.distance * 0.6)
        params.path_tracing.enabled = 0
        params.preintegrate = pre
        if env:
            r.set_environment_map(light_map)
            params.lighting.environment = abi.ENV_MAP
        else:
            r.set_environment_map(None)
        u = r.uniforms(params, 1, W, H)
        r.mask = R.mask(r, u, O.mask_margin(cfg["volume"], params.labels), int(params.labels.smoothing))
        r.majorant = R.majorant(r, u)
        ao = R.ao_volume(r, u)
        shadow = R.shadow_sweep(r, u, u.view(np.float32)[44:47])
        hdr = R.dvr(r, u, W, H, shadow=shadow, ao=ao)
        out.update({f"{name}_params": np.frombuffer(bytes(params), np.uint8), f"{name}_uniforms": u,
                    f"{name}_ao": ao, f"{name}_shadow": shadow, f"{name}_hdr": hdr})
        if env:
            out["map_env_diffuse"] = r.env_diffuse
    out["mask"], out["majorant"] = r.mask, r.majorant
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_raymarch.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def modes_fixture():
    """mask.comp, majorant.comp and pt.comp in each of scene.MODE_CASES."""
    n, size, frames, spf = 24, 24, 2, 2
    cfg = scene.small_config(n=n, size=size, spp=frames * spf)
    out = {"hu": cfg["hu"], "labels": cfg["labels_vol"], "soft": cfg["soft"], "spacing": np.array(cfg["spacing"]),
           "width": size, "height": size, "frames": frames}
    for name in scene.MODE_CASES:
        r = O.CpuRenderer(cfg["volume"], cfg["tf"], cfg["hu"])
        g = r.geo
        params = scene.frame_params_for(cfg, list(g.center), g.diagonal, clip_sagittal=True, spf=spf)
        params.camera.distance = abi.f32(params.camera.distance * 0.45)  # the phantom fills the image
        soft = scene.mode_case(name, params, list(g.center))
        r.set_labels(cfg["labels_vol"], cfg["soft"] if soft else None)
        r.resize(size, size)
        r.normals = R.normals(r, r._uniforms_geometry_only())
        u1 = r.uniforms(params, 1, size, size)
        if int(params.labels.mode) != abi.LABEL_OFF:
            r.mask = R.mask(r, u1, O.mask_margin(cfg["volume"], params.labels), int(params.labels.smoothing))
        else:
            r.mask = np.zeros(r.density.shape + (2,), np.uint16)  # not read in mode Off
        r.majorant = R.majorant(r, u1)
        acc = np.zeros((size, size, 4), np.float32)
        alb, nor = np.zeros_like(acc), np.zeros_like(acc)
        hdr = np.zeros((size, size, 4), np.uint16)
        for f in range(frames):
            r.accumulated = f * spf
            u = r.uniforms(params, f + 1, size, size)
            R.pt_frame(r, u, acc, alb, nor, hdr)
        out.update({f"{name}_params": np.frombuffer(bytes(params), np.uint8), f"{name}_soft": int(soft),
                    f"{name}_uniforms": u1, f"{name}_mask": r.mask, f"{name}_majorant": r.majorant,
                    f"{name}_accum": acc, f"{name}_albedo": alb, f"{name}_normal": nor})
        print(name, "background share", float(acc[..., 3].mean()) / (frames * spf),
              "radiance mean", float(acc[..., :3].mean()))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_modes.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    which = sys.argv[1:] or ["main", "light_map", "raymarch", "modes"]
    if "main" in which:
        main()
    if "light_map" in which:
        light_map_fixture()
    if "raymarch" in which:
        raymarch_fixture()
    if "modes" in which:
        modes_fixture()
