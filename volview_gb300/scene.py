"""Seeded synthetic CT scenes that stand in for the reference's DICOM datasets.

No CT data ships with the reference (its `data/` holds download lists only), so
every benchmark and test volume is generated here from a seed:

* `small_phantom` — 128^3 int16 HU at 1 mm: air -1000, an ellipsoid body 0+-40,
  a 4 mm skull shell 1000+-80 around a brain, two lungs -800+-50; labels in 10
  classes by region; a signed distance to each label boundary, clamped to +-3 mm,
  as the soft margin.
* `head_neck_phantom` — 512x512x400 int16 HU at 0.5x0.5x1 mm: skull, spine,
  30 tubular vessels at 400+-50 HU, 6 organ ellipsoids, airway, 120 labels; the
  soft margin stored as FP16 before quantisation.

The per-label render parameters follow the viewer's recipes: `density_stats`
(crates/app/src/labels.rs:550-~600), `Group::optics` / `subsurface` / `coat`
(labels.rs:177-237) and `surface_texture` (labels.rs:662-688).
"""
import math

import numpy as np

from . import abi

HU_MIN, HU_MAX = -1024.0, 3071.0
BINS = int(HU_MAX - HU_MIN) + 1

# Group recipes (crates/app/src/labels.rs:177-237, 662-688).
SKELETON, LUNGS, VESSELS, OTHER, MUSCLES, BRAIN = "skeleton", "lungs", "vessels", "other", "muscles", "brain"
SUBSURFACE = {SKELETON: 0.15, LUNGS: 0.15, VESSELS: 0.45, OTHER: 0.5, MUSCLES: 0.5, BRAIN: 0.5}
COAT = {SKELETON: 0.0, LUNGS: 0.3, VESSELS: 0.8, OTHER: 0.5, MUSCLES: 0.4, BRAIN: 0.5}
SCATTERING = {"bone": (2.29, 0.716), "soft": (1.89, 1.286), "brain": (2.42, 1.611)}
SURFACE = {SKELETON: (0.0, 0.0, 0.0, 0.0), LUNGS: (2.0, 0.12, 0.25, 15.0), VESSELS: (1.0, 0.06, 0.1, 6.0),
           OTHER: (1.0, 0.06, 0.15, 6.0), MUSCLES: (1.0, 0.08, 0.25, 3.0), BRAIN: (1.0, 0.06, 0.15, 6.0)}


def optics(group):
    """Group::optics: mu_s'(lambda) = a (lambda / 500 nm)^-b at 650/550/450 nm."""
    a, b = SCATTERING["bone" if group == SKELETON else "brain" if group == BRAIN else "soft"]
    a32, b32 = np.float32(a), np.float32(b)
    return [float(a32 * np.float32(np.float32(nm) / np.float32(500.0)) ** -b32) for nm in (650.0, 550.0, 450.0)] + [1.0]


def density_stats(hist):
    """Hybrid opacity ramp and texture statistics of one label (labels.rs:550-~600)."""
    total = int(hist.sum())
    cum = np.cumsum(hist, dtype=np.int64)

    def pct(p):
        target = max(int(math.ceil(p * total)), 1)
        i = int(np.searchsorted(cum, target, side="left"))
        i = min(i, BINS - 1)
        return float(np.float32(i) / np.float32(BINS - 1))

    p02, p10, p25, p50, p75 = (pct(p) for p in (0.02, 0.10, 0.25, 0.5, 0.75))
    if p25 < float(np.float32(-300.0 - HU_MIN) / np.float32(BINS - 1)):
        return [0.0, 1e-3, p50, -1.0]
    mw = float(np.float32(10.0) / np.float32(BINS - 1))
    return [p02, max(p10, float(np.float32(p02) + np.float32(mw))), p50,
            max(float(np.float32(p75) - np.float32(p25)), mw)]


def label_histograms(labels, hu):
    """HU histogram per label value, one HU per bin (labels.rs:511-547)."""
    b = np.clip(hu.astype(np.float32) - np.float32(HU_MIN), 0, BINS - 1).astype(np.int64)
    idx = labels.astype(np.int64).ravel() * BINS + b.ravel()
    return np.bincount(idx, minlength=256 * BINS).reshape(256, BINS)


def label_params(labels, hu, entries, mode=abi.LABEL_HYBRID, ghost_groups=(), tint=0.7, extinction=0.5):
    """LabelSet::params (labels.rs:463-502) for `entries`: value -> (group, rgb, roughness)."""
    p = abi.label_params_default()
    p.mode = mode
    p.tint = tint
    p.extinction = extinction
    hist = label_histograms(labels, hu)
    for v, (group, rgb, rough) in entries.items():
        p.colors[v][:] = [rgb[0], rgb[1], rgb[2], 1.0]
        p.materials[v][:] = [rough, 0.0, SUBSURFACE[group], COAT[group]]
        p.optics[v][:] = optics(group)
        p.surface[v][:] = SURFACE[group]
        p.ghost[v] = 1 if group in ghost_groups else 0
        p.density[v][:] = density_stats(hist[v])
    return p


def soft_grid(labels, spacing, factor=1, sd_clamp=3.0, sd_dtype=np.float32):
    """Soft-label grid (best, runner-up, margin x 16, overridden) from a label volume.

    The margin is the signed distance (mm) to the nearest label boundary, stored
    as `sd_dtype`, clamped to +-`sd_clamp` and scaled so the clamp reaches the
    mask pass's certainty (4 logits). Runner-up: the label across that boundary.
    """
    from scipy import ndimage

    g = labels[::factor, ::factor, ::factor]
    gs = np.asarray(spacing, dtype=np.float64)[::-1] * factor  # (z, y, x) spacing
    boundary = np.zeros(g.shape, dtype=bool)
    for ax in range(3):
        d = np.diff(g, axis=ax) != 0
        sl_lo = [slice(None)] * 3
        sl_hi = [slice(None)] * 3
        sl_lo[ax] = slice(0, -1)
        sl_hi[ax] = slice(1, None)
        boundary[tuple(sl_lo)] |= d
        boundary[tuple(sl_hi)] |= d
    dist, ind = ndimage.distance_transform_edt(~boundary, sampling=gs, return_indices=True)
    sd = np.minimum(dist, sd_clamp).astype(sd_dtype)
    nb = g[ind[0], ind[1], ind[2]]  # label at the nearest boundary voxel
    # Runner-up: a neighbour of that boundary voxel with another label.
    second = np.where(nb != g, nb, 0).astype(np.uint8)
    same = second == 0
    if same.any():
        zi, yi, xi = ind[0][same], ind[1][same], ind[2][same]
        own = g[same]
        cand = np.zeros_like(own)
        for dz, dy, dx in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            zz = np.clip(zi + dz, 0, g.shape[0] - 1)
            yy = np.clip(yi + dy, 0, g.shape[1] - 1)
            xx = np.clip(xi + dx, 0, g.shape[2] - 1)
            v = g[zz, yy, xx]
            take = (cand == 0) & (v != own)
            cand[take] = v[take]
        second[same] = cand
    margin = np.minimum(sd.astype(np.float32) * np.float32(4.0 / sd_clamp), np.float32(15.9)) * np.float32(16.0)
    out = np.zeros(g.shape + (4,), dtype=np.uint8)
    out[..., 0] = g
    out[..., 1] = second
    out[..., 2] = margin.astype(np.uint8)
    return out


def _ellipsoid(shape, center, radii):
    """Normalised radius |(p - c) / r| over the index grid (z, y, x)."""
    z, y, x = np.ogrid[:shape[0], :shape[1], :shape[2]]
    return np.sqrt(((x - center[0]) / radii[0]) ** 2 + ((y - center[1]) / radii[1]) ** 2 +
                   ((z - center[2]) / radii[2]) ** 2).astype(np.float32)


def small_phantom(seed=1, n=128):
    """The 128^3, 1 mm phantom and its 10 region labels."""
    rng = np.random.default_rng(seed)
    s = n / 128.0
    shape = (n, n, n)
    hu = np.full(shape, -1000.0, dtype=np.float32)
    lab = np.zeros(shape, dtype=np.uint8)
    noise = rng.standard_normal(shape, dtype=np.float32)
    c = (n / 2 - 0.5, n / 2 - 0.5, n / 2 - 0.5)
    body = _ellipsoid(shape, c, (50 * s, 40 * s, 58 * s)) <= 1.0
    hu[body] = 0.0 + 40.0 * noise[body]
    z, y, x = np.ogrid[:n, :n, :n]
    # Body regions: 3 slabs along z x left/right -> labels 5..10.
    slab = np.clip(((z - (c[2] - 58 * s)) / (116 * s) * 3).astype(int), 0, 2)
    side = (x >= c[0]).astype(int)
    region = (5 + slab * 2 + side).astype(np.uint8)
    lab[body] = np.broadcast_to(region, shape)[body]
    head_c = (c[0], c[1], c[2] + 31 * s)
    r_out = _ellipsoid(shape, head_c, (34 * s, 38 * s, 26 * s))
    r_in = _ellipsoid(shape, head_c, (30 * s, 34 * s, 22 * s))
    skull = (r_out <= 1.0) & (r_in > 1.0)
    brain = r_in <= 1.0
    hu[brain] = 20.0 + 20.0 * noise[brain]
    lab[brain] = 4
    hu[skull] = 1000.0 + 80.0 * noise[skull]
    lab[skull] = 1
    for k, dx in enumerate((-20 * s, 20 * s)):
        lung = _ellipsoid(shape, (c[0] + dx, c[1], c[2] - 14 * s), (14 * s, 18 * s, 24 * s)) <= 1.0
        hu[lung] = -800.0 + 50.0 * noise[lung]
        lab[lung] = 2 + k
    hu = np.clip(np.rint(hu), -32768, 32767).astype(np.int16)
    return hu, lab


def torso_phantom(seed=1, dims=(512, 512, 800)):
    """The small phantom's recipe scaled per axis to `dims` (x, y, z) voxels of
    1 mm (the precision workload's torso): body ellipsoid 0 +- 40 HU, skull
    shell 1000 +- 80, brain 20 +- 20, two lungs -800 +- 50, 10 region labels.
    Generated 32 slices at a time."""
    nx, ny, nz = dims
    sx, sy, sz = nx / 128.0, ny / 128.0, nz / 128.0
    rng = np.random.default_rng(seed)
    hu = np.empty((nz, ny, nx), np.int16)
    lab = np.zeros((nz, ny, nx), np.uint8)
    c = (nx / 2 - 0.5, ny / 2 - 0.5, nz / 2 - 0.5)
    head_c = (c[0], c[1], c[2] + 31 * sz)
    y, x = np.ogrid[:ny, :nx]
    side = (x >= c[0]).astype(np.uint8)

    def ell(zz, center, radii):
        return (((x - center[0]) / radii[0]) ** 2 + ((y - center[1]) / radii[1]) ** 2 +
                ((zz - center[2]) / radii[2]) ** 2)

    for z0 in range(0, nz, 32):
        z1 = min(z0 + 32, nz)
        zz = np.arange(z0, z1, dtype=np.float64)[:, None, None]
        noise = rng.standard_normal((z1 - z0, ny, nx), dtype=np.float32)
        h = np.full((z1 - z0, ny, nx), -1000.0, np.float32)
        l = np.zeros((z1 - z0, ny, nx), np.uint8)
        body = ell(zz, c, (50 * sx, 40 * sy, 58 * sz)) <= 1.0
        h[body] = 40.0 * noise[body]
        slab = np.clip(((zz - (c[2] - 58 * sz)) / (116 * sz) * 3).astype(int), 0, 2).astype(np.uint8)
        region = np.broadcast_to(5 + slab * 2 + side, h.shape)
        l[body] = region[body]
        r_out = ell(zz, head_c, (34 * sx, 38 * sy, 26 * sz))
        r_in = ell(zz, head_c, (30 * sx, 34 * sy, 22 * sz))
        skull, brain = (r_out <= 1.0) & (r_in > 1.0), r_in <= 1.0
        h[brain] = 20.0 + 20.0 * noise[brain]
        l[brain] = 4
        h[skull] = 1000.0 + 80.0 * noise[skull]
        l[skull] = 1
        for k, dx in enumerate((-20 * sx, 20 * sx)):
            lung = ell(zz, (c[0] + dx, c[1], c[2] - 14 * sz), (14 * sx, 18 * sy, 24 * sz)) <= 1.0
            h[lung] = -800.0 + 50.0 * noise[lung]
            l[lung] = 2 + k
        hu[z0:z1] = np.clip(np.rint(h), -32768, 32767).astype(np.int16)
        lab[z0:z1] = l
    return hu, lab


SMALL_ENTRIES = {
    1: (SKELETON, (0.84, 0.79, 0.70), 0.42),
    2: (LUNGS, (0.58, 0.33, 0.35), 0.5),
    3: (LUNGS, (0.58, 0.33, 0.35), 0.5),
    4: (BRAIN, (0.79, 0.69, 0.58), 0.3),
    5: (MUSCLES, (0.27, 0.02, 0.016), 0.4),
    6: (MUSCLES, (0.27, 0.02, 0.016), 0.4),
    7: (OTHER, (0.42, 0.13, 0.10), 0.35),
    8: (OTHER, (0.42, 0.13, 0.10), 0.35),
    9: (MUSCLES, (0.30, 0.03, 0.02), 0.45),
    10: (MUSCLES, (0.30, 0.03, 0.02), 0.45),
}


def head_neck_phantom(seed=2, dims=(512, 512, 400), spacing=(0.5, 0.5, 1.0)):
    """The head/neck phantom: int16 HU (z, y, x) and 120 labels."""
    rng = np.random.default_rng(seed)
    X, Y, Z = dims
    sx, sy, sz = spacing
    shape = (Z, Y, X)
    hu = np.full(shape, -1000.0, dtype=np.float32)
    lab = np.zeros(shape, dtype=np.uint8)
    noise = rng.standard_normal(shape, dtype=np.float32)
    cx, cy = (X - 1) / 2.0, (Y - 1) / 2.0
    ext_z = Z * sz
    z_mm = (np.arange(Z, dtype=np.float32) + 0.5) * sz
    # Neck: elliptic cylinder below the head; head: ellipsoid.
    head_cz = 0.72 * ext_z
    head_r = (74.0, 92.0, 0.27 * ext_z)
    neck_r = (55.0, 50.0)
    y_mm = ((np.arange(Y, dtype=np.float32) - cy) * sy)[:, None]
    x_mm = ((np.arange(X, dtype=np.float32) - cx) * sx)[None, :]
    region_of = np.zeros(shape, dtype=np.uint8)
    for k in range(Z):
        zz = z_mm[k]
        head = (x_mm / head_r[0]) ** 2 + (y_mm / head_r[1]) ** 2 + ((zz - head_cz) / head_r[2]) ** 2
        neck = ((x_mm / neck_r[0]) ** 2 + ((y_mm - 8.0) / neck_r[1]) ** 2 <= 1.0) & (zz < head_cz)
        inside = (head <= 1.0) | neck
        hu[k][inside] = 40.0 + 40.0 * noise[k][inside]
        # 57 body regions (62..118): angular sectors x height bands.
        ang = np.arctan2(y_mm, x_mm)
        sector = ((ang + np.pi) / (2 * np.pi) * 8).astype(np.int32) % 8
        band = min(int(zz / (head_cz - 0.6 * head_r[2]) * 8), 7)
        reg = 62 + np.minimum(band * 8 + sector, 56)
        lab[k][inside] = np.broadcast_to(reg, (Y, X))[inside].astype(np.uint8)
        # Skull: 6 mm shell of the head ellipsoid above the neck junction.
        inner = (x_mm / (head_r[0] - 6)) ** 2 + (y_mm / (head_r[1] - 6)) ** 2 + ((zz - head_cz) / (head_r[2] - 6)) ** 2
        skull = (head <= 1.0) & (inner > 1.0) & (zz > head_cz - 0.6 * head_r[2])
        hu[k][skull] = 1000.0 + 80.0 * noise[k][skull]
        lab[k][skull] = 1
        brain = inner <= 1.0
        hu[k][brain] = 30.0 + 20.0 * noise[k][brain]
        lab[k][brain] = 56
        # Airway (hollow): a tube anterior of the spine in the neck.
        air = ((x_mm / 9.0) ** 2 + ((y_mm + 12.0) / 8.0) ** 2 <= 1.0) & (zz < head_cz - 20)
        hu[k][air] = -900.0 + 30.0 * noise[k][air]
        lab[k][air] = 57
        # Spine: vertebral bodies (labels 2..25) separated by discs, posterior.
        vert = int(zz // 10.0)
        if zz < head_cz - 0.4 * head_r[2] and (zz % 10.0) < 7.5 and vert < 24:
            body = ((x_mm / 13.0) ** 2 + ((y_mm - 22.0) / 11.0) ** 2 <= 1.0) | (
                (x_mm / 4.0) ** 2 + ((y_mm - 40.0) / 9.0) ** 2 <= 1.0)
            hu[k][body] = 700.0 + 80.0 * noise[k][body]
            lab[k][body] = 2 + vert
    # 30 vessels (labels 26..55): tubes winding up through the neck into the head.
    t = z_mm / ext_z
    for v in range(30):
        ang0 = rng.uniform(0, 2 * np.pi)
        rad0 = rng.uniform(15.0, 45.0)
        amp = rng.uniform(3.0, 12.0)
        freq = rng.uniform(1.0, 3.0)
        r = rng.uniform(1.5, 4.0)
        top = rng.uniform(0.55, 0.95)
        px = rad0 * np.cos(ang0) + amp * np.sin(2 * np.pi * freq * t + v)
        py = rad0 * np.sin(ang0) * 0.8 + amp * np.cos(2 * np.pi * freq * t * 0.7 + 2 * v)
        for k in range(Z):
            if t[k] > top:
                break
            x0 = int((px[k] / sx + cx) - r / sx - 1)
            x1 = int((px[k] / sx + cx) + r / sx + 2)
            y0 = int((py[k] / sy + cy) - r / sy - 1)
            y1 = int((py[k] / sy + cy) + r / sy + 2)
            x0, y0, x1, y1 = max(x0, 0), max(y0, 0), min(x1, X), min(y1, Y)
            if x0 >= x1 or y0 >= y1:
                continue
            xs = (np.arange(x0, x1) - cx) * sx - px[k]
            ys = ((np.arange(y0, y1) - cy) * sy - py[k])[:, None]
            m = xs[None, :] ** 2 + ys ** 2 <= r * r
            sub_hu = hu[k, y0:y1, x0:x1]
            sub_hu[m] = 400.0 + 50.0 * noise[k, y0:y1, x0:x1][m]
            lab[k, y0:y1, x0:x1][m] = 26 + v
    # 6 organs (labels 58..61, 119, 120): ellipsoids in the neck and face.
    organs = [((0.0, -25.0, 0.35), (18.0, 8.0, 14.0), 60.0),    # thyroid
              ((0.0, -40.0, 0.55), (22.0, 20.0, 16.0), 70.0),   # tongue
              ((-40.0, 5.0, 0.58), (12.0, 18.0, 20.0), 35.0),   # parotid L
              ((40.0, 5.0, 0.58), (12.0, 18.0, 20.0), 35.0),    # parotid R
              ((-30.0, -70.0, 0.74), (11.0, 11.0, 11.0), 15.0),  # eye L
              ((30.0, -70.0, 0.74), (11.0, 11.0, 11.0), 15.0)]   # eye R
    organ_labels = [58, 59, 60, 61, 119, 120]
    for label, ((ox, oy, oz), (rx, ry, rz), base) in zip(organ_labels, organs):
        k0 = max(int((oz * ext_z - rz) / sz) - 1, 0)
        k1 = min(int((oz * ext_z + rz) / sz) + 2, Z)
        for k in range(k0, k1):
            e = ((x_mm - ox) / rx) ** 2 + ((y_mm - oy) / ry) ** 2 + ((z_mm[k] - oz * ext_z) / rz) ** 2 <= 1.0
            hu[k][e] = base + 20.0 * noise[k][e]
            lab[k][e] = label
    hu = np.clip(np.rint(hu), -32768, 32767).astype(np.int16)
    return hu, lab


def head_neck_entries(seed=2):
    """120 labels with albedo and roughness drawn from U[0.1, 0.9]."""
    rng = np.random.default_rng(seed + 1000)
    groups = {1: SKELETON, 56: BRAIN, 57: LUNGS}
    for v in range(2, 26):
        groups[v] = SKELETON
    for v in range(26, 56):
        groups[v] = VESSELS
    for v in (58, 59, 60, 61, 119, 120):
        groups[v] = OTHER
    for v in range(62, 119):
        groups[v] = MUSCLES
    entries = {}
    for v in sorted(groups):
        rgb = tuple(float(np.float32(a)) for a in rng.uniform(0.1, 0.9, 3))
        rough = float(np.float32(rng.uniform(0.1, 0.9)))
        entries[v] = (groups[v], rgb, rough)
    return entries


def small_config(seed=1, n=128, size=256, spp=64, mode=abi.LABEL_HYBRID, soft=True):
    """Config of the small scene: volume, TF, labels, soft grid, frame params."""
    hu, lab = small_phantom(seed, n)
    spacing = (128.0 / n,) * 3
    vol = abi.volume_struct(hu, spacing)
    tf = abi.tf_struct(abi.PRESETS["bone"])
    labels = label_params(lab, hu, SMALL_ENTRIES, mode=mode)
    soft_data = soft_grid(lab, spacing, 1, 3.0, np.float32) if soft else None
    return dict(hu=hu, labels_vol=lab, spacing=spacing, volume=vol, tf=tf, label_params=labels,
                soft=soft_data, width=size, height=size, spp=spp, min_spacing=min(spacing))


def torso_config(seed=1, dims=(512, 512, 800), width=1920, height=1080, spp=4096, soft=True):
    """The precision workload: the small phantom scaled to a 512x512x800 torso of
    1 mm voxels, 1920x1080, 4096 paths per pixel; soft labels on a 4x coarser
    grid with FP16 margins (or none: binary label masks)."""
    hu, lab = torso_phantom(seed, dims)
    spacing = (1.0, 1.0, 1.0)
    vol = abi.volume_struct(hu, spacing)
    tf = abi.tf_struct(abi.PRESETS["bone"])
    labels = label_params(lab, hu, SMALL_ENTRIES, mode=abi.LABEL_HYBRID)
    soft_data = soft_grid(lab, spacing, 4, 3.0, np.float16) if soft else None
    return dict(hu=hu, labels_vol=lab, spacing=spacing, volume=vol, tf=tf, label_params=labels,
                soft=soft_data, width=width, height=height, spp=spp, min_spacing=min(spacing))


def head_neck_config(seed=2, dims=(512, 512, 400), spacing=(0.5, 0.5, 1.0), size=1024, spp=1024):
    hu, lab = head_neck_phantom(seed, dims, spacing)
    vol = abi.volume_struct(hu, spacing)
    tf = abi.tf_struct(abi.PRESETS["bone"])
    labels = label_params(lab, hu, head_neck_entries(seed), mode=abi.LABEL_HYBRID, ghost_groups=(SKELETON,))
    soft_data = soft_grid(lab, spacing, 3, 3.0, np.float16)
    return dict(hu=hu, labels_vol=lab, spacing=spacing, volume=vol, tf=tf, label_params=labels,
                soft=soft_data, width=size, height=size, spp=spp, min_spacing=min(spacing))


def frame_params_for(cfg, center, diagonal, clip_sagittal=False, anisotropy=0.6, spf=1,
                     denoiser=abi.DENOISE_ATROUS):
    """FrameParams with the CLI defaults (crates/app/src/main.rs:60-202)."""
    cam = abi.camera_framing(center, diagonal)
    light = abi.lighting_default()
    light.anisotropy = anisotropy
    light.environment = abi.ENV_STUDIO
    pt = abi.path_tracing_default()
    pt.samples_per_frame = spf
    pt.denoiser = denoiser
    clip = abi.clipping_default()
    if clip_sagittal:
        clip.planes[0].enabled = 1
        clip.planes[0].cut_positive = 1
        clip.planes[0].position = float(center[0])
    return abi.frame_params(cam, abi.f32(0.5 * cfg["min_spacing"]), cfg["label_params"], light, pt, clip)


# Variants of a scene's frame that exercise the reference's other rendering
# modes: the label modes Off, Tint and Isolate (common.glsl:232-351) with
# hidden labels, ghosted labels and their shells (pt.comp:286-289,
# shading.glsl:73-144), binary label masks without a soft grid
# (mask.comp:107-138), the Dome environment (pt.comp:56-82) and the thin lens
# (pt.comp:406-416).
MODE_CASES = ("off", "tint", "isolate", "ghost", "binary", "dome", "lens")


def mode_case(name, params, center):
    """Sets `params` (FrameParams of the small scene) up for mode case `name`;
    returns whether the labels come with their soft grid (False: binary masks)."""
    lp = params.labels
    if name == "off":
        lp.mode = abi.LABEL_OFF
    elif name == "tint":
        lp.mode = abi.LABEL_TINT
        lp.colors[7][3] = 0.0  # one label hidden: cut away, with the tissue near it
    elif name == "isolate":
        lp.mode = abi.LABEL_ISOLATE
        for v in (5, 6):       # muscles hidden
            lp.colors[v][3] = 0.0
    elif name == "ghost":
        lp.mode = abi.LABEL_HYBRID
        for v in (1, 2, 3):    # skeleton and lungs ghosted: shells over the rest
            lp.ghost[v] = 1
    elif name == "binary":
        lp.mode = abi.LABEL_HYBRID
        return False
    elif name == "dome":
        params.lighting.environment = abi.ENV_DOME
    elif name == "lens":
        params.path_tracing.aperture = abi.f32(6.0)
        params.path_tracing.has_focus = 1
        params.path_tracing.focus[:] = [abi.f32(center[0] + 20.0), abi.f32(center[1]), abi.f32(center[2])]
    else:
        raise ValueError(f"unknown mode case {name!r}")
    return True


def random_transfer_function(seed):
    """A seeded transfer function of six control points (HU, albedo, extinction
    0..3 per mm) spread over the density range: a test input whose LUT entries
    round up and down in FP16."""
    rng = np.random.default_rng(seed)
    hu = sorted(rng.uniform(HU_MIN, HU_MAX, 6))
    return abi.tf_struct([(float(h), tuple(float(c) for c in rng.uniform(0.0, 1.0, 3)), float(rng.uniform(0.0, 3.0)))
                          for h in hu])


def synthetic_light_map(width=64, height=32, seed=3):
    """A seeded equirectangular studio-like HDR light map, (height, width, 3) linear RGB,
    rows from the zenith down: a graded sky, a small bright sun and two soft boxes,
    standing in for the reference's HDR (data/hdri/studio_small_09_2k.hdr), which
    is not shipped."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    uu, vv = np.meshgrid(u, v)
    sky = np.stack([0.25 + 0.55 * (1 - vv), 0.28 + 0.6 * (1 - vv), 0.35 + 0.7 * (1 - vv)], -1)
    img = sky * (0.9 + 0.2 * rng.random((height, width, 1)))
    sun_u, sun_v = rng.uniform(0.2, 0.8), rng.uniform(0.15, 0.35)
    d2 = ((uu - sun_u) * 2) ** 2 + (vv - sun_v) ** 2
    img += (d2 < 0.004)[..., None] * np.array([60.0, 55.0, 45.0])
    for _ in range(2):
        cu, cv = rng.uniform(0, 1), rng.uniform(0.3, 0.6)
        box = (np.abs(uu - cu) < 0.06) & (np.abs(vv - cv) < 0.08)
        img += box[..., None] * rng.uniform(3.0, 8.0)
    return np.ascontiguousarray(img, np.float32)
