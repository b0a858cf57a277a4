"""Label inputs of the renderer from files: the soft-label cache and NIfTI-1
label maps, as volview's `seg` crate reads and writes them.

* `read_soft` / `write_soft` — the gzip-compressed VVSOFT1 cache of the
  segmentation model's decision margins (crates/seg/src/soft.rs:14-105): an
  8-byte magic, the grid dims (3 x u32 LE), the volume axis of each grid axis
  (3 x u8), the flips (3 x u8), then per node (x fastest) best label, runner-up,
  margin x 16 and an "overridden" flag. The result feeds `vv_set_labels` as the
  soft grid (`abi.soft_struct`).
* `read_labels` / `write_labels` — uint8 (or int16/uint16) NIfTI-1 label maps on
  the CT's voxel grid with a JSON sidecar of label names
  (crates/seg/src/nifti.rs:31-179), checked against the volume's grid through
  the sform (RAS) within 0.01 mm.

Host-side file formats only: they decode into the arrays the C ABI takes.
"""
import gzip
import json
import os
import struct

import numpy as np

SOFT_MAGIC = b"VVSOFT1\0"
MAX_MARGIN = 15.9   # soft.rs:14: margins beyond this many logits are stored as this
MARGIN_SCALE = 16.0  # soft.rs:16: steps of 1/16 logit
AFFINE_TOLERANCE_MM = 0.01  # nifti.rs:13


class SoftLabels:
    """soft.rs:19-30: grid dims (x, y, z), src_axis, flip and (z, y, x, 4) uint8 nodes."""

    def __init__(self, dims, src_axis, flip, data):
        self.dims = tuple(int(d) for d in dims)
        self.src_axis = tuple(int(a) for a in src_axis)
        self.flip = tuple(bool(f) for f in flip)
        self.data = np.ascontiguousarray(data, np.uint8).reshape(self.dims[2], self.dims[1], self.dims[0], 4)

    @classmethod
    def from_margins(cls, dims, src_axis, flip, best, second, margin, overridden):
        """soft.rs:33-62: margin clamped to [0, 15.9] logits, x 16, rounded half away from zero."""
        m = np.clip(np.asarray(margin, np.float32), np.float32(0.0), np.float32(MAX_MARGIN)) * np.float32(MARGIN_SCALE)
        r = np.floor(m)
        q = (r + ((m - r) >= np.float32(0.5))).astype(np.uint8)  # m >= 0, m - floor(m) exact
        data = np.stack([np.asarray(best, np.uint8).ravel(), np.asarray(second, np.uint8).ravel(), q.ravel(),
                         np.asarray(overridden, bool).ravel().astype(np.uint8)], -1)
        return cls(dims, src_axis, flip, data)

    def grid_struct(self):
        """The vv_soft_label_grid for vv_set_labels."""
        from . import abi
        return abi.soft_struct(self.data, self.src_axis, [int(f) for f in self.flip])


def write_soft(path, soft):
    """soft.rs:65-77."""
    head = SOFT_MAGIC + struct.pack("<3I", *soft.dims) + bytes(soft.src_axis) + bytes(int(f) for f in soft.flip)
    with gzip.open(path, "wb", compresslevel=1) as f:
        f.write(head)
        f.write(soft.data.tobytes())


def read_soft(path):
    """soft.rs:79-105."""
    with gzip.open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 26 or raw[:8] != SOFT_MAGIC:
        raise ValueError("not a soft label file")
    dims = struct.unpack_from("<3I", raw, 8)
    src_axis = tuple(raw[20:23])
    flip = tuple(b != 0 for b in raw[23:26])
    n = int(np.prod(dims, dtype=np.int64))
    body = raw[26:]
    if len(body) != 4 * n:
        raise ValueError("soft label file is truncated")
    return SoftLabels(dims, src_axis, flip, np.frombuffer(body, np.uint8))


def _index_to_world(volume):
    """volume.rs:23-31 in f64: direction x diag(spacing), origin."""
    d = np.array(volume.direction, np.float64).reshape(3, 3).T  # columns are the axes
    m = np.eye(4)
    m[:3, :3] = d * np.array(volume.spacing, np.float64)[None, :]
    m[:3, 3] = np.array(volume.origin, np.float64)
    return m


def ras_affine(volume):
    """nifti.rs:16-18: voxel index to NIfTI world (RAS); volio's world is LPS."""
    return np.diag([-1.0, -1.0, 1.0, 1.0]) @ _index_to_world(volume)


def _sidecar(path):
    name = os.path.basename(path)
    stem = name[:-3] if name.endswith(".gz") else name
    stem = stem[:-4] if stem.endswith(".nii") else stem
    return os.path.join(os.path.dirname(path), stem + ".json")


def write_labels(path, volume, labels, names):
    """nifti.rs:31-104: uint8 NIfTI-1 with the volume's grid as sform, gzip if
    `path` ends in .gz, and the label names (a {label: name} dict) to the sidecar."""
    dims = [int(v) for v in volume.dims]
    h = bytearray(348)
    struct.pack_into("<i", h, 0, 348)
    struct.pack_into("<8h", h, 40, 3, dims[0], dims[1], dims[2], 1, 1, 1, 1)
    struct.pack_into("<h", h, 70, 2)   # datatype: uint8
    struct.pack_into("<h", h, 72, 8)   # bitpix
    sp = [float(v) for v in volume.spacing]
    struct.pack_into("<8f", h, 76, 1.0, sp[0], sp[1], sp[2], 0.0, 0.0, 0.0, 0.0)
    struct.pack_into("<f", h, 108, 352.0)  # vox_offset
    struct.pack_into("<f", h, 112, 1.0)    # scl_slope
    h[123] = 10                            # xyzt_units: mm, s
    struct.pack_into("<h", h, 254, 1)      # sform_code: scanner
    ras = ras_affine(volume)
    for r, off in ((0, 280), (1, 296), (2, 312)):
        struct.pack_into("<4f", h, off, *ras[r])
    h[344:348] = b"n+1\0"
    body = bytes(h) + bytes(4) + np.ascontiguousarray(labels, np.uint8).tobytes()
    if path.endswith(".gz"):
        with gzip.open(path, "wb", compresslevel=1) as f:
            f.write(body)
    else:
        with open(path, "wb") as f:
            f.write(body)
    with open(_sidecar(path), "w") as f:
        json.dump({"labels": {str(k): v for k, v in sorted(names.items())}}, f, indent=2)


def read_labels(path, volume):
    """nifti.rs:106-179: the labels (x-fastest uint8, one per voxel of `volume`)
    and the names of the sidecar ({} without one). Raises ValueError where the
    Rust returns an error."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    if len(raw) < 352:
        raise ValueError("file too small for a NIfTI-1 header")
    if struct.unpack_from("<i", raw, 0)[0] != 348:
        raise ValueError("not a little-endian NIfTI-1 file")
    i16 = lambda off: struct.unpack_from("<h", raw, off)[0]  # noqa: E731
    f32 = lambda off: struct.unpack_from("<f", raw, off)[0]  # noqa: E731
    dims = [i16(42) & 0xFFFF, i16(44) & 0xFFFF, i16(46) & 0xFFFF]
    if not (i16(40) >= 3 and dims == [int(v) for v in volume.dims]):
        raise ValueError(f"label map dims {dims} do not match the volume {list(volume.dims)}")
    if i16(254) > 0:
        expected = ras_affine(volume)
        for r, off in ((0, 280), (1, 296), (2, 312)):
            for c in range(4):
                got = float(f32(off + 4 * c))
                if abs(got - expected[r, c]) > AFFINE_TOLERANCE_MM:
                    raise ValueError(f"label map is on a different grid than the volume (sform row {r} col {c}: "
                                     f"{got} vs {expected[r, c]})")
    n = dims[0] * dims[1] * dims[2]
    offset = max(int(f32(108)), 352)
    data = raw[offset:]
    dtype = i16(70)
    if dtype == 2:
        if len(data) < n:
            raise ValueError("truncated voxel data")
        labels = np.frombuffer(data[:n], np.uint8).copy()
    elif dtype in (4, 512):
        if len(data) < 2 * n:
            raise ValueError("truncated voxel data")
        v = np.maximum(np.frombuffer(data[:2 * n], "<i2").astype(np.int32), 0)  # both read as int16
        if (v > 255).any():
            raise ValueError("label values above 255")
        labels = v.astype(np.uint8)
    else:
        raise ValueError(f"unsupported NIfTI datatype {dtype} for labels")
    names = {}
    try:
        with open(_sidecar(path)) as f:
            names = {int(k): v for k, v in json.load(f)["labels"].items()}
    except FileNotFoundError:
        pass
    return labels, names
