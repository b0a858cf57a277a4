"""The label file formats of volview's seg crate (CPU): the VVSOFT1 soft-label
cache (crates/seg/src/soft.rs) and NIfTI-1 label maps (crates/seg/src/nifti.rs)."""
import gzip
import json
import struct

import numpy as np
import pytest

from volview_gb300 import abi, seg_io


def test_soft_margins_quantised_as_the_writer_does():
    """soft.rs:44-55: clamp to [0, 15.9], x 16, round half away from zero."""
    m = np.array([-1.0, 0.0, 1 / 32, 0.0937, 1.0, 15.9, 40.0], np.float32)
    s = seg_io.SoftLabels.from_margins((7, 1, 1), (0, 1, 2), (0, 0, 0), np.arange(7), np.arange(7) + 1, m,
                                       np.array([0, 1, 0, 0, 0, 0, 1], bool))
    d = s.data.reshape(-1, 4)
    assert d[:, 2].tolist() == [0, 0, 1, 1, 16, 254, 254]
    assert d[:, 0].tolist() == list(range(7)) and d[:, 1].tolist() == list(range(1, 8))
    assert d[:, 3].tolist() == [0, 1, 0, 0, 0, 0, 1]


def test_soft_file_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    data = rng.integers(0, 256, (3, 4, 5, 4), np.uint8)
    s = seg_io.SoftLabels((5, 4, 3), (2, 0, 1), (1, 0, 1), data)
    path = str(tmp_path / "labels.soft")
    seg_io.write_soft(path, s)
    raw = gzip.decompress(open(path, "rb").read())
    # soft.rs:65-77, byte for byte.
    assert raw == b"VVSOFT1\0" + struct.pack("<3I", 5, 4, 3) + bytes([2, 0, 1]) + bytes([1, 0, 1]) + data.tobytes()
    back = seg_io.read_soft(path)
    assert back.dims == (5, 4, 3) and back.src_axis == (2, 0, 1) and back.flip == (True, False, True)
    assert np.array_equal(back.data, data)
    g = back.grid_struct()
    assert list(g.dims) == [5, 4, 3] and list(g.src_axis) == [2, 0, 1] and list(g.flip) == [1, 0, 1]


def test_soft_file_rejects_bad_input(tmp_path):
    bad = tmp_path / "bad.soft"
    bad.write_bytes(gzip.compress(b"NOTSOFT\0" + bytes(30)))
    with pytest.raises(ValueError, match="not a soft label file"):
        seg_io.read_soft(str(bad))
    short = tmp_path / "short.soft"
    short.write_bytes(gzip.compress(b"VVSOFT1\0" + struct.pack("<3I", 2, 2, 2) + bytes(6) + bytes(31)))
    with pytest.raises(ValueError, match="truncated"):
        seg_io.read_soft(str(short))


def _volume(dims=(6, 5, 4)):
    hu = np.zeros(dims[::-1], np.int16)
    v = abi.volume_struct(hu, (0.5, 0.75, 1.25))
    v.origin[:] = [10.0, -20.0, 30.0]
    return v, hu


@pytest.mark.parametrize("name", ["seg.nii", "seg.nii.gz"])
def test_nifti_round_trip_with_sidecar(tmp_path, name):
    vol, hu = _volume()
    labels = np.random.default_rng(2).integers(0, 120, hu.size, np.uint8)
    path = str(tmp_path / name)
    seg_io.write_labels(path, vol, labels, {3: "liver", 1: "skull"})
    raw = open(path, "rb").read()
    raw = gzip.decompress(raw) if name.endswith(".gz") else raw
    assert struct.unpack_from("<i", raw, 0)[0] == 348 and raw[344:348] == b"n+1\0"
    assert struct.unpack_from("<4h", raw, 40) == (3, 6, 5, 4)
    # The sform is the RAS voxel-to-world transform: LPS with x and y negated.
    assert struct.unpack_from("<4f", raw, 280) == pytest.approx((-0.5, 0.0, 0.0, -10.0))
    assert struct.unpack_from("<4f", raw, 296) == pytest.approx((0.0, -0.75, 0.0, 20.0))
    assert struct.unpack_from("<4f", raw, 312) == pytest.approx((0.0, 0.0, 1.25, 30.0))
    got, names = seg_io.read_labels(path, vol)
    assert np.array_equal(got, labels)
    assert names == {1: "skull", 3: "liver"}
    assert json.load(open(str(tmp_path / "seg.json")))["labels"] == {"1": "skull", "3": "liver"}


def test_nifti_checks_the_grid_and_datatypes(tmp_path):
    vol, hu = _volume()
    labels = np.zeros(hu.size, np.uint8)
    path = str(tmp_path / "seg.nii")
    seg_io.write_labels(path, vol, labels, {})
    other, _ = _volume((6, 5, 3))
    with pytest.raises(ValueError, match="do not match"):
        seg_io.read_labels(path, other)
    moved, _ = _volume()
    moved.origin[0] = 10.5
    with pytest.raises(ValueError, match="different grid"):
        seg_io.read_labels(path, moved)
    # int16 labels (datatype 4) are read too, negative values as 0, above 255 rejected.
    raw = bytearray(open(path, "rb").read())
    struct.pack_into("<h", raw, 70, 4)
    vals = np.arange(hu.size, dtype=np.int16) % 200 - 5
    body = bytes(raw[:352]) + vals.astype("<i2").tobytes()
    p16 = tmp_path / "seg16.nii"
    p16.write_bytes(body)
    got, names = seg_io.read_labels(str(p16), vol)
    assert np.array_equal(got, np.maximum(vals, 0).astype(np.uint8)) and names == {}
    p16.write_bytes(bytes(raw[:352]) + np.full(hu.size, 300, "<i2").tobytes())
    with pytest.raises(ValueError, match="above 255"):
        seg_io.read_labels(str(p16), vol)
    struct.pack_into("<h", raw, 70, 16)
    p32 = tmp_path / "seg32.nii"
    p32.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="unsupported NIfTI datatype 16"):
        seg_io.read_labels(str(p32), vol)
