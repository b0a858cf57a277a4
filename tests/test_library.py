"""The C-ABI library on a machine without a GPU: it loads, exports every
symbol the headers declare, and its host-side defaults match the reference's."""
import ctypes as C
import os
import re

import pytest

from volview_gb300 import abi
from volview_gb300 import renderer as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(vv_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol():
    lib = R.load()
    names = declared("volpt.h") + declared("volpt_probe.h")
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    bound = {e[0] for e in R.EXPORTS + R.PROBES}
    assert set(names) <= bound, set(names) - bound


def test_defaults_match_reference():
    lib = R.load()
    L = abi.Lighting()
    lib.vv_lighting_default(C.byref(L))
    assert bytes(L) == bytes(abi.lighting_default())
    lp = abi.LabelParams()
    lib.vv_label_params_default(C.byref(lp))
    assert bytes(lp) == bytes(abi.label_params_default())
    pt = abi.PathTracing()
    lib.vv_path_tracing_default(C.byref(pt))
    assert bytes(pt) == bytes(abi.path_tracing_default())
    cl = abi.Clipping()
    lib.vv_clipping_default(C.byref(cl))
    assert bytes(cl) == bytes(abi.clipping_default())
    cam = abi.OrbitCamera()
    lib.vv_orbit_camera_framing((C.c_float * 3)(1.0, 2.0, 3.0), 217.5, C.byref(cam))
    assert bytes(cam) == bytes(abi.camera_framing((1.0, 2.0, 3.0), 217.5))


def test_struct_sizes_match_header():
    assert C.sizeof(abi.FrameParams) == C.sizeof(abi.OrbitCamera) + 8 + C.sizeof(abi.LabelParams) + \
        C.sizeof(abi.Lighting) + 8 + C.sizeof(abi.Clipping) + C.sizeof(abi.PathTracing) + 4
    assert C.sizeof(abi.LabelParams) == 24 + 5 * 256 * 16 + 256


def test_fails_loudly_without_a_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(R.VolptError) as e:
        R.Context(0)
    assert e.value.status == abi.VV_ERR_CUDA
