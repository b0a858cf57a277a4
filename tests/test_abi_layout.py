"""The Python mirror of the C ABI against the header itself (CPU): a small C
program compiled with include/volpt.h prints every struct's size and every
member's offset, and the ctypes structures of volview_gb300/abi.py must agree
member for member (the tests and the bench pass these structures to the
library by pointer)."""
import os
import shutil
import subprocess

import ctypes as C
import pytest

from volview_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "vv_volume": abi.Volume, "vv_control_point": abi.ControlPoint, "vv_transfer_function": abi.TransferFunction,
    "vv_soft_label_grid": abi.SoftLabelGrid, "vv_environment_map": abi.EnvironmentMap,
    "vv_orbit_camera": abi.OrbitCamera, "vv_label_params": abi.LabelParams, "vv_lighting": abi.Lighting,
    "vv_clip_plane": abi.ClipPlane, "vv_clipping": abi.Clipping, "vv_path_tracing": abi.PathTracing,
    "vv_frame_params": abi.FrameParams, "vv_renderer_info": abi.RendererInfo, "vv_precision": abi.Precision,
    "vv_batch_request": abi.BatchRequest,
}


def _layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "volpt.h"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        table[(cname, field)] = int(value)
    return table


def test_ctypes_structures_match_the_header(tmp_path):
    table = _layout(tmp_path)
    for cname, cls in STRUCTS.items():
        assert C.sizeof(cls) == table[(cname, "size")], cname
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == table[(cname, field)], (cname, field)


def test_enum_values_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = {"VV_OK": abi.VV_OK, "VV_ERR_ARG": abi.VV_ERR_ARG, "VV_ERR_STATE": abi.VV_ERR_STATE,
             "VV_ERR_LIMIT": abi.VV_ERR_LIMIT, "VV_DENOISE_ATROUS": abi.DENOISE_ATROUS,
             "VV_DENOISE_OIDN": abi.DENOISE_OIDN, "VV_DENOISE_LEARNED": abi.DENOISE_LEARNED,
             "VV_VOLUME_SHADOW": abi.VOLUME_SHADOW, "VV_VOLUME_AO": abi.VOLUME_AO,
             "VV_DENSITY_BF16": abi.DENSITY_BF16, "VV_DENSITY_FP32": abi.DENSITY_FP32, "VV_SUMS_KAHAN": abi.SUMS_KAHAN,
             "VV_UNIFORMS_BYTES": 21200}
    body = "".join(f'    printf("{n} %d\\n", (int){n});\n' for n in names)
    src, exe = tmp_path / "enums.c", tmp_path / "enums"
    src.write_text(f'#include <stdio.h>\n#include "volpt.h"\nint main(void) {{\n{body}    return 0;\n}}\n')
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                        text=True).stdout.splitlines())
    for n, v in names.items():
        assert int(out[n]) == v, n
