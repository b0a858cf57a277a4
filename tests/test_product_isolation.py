"""The product does not reach the oracle (CPU, static): no module of the
volview_gb300 package imports `oracle`, and no CUDA or C++ source of the
library includes an oracle header. The oracle is the checker; a product path
through it would be a CPU fallback."""
import ast
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "volview_gb300")


def _python_modules():
    for name in sorted(os.listdir(PKG)):
        if name.endswith(".py"):
            yield os.path.join(PKG, name)


def test_package_modules_do_not_import_the_oracle():
    for path in _python_modules():
        tree = ast.parse(open(path).read(), path)
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                names = [node.module or ""]
            else:
                continue
            for n in names:
                assert n.split(".")[0] != "oracle", f"{path}:{node.lineno} imports {n}"


def test_library_sources_do_not_include_oracle_headers():
    csrc = os.path.join(PKG, "csrc")
    include = re.compile(r'^\s*#\s*include\s*[<"]([^>"]+)[>"]', re.M)
    for name in sorted(os.listdir(csrc)):
        if not name.endswith((".cu", ".cuh", ".cpp", ".h")):
            continue
        for inc in include.findall(open(os.path.join(csrc, name)).read()):
            assert "oracle" not in inc, f"{name} includes {inc}"
