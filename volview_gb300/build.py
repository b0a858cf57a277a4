"""Builds libvolpt.so (the CUDA path tracer behind include/volpt.h) in-tree.

Every translation unit is compiled for sm_103a only, in parallel, then linked
with a static CUDA runtime so the library loads without LD_LIBRARY_PATH.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvolpt.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["vv_volume.cu", "vv_pt.cu", "vv_pt_exact.cu", "vv_wavefront.cu", "vv_raymarch.cu", "vv_post.cu",
           "vv_noalloc.cu", "vv_nn.cu", "vv_nn_tc.cu", "vv_host.cpp"]
# Compiled once per storage format (VV_DFMT = 0..3: R16_UNORM, FP16, BF16,
# FP32 density with the RG16_UNORM mask; 4, 5: FP16 / BF16 density and mask),
# each into its own namespace, so each format's samplers are specialised for it.
PER_FORMAT = {"vv_pt.cu", "vv_pt_exact.cu", "vv_wavefront.cu", "vv_raymarch.cu"}
FORMATS = 6
# The parity build of the path probe: the oracle's texture-unit arithmetic and
# no multiply-add contraction (every product and sum rounded on its own).
UNIT_FLAGS = {"vv_pt_exact.cu": ["-DVV_EXACT=1", "--fmad=false"]}
# Host code never contracts a*b+c into an FMA (Rust, whose host math the
# renderer restates, does not either; gcc does by default on Arm).
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def build(verbose=False, force=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "volpt.h"))
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    newest = max(os.path.getmtime(p) for p in srcs + headers + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and not extra:
        return LIB
    units = []  # (source, object, defines)
    for s in srcs:
        base = os.path.join(BUILD, os.path.basename(s))
        if os.path.basename(s) in PER_FORMAT:
            units += [(s, f"{base}.f{k}.o", [f"-DVV_DFMT={k}"]) for k in range(FORMATS)]
        else:
            units.append((s, base + ".o", []))
    objs = [o for _, o, _ in units]
    running, jobs = [], max(2, os.cpu_count() or 2)

    def finish(entry):
        s, p = entry
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {s}:\n{err[-8000:]}")
        if verbose and err.strip():
            print(err, file=sys.stderr)

    for s, o, defs in units:
        lang = ["-x", "cu"] if s.endswith(".cu") else ["-x", "c++"]
        cmd = [nvcc(), *ARCH, *NVFLAGS, *UNIT_FLAGS.get(os.path.basename(s), []), *defs, *extra, *lang, "-c", s,
               "-o", o]
        if s.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        if len(running) >= jobs:
            finish(running.pop(0))
        running.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    for entry in running:
        finish(entry)
    link = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB + ".tmp", *objs]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
