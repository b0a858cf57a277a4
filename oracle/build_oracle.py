"""Compiles the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The oracle restates the reference's path on the CPU (oracle.hpp). Flags fix the
floating-point conventions that glsl.hpp documents: single-precision literals,
no FMA contraction (so x86 and Arm hosts give the same results).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["oracle_host.cpp", "oracle_shaders.cpp", "oracle_api.cpp"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
FLAGS = ["-std=c++20", "-O2", "-fPIC", "-fsingle-precision-constant", "-ffp-contract=off",
         "-fno-strict-aliasing", "-pthread", "-Wall", "-Wno-unused-variable", "-Wno-pedantic"]


# The FP64 instance: the same restatement with `float` defined as `double`
# (prelude.hpp), one translation unit, literals left at their single-precision
# values (no -fsingle-precision-constant: the shaders' constants are float
# literals with an f suffix).
SOURCES64 = ["oracle_api64.cpp"]
LIB64 = os.path.join(OUT_DIR, "liboracle64.so")
FLAGS64 = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fno-strict-aliasing", "-pthread", "-Wall",
           "-Wno-unused-variable", "-Wno-pedantic"]


def build64(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(HERE, s) for s in SOURCES64 + SOURCES] + \
        [os.path.join(HERE, f) for f in ("glsl.hpp", "oracle.hpp", "prelude.hpp")] + \
        [os.path.join(HERE, "..", "include", "volpt.h")]
    if os.path.exists(LIB64) and all(os.path.getmtime(LIB64) >= os.path.getmtime(d) for d in deps):
        return LIB64
    r = subprocess.run(["g++", *FLAGS64, "-shared", *[os.path.join(HERE, s) for s in SOURCES64], "-o", LIB64],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"FP64 oracle build failed:\n{r.stderr[-6000:]}")
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    return LIB64


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "glsl.hpp"), os.path.join(HERE, "oracle.hpp"), os.path.join(HERE, "prelude.hpp"),
                   os.path.join(HERE, "..", "include", "volpt.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        build64(verbose)
        return LIB
    objs = []
    procs = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s).replace(".cpp", ".o"))
        objs.append(o)
        procs.append(subprocess.Popen(["g++", *FLAGS, "-c", s, "-o", o],
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for p, s in zip(procs, srcs):
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"oracle build failed for {s}:\n{err[-6000:]}")
        if verbose and err:
            print(err, file=sys.stderr)
    subprocess.run(["g++", "-shared", "-pthread", *objs, "-o", LIB], check=True)
    build64(verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
