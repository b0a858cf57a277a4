"""Builds the reference's own compute shaders as CPU code (test infrastructure).

The reference's hot path is GLSL (``shaders/*.comp``), compiled for Vulkan. No GLSL
compiler, Vulkan loader or software renderer exists on either machine, so this
recipe compiles the shader sources themselves as C++20 against ``glsl.hpp`` (a
GLSL compatibility layer written for this project): the same arithmetic the GPU
would run, executed on the host cores.

The sources are read where they lie (``<reference>/shaders``) and never copied
into the repository. Six textual rewrites turn GLSL into C++; everything else is
done by macros in ``glsl.hpp`` and the prelude below:

1. the ``#version`` and ``#extension`` lines are dropped;
2. ``#include "x.glsl"`` is inlined (after the same rewrites);
3. ``out T name`` / ``inout T name`` parameters become ``T& name``;
4. ``float[](a, b, c)`` array constructors become ``{a, b, c}``;
5. the shader's ``main`` is renamed ``shader_main``;
6. ``vecN(rand(), rand())`` becomes ``vecN{rand(), rand()}``: GLSL evaluates
   arguments left to right, C++ only guarantees that order in braced lists.

Outputs go to ``oracle/_ref/`` only: ``<shader>.cpp`` (generated) and
``libref_<shader>.so``. Each library exports the entry points of a hand-written
harness (``oracle/ref_harness/<shader>.inc``) that binds buffers to the shader's
textures and images and runs its invocations.

Usage: python oracle/build_ref.py [--reference DIR] [--generate-only]
"""
import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHADERS = ["pt", "majorant", "normals", "mask", "denoise", "tonemap", "bloom", "dvr", "shadow", "ao"]
CXXFLAGS = ["-std=c++20", "-O2", "-fPIC", "-shared", "-fsingle-precision-constant",
            "-ffp-contract=off", "-fno-strict-aliasing", "-w", "-pthread"]

PRELUDE = r"""
// Invocation built-ins, per host thread.
inline thread_local uvec3 gl_GlobalInvocationID;
inline thread_local uvec3 gl_LocalInvocationID;
inline thread_local uint gl_LocalInvocationIndex;
// Global shader variables (the path tracer's `uint rng;`) become per-thread:
// `uint (*rng_slot());` redeclares this function.
inline uint* rng_slot() { static thread_local uint v; return &v; }
#define rng (*rng_slot())
// Workgroup barrier of the running workgroup (bloom.comp's exposure pass).
inline std::barrier<>* g_barrier = nullptr;
inline void barrier() { if (g_barrier) g_barrier->arrive_and_wait(); }
#define layout(...)
#define uniform struct
#define in
#define readonly
#define writeonly
#define shared static
"""


def transform(path, seen=None):
    """Returns the C++ text of GLSL file `path` with the rewrites above applied."""
    seen = seen if seen is not None else set()
    out = []
    base = os.path.dirname(path)
    with open(path) as f:
        for line in f:
            s = line.strip()
            if s.startswith("#version") or s.startswith("#extension"):
                out.append("\n")
                continue
            m = re.match(r'\s*#include\s+"([^"]+)"', line)
            if m:
                inc = os.path.join(base, m.group(1))
                if inc not in seen:
                    seen.add(inc)
                    out.append(f"// ---- inlined {m.group(1)}\n")
                    out.append(transform(inc, seen))
                continue
            line = re.sub(r"\b(?:out|inout)\s+(\w+)\s+(\w+)", r"\1& \2", line)
            line = re.sub(r"float\[\]\((.*)\);", r"{\1};", line)
            line = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", line)
            line = re.sub(r"\b(vec[234])\((rand\(\)(?:,\s*rand\(\))+)\)", r"\1{\2}", line)
            out.append(line)
    return "".join(out)


def generate(reference, name):
    src = os.path.join(reference, "shaders", f"{name}.comp")
    body = transform(src)
    harness = os.path.join(HERE, "ref_harness", f"{name}.inc")
    text = [
        f"// Generated by oracle/build_ref.py from shaders/{name}.comp. Not tracked.\n",
        "#include <barrier>\n#include <thread>\n#include <vector>\n",
        f'#include "{os.path.join(HERE, "glsl.hpp")}"\n',
        f"namespace ref_{name} {{\nGLSL_USING\n",
        PRELUDE,
        f'#line 1 "shaders/{name}.comp"\n',
        body,
        "\n#undef layout\n#undef uniform\n#undef in\n#undef readonly\n#undef writeonly\n#undef shared\n",
        f'#include "{harness}"\n',
        "}  // namespace\n",
    ]
    path = os.path.join(OUT, f"{name}.cpp")
    with open(path, "w") as f:
        f.write("".join(text))
    return path


def compile_one(name):
    src = os.path.join(OUT, f"{name}.cpp")
    lib = os.path.join(OUT, f"libref_{name}.so")
    cmd = ["g++", *CXXFLAGS, src, "-o", lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {name} failed:\n{r.stderr[-4000:]}")
    return lib


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("VOLVIEW_REFERENCE", "/root/reference"))
    ap.add_argument("--generate-only", action="store_true")
    ap.add_argument("--only", nargs="*", default=None)
    a = ap.parse_args(argv)
    names = a.only or SHADERS
    os.makedirs(OUT, exist_ok=True)
    if os.path.isdir(os.path.join(a.reference, "shaders")):
        for n in names:
            generate(a.reference, n)
    elif not all(os.path.exists(os.path.join(OUT, f"{n}.cpp")) for n in names):
        print("reference shaders not found and no generated sources present", file=sys.stderr)
        return 1
    if a.generate_only:
        return 0
    with ThreadPoolExecutor(max_workers=len(names)) as ex:
        for lib in ex.map(compile_one, names):
            print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
