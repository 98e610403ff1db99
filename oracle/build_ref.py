"""Build the reference's own code that compiles here, into oracle/_ref/
(git-ignored).  Test infrastructure only; it needs the reference tree,
found at $VCR_REFERENCE_DIR (default /root/reference), and is skipped where
that is absent.

  * Grid3D<float> (.xyz Load/Save, GetMajorant), compiled from its header
    as it lies, behind oracle/ref_grid3d.cpp -> _ref/ref_grid3d.
  * The compute shaders PathTracer.comp and ShadowVolume.comp, run on the
    CPU: `transliterate` rewrites only what a C++ compiler cannot parse —
      - the #version and local_size layout lines, and the descriptor
        declarations (layout(...) uniform ...), which glsl_shim.h and
        ref_shaders.cpp declare under the same names;
      - the parameter qualifiers: `in` dropped, `out` / `inout` as C++
        references;
      - `lowp` dropped;
      - float literals given the `f` suffix (a GLSL literal is a float,
        a C++ one a double);
      - the invocation-private global (rng_state) made thread_local;
      - main renamed shader_main —
    and writes the result to _ref/<name>.cpp, which oracle/ref_shaders.cpp
    includes over the GLSL pieces of oracle/glsl_shim.h ->
    _ref/libref_shaders.so.  The bodies are the reference's, unedited.

Not built, and why:
  * Tests.cpp (the CPU radix-sort fixture): needs an MSVC-only cast fixed
    (Tests.cpp:135) and imgui through stdafx.h, i.e. an edited copy of the
    source; its fixture (Tests.cpp:113-131) is restated in oracle_sort.cpp.
  * the photon-mapping and photon-beam shaders: shared-memory work groups,
    barriers and atomics over storage buffers, which a per-invocation C++
    loop does not reproduce.
"""
from __future__ import annotations

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("VCR_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
EXE = os.path.join(OUT, "ref_grid3d")


def available() -> bool:
    return os.path.exists(os.path.join(REF, "CloudRendering-Vulkan", "Grid3D.h"))


def build(verbose: bool = False) -> str | None:
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_grid3d.cpp")
    if os.path.exists(EXE) and os.path.getmtime(EXE) >= os.path.getmtime(src):
        return EXE
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(REF, "CloudRendering-Vulkan"), "-I",
           os.path.join(REF, "include"), src, "-o", EXE]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference Grid3D harness failed to build:\n{res.stderr}")
    if verbose:
        print(f"built {EXE}")
    return EXE


SHADERS = ("PathTracer.comp", "ShadowVolume.comp")
SHADER_LIB = os.path.join(OUT, "libref_shaders.so")


def transliterate(text: str) -> str:
    """GLSL compute shader -> C++ over glsl_shim.h (see the module doc)."""
    text = re.sub(r"^\s*#version[^\n]*\n", "", text, flags=re.M)
    text = re.sub(r"layout\s*\(\s*local_size[^)]*\)\s*in\s*;", "", text)
    # descriptor blocks: layout(...) uniform Name { ... } instance;
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+\w+\s*\{.*?\}\s*\w+\s*;", "", text, flags=re.S)
    # images and samplers: layout(...) uniform [qualifiers] type name;
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform(\s+\w+)+\s*;", "", text)
    # parameter qualifiers (inside parameter lists: followed by , or ))
    text = re.sub(r"\b(?:inout|out)\s+(const\s+)?(\w+)\s+(\w+)(?=\s*[,)])", r"\1\2& \3", text)
    text = re.sub(r"\bin\s+(const\s+)?(\w+)\s+(\w+)(?=\s*[,)])", r"\1\2 \3", text)
    text = re.sub(r"\blowp\s+", "", text)
    # float literals: 1.0 -> 1.0f, 3.4e+38 -> 3.4e+38f (not 1.0f, not integers)
    text = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", text)
    text = re.sub(r"^uint rng_state\b", "thread_local uint rng_state", text, flags=re.M)
    text = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", text)
    return text


def shaders_available() -> bool:
    return all(os.path.exists(os.path.join(REF, "shaders", n)) for n in SHADERS)


def build_shaders(verbose: bool = False) -> str | None:
    if not shaders_available():
        return None
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in ("ref_shaders.cpp", "glsl_shim.h", "build_ref.py")]
    for name in SHADERS:
        src = os.path.join(REF, "shaders", name)
        with open(src) as f:
            cpp = transliterate(f.read())
        out = os.path.join(OUT, name + ".cpp")
        if not os.path.exists(out) or open(out).read() != cpp:
            with open(out, "w") as f:
                f.write(f"// transliterated from {name} by oracle/build_ref.py; not edited by hand\n" + cpp)
        deps.append(out)
    if os.path.exists(SHADER_LIB) and os.path.getmtime(SHADER_LIB) >= max(os.path.getmtime(d) for d in deps):
        return SHADER_LIB
    cmd = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-w",
           "-I", HERE, os.path.join(HERE, "ref_shaders.cpp"), "-o", SHADER_LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference shader harness failed to build:\n{res.stderr[-4000:]}")
    if verbose:
        print(f"built {SHADER_LIB}")
    return SHADER_LIB


if __name__ == "__main__":
    build(verbose=True)
    build_shaders(verbose=True)
