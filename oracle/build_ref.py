"""Build the reference's own host C++ that compiles as it lies: Grid3D<float>
(.xyz Load/Save, GetMajorant) behind oracle/ref_grid3d.cpp, into
oracle/_ref/ (git-ignored).  Test infrastructure only; it needs the
reference tree, found at $VCR_REFERENCE_DIR (default /root/reference), and
is skipped where that is absent.

Not built, and why:
  * Tests.cpp (the CPU radix-sort fixture): needs an MSVC-only cast fixed
    (Tests.cpp:135) and imgui through stdafx.h, i.e. an edited copy of the
    source; its fixture (Tests.cpp:113-131) is restated in oracle_sort.cpp.
  * the shaders (the whole light-transport path): GLSL that needs a Vulkan
    device, which this machine does not have.
"""
from __future__ import annotations

import os
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


if __name__ == "__main__":
    build(verbose=True)
