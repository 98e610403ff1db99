"""Build libvcr.so (the CUDA kernels + C-ABI) in-tree for sm_103a.

Every translation unit compiles in parallel with nvcc, then one link step
produces ``cloudrendering-vulkan_gb300/libvcr.so``.  Float semantics: device
code is compiled with ``-fmad=false`` (FMAs are written out explicitly) and
host code with ``-ffp-contract=off``, so the CPU oracle can reproduce results
bit for bit; the one exception is ``pt_wavefront_fast.cu``, the tracker's
opt-in fast-math instantiation (see FILE_FLAGS).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvcr.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I", os.path.join(HERE, "..", "include"),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources() -> list[str]:
    out = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu")]
    out += [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".cpp")]
    return out


# Per-file flags: the fast-math instantiation of the tracker contracts
# multiply-adds and uses the hardware transcendental approximations.
FILE_FLAGS = {"pt_wavefront_fast.cu": (["-fmad=false"], ["-fmad=true", "-DVCR_FAST_MATH"])}


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps += [os.path.join(HOST, h) for h in os.listdir(HOST) if h.endswith(".h")]
    deps.append(os.path.join(HERE, "..", "include", "vcr", "abi.h"))
    deps.append(os.path.join(HERE, "..", "include", "vcr", "render_technique.hpp"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    drop, add = FILE_FLAGS.get(os.path.basename(src), ([], []))
    cmd = [_nvcc()] + [f for f in NVCC_FLAGS if f not in drop] + add + extra + lang + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or []), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
