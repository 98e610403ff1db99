"""Build the CPU oracle (test infrastructure) into oracle/liboracle.so.

g++ -O3 -std=c++17 -ffp-contract=off -fopenmp: no implicit FMA contraction,
so the oracle's float arithmetic is exactly the sequence its source spells
out.  No -march=native: the library must give the same bits on x86-64 and
aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = ["oracle_pt.cpp", "oracle_sort.cpp", "oracle_ppb.cpp", "oracle_ppm.cpp", "oracle_nrc.cpp",
           "oracle_structs.cpp"]
HEADERS = ["oracle_math.h", "oracle_scene.h", "oracle_lbvh.h"]


def build(verbose: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "vcr", "abi.h")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB] + srcs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
