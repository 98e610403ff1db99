"""Regenerates the golden fixtures in this folder.

* grid3d_*: outputs of the reference's own Grid3D<float> (Grid3D.h: Load
  :44-90, Save :166-178, GetMajorant :180-192), driven by the harness that
  oracle/build_ref.py compiles from the reference's header.  Needs the
  reference tree; the fixtures then let every machine check the project's
  .xyz reader and writer against what the reference itself wrote and read.
* sort_fixture_keys.txt: the key array of Tests.cpp:113-131 (176 draws of
  std::uniform_int_distribution<unsigned>(0, 255) over std::mt19937(1)),
  produced by the oracle's replay of those library calls with libstdc++.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cloudrendering-vulkan_gb300"))

import vcr  # noqa: E402
from oracle import build_ref, oracle as orc  # noqa: E402


def header(dims, voxel):
    return np.array(dims, np.uint32).tobytes() + np.array(voxel, np.float64).tobytes()


def main():
    keys = orc.sort_fixture_keys()
    np.savetxt(os.path.join(HERE, "sort_fixture_keys.txt"), keys, fmt="%d")
    if not build_ref.available():
        print("reference tree absent: grid3d fixtures not regenerated")
        return
    exe = build_ref.build()
    with tempfile.TemporaryDirectory() as tmp:
        # 1. the reference's Save of a seeded 9x4x3 grid (memory order x fastest), then its Load
        X, Y, Z = 9, 4, 3
        data = np.random.default_rng(11).random((Z, Y, X), dtype=np.float32)
        src = os.path.join(tmp, "in.bin")
        with open(src, "wb") as f:
            f.write(header((X, Y, Z), (0.5, 0.25, 0.125)) + data.tobytes())
        saved = os.path.join(HERE, "grid3d_ref_save_9x4x3.xyz")
        subprocess.run([exe, "save", src, saved], check=True, timeout=60)
        subprocess.run([exe, "load", saved, os.path.join(HERE, "grid3d_ref_load_9x4x3.bin")], check=True, timeout=60)
        # 2. the reference's Load of a seeded 12x7x5 grid written by the project's writer
        X, Y, Z = 12, 7, 5
        data = np.random.default_rng(12).random((Z, Y, X), dtype=np.float32)
        ours = os.path.join(tmp, "ours.xyz")
        vcr.xyz_write(ours, vcr.grid_desc((X, Y, Z), (1.0, 2.0, 3.0)), data)
        subprocess.run([exe, "load", ours, os.path.join(HERE, "grid3d_ref_load_ours_12x7x5.bin")], check=True,
                       timeout=60)
    print("wrote", sorted(f for f in os.listdir(HERE) if not f.endswith(".py")))


if __name__ == "__main__":
    main()
