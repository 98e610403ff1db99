"""The benchmark's CPU reference leg builds its scene from the oracle alone:
the structs equal the library's byte for byte, and a process that sets up
the leg and renders through it never maps libvcr.so."""
import ctypes as C
import os
import subprocess
import sys

import vcr
from vcr import configs
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bytes(s):
    return bytes(C.string_at(C.addressof(s), C.sizeof(s)))


def test_oracle_scene_structs_equal_the_library_ones():
    for sc in configs.ALL:
        desc, cloud, cam, prm = orc.scene_structs(sc)
        assert _bytes(desc) == _bytes(sc.grid_desc())
        assert _bytes(cloud) == _bytes(sc.cloud())
        assert _bytes(cam) == _bytes(sc.camera())
        assert _bytes(prm) == _bytes(sc.params())


def test_reference_leg_loads_no_product_library():
    code = r"""
import os, sys
sys.path.insert(0, %r)
import bench
from vcr import configs
from dataclasses import replace
sc = replace(configs.C5_NRC, size=(64, 32, 64), width=96, height=54)
os_ = bench.OracleScene(sc, threads=2)
paths, dt = os_.pass_rows(4, 1)
assert paths == 96 * 4, paths
maps = open("/proc/self/maps").read()
assert "liboracle.so" in maps
assert "libvcr.so" not in maps, "the reference leg mapped libvcr.so"
print("ok")
""" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
