"""The project's .xyz reader/writer and global majorant against the
reference's own Grid3D<float> (Grid3D.h: Load :44-90, Save :166-178,
GetMajorant :180-192), compiled from its header by oracle/build_ref.py.
Runs where the reference tree is present; skipped elsewhere."""
import subprocess

import numpy as np
import pytest

import vcr
from oracle import build_ref

pytestmark = pytest.mark.skipif(not build_ref.available(), reason="reference tree absent")


def _run(*args):
    subprocess.run([build_ref.build(), *map(str, args)], check=True, timeout=60)


def _ref_load(path, out):
    _run("load", path, out)
    raw = open(out, "rb").read()
    dims = tuple(int(v) for v in np.frombuffer(raw[:12], np.uint32))
    vs = np.frombuffer(raw[12:36], np.float64)
    maj = float(np.frombuffer(raw[36:40], np.float32)[0])
    return dims, vs, maj, np.frombuffer(raw[40:], np.float32)


def test_reference_loader_reads_our_files(tmp_path):
    rng = np.random.default_rng(3)
    X, Y, Z = 12, 7, 5
    data = rng.random((Z, Y, X), dtype=np.float32)  # x fastest in memory
    desc = vcr.grid_desc((X, Y, Z), (0.5, 0.25, 0.125))
    vcr.xyz_write(str(tmp_path / "a.xyz"), desc, data)
    dims, vs, maj, mem = _ref_load(tmp_path / "a.xyz", tmp_path / "a.bin")
    assert dims == (X, Y, Z)
    np.testing.assert_array_equal(vs, [0.5, 0.25, 0.125])
    np.testing.assert_array_equal(mem, data.ravel())  # the reference's memory order is ours
    assert maj == float(data.max())  # GetMajorant
    d2, back = vcr.xyz_read(str(tmp_path / "a.xyz"))
    np.testing.assert_array_equal(back, data)


def test_our_reader_reads_what_the_reference_loader_reads(tmp_path):
    """A file the reference's Save wrote is read by our reader exactly as by
    its own Load, including Save's x<->z transposition (Save writes memory
    order, Load expects z fastest)."""
    rng = np.random.default_rng(4)
    for dims in ((6, 6, 6), (9, 4, 3)):
        X, Y, Z = dims
        data = rng.random((Z, Y, X), dtype=np.float32)
        raw = np.array(dims, np.uint32).tobytes() + np.array([1.0, 2.0, 3.0], np.float64).tobytes() + data.tobytes()
        (tmp_path / "in.bin").write_bytes(raw)
        _run("save", tmp_path / "in.bin", tmp_path / "b.xyz")
        _, _, maj, mem = _ref_load(tmp_path / "b.xyz", tmp_path / "b.bin")
        desc, ours = vcr.xyz_read(str(tmp_path / "b.xyz"))
        assert tuple(desc.size) == dims
        np.testing.assert_array_equal(ours.ravel(), mem)
        assert maj == float(data.max())
        if X == Y == Z:  # on a cube the round trip is the transpose x <-> z
            np.testing.assert_array_equal(ours, data.transpose(2, 1, 0))
