"""The standalone grid tool on the CPU: generated files equal the generator
(and the oracle's restatement of it), info reports the header, majorant and
device bytes, slices become PNG files."""
import json
import os
import struct
import zlib

import numpy as np

import vcr
from oracle import oracle as orc
from vcr import grid_tool


def _run(capsys, *argv):
    assert grid_tool.main([str(a) for a in argv]) == 0
    return json.loads(capsys.readouterr().out.strip().splitlines()[-1])


def test_generate_info_and_slice(tmp_path, capsys):
    path = tmp_path / "c.xyz"
    out = _run(capsys, "generate", "--size", 20, 12, 9, "--seed", 5, "--octaves", 3, "-o", path)
    assert out["size"] == [20, 12, 9]
    desc, data = vcr.xyz_read(str(path))
    fbm = vcr.fbm_desc(seed=5, octaves=3)
    np.testing.assert_array_equal(data, vcr.fbm_fill_host((20, 12, 9), fbm))
    np.testing.assert_array_equal(data, orc.fbm_fill((20, 12, 9), seed=5, octaves=3))
    np.testing.assert_allclose(desc.voxel_size[:], [1.0 / 20] * 3)
    info = _run(capsys, "info", path)
    assert info["majorant"] == float(data.max()) and info["size"] == [20, 12, 9]
    # 3 x 2 x 2 bricks; pyramid 12 + 2 + 1 + 1 cells, padded to 4 floats a level
    assert info["device_bytes"] == {"fp32": 12 * 2048 + 48 + 4 * (12 + 4 + 4 + 4),
                                    "fp16": 12 * 1024 + 48 + 4 * (12 + 4 + 4 + 4),
                                    "bf16": 12 * 1024 + 48 + 4 * (12 + 4 + 4 + 4)}
    png = tmp_path / "s.png"
    sl = _run(capsys, "slice", path, "--axis", "y", "--index", 4, "-o", png)
    assert sl["shape"] == [9, 20]
    raw = png.read_bytes()
    w, h = struct.unpack(">II", raw[16:24])
    assert (w, h) == (20, 9)
    assert os.path.getsize(png) > 0 and zlib.crc32(raw) != 0
