"""The grid tool's device steps: the stored grid read back dense equals the
oracle's decoded bricks for every precision (odd sizes included), the
device generator writes the host generator's file, and convert reports the
quantisation error it wrote."""
import json

import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import grid_tool

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [vcr.PREC_FP32, vcr.PREC_FP16, vcr.PREC_BF16])
@pytest.mark.parametrize("size", [(16, 16, 16), (45, 37, 51)])
def test_read_dense_is_the_decoded_grid(cuda, prec, size):
    dense = orc.fbm_fill(size, seed=9, octaves=4)
    with vcr.Context() as ctx:
        ctx.grid_upload(vcr.grid_desc(size, (1.0 / max(size),) * 3), dense, prec)
        got = ctx.grid_read_dense()
    np.testing.assert_array_equal(got, orc.Grid(dense, prec).decoded())
    if prec == vcr.PREC_FP32:
        np.testing.assert_array_equal(got, dense)


def test_device_generate_and_convert(cuda, tmp_path, capsys):
    host, dev = tmp_path / "h.xyz", tmp_path / "d.xyz"
    for path, extra in ((host, []), (dev, ["--device"])):
        assert grid_tool.main(["generate", "--size", "33", "20", "17", "--seed", "4", "-o", str(path)] + extra) == 0
    np.testing.assert_array_equal(vcr.xyz_read(str(dev))[1], vcr.xyz_read(str(host))[1])
    capsys.readouterr()
    out16 = tmp_path / "c16.xyz"
    assert grid_tool.main(["convert", str(host), "--precision", "fp16", "-o", str(out16)]) == 0
    rep = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    src = vcr.xyz_read(str(host))[1]
    back = vcr.xyz_read(str(out16))[1]
    np.testing.assert_array_equal(back, orc.Grid(src, vcr.PREC_FP16).decoded())
    assert rep["max_abs_error"] == float(np.abs(back.astype(np.float64) - src).max())
    assert 0 < rep["max_error_over_majorant"] < 2 ** -10  # half precision, relative to the brick maximum
