"""CPU tests of the C-ABI library: it loads, exports every symbol the public
header declares, rejects bad arguments with status codes, and its host-side
helpers restate the reference's struct logic."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import vcr
from vcr import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "vcr", f) for f in sorted(os.listdir(os.path.join(ROOT, "include", "vcr")))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        names |= set(re.findall(r"VCR_API\s+[\w\s\*]+?\b(vcr_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    L = vcr.lib()
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    # the Python mirror binds exactly what the header declares
    assert names <= set(_abi.SIGNATURES) | _abi_extra(), sorted(names - set(_abi.SIGNATURES))


def _abi_extra():
    return set(getattr(_abi, "EXTRA_SIGNATURES", {}))


def test_null_and_bad_arguments_return_status_codes():
    L = vcr.lib()
    assert L.vcr_create(None, None) == _abi.ERR_INVALID
    assert L.vcr_set_cloud(None, None) == _abi.ERR_INVALID
    assert L.vcr_pt_pass(None, None, None) == _abi.ERR_INVALID
    assert L.vcr_readback(None, 0, None, 0) == _abi.ERR_INVALID
    assert L.vcr_destroy(None) == _abi.OK
    assert L.vcr_version() >= 0x100


def test_phase_g_matches_parameters_setphaseg():
    p = _abi.Params()
    vcr.params_set_phase_g(p, 0.857)
    g = np.float32(0.857)
    assert p.phase_g == g
    assert p.phase_one_plus_g2 == np.float32(1) + g * g
    assert p.phase_one_minus_g2 == np.float32(1) - g * g
    assert p.phase_one_over_2g == np.float32(0.5) / g
    assert p.isotropic == 0
    vcr.params_set_phase_g(p, 0.99)  # clamped to 0.95 (UniformBuffers.h:97)
    assert p.phase_g == np.float32(0.95)
    vcr.params_set_phase_g(p, 0.00001)
    assert p.isotropic == 1
    vcr.params_set_phase_g(p, 2.0)  # out of [-1, 1]: ignored
    assert p.isotropic == 1


def test_cloud_bounds_match_setcloudproperties():
    d = vcr.grid_desc((100, 50, 80), (0.01, 0.01, 0.01))
    c = vcr.cloud_from_grid(d, 1000.0, 200.0)
    # cloudSize = voxel * count * baseScaling; x,y centred, z from 0 (main.cpp:147-162)
    assert tuple(c.bounds_min) == (-500.0, -250.0, 0.0)
    assert tuple(c.bounds_max) == (500.0, 250.0, 800.0)
    assert c.base_scaling == 1000.0 and c.density_scaling == 200.0


def test_camera_matches_cameraproperties_defaults():
    cam = vcr.camera_look((0, 0, -800), (0, 0, 1), 120.0, 50.0, 800, 600)
    assert (cam.half_width, cam.half_height) == (400, 300)
    assert tuple(cam.right) == (1.0, 0.0, 0.0) and tuple(cam.up) == (0.0, 1.0, 0.0)
    py = 2 * math.tan(math.radians(60)) * 50 / 600
    assert abs(cam.pixel_size_y - py) < 1e-6
    assert abs(cam.pixel_size_x - py * 300 / 400) < 1e-6


def test_shadow_volume_setup_is_orthonormal_and_covers_the_cloud():
    sv = vcr.shadow_volume_setup((1, -1, 0), (-0.5, -0.5, 0), (0.5, 0.5, 1), 500)
    L, R, U = (np.array(v) for v in (sv.light_dir, sv.right, sv.up))
    for a, b in ((L, R), (L, U), (R, U)):
        assert abs(a @ b) < 1e-6
    B = np.array(sv.basis_change).reshape(3, 3)
    np.testing.assert_allclose(B @ np.stack([R, U, L], 1), np.eye(3), atol=1e-6)
    radius = math.sqrt(3) / 2
    assert abs(sv.voxel_size - 2 * radius / 499) < 1e-7


def test_xyz_roundtrip_and_file_order(tmp_path):
    size = (5, 3, 4)
    rng = np.random.default_rng(0)
    data = rng.random(size[::-1], dtype=np.float32)  # [z][y][x] == x fastest in memory
    d = vcr.grid_desc(size, (0.1, 0.2, 0.3))
    path = str(tmp_path / "g.xyz")
    vcr.xyz_write(path, d, data)
    raw = open(path, "rb").read()
    assert np.frombuffer(raw[:12], np.uint32).tolist() == list(size)
    assert np.frombuffer(raw[12:36], np.float64).tolist() == [0.1, 0.2, 0.3]
    body = np.frombuffer(raw[36:], np.float32)
    # GridData::save order: z fastest, x slowest (GridData.h:1-2, :12)
    np.testing.assert_array_equal(body, data.transpose(2, 1, 0).ravel())
    d2, back = vcr.xyz_read(path)
    assert tuple(d2.size) == size
    np.testing.assert_array_equal(back, data)


def test_xyz_read_errors(tmp_path):
    with pytest.raises(vcr.VcrError):
        vcr.xyz_read(str(tmp_path / "missing.xyz"))
    p = tmp_path / "short.xyz"
    p.write_bytes(np.array([4, 4, 4], np.uint32).tobytes() + np.zeros(3).tobytes() + b"\0" * 16)
    with pytest.raises(vcr.VcrError):
        vcr.xyz_read(str(p))


def test_create_without_gpu_fails_cleanly():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(vcr.VcrError):
        vcr.Context()


def test_wait_limits_round_trip_and_defaults():
    d = vcr.wait_limits()
    assert d == {"sort_lookback": 1 << 22, "stage_wait": 1 << 24}
    try:
        vcr.set_wait_limits(sort_lookback=0)
        assert vcr.wait_limits() == {"sort_lookback": 0, "stage_wait": 1 << 24}
        vcr.set_wait_limits(stage_wait=7)
        assert vcr.wait_limits() == {"sort_lookback": 0, "stage_wait": 7}
    finally:
        vcr.set_wait_limits()
    assert vcr.wait_limits() == d
    assert vcr.lib().vcr_get_wait_limits(None) == vcr.ERR_INVALID
