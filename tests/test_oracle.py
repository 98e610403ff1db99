"""CPU tests of the oracle: its math against closed forms and libm bounds,
its reduced-precision encoders against numpy / torch, its generator against
the product's host generator, and statistical properties of its trackers."""
import math

import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs


def test_log_exp_sincos_error_bounds():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.random(20000, dtype=np.float32) + np.float32(1e-7),
                         np.float32(2.0) ** rng.integers(-24, 0, 2000).astype(np.float32)])
    for x in xs[:6000]:
        ref = math.log(float(x))
        got = orc.olog(float(x))
        assert abs(got - ref) <= 4e-7 * max(1.0, abs(ref)), (x, got, ref)
    for x in np.linspace(-80, 5, 3001, dtype=np.float32):
        ref = math.exp(float(x))
        assert abs(orc.oexp(float(x)) - ref) <= 3e-7 * ref, x
    for u in np.linspace(0, 1, 4001, dtype=np.float32):
        s, c = orc.sincos2pi(float(u))
        assert abs(s - math.sin(2 * math.pi * float(u))) < 5e-7
        assert abs(c - math.cos(2 * math.pi * float(u))) < 5e-7
    assert orc.olog(0.0) == -math.inf
    assert orc.olog(1.0) == 0.0


def test_f16_bf16_encoders_match_round_to_nearest_even():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.random(50000, dtype=np.float32),
                         (rng.random(5000, dtype=np.float32) * np.float32(1e-4)),
                         np.float32([0.0, 1.0, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08, 0.99951171875])])
    L = orc.lib()
    got16 = np.array([L.oracle_f32_to_f16(float(x)) for x in xs], np.uint16)
    np.testing.assert_array_equal(got16, xs.astype(np.float16).view(np.uint16))
    torch = pytest.importorskip("torch")
    gotbf = np.array([L.oracle_f32_to_bf16(float(x)) for x in xs], np.uint16)
    ref = torch.from_numpy(xs).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    np.testing.assert_array_equal(gotbf, ref)


def test_fbm_oracle_equals_product_host_generator():
    size = (40, 24, 33)
    fb = vcr.fbm_desc(seed=7, octaves=6)
    a = orc.fbm_fill(size, seed=7, octaves=6)
    b = vcr.fbm_fill_host(size, fb)
    assert a.tobytes() == b.tobytes()
    assert 0.0 <= a.min() and a.max() <= 1.0 and a.max() > 0.5


def test_grid_majorant_bounds_every_trilinear_sample():
    """Every pyramid level: no trilinear sample inside a cell exceeds the
    cell's majorant, also right at and next to the cell faces (where the
    footprint reaches into the neighbouring bricks)."""
    size = (20, 17, 12)
    dense = orc.fbm_fill(size, seed=3, octaves=4)
    for prec in (0, 1, 2):
        g = orc.Grid(dense, prec)
        cloud = vcr.cloud_from_grid(vcr.grid_desc(size, (1 / 20,) * 3), 1.0, 8.0)
        b0 = np.array(cloud.bounds_min, np.float32)
        b1 = np.array(cloud.bounds_max, np.float32)
        rng = np.random.default_rng(prec)
        pts = (b0 + (b1 - b0) * rng.random((20000, 3))).astype(np.float32)
        brick = (b1 - b0) / np.array(size) * 8
        faces = np.round((pts[:6000] - b0) / brick) * brick + b0  # on brick faces (all levels' faces are among them)
        faces += rng.choice([-1e-6, 0.0, 1e-6], faces.shape) * (b1 - b0)
        pts = np.concatenate([pts, np.clip(faces, b0, b1).astype(np.float32)])
        vals = g.sample(cloud, pts)
        for level in range(4):
            maj = g.majorants(level)
            dims = np.array(g.level_dims(level))
            cells = np.minimum(np.floor((pts - b0) / (brick * (1 << level))).astype(int), dims - 1)
            cells = np.maximum(cells, 0)
            lin = cells[:, 0] + dims[0] * (cells[:, 1] + dims[1] * cells[:, 2])
            assert np.all(vals <= maj[lin]), (prec, level)
            assert g.max_density() == maj.max(), (prec, level)


def _small_scene(tracker, size=(32, 32, 32), ds=8.0):
    sc = configs.Scene("t", size, 4, ds, 16, 16, 1)
    dense = orc.fbm_fill(size, seed=1, octaves=4)
    g = orc.Grid(dense, 0)
    return sc, g


def test_oracle_pt_deterministic_and_resumable():
    sc, g = _small_scene(vcr.TRACKER_DDA)
    cloud, cam, prm = sc.cloud(), sc.camera(16, 16), sc.params(vcr.TRACKER_DDA)
    s1, _ = g.pt_pass(cloud, cam, prm, 16, 16, seed=5, pass_index=3)
    s2, _ = g.pt_pass(cloud, cam, prm, 16, 16, seed=5, pass_index=3)
    assert s1.tobytes() == s2.tobytes()
    # accumulate passes 0..3 in one buffer == pass-by-pass sums (resume)
    acc = np.zeros((16, 16, 3))
    for k in range(4):
        g.pt_pass(cloud, cam, prm, 16, 16, seed=5, pass_index=k, sum_img=acc)
    parts = sum(g.pt_pass(cloud, cam, prm, 16, 16, seed=5, pass_index=k)[0] for k in range(4))
    np.testing.assert_array_equal(acc, parts)


def test_global_and_dda_trackers_agree_in_expectation():
    """Both trackers are unbiased estimators of the same image."""
    sc, g = _small_scene(vcr.TRACKER_DDA, size=(24, 24, 24), ds=6.0)
    cloud, cam = sc.cloud(), sc.camera(8, 8)
    res = {}
    for tr in (vcr.TRACKER_GLOBAL, vcr.TRACKER_DDA):
        prm = sc.params(tr)
        s, _ = g.pt_pass(cloud, cam, prm, 8, 8, seed=11, spp=3000)
        res[tr] = s / 3000
    a, b = res[0].mean(), res[1].mean()
    assert abs(a - b) < 0.02 * a, (a, b)


def test_homogeneous_transmittance_matches_beer_lambert():
    """A constant-density cube, albedo 0, no sky except along the view ray:
    the camera sees sky * exp(-sigma * chord) through the centre pixel."""
    size = (16, 16, 16)
    dense = np.full(size[::-1], 0.5, np.float32)
    g = orc.Grid(dense, 0)
    sc = configs.Scene("h", size, 1, 4.0, 3, 3, 1, albedo=0.0, max_events=1)
    cloud, cam = sc.cloud(), sc.camera(2, 2)
    for tr in (vcr.TRACKER_GLOBAL, vcr.TRACKER_DDA):
        prm = sc.params(tr)
        prm.light_intensity = 0.0
        n = 20000
        s, _ = g.pt_pass(cloud, cam, prm, 2, 2, seed=1, spp=n, crop=(1, 1, 1, 1))
        est = s[1, 1, 0] / n / 0.1
        exact = math.exp(-4.0 * 0.5 * 1.0)
        assert abs(est - exact) < 4 * math.sqrt(exact * (1 - exact) / n) + 1e-3, (tr, est, exact)
