"""CPU tests of the photon-mapping oracle: it converges to the path
tracer's image (same scene, independent estimator), is deterministic, and
its per-pixel N/R/flux update follows the progressive photon mapping rule."""
import numpy as np

import vcr
from oracle import oracle as orc
from oracle import oracle_ppm as opm
from vcr import configs


def _scene():
    size = (32, 32, 32)
    g = orc.Grid(orc.fbm_fill(size, seed=3, octaves=4), 0)
    desc = vcr.grid_desc(size, (1 / 32,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 8.0)
    cloud.max_extinction = max(g.max_density(), 0.01)
    return g, cloud, configs.C2_PPM


def test_photon_map_converges_to_the_path_traced_image():
    g, cloud, sc = _scene()
    W = H = 10
    cam, prm = sc.camera(W, H), sc.params(vcr.TRACKER_DDA)
    pt = g.pt_pass(cloud, cam, prm, W, H, seed=1, spp=3000)[0] / 3000
    st = opm.init_stats(W, H, 0.04)
    K = 24
    for k in range(K):
        s, out = opm.ppm_pass(g, cloud, cam, prm, 30000, 1 << 22, 0.7, W, H, st, seed=2, pass_index=k)
    pm = s / K
    assert out["info"]["dropped"] == 0
    assert abs(pm.mean() / pt.mean() - 1.0) < 0.04, (pm.mean(), pt.mean())


def test_progressive_update_rule_and_determinism():
    g, cloud, sc = _scene()
    W = H = 8
    cam, prm = sc.camera(W, H), sc.params(vcr.TRACKER_DDA)
    st1, st2 = opm.init_stats(W, H, 0.05), opm.init_stats(W, H, 0.05)
    prev = st1.copy()
    s1, o1 = opm.ppm_pass(g, cloud, cam, prm, 5000, 1 << 20, 0.7, W, H, st1, seed=4, pass_index=0)
    s2, _ = opm.ppm_pass(g, cloud, cam, prm, 5000, 1 << 20, 0.7, W, H, st2, seed=4, pass_index=0)
    assert s1.tobytes() == s2.tobytes() and st1.tobytes() == st2.tobytes()
    # radius only shrinks where photons were found; N grows by alpha M
    shrunk = st1[..., 1] < prev[..., 1]
    assert shrunk.any()
    np.testing.assert_array_equal(st1[..., 0] > 0, shrunk)
    alpha = float(np.float32(0.7))  # alpha travels as a float32
    n = st1[..., 0][shrunk]
    m = np.round(n / alpha)  # first pass: N' = alpha M
    np.testing.assert_array_equal(n, alpha * m)
    ratio = (alpha * m) / m
    np.testing.assert_allclose(st1[..., 1][shrunk], prev[..., 1][shrunk] * ratio ** (1 / 3), rtol=1e-12)
    assert np.all(st1[..., 5:8] >= 0)


def _march(g, cloud, prm, W, H, k, sum_img=None, photons=3000, r0=0.08, alpha=0.8):
    sv = vcr.shadow_volume_setup(configs.sun_travel_dir(), cloud.bounds_min, cloud.bounds_max, 24)
    tex = g.sv_build(cloud, sv)
    cam = configs.C2_PPM.camera(W, H)
    return opm.ppm_march_pass(g, cloud, cam, prm, sv, tex, photons, 1 << 20, r0, alpha, 1.0 / 32, 1.0 / 8, W, H,
                              sum_img, seed=5, pass_index=k)


def test_march_estimate_of_an_empty_cloud_is_the_sky():
    """VCR_PPM_MARCH over a zero-density grid: no extinction and no
    in-scattering, so every pixel is the sky along its camera ray."""
    size = (16, 16, 16)
    g = orc.Grid(np.zeros(size[::-1], np.float32), 0)
    desc = vcr.grid_desc(size, (1 / 16,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 8.0)
    cloud.max_extinction = 0.01
    prm = configs.C2_PPM.params(vcr.TRACKER_DDA)
    prm.sky_mode = vcr.SKY_GRADIENT
    W = H = 12
    s, n, _ = _march(g, cloud, prm, W, H, 0)
    assert n == 0
    sky = orc.Grid(np.zeros(size[::-1], np.float32), 0).pt_pass(
        cloud, configs.C2_PPM.camera(W, H), prm, W, H, seed=1)[0]  # escaping paths carry the sky
    np.testing.assert_array_equal(s, sky)


def test_march_radius_follows_update_radius_and_is_deterministic():
    """The global radius of pass k is RenderTechniquePPM::UpdateRadius's
    r_1 = R0, r_n = r_(n-1) ((n - 1 + alpha) / n)^0.33333 (float); two runs
    of a pass give the same bits."""
    g, cloud, sc = _scene()
    prm = sc.params(vcr.TRACKER_DDA)
    prm.rng_mode = vcr.RNG_XORSHIFT
    W = H = 8
    r = []
    for k in range(4):
        s1, _, rk = _march(g, cloud, prm, W, H, k)
        s2, _, _ = _march(g, cloud, prm, W, H, k)
        assert s1.tobytes() == s2.tobytes()
        r.append(rk)
    a = np.float32(0.8)
    exp = [np.float32(0.08)]
    for n in range(2, 5):
        exp.append(np.float32(exp[-1] * np.power((np.float32(n - 1) + a) / np.float32(n), np.float32(0.33333))))
    np.testing.assert_allclose(r, exp, rtol=2e-7)
    assert r[0] > r[1] > r[2] > r[3]
