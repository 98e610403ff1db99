"""GPU tests of volumetric progressive photon mapping through the C-ABI,
against the oracle: stored photons (in photon/event order), the photon tree,
the per-pixel FP64 statistics and the image, bit for bit, over several
progressive passes; and the reference's ray-marched estimate
(VCR_PPM_MARCH, PPM_PE.comp:443-546) bit for bit in both RNG modes."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from oracle import oracle_ppm as opm
from vcr import configs

pytestmark = pytest.mark.gpu


def _scene():
    size = (40, 32, 40)
    dense = orc.fbm_fill(size, seed=6, octaves=5)
    g = orc.Grid(dense, 0)
    desc = vcr.grid_desc(size, (1 / 40,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 16.0)
    cloud.max_extinction = max(g.max_density(), 0.01)
    return dense, g, desc, cloud, configs.C2_PPM


@pytest.mark.parametrize("level", [0, 2])
def test_ppm_passes_bit_exact(cuda, level):
    dense, g, desc, cloud, sc = _scene()
    W, H = 48, 32
    cam, prm = sc.camera(W, H), sc.params(vcr.TRACKER_DDA)
    photons, cap, r0, alpha = 4000, 1 << 18, 0.03, 0.7
    st = opm.init_stats(W, H, r0)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_tuning(majorant_level=level)
        ctx.set_cloud(cloud)
        ctx.set_camera(cam)
        ctx.set_params(prm)
        ctx.set_frame(W, H)
        ctx.ppm_setup(photons, cap, r0, alpha)
        for k in range(3):
            ctx.ppm_pass(seed=21, pass_index=k)
            ctx.synchronize()
            s_o, o = opm.ppm_pass(g, cloud, cam, prm, photons, cap, alpha, W, H, st, seed=21, pass_index=k,
                                  level=level, want_photons=True)
            info = ctx.ppm_info()
            assert info["photons_stored"] == o["info"]["photons_stored"] > 1000
            assert info["dropped"] == 0
            # photons: the GPU appends in any order; its uid order is the oracle's order
            uid = ctx.ppm_read("uid")
            perm = np.argsort(uid, kind="stable")
            np.testing.assert_array_equal(uid[perm], o["uid"])
            ph = np.concatenate([ctx.ppm_read(k)[perm] for k in ("pos", "power", "dir")], axis=1)
            np.testing.assert_array_equal(ph, o["photons"])
            # tree: leaves map to the same photons
            inv = np.empty_like(perm)
            inv[perm] = np.arange(len(perm))
            np.testing.assert_array_equal(inv[ctx.ppm_read("order")], o["order"])
            np.testing.assert_array_equal(ctx.ppm_read("left"), o["left"])
            np.testing.assert_array_equal(ctx.ppm_read("right"), o["right"])
            np.testing.assert_array_equal(ctx.ppm_read("stats"), st)
            np.testing.assert_array_equal(ctx.image_sum(), s_o)
            tested, ms = ctx.gather_stats("ppm")  # leaf photons the gather tested
            assert tested > 0 and ms > 0.0
        assert ctx.pass_count() == 3
        m = ctx.image_mean()
        np.testing.assert_allclose(m, (s_o / 3).astype(np.float32), rtol=1e-6)


def test_ppm_capacity_overflow_is_reported(cuda):
    dense, g, desc, cloud, sc = _scene()
    W, H = 16, 16
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(sc.camera(W, H))
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_frame(W, H)
        ctx.ppm_setup(20000, 1000, 0.05, 0.7)
        ctx.ppm_pass(seed=1, pass_index=0)
        ctx.synchronize()
        info = ctx.ppm_info()
        assert info["photons_stored"] == 1000 and info["dropped"] > 0
        assert np.isfinite(ctx.image_mean()).all()


@pytest.mark.parametrize("rng_mode", [vcr.RNG_XORSHIFT, vcr.RNG_PCG])
def test_ppm_march_estimate_bit_exact(cuda, rng_mode):
    """The reference's estimate: back-to-front march (start jittered),
    shadow-volume direct light, the ambient sky term, the photon map within
    the global radius of UpdateRadius (RenderTechniquePPM.cpp:302-312);
    three progressive passes, the sums equal to the oracle's bit for bit."""
    dense, g, desc, cloud, sc = _scene()
    W, H = 48, 32
    cam, prm = sc.camera(W, H), sc.params(vcr.TRACKER_DDA)
    prm.rng_mode, prm.sky_mode = rng_mode, vcr.SKY_GRADIENT
    sv = vcr.shadow_volume_setup(configs.sun_travel_dir(), cloud.bounds_min, cloud.bounds_max, 48)
    photons, cap, r0, alpha, step, amb = 4000, 1 << 18, 0.06, 0.8, 1.0 / 64, 1.0 / 16
    o_sum = np.zeros((H, W, 3), np.float64)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(cam)
        ctx.set_params(prm)
        ctx.set_frame(W, H)
        ctx.ppm_setup(photons, cap, r0, alpha, estimator=vcr.PPM_MARCH, march_step=step, ambient_step=amb)
        with pytest.raises(vcr.VcrError):  # the direct term needs the shadow volume
            ctx.ppm_pass(seed=21, pass_index=0)
        ctx.shadow_volume_build(sv)
        ctx.synchronize()
        sv_tex = ctx.shadow_volume(48)
        radii = []
        for k in range(3):
            ctx.ppm_pass(seed=21, pass_index=k)
            ctx.synchronize()
            o_sum, n, r = opm.ppm_march_pass(g, cloud, cam, prm, sv, sv_tex, photons, cap, r0, alpha, step, amb, W,
                                             H, o_sum, seed=21, pass_index=k)
            assert ctx.ppm_info()["photons_stored"] == n > 1000
            np.testing.assert_array_equal(ctx.image_sum(), o_sum)
            radii.append(r)
            tested, ms = ctx.gather_stats("ppm")
            assert tested > 0 and ms > 0.0
        assert ctx.pass_count() == 3
    assert radii[0] == np.float32(r0) and radii[0] > radii[1] > radii[2]
    assert np.isfinite(o_sum).all() and o_sum.max() > 0.05
    with vcr.Context() as ctx:  # bad march parameters
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_frame(W, H)
        with pytest.raises(vcr.VcrError):
            ctx.ppm_setup(photons, cap, r0, alpha, estimator=vcr.PPM_MARCH, march_step=0.0, ambient_step=amb)
