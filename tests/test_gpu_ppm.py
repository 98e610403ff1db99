"""GPU tests of volumetric progressive photon mapping through the C-ABI,
against the oracle: stored photons (in photon/event order), the photon tree,
the per-pixel FP64 statistics and the image, bit for bit, over several
progressive passes."""
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
