"""Edge cases through the C-ABI against the oracle: one-pixel frames, odd
frame sizes and crops on the last row / column, a grid whose sides are not
multiples of the brick, a camera inside the cloud (the reference's entry
rule, PathTracer.comp:380-382), an all-zero cloud, a one-pixel batch view,
cache calls with nothing to do, and photon passes that store nothing."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs

pytestmark = pytest.mark.gpu


def _scene(size=(45, 37, 51), seed=4, dense=None):
    if dense is None:
        dense = orc.fbm_fill(size, seed=seed, octaves=4)
    og = orc.Grid(dense, 0)
    desc = vcr.grid_desc(size, (1.0 / max(size),) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 16.0)
    cloud.max_extinction = max(og.max_density(), 0.01)
    return dense, og, desc, cloud


def _pass_both(ctx, og, cloud, cam, prm, W, H, crop, seed=3, pass_index=1, level=2):
    ctx.set_camera(cam)
    ctx.set_params(prm)
    ctx.set_frame(W, H)
    ctx.set_tuning(majorant_level=level, dda_steps=4, stage_majorants=1, block_threads=256)
    ctx.pt_pass(seed=seed, pass_index=pass_index, crop=crop)
    ctx.synchronize()
    got = ctx.image_sum()
    ref, _ = og.pt_pass(cloud, cam, prm, W, H, seed=seed, pass_index=pass_index, crop=crop, level=level)
    return got, ref


@pytest.mark.parametrize("tracker", [vcr.TRACKER_DDA, vcr.TRACKER_GLOBAL])
def test_small_odd_frames_and_edge_crops(cuda, tracker):
    dense, og, desc, cloud = _scene()
    sc = configs.C1_PT
    prm = sc.params(tracker)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        for (W, H), crop in [((1, 1), (0, 0, 0, 0)), ((37, 23), (0, 0, 0, 0)), ((37, 23), (36, 22, 1, 1)),
                             ((37, 23), (36, 0, 1, 23)), ((37, 23), (0, 22, 37, 1))]:
            # a camera needs a 2x2 raster at least; a 1x1 frame renders its first pixel
            cam = vcr.camera_look((0.05, 0.0, -0.5), (0.0, 0.0, 1.0), 70.0, 0.1, max(W, 2), max(H, 2))
            got, ref = _pass_both(ctx, og, cloud, cam, prm, W, H, crop)
            np.testing.assert_array_equal(got, ref, err_msg=f"{W}x{H} crop {crop}")


def test_camera_inside_the_cloud(cuda):
    dense, og, desc, cloud = _scene()
    prm = configs.C1_PT.params(vcr.TRACKER_DDA)
    W, H = 24, 20
    cam = vcr.camera_look((0.0, 0.0, 0.45), (0.3, 0.1, 1.0), 80.0, 0.1, W, H)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        got, ref = _pass_both(ctx, og, cloud, cam, prm, W, H, (0, 0, 0, 0))
    np.testing.assert_array_equal(got, ref)


def test_all_zero_cloud_renders_the_sky(cuda):
    size = (16, 16, 16)
    dense, og, desc, cloud = _scene(size, dense=np.zeros((16, 16, 16), np.float32))
    sc = configs.C1_PT
    prm = sc.params(vcr.TRACKER_DDA)
    W, H = 20, 12
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(sc.camera(W, H))
        ctx.set_params(prm)
        ctx.set_frame(W, H)
        for k in range(3):
            ctx.pt_pass(seed=1, pass_index=k)
        ctx.synchronize()
        img = ctx.image_mean()
        paths, lookups, events, cells = ctx.counters()
        # photon passes that store nothing still produce the background
        ctx.ppm_setup(photons=2048, capacity=4096, radius=0.05, alpha=0.7)
        ctx.ppm_pass(seed=2, pass_index=0)
        ctx.synchronize()
        assert ctx.ppm_info()["photons_stored"] == 0
        ppm_img = ctx.image_sum()
        ctx.reset()
        ctx.ppb_setup(512, 4096, 0.05, 0.8)
        ctx.ppb_pass(seed=2, pass_index=0)
        ctx.synchronize()
        ppb_img = ctx.image_sum()
    np.testing.assert_array_equal(img, np.float32(0.1))
    assert events == 0
    # every free flight escapes: each pixel sees the whole sky, including
    # rays that only graze the box (an escaped flight is farther than any
    # exit distance, however the two box intersections round)
    o_ppb, _ = orc.ppb_pass(og, cloud, sc.camera(W, H), prm, 512, 4096, 0.05, 0.8, W, H, seed=2, pass_index=0)
    np.testing.assert_array_equal(np.unique(o_ppb), [np.float64(np.float32(0.1))])
    np.testing.assert_array_equal(ppb_img, o_ppb)
    np.testing.assert_array_equal(ppm_img, o_ppb)


def test_one_pixel_batch_view(cuda):
    dense, og, desc, cloud = _scene()
    sc = configs.C1_PT
    cam = vcr.camera_look((0.0, 0.0, -0.5), (0.0, 0.0, 1.0), 60.0, 0.1, 2, 2)
    sun = configs.sun_travel_dir(40.0)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_tuning(majorant_level=2, dda_steps=4, stage_majorants=1, block_threads=256)
        ctx.batch_setup([(cam, 1, 1, sun)])
        ctx.batch_pass(seed=8, pass_index=3)
        ctx.synchronize()
        got = ctx.batch_read(0)
    prm = sc.params(vcr.TRACKER_DDA)
    for a in range(3):
        prm.sun_dir[a] = sun[a]
    ref, _ = og.pt_pass(cloud, cam, prm, 1, 1, seed=8, pass_index=3, level=2)
    np.testing.assert_array_equal(got, ref)


def test_cache_calls_with_nothing_to_do(cuda):
    import torch
    dense, og, desc, cloud = _scene()
    sc = configs.C1_PT
    W, H = 16, 16
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = 2
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_params(prm)
        # a camera that looks away from the cloud: no path reaches the cache
        ctx.set_camera(vcr.camera_look((0.0, 0.0, -0.5), (0.0, 0.0, -1.0), 60.0, 0.1, W, H))
        ctx.set_frame(W, H)
        ctx.nrc_setup(train_samples=1024, query_capacity=W * H, seed=1)
        out = torch.zeros(3, dtype=torch.float32, device=cuda)
        ctx.nrc_forward(0, 0, out.data_ptr())  # zero records: a no-op
        with pytest.raises(vcr.VcrError):
            ctx.nrc_fit(0, 0, 1)  # nothing to fit on is an error
        ctx.pt_pass(seed=1, pass_index=0)
        ctx.synchronize()
        assert ctx.nrc_info()["queries"] == 0
        np.testing.assert_array_equal(ctx.image_sum(), np.float64(np.float32(0.1)))
