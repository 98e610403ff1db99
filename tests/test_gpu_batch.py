"""GPU tests of batched multi-view tracking through the C-ABI: every view
of a batch pass equals the oracle's single-view pass with the view's seed,
camera and sun (bit-exact at 1 spp), graph replays equal direct passes, and
the autotuner keeps the sums clean."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs

pytestmark = pytest.mark.gpu

SEED_STEP = 0x9E3779B9


def _views():
    """Three small views of uneven size around the C1 cloud, three suns."""
    out = []
    specs = [((0.0, 0.05, -0.45), 70.0, 48, 40, 10.0), ((0.6, 0.2, 0.5), 55.0, 32, 32, 45.0),
             ((-0.3, -0.1, -0.35), 80.0, 24, 56, 70.0)]
    for pos, fov, w, h, elev in specs:
        target = np.array([0.0, 0.0, 0.5])
        fwd = target - np.array(pos)
        fwd = tuple(fwd / np.linalg.norm(fwd))
        cam = vcr.camera_look(pos, fwd, fov, 0.1, w, h)
        out.append((cam, w, h, configs.sun_travel_dir(elev, 180.0)))
    return out


def _setup(ctx, sc, level=2):
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, 0)
    ctx.grid_upload(sc.grid_desc(), dense)
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    ctx.set_cloud(cloud)
    ctx.set_params(sc.params(vcr.TRACKER_DDA))
    ctx.set_tuning(majorant_level=level, dda_steps=4, stage_majorants=1, block_threads=256)
    return og, cloud


def _oracle_view(og, cloud, sc, view, v, seed, pass_index, spp=1, level=2):
    cam, w, h, sun = view
    prm = sc.params(vcr.TRACKER_DDA)
    for a in range(3):
        prm.sun_dir[a] = sun[a]
    s, _ = og.pt_pass(cloud, cam, prm, w, h, seed=(seed + SEED_STEP * v) % (1 << 32), pass_index=pass_index,
                      spp=spp, level=level)
    return s


def test_batch_views_match_the_single_view_oracle(cuda):
    sc = configs.C1_PT
    views = _views()
    with vcr.Context() as ctx:
        og, cloud = _setup(ctx, sc)
        ctx.batch_setup(views)
        ctx.batch_pass(seed=11, pass_index=2)
        ctx.synchronize()
        got = [ctx.batch_read(v) for v in range(len(views))]
        info = ctx.batch_info()
    assert info["views"] == 3 and info["passes"] == 1 and info["samples"] == 1
    assert info["pixels"] == sum(w * h for _, w, h, _ in views)
    for v, view in enumerate(views):
        ref = _oracle_view(og, cloud, sc, view, v, 11, 2)
        np.testing.assert_array_equal(got[v], ref)
        assert (ref > 0.1).any()  # the view sees lit cloud


def test_batch_with_four_samples_per_pixel(cuda):
    sc = configs.C1_PT
    views = _views()[:2]
    with vcr.Context() as ctx:
        og, cloud = _setup(ctx, sc, level=1)
        ctx.set_tuning(majorant_level=1, dda_steps=8, stage_majorants=1, block_threads=128)
        ctx.batch_setup(views)
        ctx.batch_pass(seed=5, pass_index=0, spp=4)
        ctx.synchronize()
        got = [ctx.batch_read(v) for v in range(len(views))]
        assert ctx.batch_info()["samples"] == 4
    for v, view in enumerate(views):
        ref = _oracle_view(og, cloud, sc, view, v, 5, 0, spp=4, level=1)
        # four float radiances per pixel summed in FP64 in another order
        np.testing.assert_allclose(got[v], ref, rtol=1e-12, atol=0)


def test_graph_replays_equal_direct_passes(cuda):
    sc = configs.C1_PT
    views = _views()
    with vcr.Context() as ctx:
        _setup(ctx, sc)
        ctx.batch_setup(views)
        for k in range(3):
            ctx.batch_pass(seed=9, pass_index=4 + k)
        ctx.synchronize()
        direct = [ctx.batch_read(v) for v in range(len(views))]
        ctx.batch_reset()
        ctx.batch_graph_record(seed=9, pass_index=4)
        ctx.batch_graph_replay(2)
        ctx.batch_graph_replay(1)
        ctx.synchronize()
        replayed = [ctx.batch_read(v) for v in range(len(views))]
        info = ctx.batch_info()
    assert info["passes"] == 3 and info["samples"] == 3
    for a, b in zip(direct, replayed):
        np.testing.assert_array_equal(a, b)


def test_batch_autotune_picks_a_candidate_and_clears(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        _setup(ctx, sc)
        ctx.batch_setup(_views())
        t = ctx.batch_autotune(seed=1, spp=2)
        assert t["majorant_level"] in (0, 1, 2, 3) and t["dda_steps"] in (2, 8, 16) and t["block_threads"] in (128, 256)
        assert ctx.get_tuning() == t
        info = ctx.batch_info()
        assert info["passes"] == 0 and info["samples"] == 0
        assert all(not ctx.batch_read(v).any() for v in range(3))


def test_batch_rejects_unsupported_setups(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        _setup(ctx, sc)
        with pytest.raises(vcr.VcrError):
            ctx.batch_pass(seed=1)  # no batch yet
        with pytest.raises(vcr.VcrError):
            ctx.batch_setup([])
        ctx.batch_setup(_views())
        prm = sc.params(vcr.TRACKER_GLOBAL)
        ctx.set_params(prm)
        with pytest.raises(vcr.VcrError):
            ctx.batch_pass(seed=1)
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.batch_pass(seed=1)
        ctx.synchronize()
