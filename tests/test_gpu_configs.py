"""Parity at the full sizes of the scene configurations.

The shipped kernels run on each configuration's own grid, image and photon
or beam counts, with the tuning the benchmark uses, and are compared with
the oracle on the same inputs:

* C5, the benchmark scene (1024x512x1024 fBm, 8 octaves, FP16 8^3 bricks,
  sigma_t = 32 rho, 1920x1080): bricks and every majorant level, then whole
  frames of the DDA wavefront tracker at the benchmark's tuning (majorant
  level 3 staged in shared memory, 16 cells a step, 256-thread CTAs) and at
  level 2; every pixel's radiance and path statistics.  Also the frame whose
  paths end in the radiance cache at the 2nd event (zero network: exactly
  the truncated paths).  Reference loop: PathTracer.comp:366-425.
* C4 (512^3, FP16 and BF16 bricks, 64 views of uneven size, 8 suns, 4 spp):
  one batched launch; every view equals the oracle's single-view pass.
* C2 (256^3, sigma_t = 16 rho, 1,048,576 photons a pass, 960x540): stored
  photons, photon tree, per-pixel FP64 statistics and the image, over two
  progressive passes.  Reference: PPM_PT.comp:452-489, PPM_PE.comp:304-375.
* C3 (256^3, about 262,144 beams a pass, 1280x720): beam slots, all
  segments with their 30-bit Morton codes, the sort permutation, the LBVH
  topology and boxes bit for bit, and the gather on a pixel crop.
  Reference: PPB_PT.comp:317-539, PPB_RadixSort_LocalSort.comp:154-252,
  PPB_GenerateHierarchy.comp:62-168, PPB_PE.comp:408-466.

Bars: integer and index work bit-exact; per-sample radiance within 1e-5
relative where the path decisions (events, lookups) agree, which must be at
least 99 % of paths (the arithmetic is pinned, so in practice all of them
agree and the images are identical); FP64 sums of several samples within
1e-12 relative.
"""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from oracle import oracle_ppm as opm
from vcr import configs

pytestmark = pytest.mark.gpu

RTOL = 1e-5
SEED_STEP = 0x9E3779B9


def _compare_frame(g_sum, g_st, o_sum, o_st):
    agree = np.all(g_st[..., :2] == o_st[..., :2], axis=-1)
    frac = agree.mean()
    assert frac >= 0.99, f"only {frac:.5f} of paths made the same decisions"
    rel = np.abs(g_sum - o_sum) / np.maximum(np.abs(o_sum), 1e-30)
    bad = (rel > RTOL) & agree[..., None]
    assert not bad.any(), f"{bad.sum()} channels differ by > {RTOL}"
    return frac, float((g_sum == o_sum).all(axis=-1).mean())


@pytest.fixture(scope="module")
def c5_oracle():
    sc = configs.C5_NRC
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, sc.precision)
    del dense
    return sc, og


def test_c5_bricks_and_majorants_at_full_size(cuda, c5_oracle):
    sc, og = c5_oracle
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.synchronize()
        for level in range(4):
            np.testing.assert_array_equal(ctx.majorants(level), og.majorants(level), err_msg=f"level {level}")
        np.testing.assert_array_equal(ctx.grid_read_dense().reshape(-1), og.decoded().reshape(-1))


@pytest.mark.parametrize("tuning", [dict(majorant_level=3, dda_steps=16, stage_majorants=1, block_threads=256),
                                    dict(majorant_level=2, dda_steps=8, stage_majorants=1, block_threads=128)])
def test_c5_full_frames_match_the_oracle(cuda, c5_oracle, tuning):
    sc, og = c5_oracle
    W, H = sc.width, sc.height
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    cam, prm = sc.camera(), sc.params(vcr.TRACKER_DDA)
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        ctx.set_tuning(**tuning)
        for k in (0, 1):
            ctx.reset()
            ctx.pt_pass(seed=5, pass_index=k, flags=vcr.PASS_RECORD_STATS)
            ctx.synchronize()
            g_sum, g_st = ctx.image_sum(), ctx.path_stats()
            paths, lookups, events, cells = ctx.counters()
            o_sum, o_st = og.pt_pass(cloud, cam, prm, W, H, seed=5, pass_index=k, flags=vcr.PASS_RECORD_STATS,
                                     level=tuning["majorant_level"])
            frac, exact = _compare_frame(g_sum, g_st, o_sum, o_st)
            assert paths == W * H
            assert lookups == int(o_st[..., 1].sum()) and events == int(o_st[..., 0].sum())
            assert cells == int(o_st[..., 3].sum())
            assert events > W * H  # the frame sees dense cloud


def test_c5_passes_in_one_launch_match_the_oracle(cuda, c5_oracle):
    """Three consecutive passes of the benchmark scene in one launch
    (vcr_pt_passes, the benchmark's timed form): the sums equal the
    oracle's three passes up to the order of the FP64 additions."""
    sc, og = c5_oracle
    W, H = sc.width, sc.height
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    cam, prm = sc.camera(), sc.params(vcr.TRACKER_DDA)
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        ctx.set_tuning(majorant_level=3, dda_steps=16, stage_majorants=1, block_threads=256)
        ctx.pt_passes(seed=9, first=4, count=3)
        ctx.synchronize()
        g_sum = ctx.image_sum()
        lookups = ctx.counters()[1]
    o_sum = None
    o_look = 0
    for k in range(4, 7):
        o_sum, o_st = og.pt_pass(cloud, cam, prm, W, H, seed=9, pass_index=k, sum_img=o_sum,
                                 flags=vcr.PASS_RECORD_STATS, level=3)
        o_look += int(o_st[..., 1].sum())
    np.testing.assert_allclose(g_sum, o_sum, rtol=1e-12, atol=0)
    assert lookups == o_look


def test_c5_fast_math_frame_against_the_oracle(cuda, c5_oracle):
    """The opt-in fast-math tracker (vcr_tuning.fast_math: contracted FMAs,
    hardware log / exp / sincos) on a full C5 frame: the share of paths
    whose decisions (events, lookups) match the bit-exact oracle's, and the
    relative radiance difference where they do.  Its figures are printed;
    the bars are those the fast build measured with margin, not the exact
    build's bit-exactness."""
    sc, og = c5_oracle
    W, H = sc.width, sc.height
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    cam, prm = sc.camera(), sc.params(vcr.TRACKER_DDA)
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        ctx.set_tuning(majorant_level=3, dda_steps=16, stage_majorants=1, block_threads=256, fast_math=1)
        ctx.pt_pass(seed=5, pass_index=0, flags=vcr.PASS_RECORD_STATS)
        ctx.synchronize()
        g_sum, g_st = ctx.image_sum(), ctx.path_stats()
    o_sum, o_st = og.pt_pass(cloud, cam, prm, W, H, seed=5, pass_index=0, flags=vcr.PASS_RECORD_STATS, level=3)
    agree = np.all(g_st[..., :2] == o_st[..., :2], axis=-1)
    hit = o_st[..., 1] > 0  # paths with at least one density lookup
    rel = np.abs(g_sum - o_sum) / np.maximum(np.abs(o_sum), 1e-30)
    ra = rel[agree & hit]
    img_rel = abs(g_sum.sum() - o_sum.sum()) / o_sum.sum()
    print(f"\nfast math: decisions agree on {agree.mean():.5f} of paths ({agree[hit].mean():.5f} of those with a "
          f"lookup); where they agree, relative radiance difference median {np.median(ra):.2e}, "
          f"99th pct {np.percentile(ra, 99):.2e}, max {ra.max():.2e}; frame sum differs by {img_rel:.2e}")
    assert agree.mean() >= 0.95
    assert np.percentile(ra, 99) <= 1e-4
    assert img_rel <= 1e-2


def test_c5_paths_ending_in_the_cache_match_the_oracle(cuda, c5_oracle):
    """The cached frame's tracker at C5: paths end at their 2nd event in the
    cache; with an all-zero network the image is exactly the oracle's
    truncated paths, and one query is made per path that got there."""
    sc, og = c5_oracle
    W, H = sc.width, sc.height
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = sc.extra["nrc_events"]
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        ctx.set_params(prm)
        ctx.set_tuning(majorant_level=3, dda_steps=16, stage_majorants=1, block_threads=256)
        ctx.nrc_setup(train_samples=sc.extra["train_samples"], query_capacity=W * H, seed=1)
        ctx.nrc_set_weights(np.zeros(ctx.NRC_WEIGHTS, np.float32))
        ctx.pt_pass(seed=4, pass_index=0, flags=vcr.PASS_RECORD_STATS)
        ctx.synchronize()
        g_sum, g_st = ctx.image_sum(), ctx.path_stats()
        queries = ctx.nrc_info()["queries"]
    o_sum, o_st = og.pt_pass(cloud, sc.camera(), prm, W, H, seed=4, pass_index=0, flags=vcr.PASS_RECORD_STATS,
                             level=3)
    _compare_frame(g_sum, g_st, o_sum, o_st)
    assert queries == int((o_st[..., 0] >= 2).sum()) > W * H // 20


@pytest.mark.parametrize("precision", [vcr.PREC_FP16, vcr.PREC_BF16])
def test_c4_batched_views_at_full_size(cuda, precision):
    sc = configs.C4_BATCH
    views = configs.c4_views(sc.extra["views"])
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, precision)
    del dense
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    spp, seed, pass_index, level = sc.spp, 13, 1, 2
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, precision=precision)
        ctx.set_cloud(cloud)
        for level_check in range(4):
            np.testing.assert_array_equal(ctx.majorants(level_check), og.majorants(level_check))
        ctx.set_tuning(majorant_level=level, dda_steps=16, stage_majorants=1, block_threads=256)
        ctx.batch_setup(views)
        ctx.batch_pass(seed=seed, pass_index=pass_index, spp=spp)
        ctx.synchronize()
        picks = range(len(views))
        got = {v: ctx.batch_read(v) for v in picks}
        info = ctx.batch_info()
    assert info["views"] == 64 and info["samples"] == spp
    assert info["pixels"] == sum(w * h for _, w, h, _ in views)
    for v in picks:
        cam, w, h, sun = views[v]
        prm = sc.params(vcr.TRACKER_DDA)
        for a in range(3):
            prm.sun_dir[a] = sun[a]
        ref, _ = og.pt_pass(cloud, cam, prm, w, h, seed=(seed + SEED_STEP * v) % (1 << 32), pass_index=pass_index,
                            spp=spp, level=level)
        # four float radiances per pixel summed in FP64 in another order
        np.testing.assert_allclose(got[v], ref, rtol=1e-12, atol=0, err_msg=f"view {v}")
        assert (ref > 0.1).any()


def test_c2_photon_mapping_at_full_size(cuda):
    sc = configs.C2_PPM
    ex = sc.extra
    W, H = sc.width, sc.height
    photons, cap = ex["photons"], 8 * ex["photons"]
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    g = orc.Grid(dense, sc.precision)
    del dense
    cloud = sc.cloud()
    cloud.max_extinction = max(g.max_density(), 0.01)
    cam, prm = sc.camera(), sc.params(vcr.TRACKER_DDA)
    st = opm.init_stats(W, H, ex["r0"])
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        ctx.ppm_setup(photons, cap, ex["r0"], ex["alpha"])
        for k in range(2):
            ctx.ppm_pass(seed=21, pass_index=k)
            ctx.synchronize()
            s_o, o = opm.ppm_pass(g, cloud, cam, prm, photons, cap, ex["alpha"], W, H, st, seed=21, pass_index=k,
                                  want_photons=True)
            info = ctx.ppm_info()
            assert info["photons_stored"] == o["info"]["photons_stored"] > photons
            assert info["dropped"] == 0
            uid = ctx.ppm_read("uid")
            perm = np.argsort(uid, kind="stable")
            np.testing.assert_array_equal(uid[perm], o["uid"])
            ph = np.concatenate([ctx.ppm_read(f)[perm] for f in ("pos", "power", "dir")], axis=1)
            np.testing.assert_array_equal(ph, o["photons"])
            inv = np.empty_like(perm)
            inv[perm] = np.arange(len(perm))
            np.testing.assert_array_equal(inv[ctx.ppm_read("order")], o["order"])
            np.testing.assert_array_equal(ctx.ppm_read("left"), o["left"])
            np.testing.assert_array_equal(ctx.ppm_read("right"), o["right"])
            np.testing.assert_array_equal(ctx.ppm_read("stats"), st)
            np.testing.assert_array_equal(ctx.image_sum(), s_o)
        assert (st[..., 0] > 0).mean() > 0.2  # pixels gathered photons


def test_c3_photon_beams_at_full_size(cuda):
    sc = configs.C3_PPB
    W, H = sc.width, sc.height
    r0, alpha, cap = 0.02, 0.8, 1 << 24
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    g = orc.Grid(dense, sc.precision)
    del dense
    cloud = sc.cloud()
    cloud.max_extinction = max(g.max_density(), 0.01)
    cam, prm = sc.camera(), sc.params(vcr.TRACKER_DDA)
    crop = (W // 2 - 32, H // 2 - 16, 64, 32)
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_cloud(cloud)
        probe = 16384
        ctx.ppb_setup(probe, cap, r0, alpha)
        ctx.ppb_pass(seed=1, pass_index=0)
        ctx.synchronize()
        photons = int(sc.extra["beams"] / max(float(ctx.ppb_read("nbeams", probe).sum()) / probe, 1e-3))
        ctx.ppb_setup(photons, cap, r0, alpha)
        ctx.reset()
        ctx.ppb_pass(seed=11, pass_index=2, crop=crop)
        ctx.synchronize()
        info = ctx.ppb_info()
        gb = {k: ctx.ppb_read(k, photons) for k in ("nbeams", "slots", "seg_a", "seg_b", "seg_beam", "codes",
                                                     "order", "left", "right", "node_lo", "node_hi", "leaf_lo",
                                                     "leaf_hi")}
        g_sum = ctx.image_sum()
    o_sum, ob = orc.ppb_pass(g, cloud, cam, prm, photons, cap, r0, alpha, W, H, seed=11, pass_index=2, crop=crop)
    beams = int(gb["nbeams"].sum())
    assert 0.8 * sc.extra["beams"] < beams < 1.25 * sc.extra["beams"]
    assert info["segments"] == ob["info"]["segments"] > 4_000_000 and info["dropped"] == 0
    for k in gb:
        np.testing.assert_array_equal(gb[k], ob[k], err_msg=k)
    # the permutation is the stable order of the codes, the tree is over them
    np.testing.assert_array_equal(gb["order"], np.argsort(gb["codes"], kind="stable").astype(np.uint32))
    x0, y0, cw, ch = crop
    gs, os_ = g_sum[y0:y0 + ch, x0:x0 + cw], o_sum[y0:y0 + ch, x0:x0 + cw]
    rel = np.abs(gs - os_) / np.maximum(np.abs(os_), 1e-30)
    assert rel.max() <= RTOL, rel.max()
    assert os_.max() > 0.05
