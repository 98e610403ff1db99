"""GPU parity tests of the density grid, the DDA and the path tracers against
the CPU oracle, called through the C-ABI.

Bar: bit-exact for the grid (generator, bricks, majorants, samples) and the
DDA cell sequence; per-sample radiance within 1e-5 relative wherever the
path decisions agree (same event and lookup counts), on >= 99% of pixels.
"""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _dev(t, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(t)).to(cuda)


@pytest.fixture(scope="module")
def small():
    size = (48, 40, 36)
    return size, orc.fbm_fill(size, seed=5, octaves=5)


@pytest.mark.parametrize("prec", [vcr.PREC_FP32, vcr.PREC_FP16, vcr.PREC_BF16])
def test_generated_grid_bricks_and_majorants_bit_exact(cuda, small, prec):
    import torch
    size, dense = small
    desc = vcr.grid_desc(size, (1 / 48,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 8.0)
    og = orc.Grid(dense, prec)
    for how in ("generate", "upload"):
        with vcr.Context() as ctx:
            if how == "generate":
                ctx.grid_generate(desc, vcr.fbm_desc(seed=5, octaves=5), prec)
            else:
                ctx.grid_upload(desc, dense, prec)
            ctx.set_cloud(cloud)
            mx, nb = ctx.grid_info()
            assert nb == og.nb
            assert mx == og.max_density()
            for level in range(4):
                np.testing.assert_array_equal(ctx.majorants(level), og.majorants(level))
            b0, b1 = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
            pts = (b0 + (b1 - b0) * np.random.default_rng(prec).random((100000, 3)) * 1.1 - 0.05 * (b1 - b0))
            pts = pts.astype(np.float32)
            d_pos = _dev(pts, cuda)
            d_out = torch.empty(len(pts), dtype=torch.float32, device=cuda)
            ctx.grid_sample(d_pos.data_ptr(), d_out.data_ptr(), len(pts))
            torch.cuda.synchronize()
            np.testing.assert_array_equal(d_out.cpu().numpy(), og.sample(cloud, pts))


@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_dda_cell_sequence_bit_exact(cuda, small, level):
    import torch
    size, dense = small
    desc = vcr.grid_desc(size, (1 / 48,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 8.0)
    og = orc.Grid(dense, 0)
    rng = np.random.default_rng(2)
    n, mc = 20000, 64
    o = (rng.random((n, 3)) * 3 - 1.5).astype(np.float32)
    o[: n // 2] = (rng.random((n // 2, 3)) * [1, 0.8, 0.75] + [-0.5, -0.4, 0]).astype(np.float32)  # inside
    d = rng.normal(size=(n, 3))
    d[:100, 1:] = 0  # axis-aligned rays
    d[100:200, 2] = 0
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_tuning(majorant_level=level)
        d_o, d_d = _dev(o, cuda), _dev(d, cuda)
        cells = torch.zeros((n, mc), dtype=torch.int32, device=cuda)
        tt = torch.zeros((n, mc, 2), dtype=torch.float32, device=cuda)
        cnt = torch.zeros(n, dtype=torch.int32, device=cuda)
        ctx.dda_trace(d_o.data_ptr(), d_d.data_ptr(), n, mc, cells.data_ptr(), tt.data_ptr(), cnt.data_ptr())
        torch.cuda.synchronize()
    oc, ot, on = og.dda_trace(cloud, o, d, mc, level)
    np.testing.assert_array_equal(cnt.cpu().numpy().view(np.uint32), on)
    assert on.max() > (4 >> level) and (on == 0).sum() > 10
    mask = np.arange(mc)[None, :] < on[:, None]
    np.testing.assert_array_equal(cells.cpu().numpy().view(np.uint32)[mask], oc[mask])
    np.testing.assert_array_equal(tt.cpu().numpy()[mask], ot[mask])


def _compare_pass(gpu_sum, gpu_stats, o_sum, o_stats, crop):
    x0, y0, w, h = crop
    gs, os_ = gpu_sum[y0:y0 + h, x0:x0 + w], o_sum[y0:y0 + h, x0:x0 + w]
    gst, ost = gpu_stats[y0:y0 + h, x0:x0 + w], o_stats[y0:y0 + h, x0:x0 + w]
    agree = np.all(gst[..., :2] == ost[..., :2], axis=-1)
    frac = agree.mean()
    assert frac >= 0.99, f"only {frac:.4f} of paths made the same decisions"
    denom = np.maximum(np.abs(os_), 1e-30)
    rel = np.abs(gs - os_) / denom
    bad = (rel > RTOL) & agree[..., None]
    assert not bad.any(), f"{bad.sum()} channels differ by > {RTOL} (max rel {rel[agree].max()})"
    return frac, float((gs == os_).all(axis=-1).mean())


def _render_both(ctx, og, cloud, cam, prm, W, H, crop, seed, pass_index, spp=1, sv=None, sv_tex=None):
    ctx.set_cloud(cloud)
    ctx.set_camera(cam)
    ctx.set_params(prm)
    ctx.set_frame(W, H)
    ctx.pt_pass(seed=seed, pass_index=pass_index, spp=spp, crop=crop, flags=vcr.PASS_RECORD_STATS)
    ctx.synchronize()
    g_sum, g_st = ctx.image_sum(), ctx.path_stats()
    o_sum, o_st = og.pt_pass(cloud, cam, prm, W, H, seed=seed, pass_index=pass_index, spp=spp, crop=crop,
                             flags=vcr.PASS_RECORD_STATS, sv=sv, sv_tex=sv_tex)
    return g_sum, g_st, o_sum, o_st


def test_shadow_volume_build_and_reference_mode_pass(cuda):
    """Reference-parity mode: xorshift streams seeded seed*(x + y*paddedW),
    shadow-volume NEE, gradient sky, albedo 1, no event cap."""
    size = (32, 32, 32)
    dense = orc.fbm_fill(size, seed=2, octaves=4)
    og = orc.Grid(dense, 0)
    desc = vcr.grid_desc(size, (1 / 32,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 6.0)
    sv = vcr.shadow_volume_setup(configs.sun_travel_dir(), cloud.bounds_min, cloud.bounds_max, 40)
    W = H = 48
    cam = vcr.camera_look((0, 0, -1), (0, 0, 1), 90.0, 0.1, W, H)
    prm = _abi_params(albedo=1.0, max_events=0, rng=vcr.RNG_XORSHIFT, nee=vcr.NEE_SHADOW_VOLUME,
                      sky=vcr.SKY_GRADIENT, tracker=vcr.TRACKER_GLOBAL)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        cloud.max_extinction = max(og.max_density(), 0.01)
        ctx.set_cloud(cloud)
        ctx.shadow_volume_build(sv)
        ctx.synchronize()
        g_sv = ctx.shadow_volume(40)
        o_sv = og.sv_build(cloud, sv)
        np.testing.assert_array_equal(g_sv, o_sv)
        out = _render_both(ctx, og, cloud, cam, prm, W, H, (0, 0, W, H), seed=12345, pass_index=0, sv=sv,
                           sv_tex=o_sv)
    _compare_pass(*out, (0, 0, W, H))
    assert out[1][..., 0].sum() > 100  # scatter events happened


def _abi_params(albedo, max_events, rng, nee, sky, tracker, g=0.857):
    p = configs.C1_PT.params(tracker)
    vcr.params_set_phase_g(p, g)
    p.albedo, p.max_events, p.rng_mode, p.nee_mode, p.sky_mode = albedo, max_events, rng, nee, sky
    return p


@pytest.mark.parametrize("tracker", [vcr.TRACKER_GLOBAL, vcr.TRACKER_DDA])
def test_c1_pass_matches_oracle_on_64x64_crop(cuda, tracker):
    """C1 (128^3 FP32, sigma_t = 8 rho, 512x512, <= 64 events): one pass on a
    64x64 crop through the middle of the cloud, per-sample radiance."""
    sc = configs.C1_PT
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, 0)
    crop = (224, 224, 64, 64)
    with vcr.Context() as ctx:
        ctx.grid_generate(sc.grid_desc(), sc.fbm(), vcr.PREC_FP32)
        cloud = sc.cloud()
        cloud.max_extinction = max(og.max_density(), 0.01)
        out = _render_both(ctx, og, cloud, sc.camera(), sc.params(tracker), sc.width, sc.height, crop, seed=7,
                           pass_index=3)
        paths, lookups, events, cells = ctx.counters()
    frac, exact = _compare_pass(*out, crop)
    assert paths == 64 * 64 and lookups > 64 * 64 and events > 64 * 64
    assert out[1][crop[1]:crop[1] + 64, crop[0]:crop[0] + 64, 0].sum() == events


@pytest.mark.parametrize("tuning", [dict(majorant_level=0, dda_steps=1, stage_majorants=0, block_threads=128),
                                    dict(majorant_level=1, dda_steps=64, stage_majorants=1, block_threads=256),
                                    dict(majorant_level=3, dda_steps=3, stage_majorants=1, block_threads=128),
                                    dict(majorant_level=2, dda_steps=2, stage_majorants=0, block_threads=256)])
def test_dda_tuning_knobs_keep_oracle_parity(cuda, tuning):
    """The level selects the estimator (the oracle mirrors it); the step
    count, shared-memory staging and CTA size are schedule-only."""
    sc = configs.C1_PT
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, 0)
    crop = (160, 200, 96, 64)
    with vcr.Context() as ctx:
        ctx.grid_upload(sc.grid_desc(), dense, vcr.PREC_FP32)
        ctx.set_tuning(**tuning)
        cloud = sc.cloud()
        cloud.max_extinction = max(og.max_density(), 0.01)
        ctx.set_cloud(cloud)
        ctx.set_camera(sc.camera())
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_frame(sc.width, sc.height)
        ctx.pt_pass(seed=9, pass_index=1, crop=crop, flags=vcr.PASS_RECORD_STATS)
        ctx.synchronize()
        g_sum, g_st = ctx.image_sum(), ctx.path_stats()
    o_sum, o_st = og.pt_pass(cloud, sc.camera(), sc.params(vcr.TRACKER_DDA), sc.width, sc.height, seed=9,
                             pass_index=1, crop=crop, flags=vcr.PASS_RECORD_STATS, level=tuning["majorant_level"])
    _compare_pass(g_sum, g_st, o_sum, o_st, crop)
    np.testing.assert_array_equal(g_st[..., 3], o_st[..., 3])  # DDA cell visits


def test_autotune_picks_a_valid_tuning(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=128, height=128)
        best = ctx.autotune(seed=1)
        assert best["majorant_level"] in range(4) and best["block_threads"] in (128, 256)
        assert ctx.get_tuning() == best
        assert ctx.pass_count() == 0  # autotune passes are not accumulated
        ctx.pt_pass(seed=1)
        ctx.synchronize()


@pytest.mark.parametrize("prec", [vcr.PREC_FP16, vcr.PREC_BF16])
def test_reduced_precision_dda_pass_matches_oracle(cuda, prec):
    sc = configs.C1_PT
    dense = orc.fbm_fill((64, 64, 64), seed=4, octaves=5)
    og = orc.Grid(dense, prec)
    desc = vcr.grid_desc((64, 64, 64), (1 / 64,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 12.0)
    cloud.max_extinction = max(og.max_density(), 0.01)
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense, prec)
        out = _render_both(ctx, og, cloud, sc.camera(96, 96), sc.params(vcr.TRACKER_DDA), 96, 96, (0, 0, 96, 96),
                           seed=3, pass_index=1, spp=2)
    _compare_pass(*out, (0, 0, 96, 96))


def test_multi_pass_accumulation_and_mean(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=64, height=64)
        for k in range(4):
            ctx.pt_pass(seed=1, pass_index=k)
        ctx.synchronize()
        assert ctx.pass_count() == 4
        s = ctx.image_sum()
        m = ctx.image_mean()
        np.testing.assert_allclose(m, (s / 4).astype(np.float32), rtol=1e-7)
        assert np.isfinite(s).all() and s.min() >= 0


def test_several_passes_in_one_launch_equal_single_passes(cuda):
    """vcr_pt_passes: the same paths and random streams as one vcr_pt_pass
    per pass; the FP64 sums equal up to the order of their additions."""
    sc = configs.C1_PT
    W = H = 128
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=W, height=H)
        ctx.set_tuning(majorant_level=2, dda_steps=8, stage_majorants=1, block_threads=256)
        tot = np.zeros(4, np.uint64)
        for k in range(5):
            ctx.pt_pass(seed=3, pass_index=10 + k)
            tot += np.array(ctx.counters(), np.uint64)
        ctx.synchronize()
        single = ctx.image_sum()
        ctx.reset()
        ctx.pt_passes(seed=3, first=10, count=5)
        ctx.synchronize()
        multi = ctx.image_sum()
        assert ctx.pass_count() == 5
        np.testing.assert_array_equal(np.array(ctx.counters(), np.uint64), tot)
        with pytest.raises(vcr.VcrError):
            ctx.pt_passes(seed=3, first=0, count=0)
        p = vcr._abi.PassDesc()
        p.seed, p.pass_index, p.spp, p.flags = 3, 0, 1, vcr.PASS_RECORD_STATS
        assert vcr.lib().vcr_pt_passes(ctx.h, p, 2, None) == vcr.ERR_INVALID
        prm = sc.params(vcr.TRACKER_GLOBAL)
        ctx.set_params(prm)
        with pytest.raises(vcr.VcrError):
            ctx.pt_passes(seed=3, first=0, count=2)
    np.testing.assert_allclose(multi, single, rtol=1e-12, atol=0)
    assert (single > 0).any()


@pytest.mark.parametrize("precision,size", [(vcr.PREC_FP32, (37, 21, 45)), (vcr.PREC_FP16, (37, 21, 45)),
                                            (vcr.PREC_BF16, (37, 21, 45)), (vcr.PREC_FP16, (24, 16, 40))])
def test_corner_blocks_give_the_bricks_values(cuda, precision, size):
    """Lookups through the per-cell corner blocks equal lookups that gather
    the 8 texels from the bricks, bit for bit: point samples over the whole
    box and past its faces (the clamp to the grid's edge), and a whole pass
    with its path statistics.  The blocks are built during the host upload
    (a tile layer behind each brick layer) or, when switched on after the
    upload, in one launch.  Odd sizes leave partial bricks and tiles;
    multiples of 8 add a tile layer past the last brick layer."""
    import torch
    dense = orc.fbm_fill(size, seed=9, octaves=4)
    desc = vcr.grid_desc(size, (1 / 45,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 24.0)
    rng = np.random.default_rng(4)
    lo, hi = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
    pts = (lo + (hi - lo) * rng.uniform(-0.02, 1.02, (50000, 3))).astype(np.float32)
    W = H = 64
    sc = configs.C1_PT
    out = []
    for corners in (1, 0, 2):
        with vcr.Context() as ctx:
            ctx.set_tuning(majorant_level=1, dda_steps=4, stage_majorants=1, block_threads=256,
                           corner_blocks=min(corners, 1))
            ctx.grid_upload(desc, dense, precision)
            if corners == 2:  # switched on after the upload
                ctx.set_tuning(majorant_level=1, dda_steps=4, stage_majorants=1, block_threads=256, corner_blocks=1)
            assert ctx.get_tuning()["corner_blocks"] == min(corners, 1)
            ctx.set_cloud(cloud)
            ctx.set_camera(vcr.camera_look((0.0, 0.0, -0.6), (0.0, 0.0, 1.0), 70.0, 0.1, W, H))
            ctx.set_params(sc.params(vcr.TRACKER_DDA))
            ctx.set_frame(W, H)
            dp = torch.from_numpy(pts).to(cuda)
            dv = torch.empty(len(pts), dtype=torch.float32, device=cuda)
            ctx.grid_sample(dp.data_ptr(), dv.data_ptr(), len(pts))
            ctx.pt_pass(seed=3, pass_index=1, flags=vcr.PASS_RECORD_STATS)
            ctx.synchronize()
            out.append((dv.cpu().numpy(), ctx.image_sum(), ctx.path_stats()))
    (va, ia, sa), (vb, ib, sb), (vc, ic, sc2) = out
    for v, i, s in ((va, ia, sa), (vc, ic, sc2)):
        np.testing.assert_array_equal(v, vb)
        np.testing.assert_array_equal(i, ib)
        np.testing.assert_array_equal(s, sb)
    assert (va > 0).mean() > 0.3 and sa[..., 1].sum() > 1000


def test_reuploading_a_same_size_grid_replaces_every_buffer(cuda):
    """A second grid of the same size uploaded into the same context (its
    brick, scale, majorant and corner buffers are reused) samples exactly
    as in a fresh context, also when the corner blocks were switched off
    for the upload and on again afterwards."""
    import torch
    size = (40, 24, 32)
    desc = vcr.grid_desc(size, (1 / 40,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 24.0)
    a = orc.fbm_fill(size, seed=1, octaves=4)
    b = orc.fbm_fill(size, seed=2, octaves=4) * 1.5
    lo, hi = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
    pts = (lo + (hi - lo) * np.random.default_rng(5).uniform(-0.02, 1.02, (20000, 3))).astype(np.float32)
    dp = torch.from_numpy(pts).to(cuda)

    def sample(ctx):
        ctx.set_cloud(cloud)
        dv = torch.empty(len(pts), dtype=torch.float32, device=cuda)
        ctx.grid_sample(dp.data_ptr(), dv.data_ptr(), len(pts))
        ctx.synchronize()
        return dv.cpu().numpy(), [ctx.majorants(lv) for lv in range(4)]

    with vcr.Context() as ctx:
        ctx.grid_upload(desc, b, vcr.PREC_FP16)
        want, want_maj = sample(ctx)
    for switch_off in (False, True):
        with vcr.Context() as ctx:
            ctx.grid_upload(desc, a, vcr.PREC_FP16)
            sample(ctx)
            if switch_off:
                ctx.set_tuning(corner_blocks=0)
            ctx.grid_upload(desc, b, vcr.PREC_FP16)
            if switch_off:
                ctx.set_tuning(corner_blocks=1)
            got, got_maj = sample(ctx)
        np.testing.assert_array_equal(got, want)
        for g, w in zip(got_maj, want_maj):
            np.testing.assert_array_equal(g, w)


def test_stream_ordered_readback_gives_each_pass_its_image(cuda):
    """vcr_readback_async after every pass on a side stream: each pinned
    host buffer holds the mean (and the FP64 sums) as they stood after its
    pass, equal to the synchronous read back of the same passes, although
    the later passes were queued before the copies landed."""
    import torch
    sc = configs.C1_PT
    W = H = 64
    passes = 4
    stream = torch.cuda.Stream()
    want_mean, want_sum = [], []
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=W, height=H, tracker=vcr.TRACKER_DDA)
        for k in range(passes):
            ctx.pt_pass(seed=8, pass_index=k)
            want_mean.append(ctx.image_mean())
            want_sum.append(ctx.image_sum())
    means = [torch.empty(W * H * 3, dtype=torch.float32).pin_memory() for _ in range(passes)]
    sums = [torch.empty(W * H * 3, dtype=torch.float64).pin_memory() for _ in range(passes)]
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=W, height=H, tracker=vcr.TRACKER_DDA)
        ctx.synchronize()
        for k in range(passes):
            ctx.pt_pass(seed=8, pass_index=k, stream=stream.cuda_stream)
            ctx.readback_async(vcr.BUF_IMAGE_MEAN, means[k].data_ptr(), W * H * 12, stream=stream.cuda_stream)
            ctx.readback_async(vcr.BUF_IMAGE_SUM, sums[k].data_ptr(), W * H * 24, stream=stream.cuda_stream)
        ctx.readback_wait()
        with pytest.raises(vcr.VcrError):
            ctx.readback_async(vcr.BUF_PATH_STATS, means[0].data_ptr(), W * H * 16)
    for k in range(passes):
        np.testing.assert_array_equal(means[k].numpy(), np.asarray(want_mean[k], np.float32).reshape(-1))
        np.testing.assert_array_equal(sums[k].numpy(), np.asarray(want_sum[k]).reshape(-1))
