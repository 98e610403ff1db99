"""GPU tests of the radiance cache through the C-ABI: forward pass and
loss gradient against the oracle's FP64 restatement (with the GPU's BF16
roundings), online training lowers the loss, and paths that end in the
cache render exactly the oracle's truncated paths plus the cache term."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from oracle import oracle_nrc as onrc
from vcr import configs

pytestmark = pytest.mark.gpu


def _cloud():
    desc = vcr.grid_desc((64, 32, 64), (1 / 64,) * 3)
    return desc, vcr.cloud_from_grid(desc, 1.0, 16.0)


def _ctx_with_cloud(ctx, desc, cloud, dense=None):
    if dense is None:
        dense = orc.fbm_fill((64, 32, 64), seed=3, octaves=4)
    ctx.grid_upload(desc, dense)
    ctx.set_cloud(cloud)
    return dense


def _dev_records(recs, cuda):
    import torch
    return torch.from_numpy(recs.view(np.uint8).copy()).to(cuda)


@pytest.mark.parametrize("kernel,n", [(vcr.NRC_QUERY_MMA, 1000), (vcr.NRC_QUERY_TCGEN05, 1000),
                                      (vcr.NRC_QUERY_TCGEN05, 128 * 152 * 3 + 77)])
def test_forward_matches_oracle(cuda, kernel, n):
    """Both query kernels (warp mma.sync tiles; tcgen05 128-record tiles
    with TMEM accumulators, several tiles per CTA and a ragged last one)."""
    import torch
    desc, cloud = _cloud()
    rng = np.random.default_rng(1)
    recs = onrc.random_records(n, cloud, rng)
    with vcr.Context() as ctx:
        _ctx_with_cloud(ctx, desc, cloud)
        ctx.nrc_setup(train_samples=4096, seed=7, query_kernel=kernel)
        w = ctx.nrc_get_weights()
        dr = _dev_records(recs, cuda)
        out = torch.zeros(3 * len(recs), dtype=torch.float32, device=cuda)
        ctx.nrc_forward(dr.data_ptr(), len(recs), out.data_ptr())
        got = out.cpu().numpy().reshape(-1, 3)
    ref = onrc.forward(w, recs, cloud)
    scale = np.abs(ref).mean() + 1e-3
    assert np.abs(got - ref).max() <= 3e-2 * scale, (np.abs(got - ref).max(), scale)
    assert np.abs(got - ref).mean() <= 3e-3 * scale


@pytest.mark.parametrize("kernel", [vcr.NRC_QUERY_MMA, vcr.NRC_QUERY_TCGEN05])
@pytest.mark.parametrize("levels", [8, 0])
def test_forward_with_fewer_position_levels_matches_oracle(cuda, kernel, levels):
    """position_levels = L (position_drop = 16 - L): both query kernels see
    only the first L frequency levels, as the oracle encoding with the same
    L (L = 0: no position input at all)."""
    import torch
    desc, cloud = _cloud()
    recs = onrc.random_records(700, cloud, np.random.default_rng(2))
    with vcr.Context() as ctx:
        _ctx_with_cloud(ctx, desc, cloud)
        ctx.nrc_setup(train_samples=4096, seed=7, query_kernel=kernel, position_levels=levels)
        w = ctx.nrc_get_weights()
        dr = _dev_records(recs, cuda)
        out = torch.zeros(3 * len(recs), dtype=torch.float32, device=cuda)
        ctx.nrc_forward(dr.data_ptr(), len(recs), out.data_ptr())
        got = out.cpu().numpy().reshape(-1, 3)
    try:
        onrc.set_levels(levels)
        ref = onrc.forward(w, recs, cloud)
    finally:
        onrc.set_levels(16)
    full = onrc.forward(w, recs, cloud)
    scale = np.abs(ref).mean() + 1e-3
    assert np.abs(got - ref).max() <= 3e-2 * scale, (np.abs(got - ref).max(), scale)
    assert np.abs(got - ref).mean() <= 3e-3 * scale
    assert np.abs(full - ref).mean() > 10 * np.abs(got - ref).mean()  # the knob changes the output


def test_query_kernels_agree_in_a_cached_render(cuda):
    """A cached frame with trained weights: the tcgen05 queries give the
    image of the mma.sync queries up to BF16 rounding of the activations
    (the paths and their queries are identical; only the cache term
    differs)."""
    sc = configs.C1_PT
    W = H = 128
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = 2
    with vcr.Context() as ctx:  # trained weights to query with
        configs.setup_context(ctx, sc, width=W, height=H)
        ctx.set_params(prm)
        ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, query_capacity=W * H, seed=2)
        for k in range(30):
            ctx.nrc_train_step(seed=4, pass_index=k)
        ctx.synchronize()
        w = ctx.nrc_get_weights()
    imgs = []
    for kernel in (vcr.NRC_QUERY_MMA, vcr.NRC_QUERY_TCGEN05):
        with vcr.Context() as ctx:
            configs.setup_context(ctx, sc, width=W, height=H)
            ctx.set_params(prm)
            ctx.nrc_setup(train_samples=8192, query_capacity=W * H, seed=2, query_kernel=kernel)
            ctx.nrc_set_weights(w)
            ctx.pt_pass(seed=6, pass_index=0)
            ctx.synchronize()
            imgs.append((ctx.image_sum(), ctx.nrc_info()["queries"]))
    (ia, qa), (ib, qb) = imgs
    assert qa == qb > 1000
    d = np.abs(ia - ib)
    assert d.max() <= 2e-2 * (np.abs(ia).max() + 1e-3), d.max()
    assert d.mean() <= 1e-3 * (np.abs(ia).mean() + 1e-3), d.mean()


@pytest.mark.parametrize("n", [4096, 20037])  # whole tiles; a ragged last tile and two tiles on some CTAs
def test_gradient_matches_oracle(cuda, n):
    desc, cloud = _cloud()
    rng = np.random.default_rng(2)
    recs = onrc.random_records(n, cloud, rng)
    with vcr.Context() as ctx:
        _ctx_with_cloud(ctx, desc, cloud)
        ctx.nrc_setup(train_samples=4096, seed=11)
        w = ctx.nrc_get_weights()
        dr = _dev_records(recs, cuda)
        g, loss = ctx.nrc_gradient(dr.data_ptr(), len(recs))
    gref, lref = onrc.gradient(w, recs, cloud)
    assert abs(loss - lref) <= 1e-2 * abs(lref)
    cos = float(g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)))
    rel = float(np.linalg.norm(g - gref) / np.linalg.norm(gref))
    assert cos > 0.999 and rel < 3e-2, (cos, rel)
    # padded output columns never receive gradient
    out = g[5 * 64 * 64:].reshape(64, 16)
    assert np.all(out[:, 3:] == 0)


def _grid_ctx(ctx, desc, cloud, kernel, rng):
    """A grid-encoded cache with random tables (large enough that the
    position inputs matter); returns all its parameters."""
    _ctx_with_cloud(ctx, desc, cloud)
    ctx.nrc_setup(train_samples=4096, seed=7, query_kernel=kernel, encoding=vcr.NRC_ENCODING_GRID)
    p = ctx.nrc_get_weights(tables=True)
    assert p.size == vcr.Context.NRC_WEIGHTS + onrc.GRID_PARAMS
    assert np.all(np.abs(p[vcr.Context.NRC_WEIGHTS:]) <= 1e-4)  # initial tables
    p[vcr.Context.NRC_WEIGHTS:] = rng.uniform(-0.5, 0.5, onrc.GRID_PARAMS)
    ctx.nrc_set_weights(p)
    return p


@pytest.mark.parametrize("kernel", [vcr.NRC_QUERY_MMA, vcr.NRC_QUERY_TCGEN05])
def test_grid_encoding_forward_matches_oracle(cuda, kernel):
    """The grid encoding (16 levels of trilinearly interpolated 2-feature
    tables, dense then hashed) through both query kernels against the
    oracle's restatement of it."""
    import torch
    desc, cloud = _cloud()
    rng = np.random.default_rng(8)
    recs = onrc.random_records(900, cloud, rng)
    with vcr.Context() as ctx:
        p = _grid_ctx(ctx, desc, cloud, kernel, rng)
        dr = _dev_records(recs, cuda)
        out = torch.zeros(3 * len(recs), dtype=torch.float32, device=cuda)
        ctx.nrc_forward(dr.data_ptr(), len(recs), out.data_ptr())
        got = out.cpu().numpy().reshape(-1, 3)
    w = p[:vcr.Context.NRC_WEIGHTS]
    try:
        onrc.set_grid(p[vcr.Context.NRC_WEIGHTS:])
        ref = onrc.forward(w, recs, cloud)
    finally:
        onrc.set_grid(None)
    freq = onrc.forward(w, recs, cloud)
    scale = np.abs(ref).mean() + 1e-3
    assert np.abs(got - ref).max() <= 3e-2 * scale, (np.abs(got - ref).max(), scale)
    assert np.abs(got - ref).mean() <= 3e-3 * scale
    assert np.abs(freq - ref).mean() > 10 * np.abs(got - ref).mean()  # the tables are what it read


def test_grid_encoding_gradient_matches_oracle(cuda):
    """The fused training kernel's gradient with the grid encoding: the
    network's weights and the tables (dX_0 = dY_0 W_0^T spread over each
    level's 8 vertices by float atomics) against the oracle."""
    desc, cloud = _cloud()
    rng = np.random.default_rng(9)
    recs = onrc.random_records(600, cloud, rng)
    with vcr.Context() as ctx:
        p = _grid_ctx(ctx, desc, cloud, vcr.NRC_QUERY_MMA, rng)
        dr = _dev_records(recs, cuda)
        g, loss = ctx.nrc_gradient(dr.data_ptr(), len(recs), tables=True)
    try:
        onrc.set_grid(p[vcr.Context.NRC_WEIGHTS:])
        gw, gt, lref = onrc.gradient_tables(p[:vcr.Context.NRC_WEIGHTS], recs, cloud)
    finally:
        onrc.set_grid(None)
    assert abs(loss - lref) <= 1e-2 * abs(lref)
    for got, ref in ((g[:vcr.Context.NRC_WEIGHTS], gw), (g[vcr.Context.NRC_WEIGHTS:], gt)):
        cos = float(got @ ref / (np.linalg.norm(got) * np.linalg.norm(ref)))
        rel = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        assert cos > 0.999 and rel < 3e-2, (cos, rel)
    assert np.array_equal(np.nonzero(g[vcr.Context.NRC_WEIGHTS:])[0], np.nonzero(gt)[0])


def _smooth_targets(recs, cloud):
    b0, b1 = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
    x = (recs["p"] - b0) / (b1 - b0)
    base = 0.3 + 0.12 * np.sin(2 * np.pi * x[:, 0]) * np.cos(2 * np.pi * x[:, 2]) + 0.08 * recs["v"][:, 1]
    recs["w"] = base[:, None] * np.array([1.0, 0.8, 0.6])


@pytest.mark.parametrize("encoding", [vcr.NRC_ENCODING_FREQUENCY, vcr.NRC_ENCODING_GRID])
def test_fit_converges_on_a_deterministic_target(cuda, encoding):
    desc, cloud = _cloud()
    rng = np.random.default_rng(4)
    recs = onrc.random_records(8192, cloud, rng)
    _smooth_targets(recs, cloud)
    with vcr.Context() as ctx:
        _ctx_with_cloud(ctx, desc, cloud)
        ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, seed=5, encoding=encoding)
        dr = _dev_records(recs, cuda)
        _, l0 = ctx.nrc_gradient(dr.data_ptr(), len(recs))
        ctx.nrc_fit(dr.data_ptr(), len(recs), 400)
        ctx.synchronize()
        _, l1 = ctx.nrc_gradient(dr.data_ptr(), len(recs))
        assert ctx.nrc_info()["steps"] == 400
    assert np.isfinite(l1) and l1 < 0.05 * l0, (l0, l1)


def test_moving_average_weights_serve_queries(cuda):
    """With ema_decay > 0 queries use the averaged weights: right after
    set_weights they equal the training weights (oracle forward of w); after
    training they lag behind the training weights."""
    import torch
    desc, cloud = _cloud()
    rng = np.random.default_rng(6)
    recs = onrc.random_records(2048, cloud, rng)
    _smooth_targets(recs, cloud)
    with vcr.Context() as ctx:
        _ctx_with_cloud(ctx, desc, cloud)
        ctx.nrc_setup(train_samples=4096, learning_rate=3e-3, seed=8, ema_decay=0.99)
        w = ctx.nrc_get_weights()
        ctx.nrc_set_weights(w)
        dr = _dev_records(recs, cuda)
        out = torch.zeros(3 * len(recs), dtype=torch.float32, device=cuda)
        ctx.nrc_forward(dr.data_ptr(), len(recs), out.data_ptr())
        y0 = out.cpu().numpy().reshape(-1, 3)
        ctx.nrc_fit(dr.data_ptr(), len(recs), 100)
        ctx.synchronize()
        ctx.nrc_forward(dr.data_ptr(), len(recs), out.data_ptr())
        y1 = out.cpu().numpy().reshape(-1, 3)
        w1 = ctx.nrc_get_weights()
    ref0 = onrc.forward(w, recs, cloud)
    scale = np.abs(ref0).mean() + 1e-3
    assert np.abs(y0 - ref0).mean() <= 3e-3 * scale
    ref1 = onrc.forward(w1, recs, cloud)
    t = recs["w"]
    err_avg, err_train = np.abs(y1 - t).mean(), np.abs(ref1 - t).mean()
    assert np.abs(y1 - ref1).mean() > 1e-3 * scale  # not the training weights
    assert err_avg < np.abs(ref0 - t).mean()  # but it has moved toward the targets
    assert err_train < np.abs(ref0 - t).mean()


def test_training_paths_are_calibrated_to_the_record_budget(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=128, height=128)
        ctx.nrc_setup(train_samples=16384, seed=3)
        counts = []
        for k in range(4):
            ctx.nrc_train_step(seed=5, pass_index=k)
            counts.append(ctx.nrc_info()["train_records"])
        ctx.set_camera(vcr.camera_look((0.2, 0.1, -0.4), (0.0, 0.0, 1.0), 70.0, 0.1, 128, 128))  # recalibrates
        ctx.nrc_train_step(seed=5, pass_index=9)
        ctx.nrc_train_step(seed=5, pass_index=10)
        counts.append(ctx.nrc_info()["train_records"])
    for c in counts[1:]:
        assert 0.7 * 16384 <= c <= 1.4 * 16384, counts


def test_a_step_traces_several_training_sets_in_one_launch(cuda):
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=128, height=128)
        prm = sc.params(vcr.TRACKER_DDA)
        prm.nrc_events = 2
        ctx.set_params(prm)
        ctx.nrc_setup(train_samples=8192, seed=3)
        with pytest.raises(vcr.VcrError):  # nothing traced yet
            ctx.nrc_train_more(1)
        ctx.nrc_train_step(seed=5, pass_index=0, sets=4)  # calibrates, then traces four sets
        four = ctx.nrc_info()["train_records"]
        w0 = ctx.nrc_get_weights()
        ctx.nrc_train_more(15, max_records=2048)  # walks the four sets batch by batch
        info = ctx.nrc_info()
        assert info["steps"] == 16 and np.isfinite(info["last_loss"])
        assert not np.array_equal(w0, ctx.nrc_get_weights())
        ctx.nrc_train_step(seed=5, pass_index=1)
        one = ctx.nrc_info()["train_records"]
        ctx.nrc_frame(seed=6, pass_index=2)
        frame = ctx.nrc_info()["train_records"]
        with pytest.raises(vcr.VcrError):
            ctx.nrc_train_step(seed=5, pass_index=3, sets=65)
        with pytest.raises(vcr.VcrError):
            ctx.nrc_set_learning_rate(0.0)
        ctx.nrc_set_learning_rate(5e-4)
        ctx.nrc_train_more(1)
    assert 0.7 * 4 * 8192 <= four <= 1.4 * 4 * 8192, four
    assert 0.7 * 8192 <= one <= 1.4 * 8192 and 0.7 * 8192 <= frame <= 1.4 * 8192, (one, frame)


def test_frame_equals_pass_then_train_step(cuda):
    """vcr_nrc_frame overlaps the training paths with the pass; its result
    is the sequential pass + train step (up to the order of the gradient's
    float atomics)."""
    sc = configs.C1_PT
    W = H = 96
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = 2
    res = []
    for mode in ("sequential", "frame"):
        with vcr.Context() as ctx:
            configs.setup_context(ctx, sc, width=W, height=H)
            ctx.set_params(prm)
            ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, query_capacity=W * H, seed=2)
            for k in range(4):
                if mode == "frame":
                    ctx.nrc_frame(seed=4, pass_index=k)
                else:
                    ctx.pt_pass(seed=4, pass_index=k)
                    ctx.nrc_train_step(seed=4, pass_index=k)
            ctx.synchronize()
            res.append((ctx.image_sum(), ctx.nrc_get_weights(), ctx.nrc_info()))
    (ia, wa, na), (ib, wb, nb) = res
    assert na["steps"] == nb["steps"] == 4 and na["train_records"] == nb["train_records"]
    np.testing.assert_allclose(wb, wa, rtol=0, atol=1e-5)
    np.testing.assert_allclose(ib, ia, rtol=1e-4, atol=1e-7)


@pytest.mark.parametrize("kernel", [vcr.NRC_QUERY_MMA, vcr.NRC_QUERY_TCGEN05])
def test_cached_passes_in_one_launch_equal_single_passes(cuda, kernel):
    """vcr_pt_passes with paths ending in the cache: the count passes' queries
    are answered after the launch with the same weights, so the sums equal
    count single cached passes up to the order of the FP64 additions; a
    query buffer too small for all of them is refused."""
    sc = configs.C1_PT
    W = H = 96
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = 2
    res = []
    for mode in ("single", "launch"):
        with vcr.Context() as ctx:
            configs.setup_context(ctx, sc, width=W, height=H)
            ctx.set_params(prm)
            ctx.nrc_setup(train_samples=8192, query_capacity=3 * W * H, seed=2, query_kernel=kernel)
            for k in range(2):  # train a little so that the cache term is not the initial network's
                ctx.nrc_train_step(seed=4, pass_index=k)
            if mode == "launch":
                ctx.pt_passes(seed=6, first=1, count=3)
            else:
                for k in range(1, 4):
                    ctx.pt_pass(seed=6, pass_index=k)
            ctx.synchronize()
            res.append((ctx.image_sum(), ctx.counters()))
            if mode == "launch":
                ctx.nrc_setup(train_samples=8192, query_capacity=2 * W * H, seed=2, query_kernel=kernel)
                with pytest.raises(vcr.VcrError, match="CAPACITY"):
                    ctx.pt_passes(seed=6, first=1, count=3)
    (ia, ca), (ib, cb) = res
    np.testing.assert_allclose(ib, ia, rtol=1e-12, atol=0)
    assert ia.sum() > 0


def _image_mean(ctx, passes, seed):
    ctx.reset()
    for k in range(passes):
        ctx.pt_pass(seed=seed, pass_index=k)
    ctx.synchronize()
    return float(ctx.image_mean().mean())


def test_online_training_makes_the_cached_render_consistent(cuda):
    """Paths cut at the second event lose the energy of the rest of the
    path; after online training the cache must give most of it back, so the
    cached render approaches the unbiased render's mean."""
    sc = configs.C1_PT
    W = H = 64
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=W, height=H)
        prm = sc.params(vcr.TRACKER_DDA)
        full = _image_mean(ctx, 64, seed=21)
        prm.nrc_events = 2
        ctx.set_params(prm)
        ctx.nrc_setup(train_samples=16384, learning_rate=2e-3, query_capacity=W * H, seed=3)
        ctx.nrc_set_weights(np.zeros(ctx.NRC_WEIGHTS, np.float32))
        cut = _image_mean(ctx, 64, seed=22)
        ctx.nrc_setup(train_samples=16384, learning_rate=2e-3, query_capacity=W * H, seed=3)
        for k in range(300):
            ctx.nrc_train_step(seed=5, pass_index=k)
        info = ctx.nrc_info()
        cached = _image_mean(ctx, 64, seed=23)
    assert info["steps"] == 300 and info["train_records"] > 4000 and np.isfinite(info["last_loss"])
    assert full - cut > 0.05 * full, (full, cut)
    assert abs(cached - full) < 0.35 * (full - cut), (full, cut, cached)


def test_paths_ending_in_the_cache_match_the_oracle(cuda):
    """nrc_events = 2 with an all-zero network: the image is exactly the
    oracle's truncated paths; with trained weights the cache adds a
    non-negative term only where paths reached the second event."""
    sc = configs.C1_PT
    dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves)
    og = orc.Grid(dense, 0)
    W = H = 96
    crop = (0, 0, W, H)
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = 2
    cloud = sc.cloud()
    cloud.max_extinction = max(og.max_density(), 0.01)
    with vcr.Context() as ctx:
        ctx.grid_upload(sc.grid_desc(), dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(sc.camera(W, H))
        ctx.set_params(prm)
        ctx.set_frame(W, H)
        ctx.nrc_setup(train_samples=8192, query_capacity=W * H, seed=1)
        ctx.nrc_set_weights(np.zeros(ctx.NRC_WEIGHTS, np.float32))
        ctx.pt_pass(seed=4, pass_index=0, flags=vcr.PASS_RECORD_STATS)
        ctx.synchronize()
        g0, st = ctx.image_sum(), ctx.path_stats()
        o0, ost = og.pt_pass(cloud, sc.camera(W, H), prm, W, H, seed=4, pass_index=0, flags=vcr.PASS_RECORD_STATS)
        np.testing.assert_array_equal(st[..., :2], ost[..., :2])
        np.testing.assert_array_equal(g0, o0)
        assert ctx.nrc_info()["queries"] == int((st[..., 0] >= 2).sum())
        # an all-zero ReLU network has zero gradient: start training from a fresh init
        ctx.nrc_setup(train_samples=8192, query_capacity=W * H, seed=1)
        for k in range(20):
            ctx.nrc_train_step(seed=9, pass_index=k)
        ctx.reset()
        ctx.pt_pass(seed=4, pass_index=0)
        ctx.synchronize()
        g1 = ctx.image_sum()
    ended = st[..., 0] >= 2
    assert np.all(g1 >= g0 - 1e-7)
    np.testing.assert_array_equal(g1[~ended], g0[~ended])
    assert (g1[ended] > g0[ended]).mean() > 0.5
