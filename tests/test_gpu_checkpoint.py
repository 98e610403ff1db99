"""Checkpoint / resume through the C-ABI: an interrupted render resumed
from its checkpoint in a fresh context continues exactly as the
uninterrupted one (PT sums, PPM statistics, the radiance cache's training,
a batch), and a checkpoint is refused by a context set up differently."""
import numpy as np
import pytest

import vcr
from vcr import configs

pytestmark = pytest.mark.gpu

W, H = 80, 64


def _scene(ctx, nrc=False):
    sc = configs.C1_PT
    configs.setup_context(ctx, sc, width=W, height=H)
    if nrc:
        prm = sc.params(vcr.TRACKER_DDA)
        prm.nrc_events = 2
        ctx.set_params(prm)
    return sc


def test_pt_resume_equals_uninterrupted(cuda, tmp_path):
    path = str(tmp_path / "pt.ckpt")
    with vcr.Context() as ctx:
        _scene(ctx)
        for k in range(5):
            ctx.pt_pass(seed=2, pass_index=k)
            if k == 2:
                ctx.checkpoint_save(path)
        ctx.synchronize()
        full = ctx.image_sum()
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.checkpoint_load(path)
        assert ctx.pass_count() == 3
        for k in range(3, 5):
            ctx.pt_pass(seed=2, pass_index=k)
        ctx.synchronize()
        resumed = ctx.image_sum()
        assert ctx.pass_count() == 5
    np.testing.assert_array_equal(resumed, full)


def test_ppm_statistics_resume(cuda, tmp_path):
    path = str(tmp_path / "ppm.ckpt")
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.ppm_setup(photons=1 << 14, capacity=1 << 16, radius=0.02, alpha=0.7)
        for k in range(4):
            ctx.ppm_pass(seed=3, pass_index=k)
            if k == 1:
                ctx.checkpoint_save(path)
        ctx.synchronize()
        full = ctx.ppm_read("stats")
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.ppm_setup(photons=1 << 14, capacity=1 << 16, radius=0.02, alpha=0.7)
        ctx.checkpoint_load(path)
        for k in range(2, 4):
            ctx.ppm_pass(seed=3, pass_index=k)
        ctx.synchronize()
        resumed = ctx.ppm_read("stats")
    # photon gathers add in an order set by atomics: equal to rounding
    np.testing.assert_allclose(resumed, full, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("encoding", [vcr.NRC_ENCODING_FREQUENCY, vcr.NRC_ENCODING_GRID])
def test_radiance_cache_training_resumes(cuda, tmp_path, encoding):
    """The cache's weights, Adam state and moving average (and, with the
    grid encoding, its tables' values, moments and average) survive a
    checkpoint; a cache with the other encoding refuses it."""
    path = str(tmp_path / "nrc.ckpt")
    grid = encoding == vcr.NRC_ENCODING_GRID
    with vcr.Context() as ctx:
        _scene(ctx, nrc=True)
        ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, query_capacity=W * H, seed=4, ema_decay=0.9,
                      encoding=encoding)
        for k in range(6):
            ctx.nrc_frame(seed=5, pass_index=k)
            if k == 3:
                ctx.checkpoint_save(path)
        ctx.synchronize()
        w_full, info_full = ctx.nrc_get_weights(tables=grid), ctx.nrc_info()
    with vcr.Context() as ctx:
        _scene(ctx, nrc=True)
        ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, query_capacity=W * H, seed=99, ema_decay=0.9,
                      encoding=encoding)
        ctx.checkpoint_load(path)
        for k in range(4, 6):
            ctx.nrc_frame(seed=5, pass_index=k)
        ctx.synchronize()
        w_res, info_res = ctx.nrc_get_weights(tables=grid), ctx.nrc_info()
        other = vcr.NRC_ENCODING_FREQUENCY if grid else vcr.NRC_ENCODING_GRID
        ctx.nrc_setup(train_samples=8192, learning_rate=3e-3, query_capacity=W * H, seed=99, ema_decay=0.9,
                      encoding=other)
        with pytest.raises(vcr.VcrError, match="STATE"):
            ctx.checkpoint_load(path)
    assert info_res["steps"] == info_full["steps"] == 6
    assert info_res["train_records"] == info_full["train_records"]
    assert info_res["weights"] == w_res.size
    # gradients are flushed with float atomics: the same up to their order
    np.testing.assert_allclose(w_res, w_full, rtol=0, atol=2e-5)


def test_batch_resume_and_refusals(cuda, tmp_path):
    path = str(tmp_path / "batch.ckpt")
    sc = configs.C1_PT
    views = [(sc.camera(48, 40), 48, 40, configs.sun_travel_dir(20.0)),
             (sc.camera(32, 32), 32, 32, configs.sun_travel_dir(60.0))]
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.batch_setup(views)
        for k in range(4):
            ctx.batch_pass(seed=6, pass_index=k)
            if k == 1:
                ctx.checkpoint_save(path)
        ctx.synchronize()
        full = [ctx.batch_read(v) for v in range(2)]
    with vcr.Context() as ctx:
        _scene(ctx)
        with pytest.raises(vcr.VcrError):  # no batch set up: refused, nothing changed
            ctx.checkpoint_load(path)
        ctx.batch_setup(views)
        ctx.checkpoint_load(path)
        assert ctx.batch_info()["passes"] == 2
        for k in range(2, 4):
            ctx.batch_pass(seed=6, pass_index=k)
        ctx.synchronize()
        resumed = [ctx.batch_read(v) for v in range(2)]
    for a, b in zip(full, resumed):
        np.testing.assert_array_equal(a, b)
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, width=W + 8, height=H)
        ctx.batch_setup(views)
        with pytest.raises(vcr.VcrError):  # frame size differs
            ctx.checkpoint_load(path)
        with pytest.raises(vcr.VcrError):
            ctx.checkpoint_load(str(tmp_path / "missing.ckpt"))


def test_checkpoint_of_another_scene_is_refused(cuda, tmp_path):
    """The scene hash: a checkpoint loads only into a context bound to the
    grid, cloud, camera and parameters it was rendered from."""
    path = str(tmp_path / "scene.ckpt")
    sc = configs.C1_PT
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.pt_pass(seed=2, pass_index=0)
        ctx.checkpoint_save(path)
    with vcr.Context() as ctx:  # other phase g
        _scene(ctx)
        prm = sc.params(vcr.TRACKER_DDA)
        vcr.params_set_phase_g(prm, 0.5)
        ctx.set_params(prm)
        with pytest.raises(vcr.VcrError, match="another scene"):
            ctx.checkpoint_load(path)
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.checkpoint_load(path)  # the same scene again: accepted
        assert ctx.pass_count() == 1
    with vcr.Context() as ctx:  # other grid seed, same sizes
        ctx.grid_generate(sc.grid_desc(), vcr.fbm_desc(seed=2, octaves=sc.octaves), sc.precision)
        ctx.set_cloud(sc.cloud())
        ctx.set_camera(sc.camera(W, H))
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_frame(W, H)
        with pytest.raises(vcr.VcrError, match="another scene"):
            ctx.checkpoint_load(path)
    with vcr.Context() as ctx:  # other camera
        _scene(ctx)
        ctx.set_camera(vcr.camera_look((0.0, 0.1, -0.4), (0.0, 0.0, 1.0), 90.0, 0.1, W, H))
        with pytest.raises(vcr.VcrError, match="another scene"):
            ctx.checkpoint_load(path)


def test_truncated_and_corrupt_checkpoints_are_io_errors(cuda, tmp_path):
    path = str(tmp_path / "full.ckpt")
    with vcr.Context() as ctx:
        _scene(ctx)
        ctx.pt_pass(seed=2, pass_index=0)
        ctx.checkpoint_save(path)
        data = open(path, "rb").read()
        cut = tmp_path / "cut.ckpt"
        cut.write_bytes(data[: len(data) // 2])
        with pytest.raises(vcr.VcrError) as e:
            ctx.checkpoint_load(str(cut))
        assert e.value.status == vcr.ERR_IO
        # a section length far beyond the file (first section's u64 at byte 24)
        bad = bytearray(data)
        bad[24:32] = (1 << 39).to_bytes(8, "little")
        (tmp_path / "bad.ckpt").write_bytes(bytes(bad))
        with pytest.raises(vcr.VcrError) as e:
            ctx.checkpoint_load(str(tmp_path / "bad.ckpt"))
        assert e.value.status == vcr.ERR_IO
        ctx.checkpoint_load(path)  # the intact file still loads
