"""Display image through the C-ABI: bytes equal the oracle's, for both pixel
orders and an exposure, into host and device memory, and while passes are
queued on a stream."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs

pytestmark = pytest.mark.gpu


def _render(ctx, W, H, passes, spp=1):
    sc = configs.C1_PT
    configs.setup_context(ctx, sc, width=W, height=H)
    ctx.set_tuning(majorant_level=2, dda_steps=8, stage_majorants=1, block_threads=256)
    for k in range(passes):
        ctx.pt_pass(seed=3, pass_index=k, spp=spp)
    ctx.synchronize()


@pytest.mark.parametrize("exposure,order", [(1.0, vcr.ORDER_RGBA), (2.5, vcr.ORDER_BGRA), (0.0, vcr.ORDER_RGBA)])
def test_display_matches_the_oracle(cuda, exposure, order):
    with vcr.Context() as ctx:
        _render(ctx, 96, 64, passes=3, spp=2)
        got = ctx.display(exposure, order)
        want = orc.display(ctx.image_sum(), 6, exposure, order)
    np.testing.assert_array_equal(got, want)
    assert (got[..., 3] == 255).all()
    if exposure == 1.0:
        assert got[..., :3].max() > 100  # the cloud is lit


def test_display_into_device_memory_in_stream_order(cuda):
    import torch
    W, H = 80, 48
    with vcr.Context() as ctx:
        _render(ctx, W, H, passes=1)
        stream = torch.cuda.Stream()
        for k in range(1, 4):  # queued behind the passes on the same stream
            ctx.pt_pass(seed=3, pass_index=k, stream=stream.cuda_stream)
        out = torch.zeros(H * W * 4, dtype=torch.uint8, device=cuda)
        ctx.display_to(out.data_ptr(), 1.0, vcr.ORDER_RGBA, stream=stream.cuda_stream)
        stream.synchronize()
        got = out.cpu().numpy().reshape(H, W, 4)
        want = orc.display(ctx.image_sum(), 4)
    np.testing.assert_array_equal(got, want)


def test_display_rejects_bad_arguments(cuda):
    with vcr.Context() as ctx:
        with pytest.raises(vcr.VcrError):
            ctx.display()  # no frame yet
        _render(ctx, 16, 16, passes=1)
        with pytest.raises(vcr.VcrError):
            ctx.display(exposure=-1.0)
        with pytest.raises(vcr.VcrError):
            ctx.display(order=7)
