"""Failure detection on the GPU without a fault: every device-side wait
has a limit, and a wait that runs out is reported as VCR_ERR_TIMEOUT while
the context stays usable.  The tests make the waits run out by setting
their limits to zero polls (vcr_set_wait_limits), then restore the
defaults and check that the next call works and is correct.

The waits replaced: the reference blocks on its frame fence without a limit
(vkWaitForFences with UINT64_MAX, main.cpp:606).  Nothing here hangs or
faults a GPU: a look-back that gives up leaves a wrong order inside the
output buffers (every store is bounds-checked), and a staging copy whose
wait ran out is still waited for before its CTA goes on reading the
majorants from global memory."""
import numpy as np
import pytest

import vcr
from vcr import configs

pytestmark = pytest.mark.gpu


@pytest.fixture
def zero_limits():
    yield vcr.set_wait_limits
    vcr.set_wait_limits()  # defaults, whatever the test did


def _sort_case(torch, cuda, n, seed):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    dk = torch.from_numpy(keys.view(np.int32)).to(cuda)
    ko = torch.empty(n, dtype=torch.int32, device=cuda)
    vo = torch.empty(n, dtype=torch.int32, device=cuda)
    return keys, dk, ko, vo


def test_sort_lookback_timeout_is_reported_then_the_next_sort_is_exact(cuda, zero_limits):
    import torch

    n = 1 << 22  # 2,048 tiles a pass: tiles whose predecessor has not published yet are certain
    keys, dk, ko, vo = _sort_case(torch, cuda, n, 5)
    with vcr.Context() as ctx:
        zero_limits(sort_lookback=0)
        assert vcr.wait_limits()["sort_lookback"] == 0
        statuses = []
        for _ in range(3):
            ctx.radix_sort_pairs(dk.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), n)
            try:
                ctx.synchronize()
                statuses.append(vcr.OK)
            except vcr.VcrError as e:
                statuses.append(e.status)
                assert "bounded wait ran out" in str(e)
            if vcr.ERR_TIMEOUT in statuses:
                break
        assert vcr.ERR_TIMEOUT in statuses, statuses
        ctx.synchronize()  # the error word was cleared by the report
        vcr.set_wait_limits()
        ctx.radix_sort_pairs(dk.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), n)
        ctx.synchronize()
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(vo.cpu().numpy().view(np.uint32), perm)
    np.testing.assert_array_equal(ko.cpu().numpy().view(np.uint32), keys[perm])


def test_staging_wait_timeout_is_reported_and_the_pass_is_unchanged(cuda, zero_limits):
    sc = configs.C1_PT
    W = H = 96
    images = []
    for polls in (None, 0):
        with vcr.Context() as ctx:
            configs.setup_context(ctx, sc, width=W, height=H)
            ctx.set_tuning(majorant_level=1, dda_steps=4, stage_majorants=1, block_threads=256)
            if polls is not None:
                zero_limits(stage_wait=polls)
            ctx.pt_pass(seed=3, pass_index=0)
            if polls is None:
                ctx.synchronize()
            else:
                with pytest.raises(vcr.VcrError) as e:
                    ctx.synchronize()
                assert e.value.status == vcr.ERR_TIMEOUT
                vcr.set_wait_limits()
                ctx.synchronize()  # cleared; the context still works
            images.append(ctx.image_sum())
            ctx.pt_pass(seed=3, pass_index=1)
            ctx.synchronize()
    # the CTAs whose staging wait ran out read the same majorants from global memory
    np.testing.assert_array_equal(images[0], images[1])
