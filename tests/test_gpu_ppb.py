"""GPU tests of progressive photon beams through the C-ABI, against the
oracle: LBVH topology and boxes bit-exact (including runs of equal Morton
codes), and a whole beam pass — photon emission, beam slots, segments and
keys, sort order, BVH, per-pixel gather — bit for bit."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a).to(cuda)


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 65537])
@pytest.mark.parametrize("dups", [False, True])
def test_lbvh_topology_and_boxes_bit_exact(cuda, n, dups):
    import torch
    rng = np.random.default_rng(n + 7 * dups)
    codes = rng.integers(0, 1 << 30, n).astype(np.uint32)
    if dups:
        codes = (codes >> 24) << 24  # long runs of equal keys
    order = np.argsort(codes, kind="stable").astype(np.uint32)
    sorted_codes = codes[order]
    a = np.zeros((n, 4), np.float32)
    a[:, :3] = rng.random((n, 3), dtype=np.float32)
    a[:, 3] = 0.01 + 0.02 * rng.random(n, dtype=np.float32)
    b = np.zeros((n, 4), np.float32)
    b[:, :3] = a[:, :3] + 0.05 * (rng.random((n, 3), dtype=np.float32) - 0.5)
    b[:5, :3] = a[:5, :3]  # zero-length segments
    ref = orc.lbvh(sorted_codes, order, a, b)
    m = max(n - 1, 1)
    out = {k: torch.zeros(s, dtype=t, device=cuda) for k, s, t in
           [("left", m, torch.int32), ("right", m, torch.int32), ("node_lo", (m, 4), torch.float32),
            ("node_hi", (m, 4), torch.float32), ("leaf_lo", (n, 4), torch.float32), ("leaf_hi", (n, 4), torch.float32)]}
    with vcr.Context() as ctx:
        dc, do, da, db = _dev(sorted_codes, cuda), _dev(order, cuda), _dev(a, cuda), _dev(b, cuda)
        ctx.lbvh_build(dc.data_ptr(), do.data_ptr(), da.data_ptr(), db.data_ptr(), n, out["left"].data_ptr(),
                       out["right"].data_ptr(), out["node_lo"].data_ptr(), out["node_hi"].data_ptr(),
                       out["leaf_lo"].data_ptr(), out["leaf_hi"].data_ptr())
        ctx.synchronize()
    k = n - 1
    np.testing.assert_array_equal(_u32(out["left"])[:k], ref["left"])
    np.testing.assert_array_equal(_u32(out["right"])[:k], ref["right"])
    np.testing.assert_array_equal(out["leaf_lo"].cpu().numpy(), ref["leaf_lo"])
    np.testing.assert_array_equal(out["leaf_hi"].cpu().numpy(), ref["leaf_hi"])
    np.testing.assert_array_equal(out["node_lo"].cpu().numpy()[:k], ref["node_lo"])
    np.testing.assert_array_equal(out["node_hi"].cpu().numpy()[:k], ref["node_hi"])
    if n > 1:  # every leaf is referenced exactly once
        kids = np.concatenate([ref["left"], ref["right"]])
        leaves = np.sort(kids[kids >= 0x80000000] & 0x7FFFFFFF)
        np.testing.assert_array_equal(leaves, np.arange(n))


def _scene(level=2):
    size = (48, 40, 48)
    dense = orc.fbm_fill(size, seed=2, octaves=5)
    g = orc.Grid(dense, 0)
    desc = vcr.grid_desc(size, (1 / 48,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 16.0)
    cloud.max_extinction = max(g.max_density(), 0.01)
    sc = configs.C3_PPB
    return dense, g, desc, cloud, sc


@pytest.mark.parametrize("pass_index,cap", [(0, 1 << 16), (3, 1 << 16), (1, 5000)])
def test_ppb_pass_bit_exact(cuda, pass_index, cap):
    dense, g, desc, cloud, sc = _scene()
    W, H = 64, 48
    cam = sc.camera(W, H)
    prm = sc.params(vcr.TRACKER_DDA)
    photons, r0, alpha = 700, 0.04, 0.8
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(cam)
        ctx.set_params(prm)
        ctx.set_frame(W, H)
        ctx.ppb_setup(photons, cap, r0, alpha)
        ctx.ppb_pass(seed=11, pass_index=pass_index)
        ctx.synchronize()
        info = ctx.ppb_info()
        gb = {k: ctx.ppb_read(k, photons) for k in _abi_buffers()}
        g_sum = ctx.image_sum()
        evaluated, ms = ctx.gather_stats("ppb")
    assert evaluated > 0 and ms > 0.0
    o_sum, ob = orc.ppb_pass(g, cloud, cam, prm, photons, cap, r0, alpha, W, H, seed=11, pass_index=pass_index)
    assert info["segments"] == ob["info"]["segments"] and info["dropped"] == ob["info"]["dropped"]
    assert info["radius"] == np.float32(orc.ppb_radius(r0, alpha, pass_index))
    if cap == 5000:
        assert info["dropped"] > 0
    np.testing.assert_array_equal(gb["nbeams"], ob["nbeams"])
    np.testing.assert_array_equal(gb["slots"], ob["slots"])
    for k in ("seg_a", "seg_b", "seg_beam", "codes", "order", "left", "right", "node_lo", "node_hi", "leaf_lo",
              "leaf_hi"):
        np.testing.assert_array_equal(gb[k], ob[k], err_msg=k)
    rel = np.abs(g_sum - o_sum) / np.maximum(np.abs(o_sum), 1e-30)
    assert rel.max() <= 1e-5, rel.max()
    assert o_sum.max() > 0.2  # beams contribute
    assert np.isfinite(g_sum).all()


def _abi_buffers():
    from vcr import _abi
    return list(_abi.PPB_BUFFERS)


def test_ppb_progressive_accumulation(cuda):
    dense, g, desc, cloud, sc = _scene()
    W, H = 32, 32
    with vcr.Context() as ctx:
        ctx.grid_upload(desc, dense)
        ctx.set_cloud(cloud)
        ctx.set_camera(sc.camera(W, H))
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_frame(W, H)
        ctx.ppb_setup(500, 1 << 15, 0.05, 0.7)
        radii = []
        for k in range(4):
            ctx.ppb_pass(seed=1, pass_index=k)
            radii.append(ctx.ppb_info()["radius"])
        ctx.synchronize()
        assert ctx.pass_count() == 4
        assert all(radii[i + 1] < radii[i] for i in range(3))
        m = ctx.image_mean()
        assert np.isfinite(m).all() and m.mean() > 0
        ctx.ppb_free()
        with pytest.raises(vcr.VcrError):
            ctx.ppb_pass(seed=1, pass_index=5)
