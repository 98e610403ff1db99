"""CPU tests of the photon-beam oracle: LBVH structure (each internal node
covers a contiguous leaf range, split where the keys' common prefix ends),
refit boxes contain their children, radius schedule, beam pass sanity."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc
from vcr import configs


def _ranges(left, right, n):
    """Leaf range [lo, hi] of every internal node."""
    out = {}

    def walk(node):
        lo, hi = [], []
        for c in (left[node], right[node]):
            if c & 0x80000000:
                lo.append(c & 0x7FFFFFFF)
                hi.append(c & 0x7FFFFFFF)
            else:
                a, b = walk(c)
                lo.append(a)
                hi.append(b)
        out[node] = (min(lo), max(hi))
        assert hi[0] + 1 == lo[1], "children must be adjacent ranges"
        return out[node]

    walk(0)
    return out


@pytest.mark.parametrize("n,dups", [(2, False), (9, False), (300, False), (300, True), (4097, True)])
def test_lbvh_structure(n, dups):
    rng = np.random.default_rng(n)
    codes = rng.integers(0, 1 << 30, n).astype(np.uint32)
    if dups:
        codes = (codes >> 26) << 26
    order = np.argsort(codes, kind="stable").astype(np.uint32)
    sc = codes[order]
    a = np.zeros((n, 4), np.float32)
    a[:, :3] = rng.random((n, 3))
    a[:, 3] = 0.01
    b = a.copy()
    b[:, :3] += 0.02
    t = orc.lbvh(sc, order, a, b)
    rg = _ranges(t["left"], t["right"], n)
    assert rg[0] == (0, n - 1) and len(rg) == n - 1
    # boxes contain children
    for node, (lo_i, hi_i) in rg.items():
        for c in (t["left"][node], t["right"][node]):
            clo = t["leaf_lo"][c & 0x7FFFFFFF] if c & 0x80000000 else t["node_lo"][c]
            chi = t["leaf_hi"][c & 0x7FFFFFFF] if c & 0x80000000 else t["node_hi"][c]
            assert np.all(t["node_lo"][node][:3] <= clo[:3]) and np.all(t["node_hi"][node][:3] >= chi[:3])
    # leaf boxes contain both end caps of their cylinder
    for i in range(n):
        s = order[i]
        assert np.all(t["leaf_lo"][i][:3] <= np.minimum(a[s, :3], b[s, :3]))
        assert np.all(t["leaf_hi"][i][:3] >= np.maximum(a[s, :3], b[s, :3]))


def test_radius_schedule_is_the_intended_product():
    r0, alpha = 0.05, 0.8
    r = [orc.ppb_radius(r0, alpha, k) for k in range(6)]
    expect = [r0]
    for i in range(1, 6):
        expect.append(expect[-1] * (i + alpha) / (i + 1))
    np.testing.assert_allclose(r, expect, rtol=1e-6)
    assert all(r[i + 1] < r[i] for i in range(5))


def test_oracle_beam_pass_is_deterministic_and_conserves_segments():
    size = (32, 32, 32)
    g = orc.Grid(orc.fbm_fill(size, seed=4, octaves=4), 0)
    desc = vcr.grid_desc(size, (1 / 32,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 12.0)
    cloud.max_extinction = max(g.max_density(), 0.01)
    sc = configs.C3_PPB
    cam, prm = sc.camera(24, 24), sc.params(vcr.TRACKER_DDA)
    s1, b1 = orc.ppb_pass(g, cloud, cam, prm, 300, 1 << 16, 0.05, 0.8, 24, 24, seed=5)
    s2, b2 = orc.ppb_pass(g, cloud, cam, prm, 300, 1 << 16, 0.05, 0.8, 24, 24, seed=5)
    assert s1.tobytes() == s2.tobytes()
    n = b1["info"]["segments"]
    # per-beam segments tile the beam length
    lens = b1["slots"][:, 6]
    segl = np.linalg.norm(b1["seg_b"][:, :3] - b1["seg_a"][:, :3], axis=1)
    tot = np.zeros(len(lens))
    np.add.at(tot, b1["seg_beam"], segl)
    used = np.unique(b1["seg_beam"])
    np.testing.assert_allclose(tot[used], lens[used], rtol=1e-4)
    assert n == len(b1["codes"]) and np.all(np.diff(b1["codes"][b1["order"]].astype(np.int64)) >= 0)


def test_empty_cloud_gathers_the_whole_sky():
    """Every free flight in an all-zero cloud escapes the box, so the camera
    transmittance estimate is 1 at every pixel, grazing rays included: an
    escaped flight counts as farther than the ray's box exit, however the
    exit distances computed from the camera and from the entry point round."""
    size = (16, 16, 16)
    og = orc.Grid(np.zeros(size, np.float32), 0)
    desc = vcr.grid_desc(size, (1.0 / 16,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 16.0)
    cloud.max_extinction = 0.01
    sc = configs.C1_PT
    W, H = 20, 12
    s, b = orc.ppb_pass(og, cloud, sc.camera(W, H), sc.params(vcr.TRACKER_DDA), 512, 4096, 0.05, 0.8, W, H,
                        seed=2, pass_index=0)
    np.testing.assert_array_equal(s, np.float64(np.float32(0.1)))
    # escaped transmittance samples sit beyond every beam point
    used = b["slots"][np.unique(b["seg_beam"])]
    assert len(used) and (used[:, 10:26] > 1e38).all()
