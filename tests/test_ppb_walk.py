"""The photon-beam gather's tree walk against brute force (CPU).

The oracle's walk (beam_walk, the one its gather uses and the GPU gather
matches bit for bit) over an LBVH of random beam segments: for every ray it
visits exactly the leaves whose boxes the ray's [t0, t1] crosses (the slab
test restated in float32 here), in tree order, and every segment the
estimator accepts for that ray (the closest approach inside the segment's
cylinder, PPB_PE.comp:362-404) is among them."""
import numpy as np
import pytest

from oracle import oracle as orc

B0 = np.array([-0.5, -0.25, 0.0], np.float32)
B1 = np.array([0.5, 0.25, 1.0], np.float32)


def _segments(rng, n, radius):
    a = rng.uniform(B0, B1, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[: n // 20] = np.eye(3)[rng.integers(0, 3, n // 20)]  # some along the axes
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    length = rng.uniform(0.0, 0.05, n)
    length[:5] = 0.0  # degenerate segments
    b = (a + d * length[:, None]).astype(np.float32)
    seg_a = np.concatenate([a, np.full((n, 1), radius, np.float32)], axis=1)
    seg_b = np.concatenate([b, np.zeros((n, 1), np.float32)], axis=1)
    return seg_a, seg_b


def _tree(seg_a, seg_b):
    mid = ((seg_a[:, :3] + seg_b[:, :3]) * np.float32(0.5)).astype(np.float32)
    codes = orc.morton(mid, B0, B1, 30)
    order = np.argsort(codes, kind="stable").astype(np.uint32)
    tree = orc.lbvh(codes[order], order, seg_a, seg_b)
    tree["order"] = order
    return tree


def _rays(rng, m):
    o = rng.uniform(B0, B1, (m, 3)).astype(np.float32)
    o[: m // 4] = rng.uniform(B0 - 0.3, B1 + 0.3, (m // 4, 3))  # some from outside the box
    d = rng.normal(size=(m, 3))
    d[:10] = np.eye(3)[np.arange(10) % 3] * np.where(np.arange(10) % 2, 1.0, -1.0)[:, None]  # axis-parallel
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t = np.stack([rng.uniform(0.0, 0.1, m), rng.uniform(1.0, 2.5, m)], axis=1).astype(np.float32)
    return o, d, t


def _ray_box(o, inv, t0, t1, lo, hi):
    """ray_box of the walk, in float32 (NaN-ignoring min / max as fmin / fmax)."""
    with np.errstate(invalid="ignore", over="ignore"):
        a = (lo[:, :3] - o) * inv
        b = (hi[:, :3] - o) * inv
    mn, mx = np.fmin(a, b), np.fmax(a, b)
    tn = np.fmax(np.fmax(mn[:, 0], mn[:, 1]), np.fmax(mn[:, 2], t0))
    tf = np.fmin(np.fmin(mx[:, 0], mx[:, 1]), np.fmin(mx[:, 2], t1))
    return tn <= tf


@pytest.mark.parametrize("n,radius", [(20000, 0.01), (3000, 0.05), (1, 0.02), (2, 0.02)])
def test_walk_visits_every_crossed_leaf_in_order(n, radius):
    rng = np.random.default_rng(n)
    seg_a, seg_b = _segments(rng, n, radius)
    tree = _tree(seg_a, seg_b)
    o, d, t = _rays(rng, 200)
    counts, hits = orc.ppb_walk(tree, o, d, t)
    assert counts.sum() == len(hits)
    start = 0
    accepted_total = 0
    for i in range(len(o)):
        got = hits[start:start + counts[i]]
        start += counts[i]
        assert np.all(got[1:] > got[:-1])  # depth first, left before right: leaves in tree order
        with np.errstate(divide="ignore"):
            inv = np.float32(1.0) / d[i]
        want = np.flatnonzero(_ray_box(o[i], inv, t[i, 0], t[i, 1], tree["leaf_lo"], tree["leaf_hi"]))
        np.testing.assert_array_equal(got, want)
        # the estimator's acceptance (float64, with margins) implies a visit
        pa, pb = seg_a[:, :3].astype(np.float64), seg_b[:, :3].astype(np.float64)
        ax = pb - pa
        segl = np.linalg.norm(ax, axis=1)
        ok = segl > 1e-6
        bd = np.where(ok[:, None], ax / np.maximum(segl, 1e-30)[:, None], 0.0)
        rd = d[i].astype(np.float64)
        bb = bd @ rd
        den = 1.0 - bb * bb
        w0 = o[i].astype(np.float64) - pa
        dw, ew = w0 @ rd, (bd * w0).sum(axis=1)
        with np.errstate(divide="ignore", invalid="ignore"):
            tt = (bb * ew - dw) / den
        sb = ew + tt * bb
        xc = o[i].astype(np.float64) + tt[:, None] * rd
        xb = pa + sb[:, None] * bd
        dist = np.linalg.norm(xc - xb, axis=1)
        m = 1e-4
        acc = ok & (den > 1e-3) & (tt > t[i, 0] + m) & (tt < t[i, 1] - m) & (sb > m) & (sb < segl - m) \
            & (dist < radius * (1.0 - 1e-3))
        sid = tree["order"][got]
        assert np.isin(np.flatnonzero(acc), sid).all()
        accepted_total += int(acc.sum())
    if n >= 3000:
        assert accepted_total > 100 and (counts > 0).mean() > 0.5  # the rays do meet beams


def test_leaf_boxes_hold_the_segment_cylinders():
    """Every point within the radius of a segment, with its foot on the
    segment (the estimator's region), lies in the segment's leaf box."""
    rng = np.random.default_rng(5)
    n, radius = 2000, 0.03
    seg_a, seg_b = _segments(rng, n, radius)
    tree = _tree(seg_a, seg_b)
    leaf_of = np.empty(n, np.int64)
    leaf_of[tree["order"]] = np.arange(n)
    lo, hi = tree["leaf_lo"][leaf_of, :3].astype(np.float64), tree["leaf_hi"][leaf_of, :3].astype(np.float64)
    pa, pb = seg_a[:, :3].astype(np.float64), seg_b[:, :3].astype(np.float64)
    ax = pb - pa
    segl = np.linalg.norm(ax, axis=1)
    keep = segl > 1e-6
    bd = ax[keep] / segl[keep, None]
    for _ in range(20):
        s = rng.uniform(0.0, 1.0, keep.sum())[:, None] * segl[keep, None]
        e = rng.normal(size=(keep.sum(), 3))
        e -= (e * bd).sum(axis=1, keepdims=True) * bd  # across the segment
        e /= np.linalg.norm(e, axis=1, keepdims=True)
        rho = rng.uniform(0.0, 1.0, keep.sum())[:, None] * radius
        p = pa[keep] + s * bd + rho * e
        tol = 1e-6
        assert np.all(p >= lo[keep] - tol) and np.all(p <= hi[keep] + tol)
