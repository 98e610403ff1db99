"""The oracle's DDA walk over a majorant pyramid level against geometry (CPU).

The GPU walk equals this one bit for bit (test_gpu_pt.py), so here the
oracle's cell sequence is checked against the ray itself, for every level:
its intervals tile the ray from the box entry to the exit, consecutive
cells are face neighbours stepping the way the ray points, each interval's
midpoint lies in its cell, and every cell that points sampled densely
along the ray fall in (away from cell faces) is in the sequence."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc

SIZE = (48, 40, 36)  # not multiples of the 8-voxel bricks


@pytest.fixture(scope="module")
def scene():
    dense = orc.fbm_fill(SIZE, seed=3, octaves=3)
    g = orc.Grid(dense, 0)
    desc = vcr.grid_desc(SIZE, (1 / 48,) * 3)
    cloud = vcr.cloud_from_grid(desc, 1.0, 8.0)
    return g, cloud


def _rays(rng, n):
    o = rng.uniform(-1.2, 1.2, (n, 3)).astype(np.float32)
    o[: n // 2] = rng.uniform([-0.5, -0.4, 0.0], [0.5, 0.4, 0.75], (n // 2, 3))  # inside
    d = rng.normal(size=(n, 3))
    d[:60, 1:] = 0.0  # along x
    d[60:120, 2] = 0.0  # in the xy plane
    d[120:150, :2] = 0.0  # along z
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return o, d


def _slab64(o, d, b0, b1):
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        a, b = (b0 - o) * inv, (b1 - o) * inv
    a = np.where(np.isnan(a), -np.inf, a)
    b = np.where(np.isnan(b), np.inf, b)
    return np.max(np.minimum(a, b)), np.min(np.maximum(a, b))


@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_dda_walk_follows_the_ray(scene, level):
    g, cloud = scene
    rng = np.random.default_rng(10 + level)
    n, mc = 3000, 256
    o, d = _rays(rng, n)
    cells, tt, cnt = g.dda_trace(cloud, o, d, mc, level)
    nx, ny, nz = g.level_dims(level)
    b0 = np.array(cloud.bounds_min, np.float64)
    b1 = np.array(cloud.bounds_max, np.float64)
    cs = (b1 - b0) / np.array(SIZE, np.float64) * (8 << level)
    walked = 0
    for i in range(n):
        k = int(cnt[i])
        oi, di = o[i].astype(np.float64), d[i].astype(np.float64)
        tmin, tmax = _slab64(oi, di, b0, b1)
        if not (tmax >= max(tmin, 0.0)) or tmax < 0:
            assert k == 0
            continue
        if tmax - max(tmin, 0.0) < 1e-6:
            continue  # grazing a face or an edge
        assert 0 < k < mc
        walked += 1
        c = cells[i, :k].astype(np.int64)
        cx, cy, cz = c % nx, (c // nx) % ny, c // (nx * ny)
        assert np.all((cx < nx) & (cy < ny) & (cz < nz))
        t = tt[i, :k].astype(np.float64)
        ext = tmax - max(tmin, 0.0)
        # the intervals tile [0, exit] (distances from the box entry)
        assert t[0, 0] == 0.0
        np.testing.assert_array_equal(t[1:, 0], t[:-1, 1])
        assert np.all(t[:, 1] >= t[:, 0])
        assert abs(t[-1, 1] - ext) <= 1e-5 * max(1.0, ext)
        # face neighbours, stepping along the ray's direction
        step = np.stack([np.diff(cx), np.diff(cy), np.diff(cz)], axis=1)
        assert np.all(np.abs(step).sum(axis=1) == 1)
        for a in range(3):
            moved = step[:, a] != 0
            assert np.all(np.sign(step[moved, a]) == np.sign(di[a]))
        # each interval's midpoint lies in its cell (away from cell faces)
        entry = oi + di * max(tmin, 0.0)
        tm = 0.5 * (t[:, 0] + t[:, 1])
        u = (entry + tm[:, None] * di - b0) / cs
        clear = np.all(np.abs(u - np.round(u)) > 1e-4, axis=1) & (t[:, 1] - t[:, 0] > 1e-4 * cs.min())
        own = np.floor(u).astype(np.int64)
        np.testing.assert_array_equal(own[clear], np.stack([cx, cy, cz], axis=1)[clear])
        # points sampled along the ray fall only in walked cells
        ts = np.linspace(0.0, ext, 1024)[1:-1]
        us = (entry + ts[:, None] * di - b0) / cs
        keep = np.all(np.abs(us - np.round(us)) > 1e-4, axis=1)
        si = np.floor(us[keep]).astype(np.int64)
        lin = si[:, 0] + nx * (si[:, 1] + ny * si[:, 2])
        assert np.isin(lin, c).all()
    assert walked > n // 3
