"""The photon map's radius query against a brute-force search (CPU).

The oracle's gather walk (the tree a pass builds: 30-bit Morton order,
radix tree, refit; the walk of samplePhotonMap, PPM_PE.comp:304-375) is what
the GPU gather matches bit for bit, so here it is checked against every
photon's distance: each query takes exactly the photons within its radius
(up to float rounding at the boundary), none twice, in Morton order."""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle import oracle_ppm as opm

B0 = (-0.5, -0.25, 0.0)
B1 = (0.5, 0.25, 1.0)


def _check(pos, queries, radii):
    counts, hits = opm.tree_query(pos, B0, B1, queries, radii)
    assert counts.sum() == len(hits)
    p64 = pos.astype(np.float64)
    codes = orc.morton(pos, B0, B1, 30) if len(pos) else np.zeros(0, np.uint32)
    start = 0
    for i, (q, r) in enumerate(zip(queries.astype(np.float64), radii.astype(np.float64))):
        got = hits[start:start + counts[i]]
        start += counts[i]
        assert len(np.unique(got)) == len(got)
        d2 = ((p64 - q) ** 2).sum(axis=1)
        r2 = r * r
        inside = np.flatnonzero(d2 < r2 * (1.0 - 1e-5) - 1e-12)
        maybe = np.flatnonzero(d2 <= r2 * (1.0 + 1e-5) + 1e-12)
        assert np.isin(inside, got).all(), (i, np.setdiff1d(inside, got)[:5])
        assert np.isin(got, maybe).all(), (i, np.setdiff1d(got, maybe)[:5])
        # the walk visits leaves left to right: ascending (Morton code, index)
        key = codes[got].astype(np.uint64) << np.uint64(32) | got.astype(np.uint64)
        assert np.all(key[1:] > key[:-1])
    return counts


def _queries(rng, m, scale):
    q = rng.uniform(B0, B1, (m, 3)).astype(np.float32)
    q[: m // 10] += rng.normal(0.0, 0.2, (m // 10, 3)).astype(np.float32)  # some outside the box
    r = (rng.uniform(0.0, 1.0, m) ** 2 * scale).astype(np.float32)
    r[0], r[1] = 0.0, 2.0  # an empty radius and one covering the box
    return q, r


def test_uniform_photons_match_brute_force():
    rng = np.random.default_rng(1)
    pos = rng.uniform(B0, B1, (20000, 3)).astype(np.float32)
    q, r = _queries(rng, 400, 0.12)
    counts = _check(pos, q, r)
    assert counts[1] == len(pos) and counts[0] <= 1 and counts.sum() > 20000


def test_clustered_and_duplicate_photons_match_brute_force():
    """Shared Morton codes (a cell holding thousands of photons, exact
    duplicates) give long runs of equal keys, split by index."""
    rng = np.random.default_rng(2)
    centre = np.array([0.1, 0.05, 0.6], np.float32)
    tight = centre + rng.normal(0.0, 2e-4, (30000, 3)).astype(np.float32)
    dup = np.repeat(np.array([[-0.3, 0.1, 0.2]], np.float32), 5000, axis=0)
    wide = rng.uniform(B0, B1, (5000, 3)).astype(np.float32)
    pos = np.concatenate([tight, dup, wide])
    q, r = _queries(rng, 200, 0.05)
    q[2:50] = centre + rng.normal(0.0, 5e-4, (48, 3)).astype(np.float32)
    r[2:50] = rng.uniform(1e-5, 1e-3, 48).astype(np.float32)
    q[50] = dup[0]
    r[50] = 1e-6
    counts = _check(pos, q, r)
    assert counts[50] == 5000


@pytest.mark.parametrize("n", [0, 1, 2, 3])
def test_tiny_photon_maps(n):
    rng = np.random.default_rng(10 + n)
    pos = rng.uniform(B0, B1, (n, 3)).astype(np.float32)
    q, r = _queries(rng, 50, 0.5)
    counts = _check(pos, q, r)
    assert counts[1] == n
