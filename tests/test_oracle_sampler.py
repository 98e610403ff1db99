"""The oracle's density lookup against the reference's sampler, restated
independently here (CPU).

sampleCloud reads the cloud through texture() with a sampler of linear
min / mag filtering and clamp-to-edge addressing on all three axes
(PathTracer.comp:115-119, Initializers.cpp:408-418).  Vulkan's linear
filter of a normalized coordinate s on an axis of N texels takes
u = s N - 1/2, the texels floor(u) and floor(u) + 1 clamped to [0, N - 1],
and the weights 1 - frac(u) and frac(u); three axes multiply.  That formula
is evaluated here in float64 and compared with the oracle's exact float32
trilinear (which the GPU lookup matches bit for bit)."""
import numpy as np

import vcr
from oracle import oracle as orc


def _vulkan_linear(tex, s):
    """tex: [Z, Y, X] float64; s: [n, 3] normalized (x, y, z)."""
    n = np.array(tex.shape[::-1])
    u = s * n - 0.5
    i0 = np.floor(u).astype(np.int64)
    a = u - i0
    out = np.zeros(len(s))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                idx = np.clip(i0 + np.array([dx, dy, dz]), 0, n - 1)
                w = np.where([dx, dy, dz], a, 1.0 - a).prod(axis=1)
                out += w * tex[idx[:, 2], idx[:, 1], idx[:, 0]]
    return out


def _setup(size, seed):
    rng = np.random.default_rng(seed)
    dense = rng.random(size[::-1]).astype(np.float32)
    g = orc.Grid(dense, 0)
    cloud = vcr.cloud_from_grid(vcr.grid_desc(size, (1.0 / max(size),) * 3), 1.0, 8.0)
    b0 = np.array(cloud.bounds_min, np.float64)
    b1 = np.array(cloud.bounds_max, np.float64)
    return rng, dense, g, cloud, b0, b1


def test_lookup_is_the_linear_clamp_to_edge_filter():
    size = (9, 7, 5)
    rng, dense, g, cloud, b0, b1 = _setup(size, 1)
    s = rng.random((50000, 3))
    s[:2000] = np.clip(rng.normal(0.0, 0.03, (2000, 3)), 0.0, 1.0)  # near the low faces: clamped
    s[2000:4000] = np.clip(1.0 - np.abs(rng.normal(0.0, 0.03, (2000, 3))), 0.0, 1.0)  # near the high faces
    s[4000:4008] = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float64)  # corners
    p = (b0 + s * (b1 - b0)).astype(np.float32)
    got = g.sample(cloud, p).astype(np.float64)
    s32 = (p.astype(np.float64) - b0) / (b1 - b0)  # the coordinates the float32 points stand for
    want = _vulkan_linear(dense.astype(np.float64), s32)
    # float32 coordinates, weights and lerps: at most 6.2e-7 off over 200,000
    # points of texels in [0, 1]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)


def test_texel_centres_return_the_texels():
    size = (6, 5, 4)
    rng, dense, g, cloud, b0, b1 = _setup(size, 2)
    z, y, x = np.meshgrid(*[np.arange(k) for k in size[::-1]], indexing="ij")
    s = (np.stack([x, y, z], axis=-1).reshape(-1, 3) + 0.5) / np.array(size)
    p = (b0 + s * (b1 - b0)).astype(np.float32)
    got = g.sample(cloud, p)
    np.testing.assert_allclose(got, dense.reshape(-1), rtol=0, atol=2e-6)


def test_beyond_the_outer_texel_centres_the_edge_value_holds():
    """Clamp-to-edge: between the last texel centre and the face, along an
    axis the value no longer changes."""
    size = (8, 8, 8)
    rng, dense, g, cloud, b0, b1 = _setup(size, 3)
    s = rng.random((4000, 3))
    edge = s.copy()
    edge[:, 0] = rng.uniform(0.0, 0.5 / size[0], len(s))  # inside the first half texel along x
    face = edge.copy()
    face[:, 0] = 0.0
    pe = (b0 + edge * (b1 - b0)).astype(np.float32)
    pf = (b0 + face * (b1 - b0)).astype(np.float32)
    np.testing.assert_allclose(g.sample(cloud, pe), g.sample(cloud, pf), rtol=0, atol=2e-6)
