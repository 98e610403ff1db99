"""CPU tests of the radiance-cache oracle: its analytic gradient equals
central finite differences of its loss (exact arithmetic mode), and its
encoding has the documented structure."""
import numpy as np
import pytest

import vcr
from oracle import oracle_nrc as onrc


def _cloud():
    desc = vcr.grid_desc((64, 32, 64), (1 / 64,) * 3)
    return vcr.cloud_from_grid(desc, 1.0, 16.0)


def test_analytic_gradient_equals_finite_differences():
    cloud = _cloud()
    rng = np.random.default_rng(0)
    recs = onrc.random_records(24, cloud, rng)
    w = ((rng.random(onrc.weight_count()) - 0.5) * 0.4).astype(np.float32)
    w[5 * 64 * 64:].reshape(64, 16)[:, 3:] = 0
    onrc.set_exact(True)
    try:
        g, loss = onrc.gradient(w, recs, cloud)
        idx = np.concatenate([rng.integers(0, 5 * 64 * 64, 12),
                              5 * 64 * 64 + rng.integers(0, 64, 6) * 16 + rng.integers(0, 3, 6)])
        for i in idx:
            h = 1e-5  # small enough that no ReLU kink falls inside the step
            wp, wm = w.copy(), w.copy()
            wp[i] += h
            wm[i] -= h
            step = float(wp[i]) - float(wm[i])  # the float32 perturbation actually applied
            # the loss treats y in the denominator as constant: difference the
            # numerator-only loss around the same denominators
            fd = (_loss_fixed_den(wp, w, recs, cloud) - _loss_fixed_den(wm, w, recs, cloud)) / step
            assert abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(g[i])) + 1e-9, (i, fd, g[i])
    finally:
        onrc.set_exact(False)


def _loss_fixed_den(w, w0, recs, cloud):
    y = onrc.forward(w, recs, cloud)
    y0 = onrc.forward(w0, recs, cloud)
    t = recs["w"].astype(np.float64)
    return float(np.sum((y - t) ** 2 / (y0 ** 2 + 0.01)) / (3 * len(recs)))


def test_encoding_structure():
    cloud = _cloud()
    rng = np.random.default_rng(1)
    recs = onrc.random_records(50, cloud, rng)
    e = onrc.encode(recs, cloud)
    # frequency pairs lie on the unit circle
    np.testing.assert_allclose(e[:, 0:32:2] ** 2 + e[:, 1:32:2] ** 2, 1.0, atol=2e-6)
    # band 0 of both SH blocks is the constant 1 / (2 sqrt(pi))
    np.testing.assert_allclose(e[:, 32], 0.28209479, rtol=1e-6)
    np.testing.assert_allclose(e[:, 48], 0.28209479, rtol=1e-6)
    # band 1 is proportional to the direction
    np.testing.assert_allclose(e[:, 34] / 0.48860251, recs["v"][:, 2], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("levels", [16, 8, 1, 0])
def test_position_levels_zero_the_finer_levels(levels):
    """The encoding ablation knob: only levels below `levels` are encoded,
    the rest of the 32 position inputs are 0 and the SH inputs do not
    change."""
    cloud = _cloud()
    recs = onrc.random_records(40, cloud, np.random.default_rng(3))
    full = onrc.encode(recs, cloud)
    try:
        onrc.set_levels(levels)
        e = onrc.encode(recs, cloud)
    finally:
        onrc.set_levels(16)
    k = levels
    np.testing.assert_array_equal(e[:, :2 * k], full[:, :2 * k])
    assert not e[:, 2 * k:32].any()
    np.testing.assert_array_equal(e[:, 32:], full[:, 32:])


def test_grid_encoding_interpolates_its_tables():
    """The grid encoding: a position on a vertex of level 0 (16 cells a
    side, dense) reads that vertex's two features; halfway between two
    vertices along x it reads their mean; the frequency inputs are gone."""
    cloud = _cloud()
    rng = np.random.default_rng(5)
    tab = rng.uniform(-1, 1, onrc.GRID_PARAMS).astype(np.float32)
    recs = onrc.random_records(3, cloud, rng)
    b0, b1 = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
    on_vertex = np.array([3, 5, 7]) / 16.0
    recs["p"][0] = b0 + (b1 - b0) * on_vertex
    recs["p"][1] = b0 + (b1 - b0) * ((np.array([3, 5, 7]) + np.array([0.5, 0, 0])) / 16.0)
    try:
        onrc.set_grid(tab)
        e = onrc.encode(recs, cloud)
    finally:
        onrc.set_grid(None)
    v = 17
    i0 = 3 + v * (5 + v * 7)
    np.testing.assert_allclose(e[0, 0:2], tab[2 * i0:2 * i0 + 2], rtol=1e-6, atol=1e-6)
    i1 = i0 + 1
    np.testing.assert_allclose(e[1, 0:2], 0.5 * (tab[2 * i0:2 * i0 + 2] + tab[2 * i1:2 * i1 + 2]), rtol=1e-5,
                               atol=1e-6)
    assert np.all(np.abs(e[:, :32]) <= 1.0)


def test_grid_table_gradient_equals_finite_differences():
    """With the grid encoding the tables are parameters: the analytic
    gradient of the touched table entries (dX_0 spread by trilinear
    weights) equals central differences of the loss (exact mode)."""
    cloud = _cloud()
    rng = np.random.default_rng(6)
    recs = onrc.random_records(12, cloud, rng)
    w = ((rng.random(onrc.weight_count()) - 0.5) * 0.4).astype(np.float32)
    w[5 * 64 * 64:].reshape(64, 16)[:, 3:] = 0
    tab = rng.uniform(-0.5, 0.5, onrc.GRID_PARAMS).astype(np.float32)
    onrc.set_exact(True)
    try:
        onrc.set_grid(tab)
        g, gt, loss = onrc.gradient_tables(w, recs, cloud)
        y0 = onrc.forward(w, recs, cloud)  # the loss's (stop-gradient) denominators
        t = recs["w"].astype(np.float64)

        def loss_at(table):
            onrc.set_grid(table)
            y = onrc.forward(w, recs, cloud)
            return float(np.sum((y - t) ** 2 / (y0 ** 2 + 0.01)) / (3 * len(recs)))

        touched = np.nonzero(gt)[0]
        assert touched.size > 12 * 8
        for i in rng.choice(touched, 16, replace=False):
            h = 1e-3
            tp, tm = tab.copy(), tab.copy()
            tp[i] += h
            tm[i] -= h
            step = float(tp[i]) - float(tm[i])
            fd = (loss_at(tp) - loss_at(tm)) / step
            assert abs(fd - gt[i]) <= 2e-3 * abs(gt[i]) + 1e-9, (i, fd, gt[i])
    finally:
        onrc.set_exact(False)
        onrc.set_grid(None)


def _bf16(x):
    """float64 -> float32 -> BF16 (round to nearest, ties to even) -> float64."""
    u = np.asarray(x, np.float64).astype(np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("exact", [True, False])
def test_forward_is_the_documented_network(exact):
    """64 encoded inputs -> five 64-wide ReLU layers -> 3 outputs; weights
    stored row-major by input (layer l at l * 64 * 64; the output layer 64 x
    16, its first 3 columns used); weights and activations rounded to BF16
    (not in the exact mode); sums in float64 over the inputs in order.
    Restated here in numpy: the same numbers, bit for bit."""
    cloud = _cloud()
    rng = np.random.default_rng(11)
    recs = onrc.random_records(40, cloud, rng)
    w = ((rng.random(onrc.weight_count()) - 0.5) * 0.5).astype(np.float32)
    rnd = (lambda v: np.asarray(v, np.float64)) if exact else _bf16
    onrc.set_exact(exact)
    try:
        got = onrc.forward(w, recs, cloud)
        x = rnd(onrc.encode(recs, cloud).astype(np.float64))
    finally:
        onrc.set_exact(False)
    wb = rnd(w.astype(np.float64))
    h = x
    for layer in range(6):
        cols = 64 if layer < 5 else 16
        m = wb[layer * 64 * 64: layer * 64 * 64 + 64 * cols].reshape(64, cols)
        z = np.zeros((len(h), cols))
        for i in range(64):  # the oracle's summation order
            z = z + h[:, i:i + 1] * m[i]
        h = rnd(np.maximum(z, 0.0)) if layer < 5 else z
    np.testing.assert_array_equal(got, h[:, :3])
    assert np.abs(got).max() > 0
