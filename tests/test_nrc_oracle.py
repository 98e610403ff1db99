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
