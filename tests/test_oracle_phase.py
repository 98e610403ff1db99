"""The oracle's Henyey-Greenstein phase function (hg_pdf / hg_sample, the
restatement of PathTracer.comp:247-311 that the tracker kernels match bit
for bit) against its closed forms: the density is the HG formula and
integrates to 1 over the sphere, and sampled directions are unit vectors
whose cosines with the incoming direction follow that density, with
<cos> = g, <P2(cos)> = g^2 and no preferred azimuth."""
import numpy as np
import pytest

from oracle import oracle as orc

# the bench cloud's g, moderate and backward lobes, isotropic, the clamp at 0.95
G_VALUES = [0.857, 0.5, -0.3, 0.0, 0.95]


def _hg64(g, c):
    if abs(g) < 1e-4:
        return np.full_like(c, 1.0 / (4.0 * np.pi))
    return (1.0 - g * g) / (4.0 * np.pi * (1.0 + g * g - 2.0 * g * c) ** 1.5)


@pytest.mark.parametrize("g", G_VALUES)
def test_hg_pdf_is_the_formula_and_integrates_to_one(g):
    c = np.linspace(-1.0, 1.0, 2_000_001)
    pdf, _ = orc.hg(g, c.astype(np.float32))
    c32 = c.astype(np.float32).astype(np.float64)
    ref = _hg64(g, c32)
    # float32 evaluation: d = 1 + g^2 - 2 g c cancels towards (1 - g)^2 near
    # c = 1, so its relative rounding error, and 1.5 times it in d^1.5,
    # grows as (1 + g^2 + 2 |g c|) / d
    d = 1.0 + g * g - 2.0 * g * c32
    tol = 1e-6 + 4.0 * 2.0 ** -23 * 1.5 * (1.0 + g * g + 2.0 * np.abs(g * c32)) / d
    assert np.all(np.abs(pdf - ref) <= tol * ref), float(np.max(np.abs(pdf - ref) / (tol * ref)))
    # On this grid the float64 formula integrates to 1 within 4e-8.  The
    # float32 constants 1 + g^2 and 1 - g^2 (Parameters::SetPhaseG) round by
    # up to 6e-8 of themselves, which is ~5e-5 of d at the peak of the
    # sharpest lobe, so the float32 density integrates to 1 + 1.4e-5 at
    # g = 0.95 and 1 + 2e-6 at g = 0.857.
    integral = 2.0 * np.pi * np.trapezoid(pdf.astype(np.float64), c32)
    assert abs(integral - 1.0) < 3e-5, integral
    assert abs(2.0 * np.pi * np.trapezoid(ref, c32) - 1.0) < 1e-7


def _frame(d):
    d = np.asarray(d, np.float64) / np.linalg.norm(d)
    a = np.array([1.0, 0.0, 0.0]) if abs(d[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(d, a)
    u /= np.linalg.norm(u)
    return d, u, np.cross(d, u)


@pytest.mark.parametrize("g", G_VALUES)
@pytest.mark.parametrize("incoming", [(0.0, 0.0, 1.0), (0.3, -0.5, -0.8)])
def test_hg_samples_follow_the_density(g, incoming):
    n = 200_000
    inc = np.asarray(incoming, np.float32) / np.float32(np.linalg.norm(incoming))
    _, dirs = orc.hg(g, [], n, tuple(float(v) for v in inc), seed=7)
    d = dirs.astype(np.float64)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
    w, u, v = _frame(inc.astype(np.float64))
    c = np.clip(d @ w, -1.0, 1.0)
    geff = 0.0 if abs(g) < 1e-4 else g
    # moments: E[P1] = g, E[P2] = g^2 (HG's Legendre coefficients)
    var1 = (1.0 + 2.0 * geff ** 2) / 3.0 - geff ** 2
    assert abs(c.mean() - geff) < 5.0 * np.sqrt(var1 / n), (c.mean(), geff)
    p2 = 0.5 * (3.0 * c * c - 1.0)
    assert abs(p2.mean() - geff ** 2) < 5.0 * p2.std() / np.sqrt(n), (p2.mean(), geff ** 2)
    # azimuth: the components across the incoming direction average to zero
    for axis in (u, v):
        comp = d @ axis
        assert abs(comp.mean()) < 5.0 * comp.std() / np.sqrt(n)
    # the cosines' histogram against the density integrated over each bin
    edges = np.linspace(-1.0, 1.0, 41)
    counts, _ = np.histogram(c, edges)
    fine = np.linspace(-1.0, 1.0, 400_001)
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (_hg64(geff, fine[1:]) + _hg64(geff, fine[:-1])) * np.diff(fine))])
    cdf *= 2.0 * np.pi
    expect = n * np.diff(np.interp(edges, fine, cdf))
    keep = expect > 20.0
    chi2 = float((((counts - expect) ** 2) / expect)[keep].sum())
    dof = int(keep.sum()) - 1
    assert chi2 < dof + 6.0 * np.sqrt(2.0 * dof), (chi2, dof)


def test_hg_sampling_is_deterministic_per_stream():
    _, a = orc.hg(0.857, [], 1000, (0.0, 1.0, 0.0), seed=3)
    _, b = orc.hg(0.857, [], 1000, (0.0, 1.0, 0.0), seed=3)
    _, c = orc.hg(0.857, [], 1000, (0.0, 1.0, 0.0), seed=4)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
