"""GPU tests of the stable radix sort and the Morton codes through the C-ABI:
bit-exact permutations against the oracle's restatement of the reference's
LocalSort/PrefixSum/GlobalSort pipeline and numpy's stable argsort."""
import numpy as np
import pytest

import vcr
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _to_dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(cuda)


def _from_dev(t):
    return t.cpu().numpy().view(np.uint32)


def _keys(kind, n, rng):
    if kind == "uniform32":
        return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    if kind == "morton30":
        return rng.integers(0, 1 << 30, n, dtype=np.uint64).astype(np.uint32)
    if kind == "few":
        return rng.integers(0, 5, n).astype(np.uint32) * np.uint32(0x01010101)
    if kind == "equal":
        return np.full(n, 0xDEADBEEF, np.uint32)
    if kind == "sorted":
        return np.arange(n, dtype=np.uint32)
    if kind == "reversed":
        return np.arange(n, dtype=np.uint32)[::-1].copy()
    raise ValueError(kind)


SIZES = [0, 1, 2, 31, 2047, 2048, 2049, 100000, 262144]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("kind", ["uniform32", "morton30", "few", "equal", "sorted", "reversed"])
def test_sort_permutation_bit_exact(cuda, n, kind):
    import torch
    rng = np.random.default_rng(n * 7 + len(kind))
    keys = _keys(kind, n, rng)
    perm = np.argsort(keys, kind="stable")
    with vcr.Context() as ctx:
        dk = _to_dev(keys, cuda)
        ko = torch.empty(max(n, 1), dtype=torch.int32, device=cuda)
        vo = torch.empty(max(n, 1), dtype=torch.int32, device=cuda)
        ctx.radix_sort_pairs(dk.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), n)
        ctx.synchronize()
    np.testing.assert_array_equal(_from_dev(vo)[:n], perm.astype(np.uint32))
    np.testing.assert_array_equal(_from_dev(ko)[:n], keys[perm])
    if n <= 100000:
        ok, ov = orc.lsd_sort_pairs(keys)
        np.testing.assert_array_equal(_from_dev(vo)[:n], ov)


@pytest.mark.parametrize("bits", [(0, 30), (4, 12), (0, 4), (28, 32), (3, 13), (5, 6), (0, 31)])
def test_sort_bit_ranges_and_payload(cuda, bits):
    """Only the bits [begin, end) decide the order, also when the range is
    not a multiple of the 8-bit digit (the keys' other bits are random)."""
    import torch
    n = 50001
    rng = np.random.default_rng(bits[0])
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    ok, ov = orc.lsd_sort_pairs(keys, vals, *bits)
    with vcr.Context() as ctx:
        dk, dv = _to_dev(keys, cuda), _to_dev(vals, cuda)
        ko = torch.empty(n, dtype=torch.int32, device=cuda)
        vo = torch.empty(n, dtype=torch.int32, device=cuda)
        ctx.radix_sort_pairs(dk.data_ptr(), dv.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, *bits)
        ctx.synchronize()
    np.testing.assert_array_equal(_from_dev(ko), ok)
    np.testing.assert_array_equal(_from_dev(vo), ov)
    mask = np.uint32(((1 << (bits[1] - bits[0])) - 1) << bits[0])
    perm = np.argsort(keys & mask, kind="stable")
    np.testing.assert_array_equal(_from_dev(vo), vals[perm])


@pytest.mark.parametrize("bits", [(0, 32), (0, 28), (0, 24), (0, 8)])
def test_sort_in_place(cuda, bits):
    """Even (4) and odd (3, 1) pass counts in place, and a last digit
    narrower than 8 bits (28 bits); keys above 24 bits also carry bits
    outside the sorted range."""
    n = 70000
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 28, n).astype(np.uint32)
    ok, ov = orc.lsd_sort_pairs(keys, None, *bits)
    with vcr.Context() as ctx:
        dk = _to_dev(keys, cuda)
        import torch
        dv = torch.arange(n, dtype=torch.int32, device=cuda)
        ctx.radix_sort_pairs(dk.data_ptr(), dv.data_ptr(), dk.data_ptr(), dv.data_ptr(), n, *bits)
        ctx.synchronize()
    np.testing.assert_array_equal(_from_dev(dk), ok)
    np.testing.assert_array_equal(_from_dev(dv), ov)


def test_sort_large(cuda):
    import torch
    n = (1 << 22) + 17
    g = torch.Generator(device=cuda).manual_seed(5)
    dk = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=torch.int32, device=cuda, generator=g)
    ko = torch.empty_like(dk)
    vo = torch.empty_like(dk)
    with vcr.Context() as ctx:
        ctx.radix_sort_pairs(dk.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), n)
        ctx.synchronize()
    keys = _from_dev(dk)
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(_from_dev(vo), perm)


def test_morton_codes_bit_exact(cuda):
    import torch
    rng = np.random.default_rng(9)
    b0, b1 = (-0.5, -0.25, 0.0), (0.5, 0.25, 1.0)
    pts = (rng.random((100000, 3)) * 1.2 - 0.1).astype(np.float32) * np.array([1, 0.5, 1], np.float32) \
        + np.array([-0.5, -0.25, 0], np.float32)
    pts[:10] = [[-0.5, -0.25, 0], [0.5, 0.25, 1.0], [0, 0, 0.5], [-9, 9, 0.5], [0.4999, 0.2499, 0.9999],
                [np.nextafter(np.float32(-0.5), np.float32(1)), 0, 0], [0, 0, 1 / 1024], [0, 0, 2 / 1024],
                [0.5, -0.25, 0], [0, 0, 0]]
    with vcr.Context() as ctx:
        dp = torch.from_numpy(pts).to(cuda)
        out = torch.empty(len(pts), dtype=torch.int32, device=cuda)
        for bits in (30, 24):
            bb0, bb1 = (b0, b1) if bits == 30 else ((-300.0, -300.0, -300.0), (300.0, 300.0, 300.0))
            p = pts if bits == 30 else (pts * 200).astype(np.float32)
            dp = torch.from_numpy(p).to(cuda)
            ctx.morton_codes(dp.data_ptr(), len(p), bb0, bb1, bits, out.data_ptr())
            ctx.synchronize()
            np.testing.assert_array_equal(_from_dev(out), orc.morton(p, bb0, bb1, bits))


def test_tests_cpp_fixture_keys_on_the_gpu(cuda):
    """The reference's only sort fixture (Tests.cpp:113-131: 176 keys in
    [0, 255], sorted on bits 0..7), from the pinned golden array: the GPU
    sort's permutation is the stable one."""
    import os
    import torch
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sort_fixture_keys.txt")
    keys = np.loadtxt(golden, dtype=np.uint32)
    n = len(keys)
    with vcr.Context() as ctx:
        dk = _to_dev(keys, cuda)
        ko = torch.empty(n, dtype=torch.int32, device=cuda)
        vo = torch.empty(n, dtype=torch.int32, device=cuda)
        ctx.radix_sort_pairs(dk.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), n, 0, 8)
        ctx.synchronize()
    perm = np.argsort(keys, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(_from_dev(vo), perm)
    np.testing.assert_array_equal(_from_dev(ko), keys[perm])
