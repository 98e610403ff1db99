"""CPU tests of the sort / Morton oracle against the reference's own fixture
(Tests.cpp:113-131) and known answers."""
import numpy as np
import pytest

from oracle import oracle as orc


def test_tests_cpp_fixture_sorts_stably():
    """tests::localSort: 176 keys in [0, 255] from mt19937(1), eight 1-bit
    split passes (bits 0..7) -> ascending, equal to a stable sort."""
    keys = orc.sort_fixture_keys()
    assert len(keys) == 176 and keys.max() <= 255
    out = orc.split_sort(keys, 0, 8)
    np.testing.assert_array_equal(out, np.sort(keys, kind="stable"))


@pytest.mark.parametrize("n", [1, 2, 3, 100, 1024])
def test_split_passes_are_stable_partitions(n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 16, n).astype(np.uint32)
    for bit in range(4):
        out = orc.split_sort(keys, bit, 1)
        zeros = keys[((keys >> bit) & 1) == 0]
        ones = keys[((keys >> bit) & 1) == 1]
        np.testing.assert_array_equal(out, np.concatenate([zeros, ones]))


@pytest.mark.parametrize("n,hi", [(0, 10), (1, 10), (1023, 7), (1025, 3), (5000, 1 << 30), (20000, 1 << 32)])
@pytest.mark.parametrize("bits", [(0, 32), (0, 30), (4, 12), (3, 13), (5, 6)])
def test_lsd_pipeline_equals_stable_argsort(n, hi, bits):
    rng = np.random.default_rng(n + bits[0])
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    ko, vo = orc.lsd_sort_pairs(keys, None, *bits)
    # only the bits [begin, end) decide the order (the last digit is narrower
    # when the range is not a multiple of 4 bits)
    mask = np.uint32(((1 << (bits[1] - bits[0])) - 1) << bits[0])
    perm = np.argsort(keys & mask, kind="stable")
    np.testing.assert_array_equal(vo, perm)
    np.testing.assert_array_equal(ko, keys[perm])


def test_morton_known_answers():
    b0, b1 = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    pts = np.array([[0, 0, 0], [1.0, 1.0, 1.0], [1 / 1024 + 1e-6, 0, 0], [0, 1 / 1024 + 1e-6, 0],
                    [0, 0, 1 / 1024 + 1e-6], [0.5, 0.5, 0.5], [-1, 2, 0.25]], np.float32)
    codes = orc.morton(pts, b0, b1, 30)
    assert codes[0] == 0
    assert codes[1] == (1 << 30) - 1
    assert codes[2] == 4 and codes[3] == 2 and codes[4] == 1
    assert codes[5] == 7 << 27  # 512 = bit 9 on every axis
    # clamped x = 0, y = 1023, z = 256
    z = orc.morton(np.array([[0, 0, 0.25]], np.float32), b0, b1, 30)[0]
    y = orc.morton(np.array([[0, 1.0, 0]], np.float32), b0, b1, 30)[0]
    assert codes[6] == z | y
    # 24-bit reference mode: (p - b0)/256 per axis
    c24 = orc.morton(np.array([[256.0 * 3, 0, 256.0 * 255.5]], np.float32), b0, b1, 24)
    # x = 3 -> 0b1001 (expanded), y = 0, z = 255 -> 0x249249
    assert c24[0] == (0b1001 << 2) | 0x249249
