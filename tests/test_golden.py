"""Golden fixtures from the reference's own code (tests/golden, made by
tests/golden/make_golden.py): files its Grid3D<float> wrote and arrays its
Load produced (Grid3D.h: Load :44-90, Save :166-178, GetMajorant :180-192),
and the key array of its only test fixture (Tests.cpp:113-131).  These run
everywhere, without the reference tree."""
import os

import numpy as np

import vcr
from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ref_load(name):
    raw = open(os.path.join(GOLDEN, name), "rb").read()
    dims = tuple(int(v) for v in np.frombuffer(raw[:12], np.uint32))
    voxel = np.frombuffer(raw[12:36], np.float64)
    maj = float(np.frombuffer(raw[36:40], np.float32)[0])
    return dims, voxel, maj, np.frombuffer(raw[40:], np.float32)


def test_file_saved_by_the_reference_reads_as_its_load_reads_it():
    """Grid3D::Save writes memory order and Grid3D::Load expects z fastest,
    so a saved file loads transposed; the project's reader must give the
    reference Load's array, not the array that was saved."""
    dims, voxel, maj, mem = _ref_load("grid3d_ref_load_9x4x3.bin")
    desc, ours = vcr.xyz_read(os.path.join(GOLDEN, "grid3d_ref_save_9x4x3.xyz"))
    assert tuple(desc.size) == dims == (9, 4, 3)
    np.testing.assert_array_equal(np.array(desc.voxel_size[:]), voxel)
    np.testing.assert_array_equal(ours.ravel(), mem)
    saved = np.random.default_rng(11).random((3, 4, 9), dtype=np.float32)  # what make_golden saved
    assert not np.array_equal(ours.ravel(), saved.ravel())  # the transposition is real
    assert maj == float(saved.max()) == float(ours.max())  # GetMajorant


def test_file_written_by_the_project_loads_in_the_reference():
    dims, voxel, maj, mem = _ref_load("grid3d_ref_load_ours_12x7x5.bin")
    data = np.random.default_rng(12).random((5, 7, 12), dtype=np.float32)
    assert dims == (12, 7, 5)
    np.testing.assert_array_equal(voxel, [1.0, 2.0, 3.0])
    np.testing.assert_array_equal(mem, data.ravel())  # the reference's memory order is the project's
    assert maj == float(data.max())


def test_sort_fixture_keys_are_the_pinned_ones():
    """The oracle's replay of Tests.cpp's std::mt19937(1) +
    uniform_int_distribution(0, 255) draws equals the pinned array, and the
    fixture's eight 1-bit split passes sort it stably."""
    golden = np.loadtxt(os.path.join(GOLDEN, "sort_fixture_keys.txt"), dtype=np.uint32)
    keys = orc.sort_fixture_keys()
    np.testing.assert_array_equal(keys, golden)
    np.testing.assert_array_equal(orc.split_sort(golden, 0, 8), np.sort(golden, kind="stable"))
