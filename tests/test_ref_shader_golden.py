"""The oracle against golden outputs of the reference's own compute shaders
(CPU; runs everywhere: the goldens are committed, made by
tests/golden/make_ref_shader_golden.py from PathTracer.comp and
ShadowVolume.comp run on the CPU where the reference tree was).

The same bounds as tests/test_ref_shaders.py: the RNG bit for bit, scattered
directions within 1e-6 with the same random numbers drawn, the shadow
volume within 5e-6, the reference-parity pass per pixel within 2e-4
relative on at least 99.5 % of pixels and in sum within 1e-4."""
import ctypes as C
import importlib.util
import os

import numpy as np
import pytest

from oracle import oracle as orc
from oracle.oracle import _p

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_shaders.npz")


def _make():
    spec = importlib.util.spec_from_file_location("make_ref_shader_golden",
                                                  os.path.join(HERE, "golden", "make_ref_shader_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def data():
    return np.load(GOLDEN), _make().scenes()


def test_rng_matches_the_shader(data):
    gold, s = data
    O = orc.lib()
    states = np.array([O.oracle_xorshift_init(int(v)) for v in s["seeds"]], np.uint32)
    np.testing.assert_array_equal(states, gold["init_states"])
    nums = np.zeros(1000, np.float32)
    assert O.oracle_xorshift_numbers(12345, 1000, _p(nums)) == int(gold["numbers_state_after"][0])
    np.testing.assert_array_equal(nums, gold["numbers"])


def test_scattering_matches_the_shader(data):
    gold, s = data
    O = orc.lib()
    p = s["a"]["params"]
    for i, (d, st) in enumerate(zip(s["scatter_in"], s["scatter_state"])):
        out, state = np.zeros(3, np.float32), C.c_uint32(int(st))
        O.oracle_hg_sample_xorshift(C.byref(p), _p(np.ascontiguousarray(d)), C.byref(state), _p(out))
        assert state.value == int(gold["scatter_state_after"][i])
        np.testing.assert_allclose(out, gold["scatter_out"][i], rtol=0, atol=1e-6)


@pytest.mark.parametrize("name", ["a", "b"])
def test_shadow_volume_and_pass_match_the_shader(data, name):
    gold, s = data
    c = s[name]
    og, cloud = c["og"], c["cloud"]
    o_sv = og.sv_build(cloud, c["sv"])
    np.testing.assert_allclose(o_sv.reshape(gold[f"sv_{name}"].shape), gold[f"sv_{name}"], rtol=0, atol=5e-6)
    sv_ref = np.ascontiguousarray(gold[f"sv_{name}"])  # the pass reads the shader's own shadow volume
    o_sum, o_stats = og.pt_pass(cloud, c["cam"], c["params"], c["W"], c["H"], seed=c["seed"], pass_index=0,
                                sv=c["sv"], sv_tex=sv_ref)
    ref = gold[f"pt_{name}"].astype(np.float64)
    rel = np.abs(ref - o_sum) / np.maximum(np.abs(o_sum), 1e-6)
    assert np.all(rel < 2e-4, axis=-1).mean() >= 0.995
    assert abs(ref.sum() / o_sum.sum() - 1.0) < 1e-4
    assert o_stats[..., 0].sum() > 300
