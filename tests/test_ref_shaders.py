"""The oracle against the reference's own compute shaders, run on the CPU
(CPU tests; only where the reference tree is).

oracle/build_ref.py transliterates PathTracer.comp and ShadowVolume.comp
(parameter qualifiers, descriptor declarations, float literals, main's
name: nothing of the bodies) and oracle/ref_shaders.cpp runs them over the
GLSL pieces of oracle/glsl_shim.h.  The oracle's reference-parity mode
(xorshift streams seeded seed * (x + y * padded width), global-majorant
delta tracking, shadow-volume NEE, gradient sky, albedo 1, no event cap)
restates the same code, and the GPU kernels match the oracle bit for bit
(test_gpu_pt.py), so agreement here pins the whole chain to the shaders.

Where the two compute the same operations in the same order they agree bit
for bit (RNG, background, box intersection, basis, camera ray); where the
shader calls the C library (log, sin, cos, pow) and the oracle its own
series, or divides where the oracle multiplies by a reciprocal, they agree
within float rounding, and path decisions agree."""
import ctypes as C

import numpy as np
import pytest

import vcr
from vcr import configs
from oracle import oracle as orc
from oracle import ref_shaders as rs
from oracle.oracle import _p

pytestmark = pytest.mark.skipif(not rs.available(), reason="the reference shaders are not here")


def _f3():
    return np.zeros(3, np.float32)


def _dirs(rng, n):
    d = rng.normal(size=(n, 3))
    d[:30] = np.eye(3)[np.arange(30) % 3] * np.where(np.arange(30) % 2, 1.0, -1.0)[:, None]
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def _params(g, tracker=vcr.TRACKER_GLOBAL):
    p = configs.C1_PT.params(tracker)
    vcr.params_set_phase_g(p, g)
    p.albedo, p.max_events = 1.0, 0
    p.rng_mode, p.nee_mode, p.sky_mode = vcr.RNG_XORSHIFT, vcr.NEE_SHADOW_VOLUME, vcr.SKY_GRADIENT
    return p


def _scene(size=(48, 40, 48), ds=16.0, g=0.857, sv_n=32, W=80, H=60, octaves=5):
    dense = orc.fbm_fill(size, seed=3, octaves=octaves)
    og = orc.Grid(dense, 0)
    cloud = vcr.cloud_from_grid(vcr.grid_desc(size, (1 / max(size),) * 3), 1.0, ds)
    cloud.max_extinction = max(og.max_density(), 0.01)
    sv = vcr.shadow_volume_setup(configs.sun_travel_dir(), cloud.bounds_min, cloud.bounds_max, sv_n)
    cam = vcr.camera_look((0.1, -0.05, -0.6), (0.1, 0.05, 1.0), 70.0, 0.1, W, H)
    p = _params(g)
    o_sv = og.sv_build(cloud, sv)
    return dense, og, cloud, cam, p, sv, o_sv


@pytest.fixture(scope="module")
def base():
    dense, og, cloud, cam, p, sv, o_sv = _scene()
    return dict(dense=dense, og=og, cloud=cloud, cam=cam, p=p, sv=sv, o_sv=o_sv,
                ref=rs.Scene(dense, cloud, cam, p, sv, o_sv))


def test_random_numbers_bit_exact():
    """initializeRandom / rand_xorshift / generateRandomNumber
    (PathTracer.comp:220-241) against the oracle's xorshift stream."""
    L, O = rs.lib(), orc.lib()
    rng = np.random.default_rng(0)
    for seed in rng.integers(0, 2 ** 32, 2000, dtype=np.uint64).tolist() + [0, 1, 6, 7, 2 ** 32 - 1]:
        assert L.ref_initialize_random(seed) == O.oracle_xorshift_init(seed)
    for state in (12345, 1, 0x80000000, 0xFFFFFFFF):
        a, b = np.zeros(5000, np.float32), np.zeros(5000, np.float32)
        assert L.ref_random_numbers(state, 5000, _p(a)) == O.oracle_xorshift_numbers(state, 5000, _p(b))
        np.testing.assert_array_equal(a, b)


def test_background_box_basis_and_camera_bit_exact(base):
    """sampleBackground (:104-113), intersectCloud (:154-184),
    createOrthonormalBasis (:197-206), getCameraRay (:144-151)."""
    base["ref"].bind()
    L, O = rs.lib(), orc.lib()
    rng = np.random.default_rng(1)
    dirs = _dirs(rng, 20000)
    cloud = base["cloud"]
    b0 = np.array(cloud.bounds_min, np.float32)
    b1 = np.array(cloud.bounds_max, np.float32)
    pos = rng.uniform(-1.5, 1.5, (20000, 3)).astype(np.float32)
    hits = 0
    for q, d in zip(pos, dirs):
        a, b = np.zeros(4, np.float32), _f3()
        L.ref_sample_background(_p(d), _p(a))
        O.oracle_sky_gradient(_p(d), _p(b))
        np.testing.assert_array_equal(a[:3], b)
        t0, t1, u0, u1 = C.c_float(), C.c_float(), C.c_float(), C.c_float()
        ha = L.ref_intersect_cloud(_p(q), _p(d), C.byref(t0), C.byref(t1))
        hb = O.oracle_slab(_p(b0), _p(b1), _p(q), _p(d), C.byref(u0), C.byref(u1))
        assert ha == hb
        if ha:
            hits += 1
            assert (t0.value, t1.value) == (u0.value, u1.value)
        xa, ya, xb, yb = _f3(), _f3(), _f3(), _f3()
        L.ref_onb(_p(d), _p(xa), _p(ya))
        O.oracle_onb(_p(d), _p(xb), _p(yb))
        np.testing.assert_array_equal(np.concatenate([xa, ya]), np.concatenate([xb, yb]))
    assert hits > 2000
    cam = base["cam"]
    for y in range(cam.half_height * 2):
        for x in range(cam.half_width * 2):
            pa, da, pb, db = _f3(), _f3(), _f3(), _f3()
            L.ref_camera_ray(x, y, _p(pa), _p(da))
            O.oracle_camera_ray(C.byref(cam), x, y, _p(pb), _p(db))
            np.testing.assert_array_equal(np.concatenate([pa, da]), np.concatenate([pb, db]))


@pytest.mark.parametrize("g", [0.857, 0.5, 0.0, -0.3, 0.95])
def test_scatter_ray_and_phase(base, g):
    """scatterRay (:277-311) and samplePhase / calculatePDF (:247-274): the
    same random numbers drawn (equal states after), directions within 1e-6
    (the C library's sin / cos against the oracle's own), densities within
    1e-6 relative (pow(d, 1.5) against d sqrt(d))."""
    b = base
    p = _params(g)
    rs.Scene(b["dense"], b["cloud"], b["cam"], p, b["sv"], b["o_sv"])
    L, O = rs.lib(), orc.lib()
    rng = np.random.default_rng(2)
    dirs = _dirs(rng, 5000)
    for d in dirs:
        st = int(rng.integers(1, 2 ** 32))
        a, bb, sb = _f3(), _f3(), C.c_uint32(st)
        sa = L.ref_scatter_ray(_p(d), st, _p(a))
        O.oracle_hg_sample_xorshift(C.byref(p), _p(d), C.byref(sb), _p(bb))
        assert sa == sb.value
        np.testing.assert_allclose(a, bb, rtol=0, atol=1e-6)
    wi, wo = dirs[:-1], dirs[1:]
    ref_pdf = np.array([L.ref_sample_phase(_p(x), _p(y)) for x, y in zip(wi, wo)])
    cosv = (wi[:, 0] * wo[:, 0] + wi[:, 1] * wo[:, 1]) + wi[:, 2] * wo[:, 2]  # the shader's float32 dot
    o_pdf, _ = orc.hg(g, cosv.astype(np.float32))
    np.testing.assert_allclose(ref_pdf, o_pdf, rtol=1e-6)


def test_cloud_and_shadow_volume_lookups(base):
    """sampleCloud (:115-119; the shader divides by the box extent where the
    oracle multiplies by its reciprocal) and sampleShadowVolume (:121-127)."""
    b = base
    b["ref"].bind()
    L, O = rs.lib(), orc.lib()
    cloud = b["cloud"]
    rng = np.random.default_rng(3)
    pts = rng.uniform(cloud.bounds_min, cloud.bounds_max, (20000, 3)).astype(np.float32)
    ref_c = np.array([L.ref_sample_cloud(_p(q)) for q in pts])
    np.testing.assert_allclose(ref_c, b["og"].sample(cloud, pts), rtol=0, atol=5e-6)
    ref_s = np.array([L.ref_sample_shadow_volume(_p(q)) for q in pts])
    o_s = np.array([O.oracle_sv_lookup(b["og"].h, C.byref(cloud), C.byref(b["sv"]), _p(b["o_sv"]), _p(q)) for q in pts])
    np.testing.assert_allclose(ref_s, o_s, rtol=0, atol=5e-7)


def test_find_scatter_point_decisions(base):
    """findScatterPoint (:318-361): the same collision or escape, the same
    random numbers consumed, the collision point within 1e-6."""
    b = base
    b["ref"].bind()
    L, O = rs.lib(), orc.lib()
    cloud = b["cloud"]
    rng = np.random.default_rng(4)
    pts = rng.uniform(cloud.bounds_min, cloud.bounds_max, (10000, 3)).astype(np.float32)
    dirs = _dirs(rng, 10000)
    hits = 0
    for q, d in zip(pts, dirs):
        st = int(rng.integers(1, 2 ** 32))
        qa, qb, sa, sb = q.copy(), q.copy(), C.c_uint32(st), C.c_uint32(st)
        ha = L.ref_find_scatter_point(_p(qa), _p(d), C.byref(sa))
        hb = O.oracle_find_scatter_global(b["og"].h, C.byref(cloud), _p(qb), _p(d), C.byref(sb))
        assert (ha, sa.value) == (hb, sb.value)
        hits += ha
        np.testing.assert_allclose(qa, qb, rtol=0, atol=1e-6)
    assert 1000 < hits < 9000


@pytest.mark.parametrize("n", [24, 40])
def test_shadow_volume_shader(n):
    """ShadowVolume.comp main (:77-93) against the oracle's build."""
    dense, og, cloud, cam, p, sv, _ = _scene(sv_n=n)
    ref = rs.sv_build(rs.Scene(dense, cloud, cam, p, sv, None))
    np.testing.assert_allclose(ref, og.sv_build(cloud, sv).reshape(ref.shape), rtol=0, atol=5e-6)


@pytest.mark.parametrize("size,ds,g,W,H,seed", [
    ((32, 32, 32), 6.0, 0.857, 48, 48, 12345),
    ((64, 64, 64), 16.0, 0.857, 96, 96, 777),
    ((64, 48, 64), 32.0, 0.0, 96, 96, 4242),
    ((64, 48, 64), 24.0, -0.3, 96, 96, 99),
    ((128, 64, 128), 32.0, 0.857, 128, 96, 5),
])
def test_path_tracer_shader_image(size, ds, g, W, H, seed):
    """PathTracer.comp main (:366-425) for every pixel against the oracle's
    reference-parity pass with the same shadow volume: per-pixel radiance
    within 2e-4 relative on at least 99.5 % of pixels (the C library's
    log / sin / cos / pow against the oracle's own series along paths of up
    to ~190 events), the image sums within 1e-4."""
    dense, og, cloud, _, p, sv, o_sv = _scene(size=size, ds=ds, g=g, sv_n=48, octaves=5)
    cam = vcr.camera_look((0, 0, -0.6), (0, 0, 1), 70.0, 0.1, W, H)
    ref = rs.pt_image(rs.Scene(dense, cloud, cam, p, sv, o_sv), W, H, seed)[..., :3].astype(np.float64)
    o_sum, o_stats = og.pt_pass(cloud, cam, p, W, H, seed=seed, pass_index=0, sv=sv, sv_tex=o_sv)
    rel = np.abs(ref - o_sum) / np.maximum(np.abs(o_sum), 1e-6)
    assert np.all(rel < 2e-4, axis=-1).mean() >= 0.995
    assert abs(ref.sum() / o_sum.sum() - 1.0) < 1e-4
    assert o_stats[..., 0].sum() > 300  # paths do scatter
