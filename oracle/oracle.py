"""ctypes binding of the CPU oracle (liboracle.so) — test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only as the checker or the timed CPU reference.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "cloudrendering-vulkan_gb300"))
from vcr import _abi  # noqa: E402  (struct layouts only)

_lib = None


def lib():
    global _lib
    if _lib is None:
        from . import build as _b  # type: ignore
        path = _b.build()
        L = C.CDLL(path)
        P = C.c_void_p
        u32, f = C.c_uint32, C.c_float
        sig = {
            "oracle_grid_new": (P, [P, P, C.c_int]),
            "oracle_grid_free": (None, [P]),
            "oracle_grid_max": (f, [P]),
            "oracle_grid_majorants": (None, [P, C.c_int, P]),
            "oracle_grid_decoded": (None, [P, P]),
            "oracle_grid_sample": (None, [P, C.POINTER(_abi.Cloud), P, u32, P]),
            "oracle_dda_trace": (None, [P, C.POINTER(_abi.Cloud), C.c_int, P, P, u32, u32, P, P, P]),
            "oracle_pt_pass": (C.c_int, [P, C.c_int, C.POINTER(_abi.Cloud), C.POINTER(_abi.Camera),
                                         C.POINTER(_abi.Params),
                                         C.POINTER(_abi.ShadowVolume), P, u32, u32, C.POINTER(_abi.PassDesc), P, P,
                                         C.c_int]),
            "oracle_sv_build": (None, [P, C.POINTER(_abi.Cloud), C.POINTER(_abi.ShadowVolume), P]),
            "oracle_fbm_fill": (None, [P, C.c_uint64, u32, f, f, f, P, C.c_int]),
            "oracle_display": (None, [P, C.c_size_t, C.c_double, f, u32, P]),
            "oracle_srgb_encode": (f, [f]),
            "oracle_log": (f, [f]),
            "oracle_exp": (f, [f]),
            "oracle_sincos2pi": (None, [f, C.POINTER(f), C.POINTER(f)]),
            "oracle_pcg_hash": (u32, [u32]),
            "oracle_f32_to_f16": (C.c_uint16, [f]),
            "oracle_f32_to_bf16": (C.c_uint16, [f]),
            "oracle_sort_fixture_keys": (None, [P]),
            "oracle_split_sort": (None, [P, u32, u32, u32]),
            "oracle_lsd_sort_pairs": (None, [P, P, u32, u32, u32, P, P]),
            "oracle_morton": (None, [P, u32, P, P, u32, P]),
            "oracle_params_set_phase_g": (C.c_int, [C.POINTER(_abi.Params), f]),
            "oracle_hg": (None, [C.POINTER(_abi.Params), P, u32, P, _abi.F3, u32, u32, P]),
            "oracle_sky_gradient": (None, [P, P]),
            "oracle_slab": (C.c_int, [P, P, P, P, C.POINTER(f), C.POINTER(f)]),
            "oracle_onb": (None, [P, P, P]),
            "oracle_camera_ray": (None, [C.POINTER(_abi.Camera), C.c_int, C.c_int, P, P]),
            "oracle_xorshift_init": (u32, [u32]),
            "oracle_xorshift_numbers": (u32, [u32, u32, P]),
            "oracle_hg_sample_xorshift": (None, [C.POINTER(_abi.Params), P, C.POINTER(u32), P]),
            "oracle_find_scatter_global": (C.c_int, [P, C.POINTER(_abi.Cloud), P, P, C.POINTER(u32)]),
            "oracle_sv_lookup": (f, [P, C.POINTER(_abi.Cloud), C.POINTER(_abi.ShadowVolume), P, P]),
            "oracle_cloud_from_grid": (C.c_int, [C.POINTER(_abi.GridDesc), f, f, C.POINTER(_abi.Cloud)]),
            "oracle_camera_look": (C.c_int, [C.POINTER(_abi.Camera), _abi.F3, _abi.F3, f, f, C.c_int32,
                                             C.c_int32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def scene_structs(sc, tracker=_abi.TRACKER_DDA):
    """(grid desc, cloud, camera, params) of a scene configuration, built by
    the oracle's restatement of the reference's set-up (no product code):
    the same bytes as the library's vcr_cloud_from_grid / vcr_camera_look /
    vcr_params_set_phase_g on the same arguments."""
    L = lib()
    n = max(sc.size)
    desc = _abi.GridDesc()
    for a in range(3):
        desc.size[a] = sc.size[a]
        desc.voxel_size[a] = 1.0 / n
    cloud = _abi.Cloud()
    assert L.oracle_cloud_from_grid(C.byref(desc), 1.0, sc.density_scaling, C.byref(cloud)) == 0
    cam = _abi.Camera()
    pos, fwd, fov, near = sc.camera_pose()
    assert L.oracle_camera_look(C.byref(cam), _abi.F3(*pos), _abi.F3(*fwd), fov, near, sc.width, sc.height) == 0
    p = sc.params_fields(tracker)
    assert L.oracle_params_set_phase_g(C.byref(p), sc.g) == 0
    return desc, cloud, cam, p


def hg(g: float, cosines, n_samples: int = 0, incoming=(0.0, 0.0, 1.0), seed: int = 1):
    """The oracle's HG phase function for parameter g (set as
    Parameters::SetPhaseG sets it): (pdf at `cosines`, `n_samples`
    directions scattered from `incoming`)."""
    p = _abi.Params()
    assert lib().oracle_params_set_phase_g(C.byref(p), g) == 0
    c = np.ascontiguousarray(cosines, np.float32)
    pdf = np.empty(len(c), np.float32)
    dirs = np.empty((max(n_samples, 1), 3), np.float32)
    lib().oracle_hg(C.byref(p), _p(c), len(c), _p(pdf), _abi.F3(*incoming), seed, n_samples, _p(dirs))
    return pdf, dirs[:n_samples]


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def fbm_fill(size, seed=1, octaves=6, lacunarity=2.0, gain=0.5, f0=4.0, threads=0) -> np.ndarray:
    out = np.empty((size[2], size[1], size[0]), np.float32)
    n = (C.c_uint32 * 3)(*size)
    lib().oracle_fbm_fill(C.cast(n, C.c_void_p), seed, octaves, lacunarity, gain, f0, _p(out),
                          threads or os.cpu_count() or 1)
    return out


class Grid:
    """Oracle grid: decoded texels of the requested precision + majorants."""

    def __init__(self, dense: np.ndarray, precision: int = 0):
        dense = np.ascontiguousarray(dense, np.float32)
        nz, ny, nx = dense.shape
        self.size = (nx, ny, nz)
        n = (C.c_uint32 * 3)(nx, ny, nz)
        self.h = lib().oracle_grid_new(C.cast(n, C.c_void_p), _p(dense), precision)
        self.nb = tuple((s + 7) // 8 for s in self.size)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_grid_free(self.h)
            self.h = None

    def max_density(self) -> float:
        return lib().oracle_grid_max(self.h)

    def level_dims(self, level: int):
        d = list(self.nb)
        for _ in range(level):
            d = [(x + 1) // 2 for x in d]
        return tuple(d)

    def majorants(self, level: int = 0) -> np.ndarray:
        d = self.level_dims(level)
        out = np.empty(d[0] * d[1] * d[2], np.float32)
        lib().oracle_grid_majorants(self.h, level, _p(out))
        return out

    def decoded(self) -> np.ndarray:
        out = np.empty(self.size[::-1], np.float32)
        lib().oracle_grid_decoded(self.h, _p(out))
        return out

    def sample(self, cloud, pos: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        out = np.empty(pos.shape[0], np.float32)
        lib().oracle_grid_sample(self.h, C.byref(cloud), _p(pos), pos.shape[0], _p(out))
        return out

    def dda_trace(self, cloud, o: np.ndarray, d: np.ndarray, max_cells: int, level: int = 0):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        cells = np.zeros((n, max_cells), np.uint32)
        tt = np.zeros((n, max_cells, 2), np.float32)
        cnt = np.zeros(n, np.uint32)
        lib().oracle_dda_trace(self.h, C.byref(cloud), level, _p(o), _p(d), n, max_cells, _p(cells), _p(tt), _p(cnt))
        return cells, tt, cnt

    def pt_pass(self, cloud, cam, params, width, height, seed=0, pass_index=0, spp=1, crop=(0, 0, 0, 0), flags=0,
                sum_img=None, stats=None, sv=None, sv_tex=None, threads=0, level=2):
        if sum_img is None:
            sum_img = np.zeros((height, width, 3), np.float64)
        if stats is None:
            stats = np.zeros((height, width, 4), np.uint32)
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp, p.flags = seed, pass_index, spp, flags
        for i in range(4):
            p.crop[i] = crop[i]
        svp = C.byref(sv) if sv is not None else None
        svt = _p(np.ascontiguousarray(sv_tex, np.float32)) if sv_tex is not None else None
        lib().oracle_pt_pass(self.h, level, C.byref(cloud), C.byref(cam), C.byref(params), svp, svt, width, height,
                             C.byref(p), _p(sum_img), _p(stats), threads or os.cpu_count() or 1)
        return sum_img, stats

    def sv_build(self, cloud, sv) -> np.ndarray:
        n = sv.voxel_axis_count
        out = np.empty((n, n, n), np.float32)
        lib().oracle_sv_build(self.h, C.byref(cloud), C.byref(sv), _p(out))
        return out


def display(sum_img: np.ndarray, samples: int, exposure: float = 1.0, order: int = 0) -> np.ndarray:
    """The oracle's display image (uint8 [H, W, 4]) of FP64 sums [H, W, 3]."""
    s = np.ascontiguousarray(sum_img, np.float64)
    h, w = s.shape[:2]
    out = np.empty((h, w), np.uint32)
    inv = 1.0 / samples if samples else 0.0
    lib().oracle_display(_p(s), h * w, inv, exposure, order, _p(out))
    return out.view(np.uint8).reshape(h, w, 4)


def srgb_encode(v: float) -> float:
    return lib().oracle_srgb_encode(v)


def olog(x: float) -> float:
    return lib().oracle_log(x)


def oexp(x: float) -> float:
    return lib().oracle_exp(x)


def sincos2pi(u: float):
    s, c = C.c_float(), C.c_float()
    lib().oracle_sincos2pi(u, C.byref(s), C.byref(c))
    return s.value, c.value


def sort_fixture_keys() -> np.ndarray:
    out = np.empty(176, np.uint32)
    lib().oracle_sort_fixture_keys(_p(out))
    return out


def split_sort(keys: np.ndarray, first_bit: int, nbits: int) -> np.ndarray:
    k = np.ascontiguousarray(keys, np.uint32).copy()
    lib().oracle_split_sort(_p(k), len(k), first_bit, nbits)
    return k


def lsd_sort_pairs(keys: np.ndarray, vals=None, begin=0, end=32):
    keys = np.ascontiguousarray(keys, np.uint32)
    n = len(keys)
    ko, vo = np.empty(n, np.uint32), np.empty(n, np.uint32)
    vp = _p(np.ascontiguousarray(vals, np.uint32)) if vals is not None else None
    lib().oracle_lsd_sort_pairs(_p(keys), vp, n, begin, end, _p(ko), _p(vo))
    return ko, vo


def morton(points: np.ndarray, bmin, bmax, bits: int) -> np.ndarray:
    pts = np.ascontiguousarray(points, np.float32)
    out = np.empty(len(pts), np.uint32)
    b0 = np.ascontiguousarray(bmin, np.float32)
    b1 = np.ascontiguousarray(bmax, np.float32)
    lib().oracle_morton(_p(pts), len(pts), _p(b0), _p(b1), bits, _p(out))
    return out


class _PpbOut(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("n", "slots", "nbeams", "seg_a", "seg_b", "seg_beam", "codes", "order",
                                         "left", "right", "node_lo", "node_hi", "leaf_lo", "leaf_hi")] + \
               [("capacity_out", C.c_uint32)]


def _ppb_lib():
    L = lib()
    if not getattr(L, "_ppb_bound", False):
        P, u32, f = C.c_void_p, C.c_uint32, C.c_float
        L.oracle_ppb_radius.restype = f
        L.oracle_ppb_radius.argtypes = [f, f, u32]
        L.oracle_ppb_pass.restype = C.c_int
        L.oracle_ppb_pass.argtypes = [P, C.c_int, C.POINTER(_abi.Cloud), C.POINTER(_abi.Camera),
                                      C.POINTER(_abi.Params), u32, u32, f, f, u32, u32, C.POINTER(_abi.PassDesc), P,
                                      C.POINTER(_PpbOut), C.c_int]
        L.oracle_lbvh.restype = None
        L.oracle_lbvh.argtypes = [P, P, P, P, u32, P, P, P, P, P, P]
        L.oracle_ppb_walk.restype = C.c_uint64
        L.oracle_ppb_walk.argtypes = [P, P, P, P, P, P, u32, P, P, P, u32, P, P, C.c_uint64]
        L._ppb_bound = True
    return L


def ppb_radius(r0, alpha, k) -> float:
    return _ppb_lib().oracle_ppb_radius(r0, alpha, k)


def lbvh(sorted_codes, order, seg_a, seg_b):
    n = len(sorted_codes)
    sc = np.ascontiguousarray(sorted_codes, np.uint32)
    od = np.ascontiguousarray(order, np.uint32)
    a = np.ascontiguousarray(seg_a, np.float32)
    b = np.ascontiguousarray(seg_b, np.float32)
    m = max(n - 1, 1)
    left, right = np.zeros(m, np.uint32), np.zeros(m, np.uint32)
    nlo, nhi = np.zeros((m, 4), np.float32), np.zeros((m, 4), np.float32)
    llo, lhi = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    _ppb_lib().oracle_lbvh(_p(sc), _p(od), _p(a), _p(b), n, _p(left), _p(right), _p(nlo), _p(nhi), _p(llo), _p(lhi))
    k = max(n - 1, 0)
    return dict(left=left[:k], right=right[:k], node_lo=nlo[:k], node_hi=nhi[:k], leaf_lo=llo, leaf_hi=lhi)


def ppb_walk(tree, origins, dirs, t01, cap=None):
    """The beam gather's walk over a tree from `lbvh` for each ray (origin,
    direction, [t0, t1]): (counts per ray, leaf indices visited, rays one
    after another in walk order)."""
    L = _ppb_lib()
    n = len(tree["leaf_lo"])
    k = max(n - 1, 1)

    def arr(key, shape, dt):
        a = np.zeros(shape, dt)
        v = np.asarray(tree[key], dt)
        a[:len(v)] = v
        return a

    left, right = arr("left", k, np.uint32), arr("right", k, np.uint32)
    nlo, nhi = arr("node_lo", (k, 4), np.float32), arr("node_hi", (k, 4), np.float32)
    llo = np.ascontiguousarray(tree["leaf_lo"], np.float32).reshape(-1, 4)
    lhi = np.ascontiguousarray(tree["leaf_hi"], np.float32).reshape(-1, 4)
    o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(t01, np.float32).reshape(-1, 2)
    m = len(o)
    counts = np.zeros(max(m, 1), np.uint32)
    cap = cap if cap is not None else max(1, n * max(m, 1))
    hits = np.zeros(cap, np.uint32)
    total = L.oracle_ppb_walk(_p(left), _p(right), _p(nlo), _p(nhi), _p(llo), _p(lhi), n, _p(o), _p(d), _p(t), m,
                              _p(counts), _p(hits), cap)
    assert total <= cap
    return counts[:m], hits[:total]


def ppb_pass(grid, cloud, cam, params, photons, capacity, r0, alpha, width, height, seed=0, pass_index=0,
             crop=(0, 0, 0, 0), flags=0, sum_img=None, level=2, threads=0, want_buffers=True):
    """One oracle photon-beam pass; returns (sum image, dict of buffers)."""
    L = _ppb_lib()
    if sum_img is None:
        sum_img = np.zeros((height, width, 3), np.float64)
    p = _abi.PassDesc()
    p.seed, p.pass_index, p.spp, p.flags = seed, pass_index, 1, flags
    for i in range(4):
        p.crop[i] = crop[i]
    K = min(params.max_events + 1, 65) if params.max_events else 65
    bufs = {}
    out = _PpbOut()
    nn = np.zeros(2, np.uint32)
    out.n = nn.ctypes.data
    out.capacity_out = capacity if want_buffers else 0
    if want_buffers:
        m = max(capacity - 1, 1)
        bufs = dict(slots=np.zeros((photons * K, 28), np.float32), nbeams=np.zeros(photons, np.uint32),
                    seg_a=np.zeros((capacity, 4), np.float32), seg_b=np.zeros((capacity, 4), np.float32),
                    seg_beam=np.zeros(capacity, np.uint32), codes=np.zeros(capacity, np.uint32),
                    order=np.zeros(capacity, np.uint32), left=np.zeros(m, np.uint32), right=np.zeros(m, np.uint32),
                    node_lo=np.zeros((m, 4), np.float32), node_hi=np.zeros((m, 4), np.float32),
                    leaf_lo=np.zeros((capacity, 4), np.float32), leaf_hi=np.zeros((capacity, 4), np.float32))
        for k, v in bufs.items():
            setattr(out, k, v.ctypes.data)
    L.oracle_ppb_pass(grid.h, level, C.byref(cloud), C.byref(cam), C.byref(params), photons, capacity, r0, alpha,
                      width, height, C.byref(p), _p(sum_img), C.byref(out), threads or os.cpu_count() or 1)
    n = int(nn[0])
    info = dict(segments=n, dropped=int(nn[1]))
    if want_buffers:
        for k in ("seg_a", "seg_b", "seg_beam", "codes", "order", "leaf_lo", "leaf_hi"):
            bufs[k] = bufs[k][:n]
        for k in ("left", "right", "node_lo", "node_hi"):
            bufs[k] = bufs[k][:max(n - 1, 0)]
    bufs["info"] = info
    return sum_img, bufs
