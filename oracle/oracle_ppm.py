"""ctypes binding of the oracle's photon-mapping restatement (test
infrastructure, see oracle.py)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import oracle as _o
from .oracle import _abi, _p

_bound = False


def _lib():
    global _bound
    L = _o.lib()
    if not _bound:
        P, u32, f = C.c_void_p, C.c_uint32, C.c_float
        L.oracle_ppm_pass.restype = C.c_int
        L.oracle_ppm_pass.argtypes = [P, C.c_int, C.POINTER(_abi.Cloud), C.POINTER(_abi.Camera),
                                      C.POINTER(_abi.Params), u32, u32, f, u32, u32, C.POINTER(_abi.PassDesc), P, P,
                                      P, P, P, P, P, P, C.c_int]
        L.oracle_ppm_march_pass.restype = C.c_int
        L.oracle_ppm_march_pass.argtypes = [P, C.c_int, C.POINTER(_abi.Cloud), C.POINTER(_abi.Camera),
                                            C.POINTER(_abi.Params), C.POINTER(_abi.ShadowVolume), P, u32, u32, f, f,
                                            f, f, u32, u32, C.POINTER(_abi.PassDesc), P, P, C.POINTER(f), C.c_int]
        L.oracle_ppm_tree_query.restype = C.c_uint64
        L.oracle_ppm_tree_query.argtypes = [P, u32, _abi.F3, _abi.F3, P, P, u32, P, P, C.c_uint64]
        _bound = True
    return L


def tree_query(positions, bmin, bmax, queries, radii, cap=None):
    """Photons within each query's radius, found by the gather's walk over
    the tree a pass builds on `positions`: (counts per query, input indices
    of the photons taken, queries one after another in walk order)."""
    L = _lib()
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    r = np.ascontiguousarray(radii, np.float32).reshape(-1)
    assert len(r) == len(q)
    counts = np.zeros(max(len(q), 1), np.uint32)
    cap = cap if cap is not None else max(1, len(pos) * max(len(q), 1))
    hits = np.zeros(cap, np.uint32)
    total = L.oracle_ppm_tree_query(_p(pos), len(pos), _abi.F3(*bmin), _abi.F3(*bmax), _p(q), _p(r), len(q),
                                    _p(counts), _p(hits), cap)
    assert total <= cap
    return counts[:len(q)], hits[:total]


def init_stats(width, height, r0):
    st = np.zeros((height, width, 8), np.float64)
    st[..., 1] = np.float32(r0)
    return st


def ppm_pass(grid, cloud, cam, params, photons, capacity, alpha, width, height, stats, sum_img=None, seed=0,
             pass_index=0, crop=(0, 0, 0, 0), level=2, threads=0, want_photons=False):
    """One oracle photon-mapping pass; updates `stats` in place."""
    L = _lib()
    if sum_img is None:
        sum_img = np.zeros((height, width, 3), np.float64)
    p = _abi.PassDesc()
    p.seed, p.pass_index, p.spp = seed, pass_index, 1
    for i in range(4):
        p.crop[i] = crop[i]
    nn = np.zeros(2, np.uint32)
    out = {}
    ph = uid = order = left = right = None
    if want_photons:
        out = dict(photons=np.zeros((capacity, 12), np.float32), uid=np.zeros(capacity, np.uint32),
                   order=np.zeros(capacity, np.uint32), left=np.zeros(capacity, np.uint32),
                   right=np.zeros(capacity, np.uint32))
        ph, uid, order, left, right = (_p(out[k]) for k in ("photons", "uid", "order", "left", "right"))
    L.oracle_ppm_pass(grid.h, level, C.byref(cloud), C.byref(cam), C.byref(params), photons, capacity, alpha, width,
                      height, C.byref(p), _p(stats), _p(sum_img), _p(nn), ph, uid, order, left, right,
                      threads or os.cpu_count() or 1)
    n = int(nn[0])
    info = dict(photons_stored=n, dropped=int(nn[1]))
    if want_photons:
        out["photons"] = out["photons"][:n]
        out["uid"] = out["uid"][:n]
        out["order"] = out["order"][:n]
        out["left"] = out["left"][:max(n - 1, 0)]
        out["right"] = out["right"][:max(n - 1, 0)]
    out["info"] = info
    return sum_img, out


def ppm_march_pass(grid, cloud, cam, params, sv, sv_tex, photons, capacity, r0, alpha, step, ambient_step, width,
                   height, sum_img=None, seed=0, pass_index=0, crop=(0, 0, 0, 0), level=2, threads=0):
    """One oracle pass of the reference's march estimate (VCR_PPM_MARCH);
    adds the pass's estimate to sum_img.  Returns (sum_img, stored photons,
    the pass's global radius)."""
    L = _lib()
    if sum_img is None:
        sum_img = np.zeros((height, width, 3), np.float64)
    p = _abi.PassDesc()
    p.seed, p.pass_index, p.spp = seed, pass_index, 1
    for i in range(4):
        p.crop[i] = crop[i]
    nn = np.zeros(2, np.uint32)
    r = C.c_float()
    tex = np.ascontiguousarray(sv_tex, np.float32)
    L.oracle_ppm_march_pass(grid.h, level, C.byref(cloud), C.byref(cam), C.byref(params), C.byref(sv), _p(tex),
                            photons, capacity, r0, alpha, step, ambient_step, width, height, C.byref(p),
                            _p(sum_img), _p(nn), C.byref(r), threads or os.cpu_count() or 1)
    return sum_img, int(nn[0]), float(r.value)
