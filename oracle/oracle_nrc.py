"""ctypes binding of the oracle's radiance-cache restatement (test
infrastructure, see oracle.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as _o
from .oracle import _p

RECORD = np.dtype([("p", np.float32, 3), ("v", np.float32, 3), ("s", np.float32, 3), ("w", np.float32, 3),
                   ("pix", np.uint32), ("pad", np.uint32, 3)])
assert RECORD.itemsize == 64

_bound = False


def _lib():
    global _bound
    L = _o.lib()
    if not _bound:
        P, u32 = C.c_void_p, C.c_uint32
        L.oracle_nrc_weight_count.restype = C.c_int
        L.oracle_nrc_encode.argtypes = [P, u32, P, P, P]
        L.oracle_nrc_forward.argtypes = [P, P, u32, P, P, P]
        L.oracle_nrc_gradient.restype = C.c_double
        L.oracle_nrc_gradient.argtypes = [P, P, u32, P, P, P]
        L.oracle_nrc_gradient_tables.restype = C.c_double
        L.oracle_nrc_gradient_tables.argtypes = [P, P, u32, P, P, P, P]
        L.oracle_nrc_set_grid.argtypes = [P]
        _bound = True
    return L


def weight_count() -> int:
    return _lib().oracle_nrc_weight_count()


def set_exact(exact: bool) -> None:
    """Exact mode drops the BF16 roundings (for finite differences)."""
    _lib().oracle_nrc_set_exact(1 if exact else 0)


def _box(cloud):
    b0 = np.array(cloud.bounds_min, np.float32)
    b1 = np.array(cloud.bounds_max, np.float32)
    inv = (np.float32(1.0) / (b1 - b0)).astype(np.float32)
    return b0, inv


def set_levels(levels: int) -> None:
    """Position levels the encoding computes (0..16, default 16), as the
    cache's 16 - position_drop; the inputs of the other levels are 0."""
    _lib().oracle_nrc_set_levels(int(levels))


GRID_PARAMS = 16 * (1 << 17) * 2

_grid_keep = None


def set_grid(tables) -> None:
    """The grid encoding's tables (16 x 2^17 x 2 floats, as the cache's
    parameters after its weights), or None for the frequency encoding."""
    global _grid_keep
    if tables is None:
        _grid_keep = None
        _lib().oracle_nrc_set_grid(None)
        return
    _grid_keep = np.ascontiguousarray(tables, np.float32)
    assert _grid_keep.size == GRID_PARAMS
    _lib().oracle_nrc_set_grid(_p(_grid_keep))


def gradient_tables(weights: np.ndarray, recs: np.ndarray, cloud):
    """(weight gradient, table gradient, loss) with the grid encoding set."""
    b0, inv = _box(cloud)
    g = np.zeros(weight_count(), np.float64)
    gt = np.zeros(GRID_PARAMS, np.float64)
    loss = _lib().oracle_nrc_gradient_tables(_p(np.ascontiguousarray(weights, np.float32)), _p(recs), len(recs),
                                             _p(b0), _p(inv), _p(g), _p(gt))
    return g, gt, loss


def encode(recs: np.ndarray, cloud) -> np.ndarray:
    b0, inv = _box(cloud)
    out = np.zeros((len(recs), 64), np.float32)
    _lib().oracle_nrc_encode(_p(recs), len(recs), _p(b0), _p(inv), _p(out))
    return out


def forward(weights: np.ndarray, recs: np.ndarray, cloud) -> np.ndarray:
    b0, inv = _box(cloud)
    out = np.zeros((len(recs), 3), np.float64)
    _lib().oracle_nrc_forward(_p(np.ascontiguousarray(weights, np.float32)), _p(recs), len(recs), _p(b0), _p(inv),
                              _p(out))
    return out


def gradient(weights: np.ndarray, recs: np.ndarray, cloud):
    b0, inv = _box(cloud)
    g = np.zeros(weight_count(), np.float64)
    loss = _lib().oracle_nrc_gradient(_p(np.ascontiguousarray(weights, np.float32)), _p(recs), len(recs), _p(b0),
                                      _p(inv), _p(g))
    return g, loss


def random_records(n, cloud, rng, sun=(0.866, -0.5, 0.0)) -> np.ndarray:
    r = np.zeros(n, RECORD)
    b0, b1 = np.array(cloud.bounds_min), np.array(cloud.bounds_max)
    r["p"] = b0 + (b1 - b0) * rng.random((n, 3))
    v = rng.normal(size=(n, 3))
    r["v"] = v / np.linalg.norm(v, axis=1, keepdims=True)
    s = np.array(sun, np.float64)
    r["s"] = s / np.linalg.norm(s)
    r["w"] = 0.05 + rng.random((n, 3)) * 0.5
    return r
