"""Python view of the vcr C-ABI (libvcr.so), used by the tests and bench.py.

The product is the C-ABI library and its C++ RenderTechnique classes; this
module only wraps the C entry points with numpy buffers for convenience.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import *  # noqa: F401,F403  (struct and enum names)
from ._abi import check, lib


def _ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"], "buffers must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


def grid_desc(size, voxel_size) -> _abi.GridDesc:
    d = _abi.GridDesc()
    for a in range(3):
        d.size[a] = int(size[a])
        d.voxel_size[a] = float(voxel_size[a])
    return d


def fbm_desc(seed=1, octaves=6, lacunarity=2.0, gain=0.5, base_frequency=4.0) -> _abi.FbmDesc:
    f = _abi.FbmDesc()
    f.seed, f.octaves, f.lacunarity, f.gain, f.base_frequency = seed, octaves, lacunarity, gain, base_frequency
    return f


def fbm_fill_host(size, fbm: _abi.FbmDesc) -> np.ndarray:
    """The generator on the host (same float arithmetic as the device kernel)."""
    out = np.empty((size[2], size[1], size[0]), np.float32)
    check(lib().vcr_fbm_fill_host(C.byref(grid_desc(size, (1, 1, 1))), C.byref(fbm), _ptr(out)))
    return out


def set_wait_limits(sort_lookback=None, stage_wait=None) -> None:
    """Process-wide limits of the device-side waits (vcr_set_wait_limits);
    no arguments restore the defaults."""
    if sort_lookback is None and stage_wait is None:
        check(lib().vcr_set_wait_limits(None))
        return
    cur = wait_limits()
    w = _abi.WaitLimits(cur["sort_lookback"] if sort_lookback is None else sort_lookback,
                        cur["stage_wait"] if stage_wait is None else stage_wait)
    check(lib().vcr_set_wait_limits(C.byref(w)))


def wait_limits() -> dict:
    w = _abi.WaitLimits()
    check(lib().vcr_get_wait_limits(C.byref(w)))
    return {"sort_lookback": w.sort_lookback, "stage_wait": w.stage_wait}


def params_set_phase_g(p: _abi.Params, g: float) -> None:
    check(lib().vcr_params_set_phase_g(C.byref(p), g))


def cloud_from_grid(desc: _abi.GridDesc, base_scaling: float, density_scaling: float) -> _abi.Cloud:
    c = _abi.Cloud()
    check(lib().vcr_cloud_from_grid(C.byref(desc), base_scaling, density_scaling, C.byref(c)))
    return c


def camera_look(position, forward, fov_y_deg, near_plane, width, height) -> _abi.Camera:
    cam = _abi.Camera()
    check(lib().vcr_camera_look(C.byref(cam), _abi.F3(*position), _abi.F3(*forward), fov_y_deg, near_plane,
                                int(width), int(height)))
    return cam


def shadow_volume_setup(light_dir, bmin, bmax, n) -> _abi.ShadowVolume:
    sv = _abi.ShadowVolume()
    check(lib().vcr_shadow_volume_setup(C.byref(sv), _abi.F3(*light_dir), _abi.F3(*bmin), _abi.F3(*bmax), n))
    return sv


def xyz_write(path: str, desc: _abi.GridDesc, data: np.ndarray) -> None:
    data = np.ascontiguousarray(data, np.float32)
    check(lib().vcr_xyz_write(path.encode(), C.byref(desc), _ptr(data)))


def xyz_read(path: str):
    desc = _abi.GridDesc()
    check(lib().vcr_xyz_read(path.encode(), C.byref(desc), None, 0))
    out = np.empty((desc.size[2], desc.size[1], desc.size[0]), np.float32)
    check(lib().vcr_xyz_read(path.encode(), C.byref(desc), _ptr(out), out.size))
    return desc, out


def write_png(path: str, rgba: np.ndarray) -> None:
    """8-bit RGBA image [H, W, 4] as a PNG file (zlib from the standard
    library; filter 0 on every row)."""
    import struct
    import zlib
    img = np.ascontiguousarray(rgba, np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("write_png wants an [H, W, 4] uint8 array")
    h, w = img.shape[:2]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def write_exr(path: str, rgb: np.ndarray, half: bool = False) -> None:
    """HDR image [H, W, 3] (float; the mean image) as an uncompressed
    OpenEXR file with FLOAT or, with half=True, HALF channels
    (vcr_write_exr)."""
    img = np.ascontiguousarray(rgb, np.float32)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("write_exr wants an [H, W, 3] float array")
    h, w = img.shape[:2]
    check(lib().vcr_write_exr(path.encode(), w, h, _ptr(img), _abi.EXR_HALF if half else _abi.EXR_FLOAT))


class Context:
    """One vcr_ctx: owns the device grid, frame sums and scratch."""

    def __init__(self, device: int = 0):
        L = lib()
        h = C.c_void_p()
        d = _abi.DeviceDesc(device, 0)
        check(L.vcr_create(C.byref(h), C.byref(d)))
        self.h = h
        self.width = self.height = 0
        self.grid_size = (0, 0, 0)

    def close(self):
        if self.h:
            lib().vcr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        check(st, self.h)

    # grid -------------------------------------------------------------------
    def grid_upload(self, desc, dense: np.ndarray, precision=_abi.PREC_FP32):
        dense = np.ascontiguousarray(dense, np.float32)
        self._ck(lib().vcr_grid_upload(self.h, C.byref(desc), _ptr(dense), precision))
        self.grid_size = tuple(desc.size)

    def grid_generate(self, desc, fbm, precision=_abi.PREC_FP32):
        self._ck(lib().vcr_grid_generate(self.h, C.byref(desc), C.byref(fbm), precision))
        self.grid_size = tuple(desc.size)

    def grid_read_dense(self) -> np.ndarray:
        """The stored grid decoded to dense floats [Z, Y, X] (what the
        trackers sample)."""
        X, Y, Z = self.grid_size
        out = np.empty((Z, Y, X), np.float32)
        self._ck(lib().vcr_grid_read_dense(self.h, _ptr(out), out.size))
        return out

    def grid_info(self):
        m = C.c_float()
        nb = (C.c_uint32 * 3)()
        self._ck(lib().vcr_grid_info(self.h, C.byref(m), nb))
        return m.value, tuple(nb)

    def majorants(self, level: int = 0) -> np.ndarray:
        _, nb = self.grid_info()
        d = list(nb)
        for _ in range(level):
            d = [(x + 1) // 2 for x in d]
        out = np.empty(d[0] * d[1] * d[2], np.float32)
        self._ck(lib().vcr_grid_read_majorants(self.h, level, _ptr(out), out.size))
        return out

    def set_tuning(self, majorant_level=2, dda_steps=4, stage_majorants=1, block_threads=256, corner_blocks=1,
                   fast_math=0):
        t = _abi.Tuning(majorant_level, dda_steps, stage_majorants, block_threads, corner_blocks, fast_math)
        self._ck(lib().vcr_set_tuning(self.h, C.byref(t)))

    def get_tuning(self) -> dict:
        t = _abi.Tuning()
        self._ck(lib().vcr_get_tuning(self.h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in _abi.Tuning._fields_}

    def autotune(self, seed=0, pass_index=0, spp=1, stream=0) -> dict:
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, spp
        t = _abi.Tuning()
        self._ck(lib().vcr_autotune_pt(self.h, C.byref(p), C.byref(t), C.c_void_p(stream)))
        return {f: getattr(t, f) for f, _ in _abi.Tuning._fields_}

    def grid_sample(self, d_pos: int, d_out: int, n: int, stream: int = 0):
        self._ck(lib().vcr_grid_sample(self.h, C.c_void_p(d_pos), C.c_void_p(d_out), n, C.c_void_p(stream)))

    # scene ------------------------------------------------------------------
    def set_cloud(self, cloud):
        self._ck(lib().vcr_set_cloud(self.h, C.byref(cloud)))

    def set_camera(self, cam):
        self._ck(lib().vcr_set_camera(self.h, C.byref(cam)))

    def set_params(self, p):
        self._ck(lib().vcr_set_params(self.h, C.byref(p)))

    def set_frame(self, w, h):
        self._ck(lib().vcr_set_frame(self.h, w, h))
        self.width, self.height = w, h

    def reset(self):
        self._ck(lib().vcr_reset_accumulation(self.h))

    def shadow_volume_build(self, sv, stream=0):
        self._ck(lib().vcr_shadow_volume_build(self.h, C.byref(sv), C.c_void_p(stream)))

    # passes -----------------------------------------------------------------
    def pt_pass(self, seed=0, pass_index=0, spp=1, crop=(0, 0, 0, 0), flags=0, stream=0):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp, p.flags = seed, pass_index, spp, flags
        for i in range(4):
            p.crop[i] = crop[i]
        self._ck(lib().vcr_pt_pass(self.h, C.byref(p), C.c_void_p(stream)))

    def pt_passes(self, seed=0, first=0, count=1, spp=1, crop=(0, 0, 0, 0), stream=0):
        """`count` consecutive passes (first, first + 1, ...) in one launch."""
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp, p.flags = seed, first, spp, 0
        for i in range(4):
            p.crop[i] = crop[i]
        self._ck(lib().vcr_pt_passes(self.h, C.byref(p), count, C.c_void_p(stream)))

    def counters(self):
        out = (C.c_uint64 * 4)()
        self._ck(lib().vcr_pt_counters(self.h, out))
        return tuple(out)

    def dda_trace(self, d_o, d_d, n, max_cells, d_cells, d_t, d_count, stream=0):
        self._ck(lib().vcr_dda_trace(self.h, C.c_void_p(d_o), C.c_void_p(d_d), n, max_cells, C.c_void_p(d_cells),
                                     C.c_void_p(d_t), C.c_void_p(d_count), C.c_void_p(stream)))

    def synchronize(self):
        self._ck(lib().vcr_synchronize(self.h))

    # radiance cache ---------------------------------------------------------
    NRC_WEIGHTS = 21504

    def nrc_setup(self, train_samples=65536, learning_rate=1e-3, query_capacity=1 << 21, seed=1, ema_decay=0.0,
                  tail_survival=0.0, query_kernel=0, position_levels=16, encoding=_abi.NRC_ENCODING_FREQUENCY):
        p = _abi.NrcParams(train_samples, learning_rate, query_capacity, seed, ema_decay, tail_survival, query_kernel,
                           16 - position_levels, encoding)
        self._ck(lib().vcr_nrc_setup(self.h, C.byref(p)))

    def nrc_free(self):
        self._ck(lib().vcr_nrc_free(self.h))

    def nrc_train_step(self, seed=0, pass_index=0, stream=0, sets=1):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, sets
        self._ck(lib().vcr_nrc_train_step(self.h, C.byref(p), C.c_void_p(stream)))

    def nrc_frame(self, seed=0, pass_index=0, spp=1, stream=0):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, spp
        self._ck(lib().vcr_nrc_frame(self.h, C.byref(p), C.c_void_p(stream)))

    def nrc_train_more(self, steps, max_records=0, stream=0):
        self._ck(lib().vcr_nrc_train_more(self.h, steps, max_records, C.c_void_p(stream)))

    def nrc_set_learning_rate(self, learning_rate):
        self._ck(lib().vcr_nrc_set_learning_rate(self.h, learning_rate))

    def nrc_info(self) -> dict:
        i = _abi.NrcInfo()
        self._ck(lib().vcr_nrc_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in _abi.NrcInfo._fields_}

    def nrc_get_weights(self, tables=False) -> np.ndarray:
        """The network's weights; with tables=True (grid encoding) followed
        by the encoding's tables (nrc_info()["weights"] values in all)."""
        w = np.empty(self.nrc_info()["weights"] if tables else self.NRC_WEIGHTS, np.float32)
        self._ck(lib().vcr_nrc_get_weights(self.h, _ptr(w), w.size))
        return w

    def nrc_set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        self._ck(lib().vcr_nrc_set_weights(self.h, _ptr(w), w.size))

    def nrc_forward(self, d_records, n, d_out, stream=0):
        self._ck(lib().vcr_nrc_forward(self.h, C.c_void_p(d_records), n, C.c_void_p(d_out), C.c_void_p(stream)))

    def nrc_fit(self, d_records, n, steps, stream=0):
        self._ck(lib().vcr_nrc_fit(self.h, C.c_void_p(d_records), n, steps, C.c_void_p(stream)))

    def nrc_gradient(self, d_records, n, tables=False):
        g = np.empty(self.nrc_info()["weights"] if tables else self.NRC_WEIGHTS, np.float32)
        loss = C.c_float()
        self._ck(lib().vcr_nrc_gradient(self.h, C.c_void_p(d_records), n, _ptr(g), g.size, C.byref(loss)))
        return g, loss.value

    # checkpoints ------------------------------------------------------------
    def checkpoint_save(self, path):
        self._ck(lib().vcr_checkpoint_save(self.h, os.fsencode(path)))

    def checkpoint_load(self, path):
        self._ck(lib().vcr_checkpoint_load(self.h, os.fsencode(path)))

    # batched views ----------------------------------------------------------
    def batch_setup(self, views):
        """views: list of (camera, width, height, sun_dir)."""
        arr = (_abi.ViewDesc * len(views))()
        for i, (cam, w, h, sun) in enumerate(views):
            arr[i].camera = cam
            arr[i].width, arr[i].height = w, h
            for a in range(3):
                arr[i].sun_dir[a] = sun[a]
        self._batch_sizes = [(w, h) for _, w, h, _ in views]
        self._ck(lib().vcr_batch_setup(self.h, arr, len(views)))

    def batch_free(self):
        self._ck(lib().vcr_batch_free(self.h))

    def batch_pass(self, seed=0, pass_index=0, spp=1, stream=0):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, spp
        self._ck(lib().vcr_batch_pass(self.h, C.byref(p), C.c_void_p(stream)))

    def batch_graph_record(self, seed=0, pass_index=0, spp=1):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, spp
        self._ck(lib().vcr_batch_graph_record(self.h, C.byref(p)))

    def batch_graph_replay(self, count, stream=0):
        self._ck(lib().vcr_batch_graph_replay(self.h, count, C.c_void_p(stream)))

    def batch_autotune(self, seed=0, pass_index=0, spp=1, stream=0) -> dict:
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, spp
        t = _abi.Tuning()
        self._ck(lib().vcr_batch_autotune(self.h, C.byref(p), C.byref(t), C.c_void_p(stream)))
        return {f: getattr(t, f) for f, _ in _abi.Tuning._fields_}

    def batch_read(self, view) -> np.ndarray:
        w, h = self._batch_sizes[view]
        out = np.empty((h, w, 3), np.float64)
        self._ck(lib().vcr_batch_read(self.h, view, _ptr(out), out.nbytes))
        return out

    def batch_info(self) -> dict:
        i = _abi.BatchInfo()
        self._ck(lib().vcr_batch_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in _abi.BatchInfo._fields_}

    def batch_reset(self):
        self._ck(lib().vcr_batch_reset(self.h))

    # photon mapping ---------------------------------------------------------
    def ppm_setup(self, photons, capacity, radius, alpha=0.7, estimator=0, march_step=0.0, ambient_step=0.0):
        p = _abi.PpmParams(photons, capacity, radius, alpha, estimator, march_step, ambient_step)
        self._ck(lib().vcr_ppm_setup(self.h, C.byref(p)))

    def ppm_free(self):
        self._ck(lib().vcr_ppm_free(self.h))

    def ppm_pass(self, seed=0, pass_index=0, crop=(0, 0, 0, 0), stream=0):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp = seed, pass_index, 1
        for i in range(4):
            p.crop[i] = crop[i]
        self._ck(lib().vcr_ppm_pass(self.h, C.byref(p), C.c_void_p(stream)))

    def ppm_info(self) -> dict:
        i = _abi.PpmInfo()
        self._ck(lib().vcr_ppm_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in _abi.PpmInfo._fields_}

    def ppm_read(self, name) -> np.ndarray:
        n = self.ppm_info()["photons_stored"]
        shapes = {"stats": (self.height, self.width, 8), "pos": (n, 4), "power": (n, 4), "dir": (n, 4),
                  "uid": (n,), "order": (n,), "left": (max(n - 1, 0),), "right": (max(n - 1, 0),)}
        dt = {"stats": np.float64, "pos": np.float32, "power": np.float32, "dir": np.float32}.get(name, np.uint32)
        out = np.empty(shapes[name], dt)
        self._ck(lib().vcr_ppm_read(self.h, _abi.PPM_BUFFERS[name], _ptr(out) if out.size else C.c_void_p(1),
                                    out.nbytes))
        return out

    # photon beams -----------------------------------------------------------
    def ppb_setup(self, photons, capacity, radius, alpha=0.8):
        p = _abi.PpbParams(photons, capacity, radius, alpha)
        self._ck(lib().vcr_ppb_setup(self.h, C.byref(p)))

    def ppb_free(self):
        self._ck(lib().vcr_ppb_free(self.h))

    def ppb_pass(self, seed=0, pass_index=0, crop=(0, 0, 0, 0), flags=0, stream=0):
        p = _abi.PassDesc()
        p.seed, p.pass_index, p.spp, p.flags = seed, pass_index, 1, flags
        for i in range(4):
            p.crop[i] = crop[i]
        self._ck(lib().vcr_ppb_pass(self.h, C.byref(p), C.c_void_p(stream)))

    def ppb_info(self) -> dict:
        i = _abi.PpbInfo()
        self._ck(lib().vcr_ppb_info(self.h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in _abi.PpbInfo._fields_}

    def gather_stats(self, technique):
        """(candidates the last pass's gather tested, its device ms) for
        technique "ppm" (leaf photons) or "ppb" (pixel-segment pairs)."""
        c, ms = C.c_uint64(), C.c_float()
        fn = lib().vcr_ppm_gather_stats if technique == "ppm" else lib().vcr_ppb_gather_stats
        self._ck(fn(self.h, C.byref(c), C.byref(ms)))
        return int(c.value), float(ms.value)

    def ppb_read(self, name, photons=None) -> np.ndarray:
        info = self.ppb_info()
        n, K = info["segments"], info["beam_slots"]
        shapes = {"slots": ((photons or 0) * K, 28), "nbeams": (photons or 0,), "seg_a": (n, 4), "seg_b": (n, 4),
                  "seg_beam": (n,), "codes": (n,), "order": (n,), "left": (max(n - 1, 0),),
                  "right": (max(n - 1, 0),), "node_lo": (max(n - 1, 0), 4), "node_hi": (max(n - 1, 0), 4),
                  "leaf_lo": (n, 4), "leaf_hi": (n, 4)}
        dt = np.float32 if name in ("slots", "seg_a", "seg_b", "node_lo", "node_hi", "leaf_lo", "leaf_hi") \
            else np.uint32
        out = np.empty(shapes[name], dt)
        self._ck(lib().vcr_ppb_read(self.h, _abi.PPB_BUFFERS[name], _ptr(out) if out.size else C.c_void_p(1),
                                    out.nbytes))
        return out

    def lbvh_build(self, d_codes, d_order, d_seg_a, d_seg_b, n, d_left, d_right, d_nlo, d_nhi, d_llo, d_lhi,
                   stream=0):
        v = C.c_void_p
        self._ck(lib().vcr_lbvh_build(self.h, v(d_codes), v(d_order), v(d_seg_a), v(d_seg_b), n, v(d_left),
                                      v(d_right), v(d_nlo), v(d_nhi), v(d_llo), v(d_lhi), v(stream)))

    # beam ordering primitives (device pointers) -----------------------------
    def radix_sort_pairs(self, d_kin, d_vin, d_kout, d_vout, n, begin_bit=0, end_bit=32, stream=0):
        self._ck(lib().vcr_radix_sort_pairs(self.h, C.c_void_p(d_kin), C.c_void_p(d_vin or 0) if d_vin else None,
                                            C.c_void_p(d_kout), C.c_void_p(d_vout), n, begin_bit, end_bit,
                                            C.c_void_p(stream)))

    def morton_codes(self, d_pts, n, bmin, bmax, bits, d_codes, stream=0):
        self._ck(lib().vcr_morton_codes(self.h, C.c_void_p(d_pts), n, _abi.F3(*bmin), _abi.F3(*bmax), bits,
                                        C.c_void_p(d_codes), C.c_void_p(stream)))

    # read back --------------------------------------------------------------
    def image_mean(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), np.float32)
        self._ck(lib().vcr_readback(self.h, _abi.BUF_IMAGE_MEAN, _ptr(out), out.nbytes))
        return out

    def image_sum(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), np.float64)
        self._ck(lib().vcr_readback(self.h, _abi.BUF_IMAGE_SUM, _ptr(out), out.nbytes))
        return out

    def path_stats(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.uint32)
        self._ck(lib().vcr_readback(self.h, _abi.BUF_PATH_STATS, _ptr(out), out.nbytes))
        return out

    def shadow_volume(self, n) -> np.ndarray:
        out = np.empty((n, n, n), np.float32)
        self._ck(lib().vcr_readback(self.h, _abi.BUF_SHADOW_VOLUME, _ptr(out), out.nbytes))
        return out

    def display(self, exposure=1.0, order=_abi.ORDER_RGBA, stream=0) -> np.ndarray:
        """The display image (uint8 [H, W, 4]): the accumulated mean, clamped,
        sRGB-encoded, as the reference's swapchain blit shows it."""
        out = np.empty((self.height, self.width, 4), np.uint8)
        d = _abi.DisplayDesc(exposure, order)
        self._ck(lib().vcr_display(self.h, C.byref(d), _ptr(out), out.nbytes, C.c_void_p(stream)))
        return out

    def display_to(self, d_ptr, exposure=1.0, order=_abi.ORDER_RGBA, stream=0):
        """The display image into device memory (stream-ordered)."""
        d = _abi.DisplayDesc(exposure, order)
        self._ck(lib().vcr_display(self.h, C.byref(d), C.c_void_p(d_ptr), self.width * self.height * 4,
                                   C.c_void_p(stream)))

    def readback_to(self, buf_id, d_ptr, nbytes):
        """Copy a context buffer into caller memory (host or device)."""
        self._ck(lib().vcr_readback(self.h, buf_id, C.c_void_p(d_ptr), nbytes))

    def readback_async(self, buf_id, host_ptr, nbytes, stream=0):
        """Stream-ordered read back of the mean or sum image into pinned host
        memory (lands by readback_wait)."""
        self._ck(lib().vcr_readback_async(self.h, buf_id, C.c_void_p(host_ptr), nbytes, C.c_void_p(stream)))

    def readback_wait(self):
        self._ck(lib().vcr_readback_wait(self.h))

    def image_rel_rmse(self, d_ref, d_out, stream=0):
        self._ck(lib().vcr_image_rel_rmse(self.h, C.c_void_p(d_ref), C.c_void_p(d_out), C.c_void_p(stream)))

    def pass_count(self) -> int:
        v = C.c_uint32()
        self._ck(lib().vcr_pass_count(self.h, C.byref(v)))
        return v.value
