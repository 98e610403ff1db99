"""ctypes mirror of include/vcr/abi.h.

The shared library is loaded from the package directory; there is no
fallback: if libvcr.so is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libvcr.so")

# status codes
OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_STATE, ERR_IO, ERR_UNSUPPORTED, ERR_CAPACITY = range(9)
STATUS_NAMES = ["OK", "INVALID", "CUDA", "OOM", "TIMEOUT", "STATE", "IO", "UNSUPPORTED", "CAPACITY"]

PREC_FP32, PREC_FP16, PREC_BF16 = 0, 1, 2
RNG_PCG, RNG_XORSHIFT = 0, 1
NEE_RATIO, NEE_SHADOW_VOLUME = 0, 1
SKY_CONSTANT, SKY_GRADIENT = 0, 1
TRACKER_GLOBAL, TRACKER_DDA = 0, 1
BUF_IMAGE_MEAN, BUF_IMAGE_SUM, BUF_PATH_STATS, BUF_PPM_STATS, BUF_SHADOW_VOLUME = range(5)
ORDER_RGBA, ORDER_BGRA = range(2)
PASS_RECORD_STATS, PASS_NO_ACCUMULATE = 1, 2
NRC_QUERY_DEFAULT, NRC_QUERY_MMA, NRC_QUERY_TCGEN05 = 0, 1, 2
NRC_ENCODING_FREQUENCY, NRC_ENCODING_GRID = 0, 1
PPM_GATHER, PPM_MARCH = 0, 1
EXR_HALF, EXR_FLOAT = 1, 2

F3 = C.c_float * 3


class DeviceDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32)]


class GridDesc(C.Structure):
    _fields_ = [("size", C.c_uint32 * 3), ("_pad", C.c_uint32), ("voxel_size", C.c_double * 3)]


class Cloud(C.Structure):
    _fields_ = [("bounds_min", F3), ("bounds_max", F3), ("max_extinction", C.c_float),
                ("base_scaling", C.c_float), ("density_scaling", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("position", F3), ("forward", F3), ("right", F3), ("up", F3), ("near_plane", C.c_float),
                ("pixel_size_x", C.c_float), ("pixel_size_y", C.c_float), ("half_width", C.c_int32),
                ("half_height", C.c_int32)]


class Params(C.Structure):
    _fields_ = [("max_events", C.c_uint32), ("light_intensity", C.c_float), ("phase_g", C.c_float),
                ("phase_one_plus_g2", C.c_float), ("phase_one_minus_g2", C.c_float),
                ("phase_one_over_2g", C.c_float), ("isotropic", C.c_int32), ("albedo", C.c_float),
                ("sun_dir", F3), ("sky", F3), ("sky_mode", C.c_uint32), ("rng_mode", C.c_uint32),
                ("nee_mode", C.c_uint32), ("tracker", C.c_uint32), ("nrc_events", C.c_uint32)]


class ShadowVolume(C.Structure):
    _fields_ = [("bounds_min", F3), ("bounds_max", F3), ("light_dir", F3), ("right", F3), ("up", F3),
                ("basis_change", C.c_float * 9), ("voxel_axis_count", C.c_uint32), ("voxel_size", C.c_float)]


class DisplayDesc(C.Structure):
    _fields_ = [("exposure", C.c_float), ("order", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class Tuning(C.Structure):
    _fields_ = [("majorant_level", C.c_uint32), ("dda_steps", C.c_uint32), ("stage_majorants", C.c_uint32),
                ("block_threads", C.c_uint32), ("corner_blocks", C.c_uint32),
                ("fast_math", C.c_uint32)]


class ViewDesc(C.Structure):
    _fields_ = [("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32), ("sun_dir", F3),
                ("reserved", C.c_uint32)]


class BatchInfo(C.Structure):
    _fields_ = [("views", C.c_uint32), ("passes", C.c_uint32), ("pixels", C.c_uint64), ("samples", C.c_uint64)]


class NrcParams(C.Structure):
    _fields_ = [("train_samples", C.c_uint32), ("learning_rate", C.c_float), ("query_capacity", C.c_uint32),
                ("seed", C.c_uint32), ("ema_decay", C.c_float), ("tail_survival", C.c_float),
                ("query_kernel", C.c_uint32), ("position_drop", C.c_uint32), ("encoding", C.c_uint32)]


class NrcInfo(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("last_loss", C.c_float), ("train_records", C.c_uint32),
                ("queries", C.c_uint32), ("weights", C.c_uint32)]


class PpmParams(C.Structure):
    _fields_ = [("photons", C.c_uint32), ("capacity", C.c_uint32), ("radius", C.c_float), ("alpha", C.c_float),
                ("estimator", C.c_uint32), ("march_step", C.c_float), ("ambient_step", C.c_float)]


class PpmInfo(C.Structure):
    _fields_ = [("photons_stored", C.c_uint32), ("dropped", C.c_uint32)]


PPM_BUFFERS = {"stats": 0, "pos": 1, "power": 2, "dir": 3, "uid": 4, "order": 5, "left": 6, "right": 7}


class PpbParams(C.Structure):
    _fields_ = [("photons", C.c_uint32), ("capacity", C.c_uint32), ("radius", C.c_float), ("alpha", C.c_float)]


class PpbInfo(C.Structure):
    _fields_ = [("segments", C.c_uint32), ("dropped", C.c_uint32), ("radius", C.c_float), ("beam_slots", C.c_uint32)]


PPB_BUFFERS = {"slots": 0, "nbeams": 1, "seg_a": 2, "seg_b": 3, "seg_beam": 4, "codes": 5, "order": 6, "left": 7,
               "right": 8, "node_lo": 9, "node_hi": 10, "leaf_lo": 11, "leaf_hi": 12}


class PassDesc(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("pass_index", C.c_uint32), ("spp", C.c_uint32),
                ("crop", C.c_uint32 * 4), ("flags", C.c_uint32)]


class WaitLimits(C.Structure):
    _fields_ = [("sort_lookback", C.c_uint32), ("stage_wait", C.c_uint32)]


class FbmDesc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("octaves", C.c_uint32), ("lacunarity", C.c_float), ("gain", C.c_float),
                ("base_frequency", C.c_float)]


_P = C.c_void_p
_S = C.c_int  # vcr_status
_u32, _u64, _f, _sz = C.c_uint32, C.c_uint64, C.c_float, C.c_size_t

# name -> (restype, argtypes).  The list is also the set of symbols the
# header declares; tests check that every one is exported.
SIGNATURES = {
    "vcr_create": (_S, [C.POINTER(_P), C.POINTER(DeviceDesc)]),
    "vcr_destroy": (_S, [_P]),
    "vcr_last_error": (C.c_char_p, [_P]),
    "vcr_version": (_u32, []),
    "vcr_synchronize": (_S, [_P]),
    "vcr_set_wait_limits": (_S, [C.POINTER(WaitLimits)]),
    "vcr_get_wait_limits": (_S, [C.POINTER(WaitLimits)]),
    "vcr_params_set_phase_g": (_S, [C.POINTER(Params), _f]),
    "vcr_cloud_from_grid": (_S, [C.POINTER(GridDesc), _f, _f, C.POINTER(Cloud)]),
    "vcr_camera_look": (_S, [C.POINTER(Camera), F3, F3, _f, _f, C.c_int32, C.c_int32]),
    "vcr_shadow_volume_setup": (_S, [C.POINTER(ShadowVolume), F3, F3, F3, _u32]),
    "vcr_grid_upload": (_S, [_P, C.POINTER(GridDesc), _P, C.c_int]),
    "vcr_grid_generate": (_S, [_P, C.POINTER(GridDesc), C.POINTER(FbmDesc), C.c_int]),
    "vcr_grid_info": (_S, [_P, C.POINTER(_f), C.POINTER(_u32)]),
    "vcr_grid_read_majorants": (_S, [_P, _u32, _P, _sz]),
    "vcr_set_tuning": (_S, [_P, C.POINTER(Tuning)]),
    "vcr_get_tuning": (_S, [_P, C.POINTER(Tuning)]),
    "vcr_autotune_pt": (_S, [_P, C.POINTER(PassDesc), C.POINTER(Tuning), _P]),
    "vcr_grid_sample": (_S, [_P, _P, _P, _u32, _P]),
    "vcr_xyz_read": (_S, [C.c_char_p, C.POINTER(GridDesc), _P, _sz]),
    "vcr_xyz_write": (_S, [C.c_char_p, C.POINTER(GridDesc), _P]),
    "vcr_fbm_fill_host": (_S, [C.POINTER(GridDesc), C.POINTER(FbmDesc), _P]),
    "vcr_set_cloud": (_S, [_P, C.POINTER(Cloud)]),
    "vcr_set_camera": (_S, [_P, C.POINTER(Camera)]),
    "vcr_set_params": (_S, [_P, C.POINTER(Params)]),
    "vcr_set_frame": (_S, [_P, _u32, _u32]),
    "vcr_reset_accumulation": (_S, [_P]),
    "vcr_shadow_volume_build": (_S, [_P, C.POINTER(ShadowVolume), _P]),
    "vcr_pt_pass": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_pt_passes": (_S, [_P, C.POINTER(PassDesc), _u32, _P]),
    "vcr_pt_counters": (_S, [_P, C.POINTER(_u64)]),
    "vcr_dda_trace": (_S, [_P, _P, _P, _u32, _u32, _P, _P, _P, _P]),
    "vcr_nrc_setup": (_S, [_P, C.POINTER(NrcParams)]),
    "vcr_nrc_free": (_S, [_P]),
    "vcr_nrc_train_step": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_nrc_frame": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_nrc_train_more": (_S, [_P, _u32, _u32, _P]),
    "vcr_nrc_set_learning_rate": (_S, [_P, C.c_float]),
    "vcr_nrc_info": (_S, [_P, C.POINTER(NrcInfo)]),
    "vcr_nrc_get_weights": (_S, [_P, _P, _sz]),
    "vcr_nrc_set_weights": (_S, [_P, _P, _sz]),
    "vcr_nrc_forward": (_S, [_P, _P, _u32, _P, _P]),
    "vcr_nrc_gradient": (_S, [_P, _P, _u32, _P, _sz, C.POINTER(_f)]),
    "vcr_nrc_fit": (_S, [_P, _P, _u32, _u32, _P]),
    "vcr_checkpoint_save": (_S, [_P, C.c_char_p]),
    "vcr_checkpoint_load": (_S, [_P, C.c_char_p]),
    "vcr_batch_setup": (_S, [_P, C.POINTER(ViewDesc), _u32]),
    "vcr_batch_free": (_S, [_P]),
    "vcr_batch_pass": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_batch_graph_record": (_S, [_P, C.POINTER(PassDesc)]),
    "vcr_batch_graph_replay": (_S, [_P, _u32, _P]),
    "vcr_batch_autotune": (_S, [_P, C.POINTER(PassDesc), C.POINTER(Tuning), _P]),
    "vcr_batch_read": (_S, [_P, _u32, _P, _sz]),
    "vcr_batch_info": (_S, [_P, C.POINTER(BatchInfo)]),
    "vcr_batch_reset": (_S, [_P]),
    "vcr_ppm_setup": (_S, [_P, C.POINTER(PpmParams)]),
    "vcr_ppm_free": (_S, [_P]),
    "vcr_ppm_pass": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_ppm_info": (_S, [_P, C.POINTER(PpmInfo)]),
    "vcr_ppm_gather_stats": (_S, [_P, C.POINTER(_u64), C.POINTER(_f)]),
    "vcr_ppm_read": (_S, [_P, C.c_int, _P, _sz]),
    "vcr_ppb_setup": (_S, [_P, C.POINTER(PpbParams)]),
    "vcr_ppb_free": (_S, [_P]),
    "vcr_ppb_pass": (_S, [_P, C.POINTER(PassDesc), _P]),
    "vcr_ppb_info": (_S, [_P, C.POINTER(PpbInfo)]),
    "vcr_ppb_gather_stats": (_S, [_P, C.POINTER(_u64), C.POINTER(_f)]),
    "vcr_ppb_read": (_S, [_P, C.c_int, _P, _sz]),
    "vcr_lbvh_build": (_S, [_P, _P, _P, _P, _P, _u32, _P, _P, _P, _P, _P, _P, _P]),
    "vcr_radix_sort_pairs": (_S, [_P, _P, _P, _P, _P, _u32, _u32, _u32, _P]),
    "vcr_radix_sort_pairs_noalloc": (_S, [_P, _P, _P, _P, _u32, _u32, _u32, _P]),
    "vcr_sort_noalloc_status": (_S, [_P]),
    "vcr_morton_codes": (_S, [_P, _P, _u32, F3, F3, _u32, _P, _P]),
    "vcr_readback": (_S, [_P, C.c_int, _P, _sz]),
    "vcr_readback_async": (_S, [_P, C.c_int, _P, _sz, _P]),
    "vcr_readback_wait": (_S, [_P]),
    "vcr_display": (_S, [_P, C.POINTER(DisplayDesc), _P, _sz, _P]),
    "vcr_grid_read_dense": (_S, [_P, _P, _sz]),
    "vcr_pass_count": (_S, [_P, C.POINTER(_u32)]),
    "vcr_image_rel_rmse": (_S, [_P, _P, _P, _P]),
    "vcr_write_exr": (_S, [C.c_char_p, _u32, _u32, _P, _u32]),
    "vcr_write_png": (_S, [C.c_char_p, _u32, _u32, _P]),
}

_lib = None


def lib():
    """Load libvcr.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class VcrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"vcr status {name}: {msg}")


def check(status: int, ctx=None) -> None:
    if status != OK:
        msg = lib().vcr_last_error(ctx)
        raise VcrError(status, msg.decode() if msg else "")
