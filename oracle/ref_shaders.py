"""ctypes binding of the reference's own compute shaders run on the CPU
(oracle/ref_shaders.cpp over the transliteration in oracle/build_ref.py).
Test infrastructure: available only where the reference tree is, to check
the oracle's restatement of the shader arithmetic against the shaders
themselves."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref
from .oracle import _abi, _p

_lib = None


def available() -> bool:
    return build_ref.shaders_available()


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build_shaders()
        if path is None:
            raise RuntimeError("the reference shaders are not available here")
        L = C.CDLL(path)
        P, u32, f, i32 = C.c_void_p, C.c_uint32, C.c_float, C.c_int
        sig = {
            "ref_set_scene": (None, [P, P, C.POINTER(_abi.Cloud), C.POINTER(_abi.Camera), C.POINTER(_abi.Params),
                                     C.POINTER(_abi.ShadowVolume), P]),
            "ref_pt_image": (None, [u32, u32, i32, u32, P, i32]),
            "ref_sv_build": (None, [P, i32]),
            "ref_sample_background": (None, [P, P]),
            "ref_intersect_cloud": (i32, [P, P, C.POINTER(f), C.POINTER(f)]),
            "ref_camera_ray": (None, [i32, i32, P, P]),
            "ref_initialize_random": (u32, [u32]),
            "ref_random_numbers": (u32, [u32, u32, P]),
            "ref_sample_phase": (f, [P, P]),
            "ref_onb": (None, [P, P, P]),
            "ref_scatter_ray": (u32, [P, u32, P]),
            "ref_sample_cloud": (f, [P]),
            "ref_sample_shadow_volume": (f, [P]),
            "ref_find_scatter_point": (i32, [P, P, C.POINTER(u32)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class Scene:
    """Keeps the arrays the shaders read alive while they are bound."""

    def __init__(self, dense, cloud, cam=None, params=None, sv=None, sv_tex=None):
        self.dense = np.ascontiguousarray(dense, np.float32)
        self.n = np.array(self.dense.shape[::-1], np.uint32)
        self.cloud, self.cam, self.params, self.sv = cloud, cam, params, sv
        self.sv_tex = None if sv_tex is None else np.ascontiguousarray(sv_tex, np.float32)
        self.bind()

    def bind(self):
        lib().ref_set_scene(_p(self.dense), _p(self.n), C.byref(self.cloud),
                            C.byref(self.cam) if self.cam is not None else None,
                            C.byref(self.params) if self.params is not None else None,
                            C.byref(self.sv) if self.sv is not None else None,
                            _p(self.sv_tex) if self.sv_tex is not None else None)


def pt_image(scene: Scene, width: int, height: int, seed: int, frame_count: int = 0, previous=None,
             threads: int = 0) -> np.ndarray:
    """PathTracer.comp main over the image: [H, W, 4] float32."""
    scene.bind()
    img = np.zeros((height, width, 4), np.float32) if previous is None else np.array(previous, np.float32)
    lib().ref_pt_image(width, height, seed, frame_count, _p(img), threads or os.cpu_count() or 1)
    return img


def sv_build(scene: Scene, threads: int = 0) -> np.ndarray:
    """ShadowVolume.comp main: the n^3 volume, x fastest, as [z, y, x]."""
    scene.bind()
    n = int(scene.sv.voxel_axis_count)
    out = np.zeros((n, n, n), np.float32)
    lib().ref_sv_build(_p(out), threads or os.cpu_count() or 1)
    return out
