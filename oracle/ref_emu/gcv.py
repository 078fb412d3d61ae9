"""TEST INFRASTRUCTURE: cvt::StereoGCVFilter (cvt/gfx/ifilter/StereoGCVFilter.cpp)
run through the OpenCL emulation (oracle/_ref/libpmref.so): the reference's
kernels with the launch sequence of its depthmap / apply."""
from __future__ import annotations

import ctypes

import numpy as np

from . import build_ref

_L = None


def available() -> bool:
    return build_ref.available()


def lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(build_ref.build())
        vp, c_int, c_float = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_gcv_depthmap.argtypes = [vp, vp, vp, c_int, c_int, c_float, c_float, c_float]
        L.ref_gcv_apply.argtypes = [vp, vp, vp, vp, vp, c_int, c_int, c_float, c_float, c_float]
        _L = L
    return _L


def depthmap(cam0, cam1, dmin, dmax, dt):
    a, b = (np.ascontiguousarray(x, np.float32) for x in (cam0, cam1))
    H, W = a.shape[:2]
    out = np.empty((H, W), np.float32)
    lib().ref_gcv_depthmap(out.ctypes.data, a.ctypes.data, b.ctypes.data, W, H, float(dmin), float(dmax), float(dt))
    return out


def apply(cam0, cam1, dmin, dmax, dt):
    a, b = (np.ascontiguousarray(x, np.float32) for x in (cam0, cam1))
    H, W = a.shape[:2]
    out = np.empty((H, W), np.uint8)
    d0, d1 = np.empty((H, W), np.float32), np.empty((H, W), np.float32)
    lib().ref_gcv_apply(out.ctypes.data, d0.ctypes.data, d1.ctypes.data, a.ctypes.data, b.ctypes.data, W, H,
                        float(dmin), float(dmax), float(dt))
    return out, d0, d1
