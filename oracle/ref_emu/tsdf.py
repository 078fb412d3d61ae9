"""TEST INFRASTRUCTURE: the reference's TSDFVolume kernels
(cvt/cl/kernel/TSDFVolume/TSDFVolume.cl) run through the OpenCL emulation
(oracle/_ref/libpmref.so), with the launch sizes of cvt/vision/TSDFVolume.cpp,
and the reference's Matrix4 product (cvt/math/Matrix4.h, through
libpmref_rect.so).  Signatures follow oracle.oracle.tsdf_*."""
from __future__ import annotations

import ctypes

import numpy as np

from . import build_ref

_L = None
_R = None


def available() -> bool:
    return build_ref.available()


def lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(build_ref.build())
        vp, c_int, c_float = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.ref_tsdf_clear.argtypes = [vp, c_int, c_int, c_int, c_float]
        L.ref_tsdf_add.argtypes = [vp, c_int, c_int, c_int, vp, c_int, c_int, c_float, vp, c_float]
        L.ref_tsdf_raycast.argtypes = [vp, c_int, c_int, vp, c_int, c_int, c_int, vp, vp, c_float]
        L.ref_tsdf_slice.argtypes = [vp, c_int, c_int, vp, c_int, c_int, c_int]
        _L = L
    return _L


def _m4(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(4, 4))


def mat4_mul(a, b):
    """cvt::Matrix4f a * b."""
    global _R
    if _R is None:
        _R = ctypes.CDLL(build_ref.build_rect())
        _R.ref_mat4_mul.argtypes = [ctypes.c_void_p] * 3
    out = np.empty((4, 4), np.float32)
    x, y = _m4(a), _m4(b)
    _R.ref_mat4_mul(x.ctypes.data, y.ctypes.data, out.ctypes.data)
    return out


def tsdf_clear(W, H, D, weight=0.0):
    v = np.empty((D, H, W, 2), np.float32)
    lib().ref_tsdf_clear(v.ctypes.data, W, H, D, float(weight))
    return v


def tsdf_add(vol, dmap, dscale, tg2cam, trunc):
    D, H, W = vol.shape[:3]
    dm = np.ascontiguousarray(dmap, np.float32)
    t = _m4(tg2cam)
    lib().ref_tsdf_add(vol.ctypes.data, W, H, D, dm.ctypes.data, dm.shape[1], dm.shape[0], float(dscale),
                       t.ctypes.data, float(trunc))
    return vol


def tsdf_raycast(vol, iw, ih, tcam2g, tg2cam, scale):
    D, H, W = vol.shape[:3]
    out = np.empty((ih, iw), np.float32)
    ti, t = _m4(tcam2g), _m4(tg2cam)
    lib().ref_tsdf_raycast(out.ctypes.data, iw, ih, vol.ctypes.data, W, H, D, ti.ctypes.data, t.ctypes.data,
                           float(scale))
    return out


def tsdf_slice(vol, axis, index):
    D, H, W = vol.shape[:3]
    shape = {0: (D, H), 1: (D, W), 2: (H, W)}[axis]
    out = np.empty(shape + (4,), np.float32)
    v = np.ascontiguousarray(vol)
    lib().ref_tsdf_slice(out.ctypes.data, axis, index, v.ctypes.data, W, H, D)
    return out
