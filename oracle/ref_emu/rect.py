"""TEST INFRASTRUCTURE: the reference's own rectification and warp code
(oracle/_ref/libpmref_rect.so, built by build_ref.build_rect from the
reference's sources where build_ref finds them), with the signatures of oracle.oracle.stereo_rectify
and oracle.oracle.warp.  available() is False where the sources are absent."""
from __future__ import annotations

import ctypes
import os

from . import build_ref
from .. import oracle as _orc

_L = None


def available() -> bool:
    return build_ref.available()


def lib():
    global _L
    if _L is None:
        path = build_ref.build_rect()
        if path is None:
            raise RuntimeError("reference sources absent")
        L = ctypes.CDLL(path)
        vp, c_int, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
        L.ref_rectify.argtypes = [vp] * 7 + [c_int, c_int, c_int] + [vp] * 7
        L.ref_warp.argtypes = [c_int, vp, sz, c_int, c_int, vp, sz, c_int, c_int, vp, sz]
        L.ref_conv_f_u8.argtypes = [c_int, vp, vp, sz]
        _L = L
    return _L


def stereo_rectify(cam0, cam1, E, vertical, W, H):
    return _orc._rect_call(lib().ref_rectify, cam0, cam1, E, vertical, W, H)


def warp(fmt, src, warp_map):
    return _orc._warp_call(lib().ref_warp, fmt, src, warp_map)


def conv_f_u8(kind: int, src):
    """Image::convert of float samples to 8 bits: kind 0 GRAY (sRGB), 1
    GRAYALPHA (linear), 2 RGBA/BGRA (sRGB colour, linear alpha)."""
    import numpy as np
    a = np.ascontiguousarray(np.asarray(src, np.float32).reshape(-1))
    out = np.zeros(a.size, np.uint8)
    if lib().ref_conv_f_u8(int(kind), a.ctypes.data, out.ctypes.data, a.size):
        raise ValueError("bad kind")
    return out
