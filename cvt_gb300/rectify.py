"""Stereo rectification of real pairs over libcvtpm.so: the Python mirror of
``cvt::StereoRectification`` (cvt/vision/StereoRectification.h) on top of
``StereoCameraCalibration::undistortRectify``
(cvt/vision/StereoCameraCalibration.h:199-277) and ``IWarp::apply``
(cvt/gfx/ifilter/IWarp.cpp:49-66).

A camera is a dict with "K" (3x3 intrinsics), "radial" (k1, k2, k3) and
"tangential" (p1, p2); ``extrinsics`` is the stereo extrinsics (4x4, the
second camera relative to the first), as StereoCameraCalibration holds it.

    rect = StereoRectification(cam0, cam1, E, width=1242, height=375)
    left_r = rect.undistortLeft(left, imageio.RGBA_UINT8)   # CUDA tensors
    right_r = rect.undistortRight(right, imageio.RGBA_UINT8)
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, imageio


def _camera(c: dict) -> _lib.CvtpmCamera:
    cam = _lib.CvtpmCamera()
    K = np.asarray(c["K"], np.float32).reshape(9)
    rad = np.asarray(c.get("radial", (0, 0, 0)), np.float32).reshape(3)
    tan = np.asarray(c.get("tangential", (0, 0)), np.float32).reshape(2)
    cam.intrinsics[:] = [float(v) for v in K]
    cam.radial[:] = [float(v) for v in rad]
    cam.tangential[:] = [float(v) for v in tan]
    return cam


def _camera_dict(cam: _lib.CvtpmCamera) -> dict:
    return {"K": np.array(cam.intrinsics[:], np.float32).reshape(3, 3),
            "radial": np.array(cam.radial[:], np.float32), "tangential": np.array(cam.tangential[:], np.float32)}


def _fail(rc: int):
    raise _lib.CvtpmError(rc, _lib.lib().cvtpm_last_error(None).decode())


def _rectify(first, second, extrinsics, vertical, width=0, height=0, maps=None, stream=None):
    c0, c1 = _camera(first), _camera(second)
    E = np.ascontiguousarray(np.asarray(extrinsics, np.float32).reshape(16))
    out = _lib.CvtpmRectification()
    m0 = m1 = None
    pitch = 0
    if maps is not None:
        m0, m1 = maps[0].data_ptr(), maps[1].data_ptr()
        pitch = maps[0].stride(0) * 4
    rc = _lib.lib().cvtpm_stereo_rectify(ctypes.byref(c0), ctypes.byref(c1),
                                         E.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(bool(vertical)),
                                         ctypes.byref(out), int(width), int(height), m0, m1, pitch, stream)
    if rc:
        _fail(rc)
    return {"first": _camera_dict(out.first), "second": _camera_dict(out.second),
            "extrinsics": np.array(out.extrinsics[:], np.float32).reshape(4, 4),
            "R0": np.array(out.rot_first[:], np.float32).reshape(3, 3),
            "R1": np.array(out.rot_second[:], np.float32).reshape(3, 3)}


def rectification(first: dict, second: dict, extrinsics, vertical: bool = False) -> dict:
    """The rectified calibration (host only): the two new cameras, the new
    stereo extrinsics and the rectifying rotations."""
    return _rectify(first, second, extrinsics, vertical)


def warp_apply(src: torch.Tensor, fmt: int, warp_map: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """IWarp::apply(dst, src, warp): ``src`` a CUDA tensor holding an image of
    GRAY/RGBA/BGRA float or uint8 storage, ``warp_map`` an (H, W, 2) float32
    CUDA tensor of source coordinates; returns the (H, W[, C]) result."""
    s = imageio.device_desc(src, fmt)
    if warp_map.dim() != 3 or warp_map.shape[2] != 2 or warp_map.dtype != torch.float32 or warp_map.stride(1) != 2:
        raise ValueError("warp_map must be an (H, W, 2) float32 tensor with contiguous pixels")
    H, W = warp_map.shape[:2]
    c, dt = imageio.fmt_info(fmt)
    if out is None:
        out = torch.empty((H, W) + ((c,) if c > 1 else ()), dtype=src.dtype, device=src.device)
    d = imageio.device_desc(out, fmt)
    stream = ctypes.c_void_p(torch.cuda.current_stream(src.device).cuda_stream)
    rc = _lib.lib().cvtpm_warp_apply(ctypes.byref(d), ctypes.byref(s), warp_map.data_ptr(), warp_map.stride(0) * 4,
                                     stream)
    if rc:
        _fail(rc)
    return out


class StereoRectification:
    """cvt::StereoRectification: the warp maps of both cameras for
    width x height rectified images (on the device), and undistortLeft /
    undistortRight through them."""

    def __init__(self, first: dict, second: dict, extrinsics, width: int, height: int, vertical: bool = False,
                 device: int | None = None):
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.maps = (torch.empty((height, width, 2), dtype=torch.float32, device=dev),
                     torch.empty((height, width, 2), dtype=torch.float32, device=dev))
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        self.rectified = _rectify(first, second, extrinsics, vertical, width, height, self.maps, stream)

    def undistortLeft(self, img: torch.Tensor, fmt: int, out: torch.Tensor | None = None) -> torch.Tensor:
        return warp_apply(img, fmt, self.maps[0], out)

    def undistortRight(self, img: torch.Tensor, fmt: int, out: torch.Tensor | None = None) -> torch.Tensor:
        return warp_apply(img, fmt, self.maps[1], out)
