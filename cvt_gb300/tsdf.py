"""TSDF fusion of depth maps over libcvtpm.so: the Python mirror of
``cvt::TSDFVolume`` (cvt/vision/TSDFVolume.h), on CUDA tensors.

    vol = TSDFVolume(grid_to_world, 128, 128, 128, truncation=0.05)
    vol.clear()
    vol.addDepthMap(K, E, depth)              # (H, W) float32 CUDA tensor
    d = vol.rayCastDepthMap(K, E, 640, 480, scale=-1.0)

Matrices are 4x4 row-major (cvt::Matrix4f), intrinsics 3x3.  rayCastDepthMap
returns max(-z * scale, 0) for the camera-space depth z of the first surface
along each pixel's ray (TSDFVolume.cl); with the integration's convention (z >
0 in front of the camera) a scale of -1 yields the depth.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _fail(rc: int):
    raise _lib.CvtpmError(rc, _lib.lib().cvtpm_last_error(None).decode())


def _fp(a, n):
    arr = np.ascontiguousarray(np.asarray(a, np.float32).reshape(n))
    return arr, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def projection(intrinsics, extrinsics) -> np.ndarray:
    """intrinsics.toMatrix4() * extrinsics (TSDFVolume.cpp:79-84)."""
    K, kp = _fp(intrinsics, 9)
    E, ep = _fp(extrinsics, 16)
    out = np.empty(16, np.float32)
    rc = _lib.lib().cvtpm_tsdf_projection(kp, ep, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    if rc:
        _fail(rc)
    return out.reshape(4, 4)


class TSDFVolume:
    def __init__(self, grid_to_world, width: int, height: int, depth: int, truncation: float = 0.1,
                 device: int | None = None):
        self.device = torch.cuda.current_device() if device is None else int(device)
        g, gp = _fp(grid_to_world, 16)
        h = ctypes.c_void_p()
        rc = _lib.lib().cvtpm_tsdf_create(ctypes.byref(h), self.device, gp, int(width), int(height), int(depth),
                                          float(truncation))
        if rc:
            _fail(rc)
        self._h = h
        self.width, self.height, self.depth = int(width), int(height), int(depth)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().cvtpm_tsdf_destroy(h)
            except Exception:
                pass
            self._h = None

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _proj(self, a, b):
        return projection(a, b) if b is not None else np.asarray(a, np.float32).reshape(4, 4)

    def clear(self, weight: float = 0.0) -> None:
        rc = _lib.lib().cvtpm_tsdf_clear(self._h, float(weight), self._stream())
        if rc:
            _fail(rc)

    def addDepthMap(self, proj_or_intrinsics, extrinsics_or_depth, depthmap=None, scale: float = 1.0) -> None:
        """addDepthMap(proj, depthmap, scale) or addDepthMap(intrinsics,
        extrinsics, depthmap, scale), as the two overloads of the reference."""
        if depthmap is None:
            proj, depthmap = self._proj(proj_or_intrinsics, None), extrinsics_or_depth
        else:
            proj = self._proj(proj_or_intrinsics, extrinsics_or_depth)
        if not depthmap.is_cuda or depthmap.dtype != torch.float32 or depthmap.dim() != 2 or depthmap.stride(1) != 1:
            raise ValueError("depthmap must be an (H, W) float32 CUDA tensor with contiguous rows")
        _, pp = _fp(proj, 16)
        rc = _lib.lib().cvtpm_tsdf_add_depthmap(self._h, pp, depthmap.data_ptr(), depthmap.shape[1], depthmap.shape[0],
                                                depthmap.stride(0) * 4, float(scale), self._stream())
        if rc:
            _fail(rc)

    def rayCastDepthMap(self, proj_or_intrinsics, extrinsics=None, width: int = 0, height: int = 0,
                        scale: float = 1.0, out: torch.Tensor | None = None) -> torch.Tensor:
        proj = self._proj(proj_or_intrinsics, extrinsics)
        if out is None:
            out = torch.empty((height, width), dtype=torch.float32, device=torch.device("cuda", self.device))
        _, pp = _fp(proj, 16)
        rc = _lib.lib().cvtpm_tsdf_raycast(self._h, pp, out.data_ptr(), out.shape[1], out.shape[0], out.stride(0) * 4,
                                           float(scale), self._stream())
        if rc:
            _fail(rc)
        return out

    def slice(self, axis: int, index: int) -> torch.Tensor:
        """The slice kernels (axis 0 = x, 1 = y, 2 = z): RGBA (c, c, c, 1)."""
        shape = {0: (self.depth, self.height), 1: (self.depth, self.width), 2: (self.height, self.width)}[axis]
        out = torch.empty(shape + (4,), dtype=torch.float32, device=torch.device("cuda", self.device))
        rc = _lib.lib().cvtpm_tsdf_slice(self._h, int(axis), int(index), out.data_ptr(), out.stride(0) * 4,
                                         self._stream())
        if rc:
            _fail(rc)
        return out

    def volume(self) -> torch.Tensor:
        """The (depth, height, width, 2) float32 (tsdf, weight) volume: a view
        of the library's device memory, valid while this object lives."""
        ptr = ctypes.c_void_p()
        rc = _lib.lib().cvtpm_tsdf_info(self._h, None, None, None, ctypes.byref(ptr))
        if rc:
            _fail(rc)

        class _View:
            __cuda_array_interface__ = {"shape": (self.depth, self.height, self.width, 2), "typestr": "<f4",
                                        "data": (ptr.value, False), "version": 3, "strides": None}
        return torch.as_tensor(_View(), device=torch.device("cuda", self.device))

    def saveRaw(self, path: str, weighted: bool) -> None:
        rc = _lib.lib().cvtpm_tsdf_save_raw(self._h, str(path).encode(), int(bool(weighted)))
        if rc:
            _fail(rc)

