"""The comparison baseline over libcvtpm.so: the Python mirror of
``cvt::StereoGCVFilter`` (cvt/gfx/ifilter/StereoGCVFilter.h) on CUDA tensors.

    f = StereoGCVFilter()
    d = f.depthmap(right, left, 0.0, 64.0, 1.0)      # left view, normalised
    fused, d0, d1 = f.apply(right, left, 0.0, 64.0, 1.0)

Images are (H, W, 4) float32 RGBA CUDA tensors.  The depth is normalised,
|d - dmin| / |dmax - dmin|; the map belongs to cam1, whose match in cam0
lies at x - d (the reference's convention).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def _fail(rc: int):
    raise _lib.CvtpmError(rc, _lib.lib().cvtpm_last_error(None).decode())


def _img(t: torch.Tensor, name: str) -> torch.Tensor:
    if not t.is_cuda or t.dtype != torch.float32 or t.dim() != 3 or t.shape[2] != 4:
        raise ValueError(f"{name} must be an (H, W, 4) float32 CUDA tensor")
    return t.contiguous()


def set_batch(disparities: int = 0) -> None:
    """Disparities per batch for later calls (0: automatic); results do not
    depend on it."""
    rc = _lib.lib().cvtpm_gcv_set_batch(int(disparities))
    if rc:
        _fail(rc)


def trim(device: int = 0, keep_bytes: int = 0) -> None:
    """Return the scratch pool's unused memory beyond keep_bytes to the
    device (the pool otherwise keeps its largest reservation until exit)."""
    rc = _lib.lib().cvtpm_gcv_trim(int(device), int(keep_bytes))
    if rc:
        _fail(rc)


def plan(width: int, height: int, dmin: float, dmax: float, dt: float) -> dict:
    """steps, batch, scratch bytes and kernel launches of one depthmap call."""
    steps, batch, launches = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    nbytes = ctypes.c_size_t()
    rc = _lib.lib().cvtpm_gcv_plan(int(width), int(height), float(dmin), float(dmax), float(dt), ctypes.byref(steps),
                                   ctypes.byref(batch), ctypes.byref(nbytes), ctypes.byref(launches))
    if rc:
        _fail(rc)
    return {"steps": steps.value, "batch": batch.value, "scratch_bytes": nbytes.value, "launches": launches.value}


class StereoGCVFilter:
    def _stream(self, t):
        return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)

    def depthmap(self, cam0: torch.Tensor, cam1: torch.Tensor, dmin: float, dmax: float, dt: float,
                 out: torch.Tensor | None = None) -> torch.Tensor:
        a, b = _img(cam0, "cam0"), _img(cam1, "cam1")
        if a.shape != b.shape:
            raise ValueError("cam0 and cam1 differ in size")
        H, W = a.shape[:2]
        if out is None:
            out = torch.empty((H, W), dtype=torch.float32, device=a.device)
        rc = _lib.lib().cvtpm_gcv_depthmap(out.data_ptr(), out.stride(0) * 4, a.data_ptr(), b.data_ptr(), W, H, W * 16,
                                           float(dmin), float(dmax), float(dt), self._stream(a))
        if rc:
            _fail(rc)
        return out

    def apply(self, cam0: torch.Tensor, cam1: torch.Tensor, dmin: float, dmax: float, dt: float):
        """(fused GRAY_UINT8 map, depth map of cam1's view, depth map of cam0's view)."""
        a, b = _img(cam0, "cam0"), _img(cam1, "cam1")
        if a.shape != b.shape:
            raise ValueError("cam0 and cam1 differ in size")
        H, W = a.shape[:2]
        out = torch.empty((H, W), dtype=torch.uint8, device=a.device)
        d0 = torch.empty((H, W), dtype=torch.float32, device=a.device)
        d1 = torch.empty((H, W), dtype=torch.float32, device=a.device)
        rc = _lib.lib().cvtpm_gcv_apply(out.data_ptr(), W, d0.data_ptr(), d1.data_ptr(), W * 4, a.data_ptr(),
                                        b.data_ptr(), W, H, W * 16, float(dmin), float(dmax), float(dt), self._stream(a))
        if rc:
            _fail(rc)
        return out, d0, d1
