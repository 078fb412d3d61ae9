"""The depth conversion between the stereo path and TSDF fusion over
libcvtpm.so: the Python mirror of ``cvt::Vision::disparityToDepthmap``
(cvt/vision/Vision.h:183, Vision.cpp:147-168), on CUDA tensors.

    dmap = stereo.depthMap(...)                          # disparity / depthmax
    depth = disparityToDepthmap(dmap, depthmax, f, baseline)
    vol.addDepthMap(K, E, depth)
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def disparityToDepthmap(disparity: torch.Tensor, dispscale: float, focallength: float, baseline: float,
                        dispthres: float = 0.01, out: torch.Tensor | None = None) -> torch.Tensor:
    """depth = focallength * baseline / (disparity * dispscale) where the
    scaled disparity exceeds dispthres, else 0."""
    if not disparity.is_cuda or disparity.dtype != torch.float32 or disparity.dim() != 2 or disparity.stride(1) != 1:
        raise ValueError("disparity must be an (H, W) float32 CUDA tensor with contiguous rows")
    H, W = disparity.shape
    if out is None:
        out = torch.empty((H, W), dtype=torch.float32, device=disparity.device)
    L = _lib.lib()
    rc = L.cvtpm_disparity_to_depth(out.data_ptr(), out.stride(0) * 4, disparity.data_ptr(), disparity.stride(0) * 4,
                                    W, H, float(dispscale), float(focallength), float(baseline), float(dispthres),
                                    ctypes.c_void_p(torch.cuda.current_stream(disparity.device).cuda_stream))
    if rc:
        raise _lib.CvtpmError(rc, L.cvtpm_last_error(None).decode())
    return out
