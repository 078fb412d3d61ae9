"""The reference's image formats and files, over libcvtpm.so.

Images are numpy arrays (host) or torch tensors (device) holding a
``cvt::Image``'s storage: shape (H, W) for one channel, (H, W, C) otherwise,
dtype uint8 / uint16 / int16 / float32 by format.  ``fmt`` is a
``cvt::IFormatID`` (cvt/gfx/IFormat.h:36-63), the constants below.

    arr, fmt = read_ppm("left.ppm")               # RGBA_UINT8
    rgba = to_rgbaf(torch.from_numpy(arr).cuda(), fmt)   # as read_imagef sees it
    write_pfm("disparity.pfm", dmap.cpu().numpy(), GRAY_FLOAT)
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

(GRAY_UINT8, GRAY_UINT16, GRAY_INT16, GRAY_FLOAT,
 GRAYALPHA_UINT8, GRAYALPHA_UINT16, GRAYALPHA_INT16, GRAYALPHA_FLOAT,
 RGBA_UINT8, RGBA_UINT16, RGBA_INT16, RGBA_FLOAT,
 BGRA_UINT8, BGRA_UINT16, BGRA_INT16, BGRA_FLOAT,
 BAYER_RGGB_UINT8, BAYER_GRBG_UINT8, BAYER_GBRG_UINT8,
 YUYV_UINT8, UYVY_UINT8) = range(1, 22)

_DT = (np.uint8, np.uint16, np.int16, np.float32)


def fmt_info(fmt: int):
    """(channels, numpy dtype) of a format."""
    if 1 <= fmt <= 16:
        return (1, 2, 4, 4)[(fmt - 1) // 4], _DT[(fmt - 1) % 4]
    if 17 <= fmt <= 19:
        return 1, np.uint8
    if fmt in (20, 21):
        return 2, np.uint8
    raise ValueError(f"unknown image format {fmt}")


def _shape(h: int, w: int, c: int):
    return (h, w) if c == 1 else (h, w, c)


def _fail(rc: int):
    raise _lib.CvtpmError(rc, _lib.lib().cvtpm_last_error(None).decode())


def _desc(arr, fmt: int, ptr: int, stride: int) -> _lib.CvtpmImage:
    c, dt = fmt_info(fmt)
    if (c > 1 and (arr.ndim != 3 or arr.shape[2] != c)) or (c == 1 and arr.ndim != 2):
        raise ValueError(f"format {fmt} wants shape {_shape(arr.shape[0], arr.shape[1], c)}, got {tuple(arr.shape)}")
    return _lib.CvtpmImage(int(fmt), int(arr.shape[1]), int(arr.shape[0]), int(stride), ptr)


def _host_desc(arr: np.ndarray, fmt: int) -> _lib.CvtpmImage:
    c, dt = fmt_info(fmt)
    if arr.dtype != dt:
        raise ValueError(f"format {fmt} wants dtype {np.dtype(dt).name}, got {arr.dtype}")
    if not arr.flags.c_contiguous:
        raise ValueError("host image must be C-contiguous")
    return _desc(arr, fmt, arr.ctypes.data, arr.strides[0])


def _read(fn, path: str):
    d = _lib.CvtpmImage()
    rc = fn(str(path).encode(), ctypes.byref(d))
    if rc:
        _fail(rc)
    c, dt = fmt_info(d.format)
    arr = np.empty(_shape(d.height, d.width, c), dt)
    d.data = arr.ctypes.data
    d.stride = arr.strides[0]
    rc = fn(str(path).encode(), ctypes.byref(d))
    if rc:
        _fail(rc)
    return arr, int(d.format)


def read_raw(path: str):
    """CVTRaw file (plugins/iloader/CVTRaw/CVTRawLoader.cpp) -> (array, fmt)."""
    return _read(_lib.lib().cvtpm_raw_read, path)


def write_raw(path: str, arr: np.ndarray, fmt: int) -> None:
    """CVTRaw file (plugins/isaver/CVTRaw/CVTRawSaver.cpp)."""
    d = _host_desc(arr, fmt)
    rc = _lib.lib().cvtpm_raw_write(str(path).encode(), ctypes.byref(d))
    if rc:
        _fail(rc)


def read_ppm(path: str):
    """PPM / PGM (plugins/iloader/PPM/PPMLoader.cpp) -> (array, fmt):
    RGBA_UINT8 (alpha 255) for P3/P6, GRAY_UINT8 for P2/P5."""
    return _read(_lib.lib().cvtpm_ppm_read, path)


def read_png(path: str):
    """PNG (plugins/iloader/PNG/PNGLoader.cpp) -> (array, fmt): GRAY_UINT8/16,
    GRAYALPHA_UINT8/16 or RGBA_UINT8/16 as the reference's libpng set-up
    gives them."""
    return _read(_lib.lib().cvtpm_png_read, path)


def write_png(path: str, arr: np.ndarray, fmt: int) -> None:
    """PNG (plugins/isaver/PNG/PNGSaver.cpp) of a GRAY, GRAYALPHA, RGBA or
    BGRA image of 8 or 16 bits, or of a float one converted to 8 bits as the
    reference converts it (sRGB for colour and gray, linear for alpha)."""
    d = _host_desc(np.ascontiguousarray(arr), fmt)
    rc = _lib.lib().cvtpm_png_write(str(path).encode(), ctypes.byref(d))
    if rc:
        _fail(rc)


def write_pfm(path: str, arr: np.ndarray, fmt: int) -> None:
    """PFM (plugins/isaver/PFM/PFMSaver.cpp) of a GRAY/RGBA/BGRA float image."""
    d = _host_desc(np.ascontiguousarray(arr), fmt)
    rc = _lib.lib().cvtpm_pfm_write(str(path).encode(), ctypes.byref(d))
    if rc:
        _fail(rc)


def device_desc(img: torch.Tensor, fmt: int) -> _lib.CvtpmImage:
    """cvtpm_image of a CUDA tensor holding an image's storage (rows may be
    padded: stride(0) elements per row).  A uint8 tensor of shape
    (H, row bytes) is accepted for any format (width = row bytes // bytes per
    pixel), which carries 16-bit data without a uint16 tensor type."""
    c, dt = fmt_info(fmt)
    if img.is_cuda and img.dtype == torch.uint8 and dt != np.uint8:
        bpp = c * np.dtype(dt).itemsize
        if img.dim() != 2 or img.stride(1) != 1 or img.shape[1] % bpp:
            raise ValueError("a byte tensor must be (H, W * bytes per pixel) with contiguous rows")
        return _lib.CvtpmImage(int(fmt), img.shape[1] // bpp, img.shape[0], img.stride(0), img.data_ptr())
    tdt = {np.uint8: torch.uint8, np.int16: torch.int16, np.float32: torch.float32}.get(dt)
    if dt == np.uint16:
        tdt = getattr(torch, "uint16", None)
    if not img.is_cuda or img.dtype != tdt:
        raise ValueError(f"format {fmt} wants a CUDA tensor of {tdt}, got {img.dtype} on {img.device}")
    inner = img.stride(-1) == 1 and (c == 1 or img.stride(1) == c)
    if not inner:
        raise ValueError("pixels of a row must be contiguous")
    return _desc(img, fmt, img.data_ptr(), img.stride(0) * img.element_size())


def to_rgbaf(img: torch.Tensor, fmt: int, out: torch.Tensor | None = None) -> torch.Tensor:
    """The image as the reference's kernels read it (read_imagef): an (H, W, 4)
    float32 RGBA tensor."""
    d = device_desc(img, fmt)
    if out is not None and (out.shape != (d.height, d.width, 4) or out.dtype != torch.float32 or out.stride(1) != 4):
        raise ValueError("out must be an (H, W, 4) float32 tensor with contiguous pixels")
    if out is None:
        out = torch.empty((d.height, d.width, 4), dtype=torch.float32, device=img.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(img.device).cuda_stream)
    rc = _lib.lib().cvtpm_image_to_rgbaf(ctypes.byref(d), out.data_ptr(), out.stride(0) * 4, stream)
    if rc:
        _fail(rc)
    return out
