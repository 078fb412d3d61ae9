"""ctypes binding of libcvtpm.so (include/cvtpm.h).

The library is the only compute path: if it is missing or cannot be loaded,
import fails with an error that says how to build it.  There is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os

from .params import CvtpmParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcvtpm.so")

# every symbol include/cvtpm.h declares
EXPORTS = (
    "cvtpm_version", "cvtpm_status_string", "cvtpm_params_default", "cvtpm_create", "cvtpm_destroy",
    "cvtpm_set_params", "cvtpm_get_params", "cvtpm_last_error", "cvtpm_synchronize", "cvtpm_depthmap",
    "cvtpm_depthmap_host", "cvtpm_depthmap_resumable", "cvtpm_depthmap_inpaint", "cvtpm_cost_eval", "cvtpm_cost_adjoint", "cvtpm_polish_planes", "cvtpm_depthmap_batched", "cvtpm_set_batch_knobs", "cvtpm_set_memory_budget",
    "cvtpm_set_batch_lanes", "cvtpm_get_batch_info",
    "cvtpm_set_timing", "cvtpm_reset_stats", "cvtpm_get_stats", "cvtpm_tool_fp32_peak",
    "cvtpm_tool_pd_time",
    "cvtpm_cost_eval_noalloc",
    "cvtpm_iformat_bpp", "cvtpm_image_to_rgbaf", "cvtpm_depthmap_image", "cvtpm_raw_read", "cvtpm_raw_write",
    "cvtpm_ppm_read", "cvtpm_pfm_write", "cvtpm_png_read", "cvtpm_png_write", "cvtpm_float_to_srgb_u8", "cvtpm_stereo_rectify", "cvtpm_warp_apply",
    "cvtpm_tsdf_create", "cvtpm_tsdf_destroy", "cvtpm_tsdf_info", "cvtpm_tsdf_clear", "cvtpm_tsdf_projection",
    "cvtpm_tsdf_add_depthmap", "cvtpm_tsdf_raycast", "cvtpm_tsdf_slice", "cvtpm_tsdf_save_raw",
    "cvtpm_disparity_to_depth", "cvtpm_gcv_set_batch", "cvtpm_gcv_trim", "cvtpm_gcv_plan", "cvtpm_gcv_depthmap", "cvtpm_gcv_apply",
)


class CvtpmCheckpoint(ctypes.Structure):
    _fields_ = [("iteration", ctypes.c_int), ("states", ctypes.c_void_p), ("smooth", ctypes.c_void_p)]


class CvtpmTrace(ctypes.Structure):
    _fields_ = [("winners", ctypes.c_void_p), ("valid", ctypes.c_void_p), ("states", ctypes.c_void_p)]


class CvtpmPair(ctypes.Structure):
    _fields_ = [("left", ctypes.c_void_p), ("right", ctypes.c_void_p), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("pitch", ctypes.c_size_t), ("depthmax", ctypes.c_float),
                ("dmap", ctypes.c_void_p), ("dmap_pitch", ctypes.c_size_t)]


class CvtpmImage(ctypes.Structure):
    """cvtpm_image: a cvt::Image's storage (format, size, row stride in bytes, data)."""
    _fields_ = [("format", ctypes.c_int), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("stride", ctypes.c_size_t), ("data", ctypes.c_void_p)]


class CvtpmCamera(ctypes.Structure):
    """cvtpm_camera: intrinsics (row-major 3x3), radial k1..k3, tangential p1, p2."""
    _fields_ = [("intrinsics", ctypes.c_float * 9), ("radial", ctypes.c_float * 3), ("tangential", ctypes.c_float * 2)]


class CvtpmRectification(ctypes.Structure):
    _fields_ = [("first", CvtpmCamera), ("second", CvtpmCamera), ("extrinsics", ctypes.c_float * 16),
                ("rot_first", ctypes.c_float * 9), ("rot_second", ctypes.c_float * 9)]


BATCH_MAX_CAND = 16


class CvtpmBatchInfo(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("shared_windows", ctypes.c_int), ("tuned", ctypes.c_int),
                ("ncand", ctypes.c_int), ("cand_lanes", ctypes.c_int * BATCH_MAX_CAND),
                ("cand_ms", ctypes.c_float * BATCH_MAX_CAND), ("graph_nodes", ctypes.c_longlong),
                ("replays", ctypes.c_longlong), ("phased", ctypes.c_int), ("grid_mult", ctypes.c_int),
                ("pd_rows", ctypes.c_int), ("pd_halo", ctypes.c_int),
                ("cand_grid_mult", ctypes.c_int * BATCH_MAX_CAND), ("cand_pd_rows", ctypes.c_int * BATCH_MAX_CAND),
                ("cand_pd_halo", ctypes.c_int * BATCH_MAX_CAND), ("launches", ctypes.c_longlong),
                ("tune_ms", ctypes.c_float), ("mode_ms", ctypes.c_float * 2)]

    def as_dict(self) -> dict:
        n = self.ncand
        cands = []
        for i in range(n):
            c = {"lanes": self.cand_lanes[i], "proxy_ms": self.cand_ms[i]}
            if self.cand_lanes[i] == 0:
                c.update(grid_mult=self.cand_grid_mult[i], pd_rows=self.cand_pd_rows[i], pd_halo=self.cand_pd_halo[i])
            cands.append(c)
        return {"lanes": self.lanes, "shared_windows": self.shared_windows, "tuned": self.tuned,
                "candidates": cands, "graph_nodes": self.graph_nodes, "replays": self.replays,
                "phased": self.phased, "grid_mult": self.grid_mult, "pd_rows": self.pd_rows,
                "pd_halo": self.pd_halo, "launches": self.launches, "tune_ms": self.tune_ms,
                "mode_ms": {"phase_batched": self.mode_ms[0], "one_lane": self.mode_ms[1]}}


class CvtpmStats(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("propagate_launches", ctypes.c_uint64),
                ("cost_evals", ctypes.c_uint64), ("cost_taps", ctypes.c_uint64), ("pd_launches", ctypes.c_uint64), ("pd_steps", ctypes.c_uint64),
                ("propagate_ms", ctypes.c_float), ("pd_ms", ctypes.c_float)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class CvtpmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"cvtpm status {status}: {message}")
        self.status = status


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, f, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
    P = ctypes.POINTER(CvtpmParams)
    L.cvtpm_version.restype = ctypes.c_char_p
    L.cvtpm_status_string.argtypes = [i]
    L.cvtpm_status_string.restype = ctypes.c_char_p
    L.cvtpm_params_default.argtypes = [P, i]
    L.cvtpm_create.argtypes = [ctypes.POINTER(vp), i]
    L.cvtpm_destroy.argtypes = [vp]
    L.cvtpm_set_params.argtypes = [vp, P]
    L.cvtpm_get_params.argtypes = [vp, P]
    L.cvtpm_last_error.argtypes = [vp]
    L.cvtpm_last_error.restype = ctypes.c_char_p
    L.cvtpm_synchronize.argtypes = [vp, vp]
    L.cvtpm_depthmap.argtypes = [vp, vp, sz, vp, vp, i, i, sz, i, f, i, i, f, vp, sz, ctypes.POINTER(CvtpmTrace), vp]
    L.cvtpm_depthmap_resumable.argtypes = [vp, vp, sz, vp, vp, i, i, sz, i, f, i, i, f, vp, sz,
                                           ctypes.POINTER(CvtpmTrace), ctypes.POINTER(CvtpmCheckpoint), i,
                                           ctypes.POINTER(CvtpmCheckpoint), vp]
    L.cvtpm_depthmap_host.argtypes = [vp, vp, sz, vp, vp, i, i, sz, i, f, i, i, f, vp, sz, vp]
    L.cvtpm_depthmap_inpaint.argtypes = [vp, vp, sz, vp, vp, i, i, sz, i, f, i, i, ctypes.POINTER(CvtpmTrace), vp]
    L.cvtpm_cost_eval.argtypes = [vp, vp, vp, i, i, sz, vp, i, vp, vp]
    L.cvtpm_cost_adjoint.argtypes = [vp, vp, vp, i, i, sz, vp, i, vp, vp, vp, vp, vp, vp]
    L.cvtpm_depthmap_batched.argtypes = [vp, ctypes.POINTER(CvtpmPair), i, vp]
    L.cvtpm_set_timing.argtypes = [vp, i]
    L.cvtpm_set_memory_budget.argtypes = [vp, sz]
    L.cvtpm_polish_planes.argtypes = [vp, vp, vp, i, i, sz, vp, i, i, vp, vp]
    L.cvtpm_set_batch_lanes.argtypes = [vp, i]
    L.cvtpm_get_batch_info.argtypes = [vp, ctypes.POINTER(CvtpmBatchInfo)]
    L.cvtpm_set_batch_knobs.argtypes = [vp, i, i, i]
    L.cvtpm_reset_stats.argtypes = [vp]
    L.cvtpm_get_stats.argtypes = [vp, ctypes.POINTER(CvtpmStats)]
    L.cvtpm_tool_fp32_peak.argtypes = [i, vp, ctypes.POINTER(ctypes.c_float)]
    L.cvtpm_tool_pd_time.argtypes = [vp, i, vp, ctypes.POINTER(ctypes.c_float)]
    L.cvtpm_cost_eval_noalloc.argtypes = [P, vp, vp, i, i, sz, vp, vp, vp]
    IP = ctypes.POINTER(CvtpmImage)
    L.cvtpm_iformat_bpp.argtypes = [i]
    L.cvtpm_iformat_bpp.restype = sz
    L.cvtpm_image_to_rgbaf.argtypes = [IP, vp, sz, vp]
    L.cvtpm_depthmap_image.argtypes = [vp, vp, sz, IP, IP, i, f, i, i, f, vp, sz, ctypes.POINTER(CvtpmTrace), vp]
    L.cvtpm_raw_read.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_raw_write.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_ppm_read.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_pfm_write.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_png_read.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_png_write.argtypes = [ctypes.c_char_p, IP]
    L.cvtpm_float_to_srgb_u8.argtypes = [f]
    L.cvtpm_float_to_srgb_u8.restype = ctypes.c_uint8
    CP = ctypes.POINTER(CvtpmCamera)
    L.cvtpm_stereo_rectify.argtypes = [CP, CP, ctypes.POINTER(ctypes.c_float), i, ctypes.POINTER(CvtpmRectification),
                                       i, i, vp, vp, sz, vp]
    L.cvtpm_warp_apply.argtypes = [IP, IP, vp, sz, vp]
    FP = ctypes.POINTER(ctypes.c_float)
    L.cvtpm_tsdf_create.argtypes = [ctypes.POINTER(vp), i, FP, i, i, i, f]
    L.cvtpm_tsdf_destroy.argtypes = [vp]
    IPp = ctypes.POINTER(ctypes.c_int)
    L.cvtpm_tsdf_info.argtypes = [vp, IPp, IPp, IPp, ctypes.POINTER(vp)]
    L.cvtpm_tsdf_clear.argtypes = [vp, f, vp]
    L.cvtpm_tsdf_projection.argtypes = [FP, FP, FP]
    L.cvtpm_tsdf_add_depthmap.argtypes = [vp, FP, vp, i, i, sz, f, vp]
    L.cvtpm_tsdf_raycast.argtypes = [vp, FP, vp, i, i, sz, f, vp]
    L.cvtpm_tsdf_slice.argtypes = [vp, i, i, vp, sz, vp]
    L.cvtpm_tsdf_save_raw.argtypes = [vp, ctypes.c_char_p, i]
    L.cvtpm_disparity_to_depth.argtypes = [vp, sz, vp, sz, i, i, f, f, f, f, vp]
    L.cvtpm_gcv_set_batch.argtypes = [i]
    L.cvtpm_gcv_trim.argtypes = [i, sz]
    L.cvtpm_gcv_plan.argtypes = [i, i, f, f, f, vp, vp, vp, vp]
    L.cvtpm_gcv_depthmap.argtypes = [vp, sz, vp, vp, i, i, sz, f, f, f, vp]
    L.cvtpm_gcv_apply.argtypes = [vp, sz, vp, vp, sz, vp, vp, i, i, sz, f, f, f, vp]
    for name in EXPORTS:
        if name not in ("cvtpm_version", "cvtpm_status_string", "cvtpm_last_error", "cvtpm_iformat_bpp",
                        "cvtpm_float_to_srgb_u8"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def version() -> str:
    return lib().cvtpm_version().decode()


def status_string(s: int) -> str:
    return lib().cvtpm_status_string(int(s)).decode()


def c_default_params(preset: int) -> CvtpmParams:
    p = CvtpmParams()
    rc = lib().cvtpm_params_default(ctypes.byref(p), int(preset))
    if rc:
        raise CvtpmError(rc, "cvtpm_params_default")
    return p
