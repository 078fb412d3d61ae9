"""Python mirror of ``cvt::PMHuberStereo`` (cvt/vision/PMHuberStereo.h:35-59)
over libcvtpm.so, for torch tensors on a CUDA device.

    stereo = PMHuberStereo()
    dmap = torch.empty(0, device="cuda")
    stereo.depthMap(dmap, left, right, patchsize=17, depthmax=64,
                    iterations=3, viewsamples=4)

``left``/``right`` are (H, W, 4) float32 RGBA CUDA tensors (the reference's
IFormat::RGBA_FLOAT images).  ``dmap`` is resized to (H, W) like the
reference's ``dmap.reallocate(...)`` (PMHuberStereo.cpp:278), and so is
``normalmap`` to (H, W, 4) (:286).  Size mismatches raise CVTException with
the reference's message (:66-68); every other failure raises CvtpmError.
Work runs on torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .params import CvtpmParams, default_params, PRESET_REFERENCE


class CVTException(RuntimeError):
    """The reference's cvt::CVTException for inconsistent inputs."""


def _stream_ptr(t: torch.Tensor):
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _check_img(t: torch.Tensor, name: str):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
        raise CVTException(f"{name} must be a float32 CUDA tensor")
    if t.dim() != 3 or t.shape[2] != 4:
        raise CVTException(f"{name} must be an (H, W, 4) RGBA image")
    if t.stride(2) != 1 or t.stride(1) != 4:
        raise CVTException(f"{name} rows must be contiguous RGBA pixels")


class PMHuberStereo:
    def __init__(self, device: int | None = None, params: CvtpmParams | None = None):
        L = _lib.lib()
        if device is None:
            device = torch.cuda.current_device()
        self.device = int(device)
        h = ctypes.c_void_p()
        rc = L.cvtpm_create(ctypes.byref(h), self.device)
        if rc:
            raise _lib.CvtpmError(rc, _lib.status_string(rc))
        self._h = h
        self.params = params if params is not None else default_params(PRESET_REFERENCE)
        self.set_params(self.params)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().cvtpm_destroy(h)
            except Exception:
                pass
            self._h = None

    def _check(self, rc: int):
        if rc:
            msg = _lib.lib().cvtpm_last_error(self._h).decode()
            raise _lib.CvtpmError(rc, msg)

    def set_params(self, params: CvtpmParams):
        self._check(_lib.lib().cvtpm_set_params(self._h, ctypes.byref(params)))
        self.params = params

    def set_timing(self, enable: bool):
        self._check(_lib.lib().cvtpm_set_timing(self._h, int(bool(enable))))

    def reset_stats(self):
        self._check(_lib.lib().cvtpm_reset_stats(self._h))

    def stats(self) -> dict:
        st = _lib.CvtpmStats()
        self._check(_lib.lib().cvtpm_get_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    def get_params(self) -> CvtpmParams:
        p = CvtpmParams()
        self._check(_lib.lib().cvtpm_get_params(self._h, ctypes.byref(p)))
        return p

    def depthMap(self, dmap: torch.Tensor, left: torch.Tensor, right: torch.Tensor, patchsize: int,
                 depthmax: float, iterations: int, viewsamples: int, dscale: float = -1.0,
                 normalmap: torch.Tensor | None = None, trace: dict | None = None) -> torch.Tensor:
        """PMHuberStereo::depthMap.  If ``trace`` is a dict it receives the
        integer outputs: 'winners' (2, H, W) uint8, 'valid' (H, W) uint8 and
        'states' (2, H, W, 4) float32."""
        _check_img(left, "left")
        _check_img(right, "right")
        if left.shape != right.shape:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        if left.device != right.device or left.device.index != self.device:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        if left.stride(0) != right.stride(0):
            right = right.contiguous()
            left = left.contiguous()
        H, W = left.shape[:2]
        if dmap is None:
            dmap = torch.empty((H, W), dtype=torch.float32, device=left.device)
        if dmap.shape != (H, W) or dmap.dtype != torch.float32 or not dmap.is_contiguous() or dmap.device != left.device:
            if dmap.device != left.device or dmap.dtype != torch.float32:
                raise CVTException("dmap must be a float32 tensor on the images' device")
            dmap.resize_(H, W)
        nm_ptr, nm_pitch = None, 0
        if normalmap is not None:
            if normalmap.device != left.device or normalmap.dtype != torch.float32:
                raise CVTException("normalmap must be a float32 tensor on the images' device")
            if normalmap.shape != (H, W, 4) or not normalmap.is_contiguous():
                normalmap.resize_(H, W, 4)
            nm_ptr, nm_pitch = normalmap.data_ptr(), W * 16
        tr = None
        if trace is not None:
            trace["winners"] = torch.empty((2, H, W), dtype=torch.uint8, device=left.device)
            trace["valid"] = torch.empty((H, W), dtype=torch.uint8, device=left.device)
            trace["states"] = torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device)
            tr = _lib.CvtpmTrace(trace["winners"].data_ptr(), trace["valid"].data_ptr(), trace["states"].data_ptr())
        rc = _lib.lib().cvtpm_depthmap(
            self._h, dmap.data_ptr(), W * 4, left.data_ptr(), right.data_ptr(), W, H, left.stride(0) * 4,
            int(patchsize), float(depthmax), int(iterations), int(viewsamples), float(dscale),
            nm_ptr, nm_pitch, ctypes.byref(tr) if tr is not None else None, _stream_ptr(left))
        self._check(rc)
        return dmap

    def depthMapResumable(self, dmap: torch.Tensor | None, left: torch.Tensor, right: torch.Tensor, patchsize: int,
                          depthmax: float, iterations: int, resume: dict | None = None, stop: int = -1,
                          save: bool = False, trace: dict | None = None):
        """cvtpm_depthmap_resumable: the run from resume["iteration"] (with
        resume["states"], resume["smooth"], (2, H, W, 4) float32 CUDA tensors;
        None: from the random init) up to iteration `stop` (-1: the end).
        Returns (dmap or None, checkpoint dict or None): the map when the run
        reached the end, the state before `stop` when save is true."""
        _check_img(left, "left")
        _check_img(right, "right")
        if left.shape != right.shape:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        H, W = left.shape[:2]
        if stop < 0 or stop > iterations:
            stop = iterations
        finish = stop == iterations
        if finish and dmap is None:
            dmap = torch.empty((H, W), dtype=torch.float32, device=left.device)
        rs = None
        if resume is not None:
            for k in ("states", "smooth"):
                t = resume[k]
                if t.shape != (2, H, W, 4) or t.dtype != torch.float32 or not t.is_contiguous() or t.device != left.device:
                    raise CVTException(f"resume['{k}'] must be a contiguous (2, H, W, 4) float32 tensor on the images' device")
            rs = _lib.CvtpmCheckpoint(int(resume["iteration"]), resume["states"].data_ptr(), resume["smooth"].data_ptr())
        sv, out = None, None
        if save:
            out = {"states": torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device),
                   "smooth": torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device)}
            sv = _lib.CvtpmCheckpoint(-1, out["states"].data_ptr(), out["smooth"].data_ptr())
        tr = None
        if trace is not None and finish:
            trace["winners"] = torch.empty((2, H, W), dtype=torch.uint8, device=left.device)
            trace["valid"] = torch.empty((H, W), dtype=torch.uint8, device=left.device)
            trace["states"] = torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device)
            tr = _lib.CvtpmTrace(trace["winners"].data_ptr(), trace["valid"].data_ptr(), trace["states"].data_ptr())
        rc = _lib.lib().cvtpm_depthmap_resumable(
            self._h, dmap.data_ptr() if finish else None, W * 4, left.data_ptr(), right.data_ptr(), W, H,
            left.stride(0) * 4, int(patchsize), float(depthmax), int(iterations), 4, -1.0, None, 0,
            ctypes.byref(tr) if tr is not None else None, ctypes.byref(rs) if rs is not None else None, int(stop),
            ctypes.byref(sv) if sv is not None else None, _stream_ptr(left))
        self._check(rc)
        if out is not None:
            out["iteration"] = sv.iteration
        return (dmap if finish else None), out

    def depthMapImage(self, dmap: torch.Tensor | None, left: torch.Tensor, left_fmt: int, right: torch.Tensor,
                      right_fmt: int, patchsize: int, depthmax: float, iterations: int, viewsamples: int,
                      dscale: float = -1.0, normalmap: torch.Tensor | None = None,
                      trace: dict | None = None) -> torch.Tensor:
        """PMHuberStereo::depthMap with left/right in any cvt::IFormat (CUDA
        tensors holding the storage, see ``imageio.device_desc``); each is
        read as the reference's read_imagef reads it."""
        from . import imageio
        dl, dr = imageio.device_desc(left, left_fmt), imageio.device_desc(right, right_fmt)
        if (dl.width, dl.height) != (dr.width, dr.height) or left.device != right.device:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        H, W = dl.height, dl.width
        if dmap is None:
            dmap = torch.empty((H, W), dtype=torch.float32, device=left.device)
        if dmap.shape != (H, W) or not dmap.is_contiguous():
            dmap.resize_(H, W)
        nm_ptr, nm_pitch = None, 0
        if normalmap is not None:
            if normalmap.shape != (H, W, 4) or not normalmap.is_contiguous():
                normalmap.resize_(H, W, 4)
            nm_ptr, nm_pitch = normalmap.data_ptr(), W * 16
        tr = None
        if trace is not None:
            trace["winners"] = torch.empty((2, H, W), dtype=torch.uint8, device=left.device)
            trace["valid"] = torch.empty((H, W), dtype=torch.uint8, device=left.device)
            trace["states"] = torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device)
            tr = _lib.CvtpmTrace(trace["winners"].data_ptr(), trace["valid"].data_ptr(), trace["states"].data_ptr())
        rc = _lib.lib().cvtpm_depthmap_image(
            self._h, dmap.data_ptr(), W * 4, ctypes.byref(dl), ctypes.byref(dr), int(patchsize), float(depthmax),
            int(iterations), int(viewsamples), float(dscale), nm_ptr, nm_pitch,
            ctypes.byref(tr) if tr is not None else None, _stream_ptr(left))
        self._check(rc)
        return dmap

    def depthMapHost(self, left, right, patchsize: int, depthmax: float, iterations: int, viewsamples: int,
                     dscale: float = -1.0, dmap=None):
        """depthMap on host (numpy / CPU torch) buffers: copies in, runs,
        copies out and synchronizes.  Returns the (H, W) disparity map."""
        import numpy as np
        left = np.ascontiguousarray(left, np.float32)
        right = np.ascontiguousarray(right, np.float32)
        if left.shape != right.shape or left.ndim != 3 or left.shape[2] != 4:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        H, W = left.shape[:2]
        if dmap is None:
            dmap = np.empty((H, W), np.float32)
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        rc = _lib.lib().cvtpm_depthmap_host(
            self._h, dmap.ctypes.data, W * 4, left.ctypes.data, right.ctypes.data, W, H, W * 16,
            int(patchsize), float(depthmax), int(iterations), int(viewsamples), float(dscale), None, 0, stream)
        self._check(rc)
        return dmap

    def cost(self, img1: torch.Tensor, img2: torch.Tensor, states: torch.Tensor, lr: int = 1) -> torch.Tensor:
        """Aggregated ASW cost of every pixel for a fixed state field
        (H, W, 4) (s0, s1, s2, -): x_other = s0*x + s1*y + s2."""
        _check_img(img1, "img1")
        _check_img(img2, "img2")
        if img1.shape != img2.shape or states.shape != img1.shape:
            raise CVTException("img1/img2/states shapes differ")
        states = states.contiguous()
        H, W = img1.shape[:2]
        out = torch.empty((H, W), dtype=torch.float32, device=img1.device)
        rc = _lib.lib().cvtpm_cost_eval(self._h, img1.data_ptr(), img2.data_ptr(), W, H, img1.stride(0) * 4,
                                        states.data_ptr(), int(lr), out.data_ptr(), _stream_ptr(img1))
        self._check(rc)
        return out

    def depthMapInpaint(self, dmap: torch.Tensor, left: torch.Tensor, right: torch.Tensor, patchsize: int,
                        depthmax: float, iterations: int, viewsamples: int, trace: dict | None = None) -> torch.Tensor:
        """PMHuberStereo::depthMapInpaint: disparity in pixels; ``trace`` as
        for depthMap."""
        _check_img(left, "left")
        _check_img(right, "right")
        if left.shape != right.shape or left.device != right.device or left.device.index != self.device:
            raise CVTException("Left/Right stereo images inconsistent or incompatible memory type")
        if left.stride(0) != right.stride(0):
            right = right.contiguous()
            left = left.contiguous()
        H, W = left.shape[:2]
        if dmap is None:
            dmap = torch.empty((H, W), dtype=torch.float32, device=left.device)
        if dmap.device != left.device or dmap.dtype != torch.float32:
            raise CVTException("dmap must be a float32 tensor on the images' device")
        if dmap.shape != (H, W) or not dmap.is_contiguous():
            dmap.resize_(H, W)
        tr = None
        if trace is not None:
            trace["winners"] = torch.empty((2, H, W), dtype=torch.uint8, device=left.device)
            trace["valid"] = torch.empty((H, W), dtype=torch.uint8, device=left.device)
            trace["states"] = torch.empty((2, H, W, 4), dtype=torch.float32, device=left.device)
            tr = _lib.CvtpmTrace(trace["winners"].data_ptr(), trace["valid"].data_ptr(), trace["states"].data_ptr())
        rc = _lib.lib().cvtpm_depthmap_inpaint(
            self._h, dmap.data_ptr(), W * 4, left.data_ptr(), right.data_ptr(), W, H, left.stride(0) * 4,
            int(patchsize), float(depthmax), int(iterations), int(viewsamples),
            ctypes.byref(tr) if tr is not None else None, _stream_ptr(left))
        self._check(rc)
        return dmap

    def depthMapBatched(self, pairs, outs=None, stream=None):
        """cvtpm_depthmap_batched.  pairs: list of (left, right, depthmax) with
        left/right (H, W, 4) float32 CUDA tensors; returns the (H, W) disparity
        maps (scaled like depthMap: dscale, or 1/depthmax per pair).  Passing
        the returned maps back as `outs` (same inputs) replays the captured
        graph instead of capturing a new one."""
        arr = (_lib.CvtpmPair * len(pairs))()
        if outs is None:
            outs = [None] * len(pairs)
        outs = list(outs)
        for i, (left, right, dmax) in enumerate(pairs):
            _check_img(left, "left")
            _check_img(right, "right")
            if left.shape != right.shape or left.stride(0) != right.stride(0):
                raise CVTException(f"pair {i}: left/right shapes or pitches differ")
            H, W = left.shape[:2]
            d = outs[i]
            if d is None or tuple(d.shape) != (H, W) or not d.is_contiguous() or d.dtype != torch.float32:
                d = torch.empty((H, W), dtype=torch.float32, device=left.device)
            outs[i] = d
            arr[i] = _lib.CvtpmPair(left.data_ptr(), right.data_ptr(), W, H, left.stride(0) * 4, float(dmax),
                                    d.data_ptr(), W * 4)
        self._batch_keep = (arr, outs, list(pairs))
        st = _stream_ptr(pairs[0][0]) if stream is None else stream
        self._check(_lib.lib().cvtpm_depthmap_batched(self._h, arr, len(pairs), st))
        return outs

    def set_batch_lanes(self, lanes: int) -> None:
        """Fix the lane count of depthMapBatched (0: autotune)."""
        self._check(_lib.lib().cvtpm_set_batch_lanes(self._h, int(lanes)))

    def set_batch_knobs(self, grid_mult: int = -1, pd_rows: int = 16, pd_halo: int = 4) -> None:
        """Pin the phase-batched launch knobs (grid_mult -1: autotune)."""
        self._check(_lib.lib().cvtpm_set_batch_knobs(self._h, int(grid_mult), int(pd_rows), int(pd_halo)))

    def batch_info(self) -> dict:
        info = _lib.CvtpmBatchInfo()
        self._check(_lib.lib().cvtpm_get_batch_info(self._h, ctypes.byref(info)))
        return info.as_dict()

    def polish_planes(self, img1: torch.Tensor, img2: torch.Tensor, planes: torch.Tensor, lr: int = 1,
                      steps: int = 4) -> torch.Tensor:
        """cvtpm_polish_planes on (H, W, 4) planes (a, b, c, -), in place;
        returns the final per-pixel cost."""
        _check_img(img1, "img1")
        _check_img(img2, "img2")
        if planes.shape != img1.shape or not planes.is_contiguous() or planes.dtype != torch.float32:
            raise CVTException("planes must be a contiguous float32 (H, W, 4) tensor")
        H, W = img1.shape[:2]
        cost = torch.empty((H, W), dtype=torch.float32, device=img1.device)
        self._check(_lib.lib().cvtpm_polish_planes(self._h, img1.data_ptr(), img2.data_ptr(), W, H,
                                                   img1.stride(0) * 4, planes.data_ptr(), int(lr), int(steps),
                                                   cost.data_ptr(), _stream_ptr(img1)))
        return cost

    def set_memory_budget(self, nbytes: int) -> None:
        """Device bytes the FAST path may use for its shared-window neighbour
        costs, 32 per pixel (0: evaluate neighbours per pixel; results are the
        same)."""
        self._check(_lib.lib().cvtpm_set_memory_budget(self._h, int(nbytes)))

    def cost_adjoint(self, img1: torch.Tensor, img2: torch.Tensor, planes: torch.Tensor, lr: int = 1,
                     dcost: torch.Tensor | None = None, want_planes: bool = True, want_images: bool = True):
        """cvtpm_cost_adjoint.  planes (H, W, 4) = (a, b, c, -) with
        d = a*x + b*y + c (x_other = x - d for lr = 1, x + d for lr = 0).
        Returns (cost, dplanes, dimg1, dimg2); the gradients are None when
        dcost is None or not wanted."""
        _check_img(img1, "img1")
        _check_img(img2, "img2")
        if img1.shape != img2.shape or planes.shape != img1.shape:
            raise CVTException("img1/img2/planes shapes differ")
        planes = planes.contiguous()
        H, W = img1.shape[:2]
        dev = img1.device
        cost = torch.empty((H, W), dtype=torch.float32, device=dev)
        dpl = d1 = d2 = None
        if dcost is not None:
            dcost = dcost.to(torch.float32).contiguous()
            if dcost.shape != (H, W):
                raise CVTException("dcost must be (H, W)")
            if want_planes:
                dpl = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
            if want_images:
                d1 = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
                d2 = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
        ptr = lambda t: None if t is None else t.data_ptr()
        rc = _lib.lib().cvtpm_cost_adjoint(self._h, img1.data_ptr(), img2.data_ptr(), W, H, img1.stride(0) * 4,
                                           planes.data_ptr(), int(lr), ptr(dcost), cost.data_ptr(), ptr(dpl),
                                           ptr(d1), ptr(d2), _stream_ptr(img1))
        self._check(rc)
        return cost, dpl, d1, d2
