"""TEST INFRASTRUCTURE: ctypes front end of the CPU oracle (liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use this module, as the checker or as the timed CPU baseline.  The
product never imports it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from cvt_gb300.params import CvtpmParams

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.LIB
        if not os.path.exists(path):
            build_oracle.build()
        L = ctypes.CDLL(path)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        i16p = np.ctypeslib.ndpointer(np.int16, flags="C_CONTIGUOUS")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        P = ctypes.POINTER(CvtpmParams)
        c_int, c_float = ctypes.c_int, ctypes.c_float
        L.orc_set_threads.argtypes = [c_int]
        L.orc_max_threads.restype = c_int
        L.orc_gradxy.argtypes = [f32p, c_int, c_int, f32p]
        L.orc_edge_weight.argtypes = [f32p, c_int, c_int, f32p]
        for n in ("orc_exp", "orc_wexp", "orc_acospi"):
            getattr(L, n).argtypes = [c_float]
            getattr(L, n).restype = c_float
        L.orc_pow.argtypes = [c_float, c_float]
        L.orc_pow.restype = c_float
        L.orc_exp_array.argtypes = [f32p, f32p, ctypes.c_long]
        L.orc_wexp_array.argtypes = [f32p, f32p, ctypes.c_long]
        L.orc_acospi_array.argtypes = [f32p, f32p, ctypes.c_long]
        L.orc_pow_array.argtypes = [f32p, c_float, f32p, ctypes.c_long]
        L.orc_mwc_mulmod_serial.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_mwc_mulmod_serial.restype = ctypes.c_uint64
        L.orc_mwc_mulmod.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_mwc_mulmod.restype = ctypes.c_uint64
        L.orc_mwc_stream.argtypes = [ctypes.c_uint64, c_int, f32p]
        L.orc_mwc_state.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        L.orc_philox.argtypes = [u32p, u32p, u32p]
        L.orc_philox_stream.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, c_int, f32p]
        L.orc_cost_field.argtypes = [P, f32p, f32p, c_int, c_int, f32p, f32p]
        L.orc_cost_field.restype = c_int
        L.orc_init.argtypes = [P, f32p, f32p, c_int, c_int, c_int, f32p]
        L.orc_init.restype = c_int
        opt_i16 = ctypes.c_void_p
        L.orc_propagate.argtypes = [P, f32p, f32p, c_int, c_int, c_int, c_int, c_float, f32p, f32p,
                                    opt_i16, ctypes.c_void_p, f32p, ctypes.c_void_p]
        L.orc_propagate.restype = c_int
        L.orc_view_list.argtypes = [f32p, c_int, c_int, i16p]
        L.orc_consistency.argtypes = [f32p, f32p, c_int, c_int, c_float, c_float, c_int, f32p, ctypes.c_void_p]
        L.orc_fill_state.argtypes = [f32p, c_int, c_int, c_float, c_int, f32p]
        L.orc_fill_depthmap.argtypes = [f32p, c_int, c_int, c_float, f32p]
        L.orc_fill_normalmap.argtypes = [f32p, c_int, c_int, f32p]
        L.orc_pd_step.argtypes = [f32p, f32p, f32p, f32p, f32p, f32p, c_float, c_int, c_int]
        L.orc_pd_apply.argtypes = [f32p, f32p, f32p, c_float, c_int, c_int, c_int]
        L.orc_depthmap.argtypes = [P, f32p, f32p, c_int, c_int, f32p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]
        L.orc_depthmap.restype = c_int
        L.orc_depthmap_inpaint.argtypes = [P, f32p, f32p, c_int, c_int, f32p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]
        L.orc_depthmap_inpaint.restype = c_int
        L.orc_occmap.argtypes = [f32p, f32p, c_int, c_int, c_float, c_int, f32p]
        L.orc_normal_depth.argtypes = [f32p, c_int, c_int, c_float, c_int, f32p]
        L.orc_pd_apply_inpaint.argtypes = [f32p, f32p, f32p, f32p, c_float, c_int, c_int, c_int]
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.orc_cost_field_f64.argtypes = [P, f32p, f32p, c_int, c_int, f32p, ctypes.c_double, f64p, u8p]
        L.orc_cost_field_f64.restype = c_int
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        L.orc_cost_planes_f64.argtypes = [P, f64p, f64p, c_int, c_int, f64p, c_int, ctypes.c_double, f64p, u8p, u64p]
        L.orc_cost_planes_f64.restype = c_int
        L.orc_cost_adjoint_f64.argtypes = [P, f64p, f64p, c_int, c_int, f64p, c_int, f64p, f64p, f64p, f64p, f64p,
                                           ctypes.c_double, u8p, u8p, u8p]
        L.orc_cost_adjoint_f64.restype = c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def gradxy(img):
    img = _f32(img)
    h, w = img.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    lib().orc_gradxy(img, w, h, out)
    return out


def edge_weight(img):
    img = _f32(img)
    h, w = img.shape[:2]
    out = np.empty((h, w), np.float32)
    lib().orc_edge_weight(img, w, h, out)
    return out


def cost_field(params: CvtpmParams, img1, img2, states):
    img1, img2, states = _f32(img1), _f32(img2), _f32(states)
    h, w = img1.shape[:2]
    out = np.empty((h, w), np.float32)
    rc = lib().orc_cost_field(ctypes.byref(params), img1, img2, w, h, states, out)
    assert rc == 0, rc
    return out


def cost_field_f64(params: CvtpmParams, img1, img2, states, eps: float = 1e-3):
    """FP64 cost of a fixed state field and the mask of pixels with a tap
    within eps of the sample-validity bounds."""
    img1, img2, states = _f32(img1), _f32(img2), _f32(states)
    h, w = img1.shape[:2]
    out = np.empty((h, w), np.float64)
    edge = np.empty((h, w), np.uint8)
    rc = lib().orc_cost_field_f64(ctypes.byref(params), img1, img2, w, h, states, float(eps), out, edge)
    assert rc == 0, rc
    return out, edge.astype(bool)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def cost_planes_f64(params: CvtpmParams, img1, img2, planes, lr: int = 1, eps: float = 1e-3):
    """FP64 cost of per-pixel planes (a, b, c, _) of view lr on double images;
    returns (cost, edge mask, branch signature per pixel)."""
    img1, img2, planes = _f64(img1), _f64(img2), _f64(planes)
    h, w = img1.shape[:2]
    out = np.empty((h, w), np.float64)
    edge = np.empty((h, w), np.uint8)
    sig = np.empty((h, w), np.uint64)
    rc = lib().orc_cost_planes_f64(ctypes.byref(params), img1, img2, w, h, planes, int(lr), float(eps), out, edge, sig)
    assert rc == 0, rc
    return out, edge.astype(bool), sig


def cost_adjoint_f64(params: CvtpmParams, img1, img2, planes, dcost, lr: int = 1, kink_eps: float = 0.0):
    """FP64 adjoint: returns (cost, dplanes (H,W,4), dimg1 (H,W,4), dimg2 (H,W,4));
    with kink_eps > 0 also the (H,W) masks of plane / image-1 / image-2
    entries reached by a tap within kink_eps of a kink."""
    img1, img2, planes, dcost = _f64(img1), _f64(img2), _f64(planes), _f64(dcost)
    h, w = img1.shape[:2]
    cost = np.empty((h, w), np.float64)
    dpl = np.empty((h, w, 4), np.float64)
    d1 = np.empty((h, w, 4), np.float64)
    d2 = np.empty((h, w, 4), np.float64)
    am = [np.zeros((h, w), np.uint8) for _ in range(3)]
    rc = lib().orc_cost_adjoint_f64(ctypes.byref(params), img1, img2, w, h, planes, int(lr), dcost, cost, dpl, d1, d2,
                                    float(kink_eps), *am)
    assert rc == 0, rc
    if kink_eps > 0:
        return cost, dpl, d1, d2, tuple(m.astype(bool) for m in am)
    return cost, dpl, d1, d2


def init(params: CvtpmParams, img1, img2, lr: int):
    img1, img2 = _f32(img1), _f32(img2)
    h, w = img1.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    rc = lib().orc_init(ctypes.byref(params), img1, img2, w, h, int(lr), out)
    assert rc == 0, rc
    return out


def propagate(params, img1, img2, lr, it, theta, old, smooth, viewin=None, viewsrc=None):
    img1, img2, old, smooth = _f32(img1), _f32(img2), _f32(old), _f32(smooth)
    h, w = img1.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    win = np.empty((h, w), np.uint8)
    vi = None if viewin is None else np.ascontiguousarray(viewin, np.int16)
    vs = None if viewsrc is None else _f32(viewsrc)
    rc = lib().orc_propagate(ctypes.byref(params), img1, img2, w, h, int(lr), int(it), float(theta),
                             old, smooth, _ptr(vi), _ptr(vs), out, _ptr(win))
    assert rc == 0, rc
    return out, win


def view_list(src):
    src = _f32(src)
    h, w = src.shape[:2]
    out = np.empty((h, w, 4), np.int16)
    lib().orc_view_list(src, w, h, out)
    return out


def consistency(L, R, maxdisp, maxangle, lr):
    L, R = _f32(L), _f32(R)
    h, w = L.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    valid = np.empty((h, w), np.uint8)
    lib().orc_consistency(L, R, w, h, float(maxdisp), float(maxangle), int(lr), out, _ptr(valid))
    return out, valid


def fill_state(inp, depthmax, lr):
    inp = _f32(inp)
    h, w = inp.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    lib().orc_fill_state(inp, w, h, float(depthmax), int(lr), out)
    return out


def fill_depthmap(inp, scale):
    inp = _f32(inp)
    h, w = inp.shape[:2]
    out = np.empty((h, w), np.float32)
    lib().orc_fill_depthmap(inp, w, h, float(scale), out)
    return out


def fill_normalmap(inp):
    inp = _f32(inp)
    h, w = inp.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    lib().orc_fill_normalmap(inp, w, h, out)
    return out


def pd_step(last, pin, f, wgt, lam):
    last, pin, f, wgt = _f32(last), _f32(pin), _f32(f), _f32(wgt)
    h, w = last.shape[:2]
    uout = np.empty((h, w, 4), np.float32)
    pout = np.empty((h, w, 8), np.float32)
    lib().orc_pd_step(uout, pout, last, pin, f, wgt, float(lam), w, h)
    return uout, pout


def pd_apply(output, inp, wgt, lam, iters):
    out = _f32(output).copy()
    inp, wgt = _f32(inp), _f32(wgt)
    h, w = inp.shape[:2]
    lib().orc_pd_apply(out, inp, wgt, float(lam), int(iters), w, h)
    return out


def depthmap(params: CvtpmParams, left, right, normalmap: bool = False, trace: bool = False):
    """PMHuberStereo::depthMap on the CPU.  Returns (dmap, extras) with extras
    holding 'normalmap', 'states' (2,H,W,4), 'winners' (2,H,W), 'valid' (H,W)."""
    left, right = _f32(left), _f32(right)
    h, w = left.shape[:2]
    dmap = np.empty((h, w), np.float32)
    nm = np.empty((h, w, 4), np.float32) if normalmap else None
    st = np.empty((2, h, w, 4), np.float32) if trace else None
    win = np.empty((2, h, w), np.uint8) if trace else None
    val = np.empty((h, w), np.uint8) if trace else None
    rc = lib().orc_depthmap(ctypes.byref(params), left, right, w, h, dmap, _ptr(nm), _ptr(st), _ptr(win), _ptr(val))
    assert rc == 0, rc
    return dmap, {"normalmap": nm, "states": st, "winners": win, "valid": val}


def depthmap_inpaint(params: CvtpmParams, left, right, trace: bool = False):
    """PMHuberStereo::depthMapInpaint on the CPU.  Returns (dmap in pixels,
    extras) with extras 'states' (2,H,W,4), 'winners' (2,H,W), 'valid' (H,W)."""
    left, right = _f32(left), _f32(right)
    h, w = left.shape[:2]
    dmap = np.empty((h, w), np.float32)
    st = np.empty((2, h, w, 4), np.float32) if trace else None
    win = np.empty((2, h, w), np.uint8) if trace else None
    val = np.empty((h, w), np.uint8) if trace else None
    rc = lib().orc_depthmap_inpaint(ctypes.byref(params), left, right, w, h, dmap, _ptr(st), _ptr(win), _ptr(val))
    assert rc == 0, rc
    return dmap, {"states": st, "winners": win, "valid": val}


def occmap(L, R, maxdiff, lr):
    L, R = _f32(L), _f32(R)
    h, w = L.shape[:2]
    out = np.empty((h, w), np.float32)
    lib().orc_occmap(L, R, w, h, float(maxdiff), int(lr), out)
    return out


def normal_depth(states, depthmax, lr):
    states = _f32(states)
    h, w = states.shape[:2]
    out = np.empty((h, w, 4), np.float32)
    lib().orc_normal_depth(states, w, h, float(depthmax), int(lr), out)
    return out


def pd_apply_inpaint(output, inp, wgt, mask, lam, iters):
    out = _f32(output).copy()
    inp, wgt, mask = _f32(inp), _f32(wgt), _f32(mask)
    h, w = inp.shape[:2]
    lib().orc_pd_apply_inpaint(out, inp, wgt, mask, float(lam), int(iters), w, h)
    return out


# ----------------------------------------------------------------------
# Image formats as the reference's kernels read them.  cvt::IFormatID
# (cvt/gfx/IFormat.h:36-63) -> OpenCL image format (IFormat::toCLImageFormat,
# IFormat.h:293-328) -> what read_imagef returns (OpenCL 1.2, 6.12.14.1 for
# the channel orders, 8.3.1.1 for normalized integers).  float32 numpy
# division is the correctly rounded IEEE division.


def image_to_rgbaf(arr: np.ndarray, fmt: int) -> np.ndarray:
    """(H, W[, C]) storage of format `fmt` -> (H, W, 4) float32 RGBA."""
    a = np.asarray(arr)
    if 1 <= fmt <= 16:
        kind = (fmt - 1) % 4          # 0 unorm8, 1 unorm16, 2 snorm16, 3 float
        order = ("I", "RG", "RGBA", "BGRA")[(fmt - 1) // 4]
    elif 17 <= fmt <= 19:
        kind, order = 0, "I"          # Bayer: CL_INTENSITY, CL_UNORM_INT8
    elif fmt in (20, 21):
        kind, order = 0, "RA"         # YUYV / UYVY: CL_RA, CL_UNORM_INT8
    else:
        raise ValueError(fmt)
    if kind == 0:
        v = a.astype(np.float32) / np.float32(255.0)
    elif kind == 1:
        v = a.astype(np.float32) / np.float32(65535.0)
    elif kind == 2:
        v = np.maximum(np.float32(-1.0), a.astype(np.float32) / np.float32(32767.0))
    else:
        v = a.astype(np.float32)
    if v.ndim == 2:
        v = v[..., None]
    H, W = v.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    if order == "I":
        out[...] = v[..., :1]
    elif order == "RG":
        out[..., 0], out[..., 1], out[..., 3] = v[..., 0], v[..., 1], 1.0
    elif order == "RA":
        out[..., 0], out[..., 3] = v[..., 0], v[..., 1]
    elif order == "RGBA":
        out[...] = v
    else:                             # stored B, G, R, A
        out[..., 0], out[..., 1], out[..., 2], out[..., 3] = v[..., 2], v[..., 1], v[..., 0], v[..., 3]
    return out


# ----------------------------------------------------------------------
# Stereo rectification and IWarp::apply (orc_stereo_rectify, orc_warp in
# pm_oracle.cpp).  A camera is a dict: "K" (3, 3), "radial" (3,),
# "tangential" (2,) float32.

WARP_KIND = {4: 0, 12: 1, 16: 1, 1: 2, 9: 3, 13: 3}   # IFormatID -> IWarp::apply variant


def _rect_call(fn, cam0, cam1, E, vertical, W, H):
    f = lambda a, n: np.ascontiguousarray(np.asarray(a, np.float32).reshape(n))
    map0 = np.empty((H, W, 2), np.float32)
    map1 = np.empty((H, W, 2), np.float32)
    K0n, K1n, Rl, Rr = (np.empty(9, np.float32) for _ in range(4))
    En = np.empty(16, np.float32)
    args = [f(cam0["K"], 9), f(cam0["radial"], 3), f(cam0["tangential"], 2), f(cam1["K"], 9), f(cam1["radial"], 3),
            f(cam1["tangential"], 2), f(E, 16)]
    rc = fn(*[a.ctypes.data for a in args], int(vertical), int(W), int(H), map0.ctypes.data, map1.ctypes.data,
            K0n.ctypes.data, K1n.ctypes.data, En.ctypes.data, Rl.ctypes.data, Rr.ctypes.data)
    if rc:
        raise RuntimeError("rectification failed")
    return {"map0": map0, "map1": map1, "K0": K0n.reshape(3, 3), "K1": K1n.reshape(3, 3),
            "E": En.reshape(4, 4), "R0": Rl.reshape(3, 3), "R1": Rr.reshape(3, 3)}


def _warp_call(fn, fmt, src, warp_map):
    src = np.ascontiguousarray(src)
    warp_map = np.ascontiguousarray(warp_map, np.float32)
    H, W = warp_map.shape[:2]
    kind = WARP_KIND[fmt]
    sh, sw = src.shape[:2]
    dst = np.empty((H, W) + src.shape[2:], src.dtype)
    rc = fn(kind, src.ctypes.data, src.strides[0], sw, sh, warp_map.ctypes.data, warp_map.strides[0], W, H,
            dst.ctypes.data, dst.strides[0])
    if rc:
        raise RuntimeError("warp failed")
    return dst


def _rect_lib(L):
    vp, c_int, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    L.orc_stereo_rectify.argtypes = [vp] * 7 + [c_int, c_int, c_int] + [vp] * 7
    L.orc_warp.argtypes = [c_int, vp, sz, c_int, c_int, vp, sz, c_int, c_int, vp, sz]
    return L


def stereo_rectify(cam0, cam1, E, vertical, W, H):
    """StereoCameraCalibration(cam0, cam1, E).undistortRectify on W x H maps."""
    return _rect_call(_rect_lib(lib()).orc_stereo_rectify, cam0, cam1, E, vertical, W, H)


def warp(fmt, src, warp_map):
    """IWarp::apply(dst, src, warp) for GRAY/RGBA/BGRA float and uint8 storage."""
    return _warp_call(_rect_lib(lib()).orc_warp, fmt, src, warp_map)


# ----------------------------------------------------------------------
# TSDF fusion (orc_tsdf_* in pm_oracle.cpp).  Volumes are (D, H, W, 2)
# float32 arrays of (tsdf, weight); matrices (4, 4) float32 row-major.

def _tsdf_lib():
    L = lib()
    vp, c_int, c_float = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.orc_tsdf_matrices.argtypes = [vp, vp, vp, vp]
    L.orc_tsdf_clear.argtypes = [vp, c_int, c_int, c_int, c_float]
    L.orc_tsdf_add.argtypes = [vp, c_int, c_int, c_int, vp, c_int, c_int, c_float, vp, c_float]
    L.orc_tsdf_raycast.argtypes = [vp, c_int, c_int, vp, c_int, c_int, c_int, vp, vp, c_float, c_int]
    L.orc_tsdf_slice.argtypes = [vp, c_int, c_int, vp, c_int, c_int, c_int]
    return L


def _m4(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(4, 4))


def tsdf_matrices(proj, g2w):
    """(proj * g2w, its inverse) as TSDFVolume::addDepthMap / rayCastDepthMap form them."""
    t, ti = np.empty((4, 4), np.float32), np.empty((4, 4), np.float32)
    p, g = _m4(proj), _m4(g2w)
    _tsdf_lib().orc_tsdf_matrices(p.ctypes.data, g.ctypes.data, t.ctypes.data, ti.ctypes.data)
    return t, ti


def tsdf_clear(W, H, D, weight=0.0):
    v = np.empty((D, H, W, 2), np.float32)
    _tsdf_lib().orc_tsdf_clear(v.ctypes.data, W, H, D, float(weight))
    return v


def tsdf_add(vol, dmap, dscale, tg2cam, trunc):
    """In place: TSDFVolume_add with the kernel matrix TG2CAM."""
    D, H, W = vol.shape[:3]
    dm = np.ascontiguousarray(dmap, np.float32)
    t = _m4(tg2cam)
    _tsdf_lib().orc_tsdf_add(vol.ctypes.data, W, H, D, dm.ctypes.data, dm.shape[1], dm.shape[0], float(dscale),
                             t.ctypes.data, float(trunc))
    return vol


def tsdf_raycast(vol, iw, ih, tcam2g, tg2cam, scale, max_steps=None):
    D, H, W = vol.shape[:3]
    if max_steps is None:
        max_steps = 2 * max(W, H, D) + 16
    out = np.empty((ih, iw), np.float32)
    ti, t = _m4(tcam2g), _m4(tg2cam)
    _tsdf_lib().orc_tsdf_raycast(out.ctypes.data, iw, ih, vol.ctypes.data, W, H, D, ti.ctypes.data, t.ctypes.data,
                                 float(scale), int(max_steps))
    return out


def tsdf_slice(vol, axis, index):
    D, H, W = vol.shape[:3]
    shape = {0: (D, H), 1: (D, W), 2: (H, W)}[axis]
    out = np.empty(shape + (4,), np.float32)
    _tsdf_lib().orc_tsdf_slice(out.ctypes.data, axis, index, vol.ctypes.data, W, H, D)
    return out


# ----------------------------------------------------------------------
# StereoGCVFilter (orc_gcv_* in pm_oracle.cpp).  Images (H, W, 4) float32.

def _gcv_lib():
    L = lib()
    vp, c_int, c_float = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.orc_gcv_depthmap.argtypes = [vp, vp, vp, c_int, c_int, c_float, c_float, c_float]
    L.orc_gcv_apply.argtypes = [vp, vp, vp, vp, vp, c_int, c_int, c_float, c_float, c_float]
    return L


def gcv_depthmap(cam0, cam1, dmin, dmax, dt):
    """StereoGCVFilter::depthmap: the normalised depth map of cam1's view."""
    a = np.ascontiguousarray(cam0, np.float32)
    b = np.ascontiguousarray(cam1, np.float32)
    H, W = a.shape[:2]
    out = np.empty((H, W), np.float32)
    _gcv_lib().orc_gcv_depthmap(out.ctypes.data, a.ctypes.data, b.ctypes.data, W, H, float(dmin), float(dmax),
                                float(dt))
    return out


def gcv_apply(cam0, cam1, dmin, dmax, dt):
    """StereoGCVFilter::apply: (GRAY_UINT8 fused map, d0, d1)."""
    a = np.ascontiguousarray(cam0, np.float32)
    b = np.ascontiguousarray(cam1, np.float32)
    H, W = a.shape[:2]
    out = np.empty((H, W), np.uint8)
    d0 = np.empty((H, W), np.float32)
    d1 = np.empty((H, W), np.float32)
    _gcv_lib().orc_gcv_apply(out.ctypes.data, d0.ctypes.data, d1.ctypes.data, a.ctypes.data, b.ctypes.data, W, H,
                             float(dmin), float(dmax), float(dt))
    return out, d0, d1


def disparity_to_depth(disp, dispscale, focallength, baseline, dispthres=0.01):
    """Vision::disparityToDepthmap (orc_disparity_to_depth)."""
    L = lib()
    vp, c_int, c_float = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.orc_disparity_to_depth.argtypes = [vp, vp, c_int, c_int, c_float, c_float, c_float, c_float]
    d = np.ascontiguousarray(disp, np.float32)
    out = np.empty_like(d)
    L.orc_disparity_to_depth(out.ctypes.data, d.ctypes.data, d.shape[1], d.shape[0], float(dispscale),
                             float(focallength), float(baseline), float(dispthres))
    return out
