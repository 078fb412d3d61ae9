"""Seeded synthetic rectified stereo pairs with ground-truth disparity.

The reference ships no stereo data with ground truth for this path, so every
measurement runs on generated scenes:

* Voronoi layout: ``nplanes`` sites uniform in the image; each cell carries a
  disparity plane ``d = a*x + b*y + c`` (left-view pixel coordinates) with
  ``d0 ~ U[0, dmax]`` at the site and ``(a, b) ~ U[-0.15, 0.15]^2``, redrawn
  until ``d`` stays in ``[0, dmax]`` over the whole cell.
* Texture: per-channel uniform noise blurred by a separable Gaussian
  (sigma 1.5, radius 5), min-max stretched back to [0, 1]; alpha = 1.
* Right view: ``I_R(x, y) = I_L(x + d_R(x, y), y)`` (linear interpolation in
  x), where ``d_R`` is the left ground truth forward-mapped with a z-test
  (larger disparity wins); right-view pixels that no left surface reaches take
  the smaller (background) disparity of their row neighbours.
* Left occlusion mask: ``|d_L(x) - d_R(round(x - d_L))| > 0.5`` or the match
  leaves the image.
* Optional salt noise (a fraction of pixels per view set to 1.0) and a
  per-channel gain/bias mismatch of the right view.

Everything is float32, row-major RGBA (H, W, 4).
"""
from __future__ import annotations

import dataclasses

import numpy as np
from scipy.ndimage import convolve1d


@dataclasses.dataclass
class StereoScene:
    left: np.ndarray      # (H, W, 4) float32
    right: np.ndarray     # (H, W, 4) float32
    disp_left: np.ndarray  # (H, W) float32 ground truth, left view
    disp_right: np.ndarray  # (H, W) float32 ground truth, right view
    occluded: np.ndarray  # (H, W) bool, left pixels without a visible match
    planes: np.ndarray    # (nplanes, 3) float64 (a, b, c)
    labels: np.ndarray    # (H, W) int32 Voronoi cell of each left pixel
    dmax: float

    @property
    def width(self) -> int:
        return self.left.shape[1]

    @property
    def height(self) -> int:
        return self.left.shape[0]

    def plane_field(self) -> np.ndarray:
        """Per-pixel ground-truth plane (a, b, c, 0) of the left view."""
        out = np.zeros(self.labels.shape + (4,), np.float32)
        out[..., :3] = self.planes[self.labels]
        return out


def _texture(rng: np.random.Generator, h: int, w: int) -> np.ndarray:
    r = np.arange(-5, 6, dtype=np.float64)
    g = np.exp(-0.5 * (r / 1.5) ** 2)
    g /= g.sum()
    img = np.ones((h, w, 4), np.float64)
    for ch in range(3):
        n = rng.random((h, w))
        n = convolve1d(n, g, axis=0, mode="reflect")
        n = convolve1d(n, g, axis=1, mode="reflect")
        lo, hi = n.min(), n.max()
        img[..., ch] = (n - lo) / max(hi - lo, 1e-12)
    return img


def _voronoi(rng: np.random.Generator, h: int, w: int, nplanes: int, dmax: float):
    sx = rng.random(nplanes) * w
    sy = rng.random(nplanes) * h
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    best = np.full((h, w), np.inf)
    labels = np.zeros((h, w), np.int32)
    for i in range(nplanes):
        dist = (xx - sx[i]) ** 2 + (yy - sy[i]) ** 2
        m = dist < best
        best[m] = dist[m]
        labels[m] = i
    planes = np.zeros((nplanes, 3))
    for i in range(nplanes):
        m = labels == i
        cx, cy = xx[m], yy[m]
        for _ in range(1000):
            d0 = rng.random() * dmax
            a, b = (rng.random(2) - 0.5) * 0.3
            c = d0 - a * sx[i] - b * sy[i]
            if cx.size == 0:
                break
            d = a * cx + b * cy + c
            if d.min() >= 0.0 and d.max() <= dmax:
                break
        else:  # fall back to a fronto-parallel plane
            a = b = 0.0
            c = rng.random() * dmax
        planes[i] = (a, b, c)
    return labels, planes


def _interp_row(img: np.ndarray, xs: np.ndarray) -> np.ndarray:
    """Linear interpolation of img (H, W, C) at per-pixel x positions xs (H, W),
    edge-clamped, same row."""
    h, w, _ = img.shape
    xs = np.clip(xs, 0.0, w - 1.0)
    x0 = np.floor(xs).astype(np.int64)
    x1 = np.minimum(x0 + 1, w - 1)
    a = (xs - x0)[..., None]
    rows = np.arange(h)[:, None]
    return img[rows, x0] * (1.0 - a) + img[rows, x1] * a


def make_scene(width: int, height: int, nplanes: int, dmax: float, seed: int,
               salt: float = 0.0, gain_bias: float = 0.0) -> StereoScene:
    rng = np.random.default_rng(seed)
    h, w = height, width
    labels, planes = _voronoi(rng, h, w, nplanes, dmax)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    pa, pb, pc = planes[labels, 0], planes[labels, 1], planes[labels, 2]
    dl = pa * xx + pb * yy + pc

    # right-view disparity: for every plane, the left position that lands on
    # each right pixel; keep it when it lies in that plane's cell; nearest wins.
    dr = np.full((h, w), -np.inf)
    for i, (a, b, c) in enumerate(planes):
        xl = (xx + b * yy + c) / (1.0 - a)
        inside = (xl >= 0) & (xl <= w - 1)
        xi = np.clip(np.rint(xl), 0, w - 1).astype(np.int64)
        ok = inside & (labels[np.arange(h)[:, None], xi] == i)
        d = a * xl + b * yy + c
        dr = np.where(ok & (d > dr), d, dr)
    hole = ~np.isfinite(dr)
    if hole.any():
        idx = np.arange(w)[None, :].repeat(h, 0)
        lidx = np.where(~hole, idx, -1)
        lidx = np.maximum.accumulate(lidx, axis=1)
        ridx = np.where(~hole, idx, w)
        ridx = np.minimum.accumulate(ridx[:, ::-1], axis=1)[:, ::-1]
        rows = np.arange(h)[:, None]
        lv = np.where(lidx >= 0, dr[rows, np.clip(lidx, 0, w - 1)], np.inf)
        rv = np.where(ridx < w, dr[rows, np.clip(ridx, 0, w - 1)], np.inf)
        fillv = np.minimum(lv, rv)
        fillv = np.where(np.isfinite(fillv), fillv, 0.0)
        dr = np.where(hole, fillv, dr)

    tex = _texture(rng, h, w)
    left = tex.copy()
    right = _interp_row(tex, xx + dr)
    right[..., 3] = 1.0

    xr = np.rint(xx - dl).astype(np.int64)
    out = (xr < 0) | (xr >= w)
    drl = dr[np.arange(h)[:, None], np.clip(xr, 0, w - 1)]
    occ = out | (np.abs(dl - drl) > 0.5)

    if salt > 0.0:
        for img in (left, right):
            m = rng.random((h, w)) < salt
            img[m, :3] = 1.0
    if gain_bias > 0.0:
        g = 1.0 + (rng.random(3) - 0.5) * 2.0 * gain_bias
        bias = (rng.random(3) - 0.5) * 2.0 * gain_bias
        right[..., :3] = np.clip(right[..., :3] * g + bias, 0.0, 1.0)

    return StereoScene(left=left.astype(np.float32), right=right.astype(np.float32),
                       disp_left=dl.astype(np.float32), disp_right=dr.astype(np.float32),
                       occluded=occ, planes=planes, labels=labels, dmax=float(dmax))


def batch_shapes(npairs: int = 64, seed: int = 3000):
    """Pair shapes of the batched workload: widths uniform in 320-1920,
    heights in 240-1080, disparity ranges 32-256 px, 4-24 planes; returns
    (width, height, dmax, nplanes, scene seed) per pair."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(npairs):
        w = int(rng.integers(320, 1921))
        h = int(rng.integers(240, 1081))
        dmax = float(rng.integers(32, 257))
        nplanes = int(rng.integers(4, 25))
        out.append((w, h, dmax, nplanes, seed + 1 + i))
    return out


def batch_scene(shape) -> StereoScene:
    w, h, dmax, nplanes, seed = shape
    return make_scene(w, h, nplanes, dmax, seed)


def config_scene(index: int, pair: int = 0) -> StereoScene:
    """The scene of a named workload, seeded 1000*config + pair.

    1: 640x480, 8 planes, dmax 64.
    2: 1242x375, 16 planes, dmax 128, 2% salt, +/-5% gain/bias.
    """
    seed = 1000 * index + pair
    if index == 1:
        return make_scene(640, 480, 8, 64.0, seed)
    if index == 2:
        return make_scene(1242, 375, 16, 128.0, seed, salt=0.02, gain_bias=0.05)
    raise ValueError(f"unknown scene config {index}")


def bad_pixel_rate(dmap_px: np.ndarray, scene: StereoScene, thresh: float = 1.0,
                   nonocc: bool = True) -> float:
    """Percentage of (non-occluded) left pixels whose disparity error exceeds thresh."""
    err = np.abs(dmap_px.astype(np.float64) - scene.disp_left)
    m = ~scene.occluded if nonocc else np.ones_like(scene.occluded)
    bad = ~(err <= thresh)
    return 100.0 * float(bad[m].mean()) if m.any() else 0.0


def end_point_error(dmap_px: np.ndarray, scene: StereoScene, nonocc: bool = True) -> float:
    err = np.abs(dmap_px.astype(np.float64) - scene.disp_left)
    m = ~scene.occluded if nonocc else np.ones_like(scene.occluded)
    e = err[m]
    e = e[np.isfinite(e)]
    return float(e.mean()) if e.size else float("nan")


def render_depth(K, E, width: int, height: int, spheres=((0.0, 0.0, 2.0, 0.5),),
                 planes=((0.0, 0.0, 1.0, 3.0),)) -> np.ndarray:
    """Camera-space depth (z) of the first surface along each pixel's ray, 0
    where none: spheres (cx, cy, cz, r) and planes n . X = d (nx, ny, nz, d)
    in world coordinates; K 3x3 intrinsics, E 4x4 world-to-camera.  Inputs for
    the TSDF fusion workloads."""
    Ki = np.linalg.inv(np.asarray(K, np.float64))
    Ei = np.linalg.inv(np.asarray(E, np.float64))
    v, u = np.mgrid[0:height, 0:width].astype(np.float64)
    dirs = (np.stack([u, v, np.ones_like(u)], -1) @ Ki.T) @ Ei[:3, :3].T   # camera z = 1 per unit of t
    o = Ei[:3, 3]
    best = np.full((height, width), np.inf)
    a = (dirs * dirs).sum(-1)
    for cx, cy, cz, r in spheres:
        oc = o - np.array([cx, cy, cz])
        b = dirs @ oc
        disc = b * b - a * ((oc * oc).sum() - r * r)
        t = (-b - np.sqrt(np.maximum(disc, 0.0))) / a
        best = np.where((disc > 0) & (t > 0) & (t < best), t, best)
    for nx, ny, nz, d in planes:
        n = np.array([nx, ny, nz])
        den = dirs @ n
        with np.errstate(divide="ignore", invalid="ignore"):
            t = (d - o @ n) / den
        best = np.where((t > 0) & (t < best), t, best)
    return np.where(np.isfinite(best), best, 0.0).astype(np.float32)
