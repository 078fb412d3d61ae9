"""The image adapter on the GPU: every cvt::IFormat read into RGBA float32 as
the reference's read_imagef returns it (bit-exact against the oracle's
restatement of the OpenCL conversion rules), and PMHuberStereo::depthMap on
typed images equal to the float path on the converted images."""
import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import _lib, imageio, scenes
from cvt_gb300.params import default_params, PRESET_BASELINE

pytestmark = pytest.mark.gpu


def _storage(fmt, h, w, seed):
    c, dt = imageio.fmt_info(fmt)
    rng = np.random.default_rng(seed)
    shape = (h, w) if c == 1 else (h, w, c)
    if dt == np.float32:
        return rng.standard_normal(shape).astype(np.float32)
    info = np.iinfo(dt)
    return rng.integers(info.min, info.max, size=shape, endpoint=True).astype(dt)


def _upload_padded(a, pad_bytes):
    """Rows of the array's bytes plus `pad_bytes` of padding, as a (H, stride)
    uint8 CUDA tensor viewed down to the image bytes."""
    h = a.shape[0]
    row = a.reshape(h, -1).view(np.uint8)
    buf = np.full((h, row.shape[1] + pad_bytes), 0xAB, np.uint8)
    buf[:, :row.shape[1]] = row
    return torch.from_numpy(buf).cuda()[:, :row.shape[1]]


@pytest.mark.parametrize("fmt", range(1, 22))
def test_every_format_bitexact(cuda, oracle, fmt):
    a = _storage(fmt, 11, 37, 100 + fmt)
    t = _upload_padded(a, 24)
    if np.dtype(imageio.fmt_info(fmt)[1]).itemsize == 1:
        c = imageio.fmt_info(fmt)[0]
        t = t.view(11, 37, c) if c > 1 else t              # typed uint8 view, padded rows
    got = imageio.to_rgbaf(t, fmt).cpu().numpy()
    want = oracle.image_to_rgbaf(a, fmt)
    d = bit_diff(got, want)
    assert not d.any(), f"format {fmt}: {int(d.sum())} values differ"


def test_typed_depthmap_equals_float_path(cuda, oracle):
    """Left RGBA_UINT8, right BGRA_UINT8 (the reference allows different
    formats): the same disparities, states and winners as depthMap on the
    oracle's float conversion of both."""
    from cvt_gb300.stereo import PMHuberStereo
    sc = scenes.make_scene(96, 64, 4, 16.0, seed=21)
    lu8 = np.round(sc.left * 255).astype(np.uint8)
    ru8 = np.ascontiguousarray(np.round(sc.right * 255).astype(np.uint8)[..., [2, 1, 0, 3]])
    p = default_params(PRESET_BASELINE, patchsize=7, depthmax=16.0, iterations=3, pd_iterations=20)
    st = PMHuberStereo(0, p)
    tr1, tr2 = {}, {}
    d1 = st.depthMapImage(None, torch.from_numpy(lu8).cuda(), imageio.RGBA_UINT8, torch.from_numpy(ru8).cuda(),
                          imageio.BGRA_UINT8, 7, 16.0, 3, 4, trace=tr1)
    lf = torch.from_numpy(oracle.image_to_rgbaf(lu8, imageio.RGBA_UINT8)).cuda()
    rf = torch.from_numpy(oracle.image_to_rgbaf(ru8, imageio.BGRA_UINT8)).cuda()
    d2 = st.depthMap(None, lf, rf, 7, 16.0, 3, 4, trace=tr2)
    torch.cuda.synchronize()
    assert not bit_diff(d1.cpu().numpy(), d2.cpu().numpy()).any()
    for k in ("winners", "valid", "states"):
        assert not bit_diff(tr1[k].cpu().numpy(), tr2[k].cpu().numpy()).any(), k


def test_gray_uint16_input(cuda, oracle):
    from cvt_gb300.stereo import PMHuberStereo
    sc = scenes.make_scene(64, 48, 3, 8.0, seed=22)
    g = lambda im: np.round((0.2126 * im[..., 0] + 0.7152 * im[..., 1] + 0.0722 * im[..., 2]) * 65535).astype(np.uint16)
    gl, gr = g(sc.left), g(sc.right)
    p = default_params(PRESET_BASELINE, patchsize=5, depthmax=8.0, iterations=2, pd_iterations=10)
    st = PMHuberStereo(0, p)
    bl = torch.from_numpy(gl.view(np.uint8)).cuda()
    br = torch.from_numpy(gr.view(np.uint8)).cuda()
    d1 = st.depthMapImage(None, bl, imageio.GRAY_UINT16, br, imageio.GRAY_UINT16, 5, 8.0, 2, 4)
    d2 = st.depthMap(None, torch.from_numpy(oracle.image_to_rgbaf(gl, imageio.GRAY_UINT16)).cuda(),
                     torch.from_numpy(oracle.image_to_rgbaf(gr, imageio.GRAY_UINT16)).cuda(), 5, 8.0, 2, 4)
    torch.cuda.synchronize()
    assert not bit_diff(d1.cpu().numpy(), d2.cpu().numpy()).any()


def test_typed_depthmap_errors(cuda):
    from cvt_gb300.stereo import PMHuberStereo, CVTException
    st = PMHuberStereo(0)
    a = torch.zeros((8, 8, 4), dtype=torch.uint8, device="cuda")
    b = torch.zeros((8, 9, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(CVTException):
        st.depthMapImage(None, a, imageio.RGBA_UINT8, b, imageio.RGBA_UINT8, 3, 4.0, 1, 4)
    # the C entry: sizes differ -> CVTPM_ERR_INCONSISTENT; unknown format -> invalid argument
    L = _lib.lib()
    da = imageio.device_desc(a, imageio.RGBA_UINT8)
    db = imageio.device_desc(b, imageio.RGBA_UINT8)
    import ctypes
    out = torch.empty((8, 8), device="cuda")
    assert L.cvtpm_depthmap_image(st._h, out.data_ptr(), 32, ctypes.byref(da), ctypes.byref(db), 3, 4.0, 1, 4,
                                  -1.0, None, 0, None, None) == 3
    db = imageio.device_desc(a, imageio.RGBA_UINT8)
    db.format = 42
    assert L.cvtpm_depthmap_image(st._h, out.data_ptr(), 32, ctypes.byref(da), ctypes.byref(db), 3, 4.0, 1, 4,
                                  -1.0, None, 0, None, None) == 1
    assert "unknown image format" in L.cvtpm_last_error(st._h).decode()
