"""The input side on the host (no GPU): the reference's image files read and
written by libcvtpm.so, checked against files laid out here by hand after the
reference's loaders and savers, and the format table of the image adapter.

  CVTRaw  plugins/iloader/CVTRaw/CVTRawLoader.cpp, plugins/isaver/CVTRaw/CVTRawSaver.cpp
  PPM     plugins/iloader/PPM/PPMLoader.cpp
  PFM     plugins/isaver/PFM/PFMSaver.cpp
"""
import struct

import numpy as np
import pytest

from cvt_gb300 import _lib, imageio


def _random_image(fmt, h, w, seed):
    c, dt = imageio.fmt_info(fmt)
    rng = np.random.default_rng(seed)
    shape = (h, w) if c == 1 else (h, w, c)
    if dt == np.float32:
        return rng.standard_normal(shape).astype(np.float32)
    info = np.iinfo(dt)
    return rng.integers(info.min, info.max, size=shape, endpoint=True).astype(dt)


def test_bytes_per_pixel_follow_the_format_table():
    L = _lib.lib()
    for fmt in range(1, 22):
        c, dt = imageio.fmt_info(fmt)
        assert L.cvtpm_iformat_bpp(fmt) == c * np.dtype(dt).itemsize
    assert L.cvtpm_iformat_bpp(0) == 0 and L.cvtpm_iformat_bpp(22) == 0


@pytest.mark.parametrize("fmt", range(1, 22))
def test_raw_round_trip_every_format(tmp_path, fmt):
    a = _random_image(fmt, 5, 7, fmt)
    p = tmp_path / "img.raw"
    imageio.write_raw(p, a, fmt)
    b, f = imageio.read_raw(p)
    assert f == fmt and b.dtype == a.dtype and b.shape == a.shape
    assert a.tobytes() == b.tobytes()


def test_raw_layout_and_padded_stride(tmp_path):
    """A file as CVTRawSaver writes it (header width, height, stride, format
    id; rows of `stride` bytes) with a padded stride reads back tight."""
    w, h, stride = 3, 2, 16
    rows = [bytes(range(10 * y, 10 * y + w)) + b"\xee" * (stride - w) for y in range(h)]
    p = tmp_path / "pad.raw"
    p.write_bytes(struct.pack("<4I", w, h, stride, imageio.GRAY_UINT8) + b"".join(rows))
    b, f = imageio.read_raw(p)
    assert f == imageio.GRAY_UINT8
    assert b.tolist() == [[0, 1, 2], [10, 11, 12]]
    # and the writer lays out what it was given, stride included
    a = np.arange(12, dtype=np.uint8).reshape(3, 4)
    q = tmp_path / "w.raw"
    imageio.write_raw(q, a, imageio.GRAY_UINT8)
    assert q.read_bytes() == struct.pack("<4I", 4, 3, 4, imageio.GRAY_UINT8) + a.tobytes()


@pytest.mark.parametrize("content,msg", [
    (b"", "header truncated"),
    (struct.pack("<4I", 4, 4, 4, 99), "unknown format"),
    (struct.pack("<4I", 4, 4, 4, 1) + b"\0" * 15, "truncated"),
    (struct.pack("<4I", 4, 4, 2, 1) + b"\0" * 64, "stride"),
])
def test_raw_corrupt_files_rejected(tmp_path, content, msg):
    p = tmp_path / "bad.raw"
    p.write_bytes(content)
    with pytest.raises(_lib.CvtpmError) as e:
        imageio.read_raw(p)
    assert e.value.status == 8 and msg in str(e.value)


def test_missing_file(tmp_path):
    with pytest.raises(_lib.CvtpmError) as e:
        imageio.read_raw(tmp_path / "none.raw")
    assert e.value.status == 8


def test_ppm_binary_rgb_and_gray(tmp_path):
    rgb = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3) * 7
    p = tmp_path / "a.ppm"
    p.write_bytes(b"P6\n# a comment\n3 2\n255\n" + rgb.tobytes())
    a, f = imageio.read_ppm(p)
    assert f == imageio.RGBA_UINT8 and a.shape == (2, 3, 4)
    assert (a[..., :3] == rgb).all() and (a[..., 3] == 255).all()
    g = np.arange(6, dtype=np.uint8).reshape(2, 3) * 40
    q = tmp_path / "b.pgm"
    q.write_bytes(b"P5 3 2 255\n" + g.tobytes())
    b, f = imageio.read_ppm(q)
    assert f == imageio.GRAY_UINT8 and (b == g).all()


def test_ppm_ascii(tmp_path):
    p = tmp_path / "a.ppm"
    p.write_text("P3\n2 1\n255\n# comment line\n1 2 3  4 5 6\n")
    a, f = imageio.read_ppm(p)
    assert f == imageio.RGBA_UINT8 and a.tolist() == [[[1, 2, 3, 255], [4, 5, 6, 255]]]
    q = tmp_path / "b.pgm"
    q.write_text("P2\n3 1\n255\n7 8 9\n")
    b, f = imageio.read_ppm(q)
    assert f == imageio.GRAY_UINT8 and b.tolist() == [[7, 8, 9]]


@pytest.mark.parametrize("content,status", [
    (b"P7\n1 1\n255\n\0", 8),                 # unknown type
    (b"P6\n1 1\n65535\n" + b"\0" * 6, 7),     # 16-bit: no reader in the reference
    (b"P6\n2 2\n255\n" + b"\0" * 5, 8),       # not enough data
    (b"P6\n2\n", 8),                          # header corrupt
])
def test_ppm_rejected(tmp_path, content, status):
    p = tmp_path / "bad.ppm"
    p.write_bytes(content)
    with pytest.raises(_lib.CvtpmError) as e:
        imageio.read_ppm(p)
    assert e.value.status == status


def _parse_pfm(data: bytes):
    lines = data.split(b"\n", 3)
    magic, dims, scale, body = lines
    w, h = map(int, dims.split())
    ch = 3 if magic == b"PF" else 1
    endian = "<" if float(scale) < 0 else ">"
    px = np.frombuffer(body, dtype=endian + "f4").reshape(h, w, ch)
    return magic, float(scale), px[::-1]      # stored bottom to top


def test_pfm_gray_and_rgba(tmp_path):
    g = np.arange(12, dtype=np.float32).reshape(3, 4) / 7
    p = tmp_path / "d.pfm"
    imageio.write_pfm(p, g, imageio.GRAY_FLOAT)
    magic, scale, px = _parse_pfm(p.read_bytes())
    assert magic == b"Pf" and scale == -1.0 and (px[..., 0] == g).all()
    c = np.random.default_rng(1).random((2, 3, 4), dtype=np.float32)
    q = tmp_path / "c.pfm"
    imageio.write_pfm(q, c, imageio.RGBA_FLOAT)
    magic, _, px = _parse_pfm(q.read_bytes())
    assert magic == b"PF" and (px == c[..., :3]).all()     # alpha dropped
    with pytest.raises(_lib.CvtpmError) as e:
        imageio.write_pfm(q, np.zeros((2, 2), np.uint8), imageio.GRAY_UINT8)
    assert e.value.status == 7


def test_oracle_format_table(oracle):
    """Spot values of the read_imagef conversions the GPU adapter is checked
    against: normalized integers, channel orders."""
    f = oracle.image_to_rgbaf
    u8 = np.array([[0, 255, 51]], np.uint8)
    assert f(u8, imageio.GRAY_UINT8)[0].tolist() == [[0.0] * 4, [1.0] * 4, [np.float32(0.2)] * 4]
    i16 = np.array([[-32768, 32767]], np.int16)
    assert f(i16, imageio.GRAY_INT16)[0, :, 0].tolist() == [-1.0, 1.0]
    ga = np.array([[[255, 0]]], np.uint8)
    assert f(ga, imageio.GRAYALPHA_UINT8)[0, 0].tolist() == [1.0, 0.0, 0.0, 1.0]
    bgra = np.array([[[0, 51, 255, 102]]], np.uint8)
    assert f(bgra, imageio.BGRA_UINT8)[0, 0].tolist() == f(bgra[..., [2, 1, 0, 3]], imageio.RGBA_UINT8)[0, 0].tolist()
    yuyv = np.array([[[255, 51]]], np.uint8)
    r = f(yuyv, imageio.YUYV_UINT8)[0, 0]
    assert r[0] == 1.0 and r[1] == 0.0 and r[2] == 0.0 and r[3] == np.float32(0.2)
