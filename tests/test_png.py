"""PNG files through libcvtpm.so on the host (no GPU): the decoder against
files made by an independent encoder (tests/pngtool.py over Python's zlib)
for every colour type, bit depth, filter, interlace method and zlib block
type, with the reference's libpng transformations applied to the expected
pixels; the encoder against the independent decoder; the float conversions
of the saver against the reference's own (tests/golden/make_png_golden.py);
corrupt and unsupported files; and, where the reference's data files are
present, its PNG images."""
import glob
import os
import struct
import sys
import zlib

import numpy as np
import pytest

from cvt_gb300 import _lib, imageio

sys.path.insert(0, os.path.dirname(__file__))
import pngtool  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "png_reference_golden.npz")
RNG = np.random.default_rng(5)


def expected(samples, ctype, depth, plte=None, trns=None):
    """(array, format) the reference's loader gives for these PNG samples."""
    H, W = samples.shape[:2]
    top = 65535 if depth == 16 else 255
    dt = np.uint16 if depth == 16 else np.uint8
    s = samples.astype(np.int64)
    if ctype == 3:
        pal = np.frombuffer(plte, np.uint8).reshape(-1, 3).astype(np.int64)
        alpha = np.full(len(pal), 255, np.int64)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        idx = s[..., 0]
        return np.concatenate([pal[idx], alpha[idx][..., None]], -1).astype(np.uint8), imageio.RGBA_UINT8
    if ctype == 0:
        g = s[..., 0] * (255 // ((1 << depth) - 1)) if depth < 8 else s[..., 0]
        if trns is None:
            return g.astype(dt), (imageio.GRAY_UINT16 if depth == 16 else imageio.GRAY_UINT8)
        key = struct.unpack(">H", trns)[0]
        a = np.where(s[..., 0] == key, 0, top)
        return np.stack([g, a], -1).astype(dt), (imageio.GRAYALPHA_UINT16 if depth == 16 else imageio.GRAYALPHA_UINT8)
    if ctype == 4:
        return s.astype(dt), (imageio.GRAYALPHA_UINT16 if depth == 16 else imageio.GRAYALPHA_UINT8)
    if ctype == 2:
        if trns is None:
            a = np.full((H, W), 255)
        else:
            key = np.array(struct.unpack(">HHH", trns))
            a = np.where((s == key).all(-1), 0, top)
        s = np.concatenate([s, a[..., None]], -1)
    return s.astype(dt), (imageio.RGBA_UINT16 if depth == 16 else imageio.RGBA_UINT8)


CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("ctype,depth", CASES)
def test_decoder_all_types(tmp_path, ctype, depth, interlace):
    for (W, H), level in (((13, 7), 6), ((1, 1), 0), ((33, 19), 9), ((5, 11), 1)):
        nch = pngtool.CHANNELS[ctype]
        if ctype == 3:
            n = min(1 << depth, 40)
            s = RNG.integers(0, n, (H, W, 1))
            plte = RNG.integers(0, 256, 3 * n).astype(np.uint8).tobytes()
        else:
            s = RNG.integers(0, 1 << depth, (H, W, nch))
            plte = None
        data = pngtool.encode(s, ctype, depth, interlace=interlace, plte=plte, level=level, idat_split=7)
        p = tmp_path / f"t{ctype}_{depth}_{W}.png"
        p.write_bytes(data)
        got, fmt = imageio.read_png(p)
        want, wfmt = expected(s, ctype, depth, plte)
        assert fmt == wfmt
        assert np.array_equal(got.reshape(want.shape), want), (W, H, level)


@pytest.mark.parametrize("ctype,depth", [(0, 2), (0, 8), (0, 16), (2, 8), (2, 16), (3, 4), (3, 8)])
def test_decoder_transparency(tmp_path, ctype, depth):
    W, H = 17, 9
    nch = pngtool.CHANNELS[ctype]
    plte = None
    if ctype == 3:
        n = min(1 << depth, 12)
        s = RNG.integers(0, n, (H, W, 1))
        plte = RNG.integers(0, 256, 3 * n).astype(np.uint8).tobytes()
        trns = bytes([0]) + RNG.integers(0, 256, n - 4).astype(np.uint8).tobytes()   # shorter than the palette
        s[0, 0] = 0
    else:
        s = RNG.integers(0, min(1 << depth, 6), (H, W, nch))           # few values: the key recurs
        key = s[0, 0]
        trns = struct.pack(">" + "H" * nch, *[int(v) for v in key])
    p = tmp_path / "t.png"
    p.write_bytes(pngtool.encode(s, ctype, depth, plte=plte, trns=trns))
    got, fmt = imageio.read_png(p)
    want, wfmt = expected(s, ctype, depth, plte, trns)
    assert fmt == wfmt
    assert np.array_equal(got.reshape(want.shape), want)
    assert (want[..., -1] == 0).any()


def _fixed_and_stored(raw: bytes) -> bytes:
    """zlib stream of a stored block, a fixed-Huffman block (Python's zlib
    with Z_FIXED) and an empty stored final block"""
    c = zlib.compressobj(6, zlib.DEFLATED, -15, 9, zlib.Z_FIXED)
    half = len(raw) // 2
    body = bytearray()
    first = raw[:half]
    body += bytes([0]) + struct.pack("<HH", len(first), len(first) ^ 0xffff) + first   # stored, not final
    comp = c.compress(raw[half:]) + c.flush(zlib.Z_FULL_FLUSH)
    body += comp
    body += bytes([1]) + struct.pack("<HH", 0, 0xffff)                                   # stored, final, empty
    return b"\x78\x01" + bytes(body) + struct.pack(">I", zlib.adler32(raw))


def test_decoder_mixed_blocks(tmp_path):
    """stored and fixed-Huffman blocks in one stream (Python's zlib at level
    6 writes dynamic blocks, at level 0 stored ones)"""
    W, H = 29, 13
    s = RNG.integers(0, 256, (H, W, 4))
    raw = b"".join(bytes([0]) + s[y].astype(np.uint8).tobytes() for y in range(H))
    z = _fixed_and_stored(raw)
    assert zlib.decompress(z) == raw
    data = pngtool.SIG + pngtool.chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, 6, 0, 0, 0))
    data += pngtool.chunk(b"IDAT", z) + pngtool.chunk(b"IEND", b"")
    p = tmp_path / "m.png"
    p.write_bytes(data)
    got, fmt = imageio.read_png(p)
    assert fmt == imageio.RGBA_UINT8 and np.array_equal(got, s.astype(np.uint8))


WRITABLE = [(imageio.GRAY_UINT8, 0, 8, 1), (imageio.GRAY_UINT16, 0, 16, 1), (imageio.GRAYALPHA_UINT8, 4, 8, 2),
            (imageio.GRAYALPHA_UINT16, 4, 16, 2), (imageio.RGBA_UINT8, 6, 8, 4), (imageio.RGBA_UINT16, 6, 16, 4),
            (imageio.BGRA_UINT8, 6, 8, 4), (imageio.BGRA_UINT16, 6, 16, 4)]


@pytest.mark.parametrize("fmt,ctype,depth,nch", WRITABLE)
def test_encoder_round_trips(tmp_path, fmt, ctype, depth, nch):
    dt = np.uint16 if depth == 16 else np.uint8
    for W, H in ((1, 1), (37, 23), (300, 7)):
        smooth = (np.add.outer(np.arange(H), np.arange(W))[..., None] * 3 + np.arange(nch)) % (1 << depth)
        a = np.where(RNG.random((H, W, nch)) < 0.3, RNG.integers(0, 1 << depth, (H, W, nch)), smooth).astype(dt)
        arr = a[..., 0] if nch == 1 else a
        p = tmp_path / "w.png"
        imageio.write_png(p, arr, fmt)
        s, ct, dp = pngtool.decode(p.read_bytes())
        assert (ct, dp) == (ctype, depth)
        want = a[..., [2, 1, 0, 3]] if fmt in (imageio.BGRA_UINT8, imageio.BGRA_UINT16) else a
        assert np.array_equal(s, want.astype(np.int64))
        back, bfmt = imageio.read_png(p)
        rgba = imageio.RGBA_UINT16 if depth == 16 else imageio.RGBA_UINT8
        assert bfmt == (rgba if nch == 4 else fmt)
        assert np.array_equal(back.reshape(want.shape), want)


def test_encoder_compresses():
    """a smooth 640 x 480 RGBA image: the filters and LZ77 matches make the
    file several times smaller than its pixels"""
    import tempfile
    y, x = np.mgrid[0:480, 0:640]
    a = np.stack([x % 256, y % 256, (x + y) % 256, np.full_like(x, 255)], -1).astype(np.uint8)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.png")
        imageio.write_png(p, a, imageio.RGBA_UINT8)
        assert os.path.getsize(p) < a.nbytes / 8
        back, _ = imageio.read_png(p)
        assert np.array_equal(back, a)


def test_float_conversions_match_reference(tmp_path):
    G = np.load(GOLDEN)
    x = G["x"]
    L = _lib.lib()
    got = np.array([L.cvtpm_float_to_srgb_u8(float(v)) for v in x], np.uint8)
    assert np.array_equal(got, G["gray"])
    n = x.size // 4
    # GRAY_FLOAT, GRAYALPHA_FLOAT and RGBA/BGRA_FLOAT images through the saver
    for fmt, key, shape in ((imageio.GRAY_FLOAT, "gray", (1, x.size)), (imageio.GRAYALPHA_FLOAT, "grayalpha",
                                                                        (1, x.size // 2, 2)),
                            (imageio.RGBA_FLOAT, "rgba", (1, n, 4)), (imageio.BGRA_FLOAT, "rgba", (1, n, 4))):
        img = x.reshape(shape)
        want = G[key].reshape(shape)
        if fmt == imageio.BGRA_FLOAT:
            img = np.ascontiguousarray(img[..., [2, 1, 0, 3]])
        p = tmp_path / "f.png"
        imageio.write_png(p, img, fmt)
        s, _, _ = pngtool.decode(p.read_bytes())
        assert np.array_equal(s.reshape(want.shape), want.astype(np.int64)), fmt


def test_float_conversions_live():
    from oracle.ref_emu import rect
    if not rect.available():
        pytest.skip("reference sources absent")
    x = np.random.default_rng(11).uniform(-0.5, 1.5, 4000).astype(np.float32)
    L = _lib.lib()
    assert np.array_equal(np.array([L.cvtpm_float_to_srgb_u8(float(v)) for v in x], np.uint8), rect.conv_f_u8(0, x))


def _corrupt(tmp_path, data):
    p = tmp_path / "c.png"
    p.write_bytes(data)
    d = _lib.CvtpmImage()
    return _lib.lib().cvtpm_png_read(str(p).encode(), d), _lib.lib().cvtpm_last_error(None).decode()


def test_corrupt_and_unsupported(tmp_path):
    s = RNG.integers(0, 256, (6, 5, 3))
    good = pngtool.encode(s, 2, 8)
    assert _corrupt(tmp_path, good)[0] == 0
    bad = bytearray(good)
    bad[40] ^= 1                                        # inside the IHDR or tEXt data: CRC mismatch
    assert _corrupt(tmp_path, bytes(bad)) == (8, "png read: chunk CRC mismatch")
    assert _corrupt(tmp_path, good[:-20])[0] == 8        # truncated
    assert _corrupt(tmp_path, b"GIF89a" + good[6:])[0] == 8
    # a 16-bit palette image is not a PNG type
    hdr = pngtool.SIG + pngtool.chunk(b"IHDR", struct.pack(">IIBBBBB", 4, 4, 16, 3, 0, 0, 0))
    assert _corrupt(tmp_path, hdr + pngtool.chunk(b"IEND", b""))[0] == 7
    # Adler-32 and the data length are checked when the pixels are read
    raw = b"".join(b"\x00" + bytes(15) for _ in range(5))
    z = bytearray(zlib.compress(raw))
    z[-1] ^= 1
    data = pngtool.SIG + pngtool.chunk(b"IHDR", struct.pack(">IIBBBBB", 5, 5, 8, 2, 0, 0, 0))
    data += pngtool.chunk(b"IDAT", bytes(z)) + pngtool.chunk(b"IEND", b"")
    p = tmp_path / "a.png"
    p.write_bytes(data)
    with pytest.raises(_lib.CvtpmError, match="Adler-32"):
        imageio.read_png(p)
    data = pngtool.SIG + pngtool.chunk(b"IHDR", struct.pack(">IIBBBBB", 5, 6, 8, 2, 0, 0, 0))
    data += pngtool.chunk(b"IDAT", zlib.compress(raw)) + pngtool.chunk(b"IEND", b"")
    p.write_bytes(data)
    with pytest.raises(_lib.CvtpmError, match="less image data"):
        imageio.read_png(p)
    with pytest.raises(_lib.CvtpmError):
        imageio.write_png(tmp_path / "x.png", np.zeros((2, 2), np.int16), imageio.GRAY_INT16)


def test_reference_data_images():
    from oracle.ref_emu import build_ref
    files = sorted(glob.glob(os.path.join(build_ref.REF, "data", "*.png")))
    if not files:
        pytest.skip("reference data absent")
    for f in files[:12]:
        s, ct, dp = pngtool.decode(open(f, "rb").read())
        got, fmt = imageio.read_png(f)
        plte = trns = None
        blob = open(f, "rb").read()
        pos = 8
        while pos < len(blob):
            n, t = struct.unpack(">I4s", blob[pos:pos + 8])
            if t == b"PLTE":
                plte = blob[pos + 8:pos + 8 + n]
            if t == b"tRNS":
                trns = blob[pos + 8:pos + 8 + n]
            pos += 12 + n
        want, wfmt = expected(s, ct, dp, plte, trns)
        assert fmt == wfmt, f
        assert np.array_equal(got.reshape(want.shape), want), f


def test_header_larger_than_its_data_is_refused(tmp_path):
    """a 20000 x 20000 header over a few bytes of IDAT: refused before the
    decoder allocates for it (DEFLATE expands at most 1032:1)"""
    raw = zlib.compress(b"\x00" * 1000)
    data = pngtool.SIG + pngtool.chunk(b"IHDR", struct.pack(">IIBBBBB", 20000, 20000, 8, 0, 0, 0, 0))
    data += pngtool.chunk(b"IDAT", raw) + pngtool.chunk(b"IEND", b"")
    p = tmp_path / "big.png"
    p.write_bytes(data)
    with pytest.raises(_lib.CvtpmError, match="less image data"):
        imageio.read_png(p)          # the 400 MB output array is allocated lazily and never written
