"""A small PNG encoder and decoder for the tests, written from the PNG
specification over Python's zlib module: it makes files of every colour
type, bit depth, filter and interlace method for the library's decoder, and
decodes the library's files independently of it."""
from __future__ import annotations

import struct
import zlib

import numpy as np

SIG = b"\x89PNG\r\n\x1a\n"
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def chunk(t: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xffffffff)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """one row of samples (pixels x channels, ints) in PNG byte order"""
    flat = samples.reshape(-1).astype(np.int64)
    if depth == 16:
        return flat.astype(">u2").tobytes()
    if depth == 8:
        return flat.astype(np.uint8).tobytes()
    per = 8 // depth
    out = bytearray((len(flat) + per - 1) // per)
    for i, v in enumerate(flat):
        out[i // per] |= int(v) << (8 - depth - (i % per) * depth)
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter(row: bytes, prior: bytes, ftype: int, bpp: int) -> bytes:
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prior[i]
        c = prior[i - bpp] if i >= bpp else 0
        pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ftype]
        out[i] = (row[i] - pred) & 0xff
    return bytes(out)


def encode(samples: np.ndarray, ctype: int, depth: int, *, interlace: bool = False, plte: bytes | None = None,
           trns: bytes | None = None, level: int = 6, filters=(0, 1, 2, 3, 4), idat_split: int = 0) -> bytes:
    """samples: (H, W, channels) ints.  Rows cycle through `filters`."""
    H, W = samples.shape[:2]
    nch = CHANNELS[ctype]
    bits = depth * nch
    bpp = max(1, bits // 8)
    raw = bytearray()
    k = 0
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prior = bytes((sub.shape[1] * bits + 7) // 8)
        for r in range(sub.shape[0]):
            row = _pack_row(sub[r], depth)
            f = filters[k % len(filters)]
            k += 1
            raw += bytes([f]) + _filter(row, prior, f, bpp)
            prior = row
    z = zlib.compress(bytes(raw), level)
    out = SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, 1 if interlace else 0))
    out += chunk(b"tEXt", b"Comment\x00made by the tests")
    if plte is not None:
        out += chunk(b"PLTE", plte)
    if trns is not None:
        out += chunk(b"tRNS", trns)
    if idat_split:
        for i in range(0, len(z), idat_split):
            out += chunk(b"IDAT", z[i:i + idat_split])
    else:
        out += chunk(b"IDAT", z)
    return out + chunk(b"IEND", b"")


def decode(data: bytes):
    """(samples (H, W, channels) int64, ctype, depth) of a non-interlaced or
    interlaced PNG, no transformations."""
    assert data[:8] == SIG
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n, t = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(t + body) & 0xffffffff
        if t == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif t == b"IDAT":
            idat += body
        pos += 12 + n
    W, H, depth, ctype, _, _, il = hdr
    nch = CHANNELS[ctype]
    bits = depth * nch
    bpp = max(1, bits // 8)
    raw = zlib.decompress(idat)
    out = np.zeros((H, W, nch), np.int64)
    p = 0
    for x0, y0, dx, dy in (ADAM7 if il else [(0, 0, 1, 1)]):
        if W <= x0 or H <= y0:
            continue
        pw, ph = (W - x0 + dx - 1) // dx, (H - y0 + dy - 1) // dy
        ln = (pw * bits + 7) // 8
        prior = bytearray(ln)
        for r in range(ph):
            f = raw[p]
            row = bytearray(raw[p + 1:p + 1 + ln])
            for i in range(ln):
                a = row[i - bpp] if i >= bpp else 0
                b = prior[i]
                c = prior[i - bpp] if i >= bpp else 0
                row[i] = (row[i] + [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]) & 0xff
            if depth == 16:
                vals = np.frombuffer(bytes(row), ">u2").astype(np.int64)
            elif depth == 8:
                vals = np.frombuffer(bytes(row), np.uint8).astype(np.int64)
            else:
                vals = np.array([(row[i * depth // 8] >> (8 - depth - (i * depth) % 8)) & ((1 << depth) - 1)
                                 for i in range(pw * nch)], np.int64)
            out[y0 + r * dy, x0::dx][:pw] = vals[:pw * nch].reshape(pw, nch)
            prior = row
            p += 1 + ln
    return out, ctype, depth
