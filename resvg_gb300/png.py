"""Minimal PNG reader/writer (RGBA8 / RGB8 / gray / palette, 8-bit, non-interlaced).

Used to read resvg's golden images and to write debug renders.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def _unfilter(raw: bytes, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    pos = 0
    for y in range(h):
        ft = raw[pos]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=pos + 1).astype(np.int32)
        pos += 1 + stride
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        else:
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if ft == 1:
                    p = a
                elif ft == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out


def read_png(path: str) -> np.ndarray:
    """Returns an (h, w, 4) uint8 RGBA (straight alpha) array."""
    with open(path, "rb") as fh:
        return decode_png(fh.read())


def decode_png(data: bytes) -> np.ndarray:
    """An (h, w, 4) uint8 RGBA (straight alpha) array from PNG bytes; 16-bit
    samples keep their high byte."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
    pos = 8
    idat = b""
    plte = None
    trns = None
    while pos < len(data):
        ln, tp = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if tp == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif tp == b"IDAT":
            idat += body
        elif tp == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif tp == b"tRNS":
            trns = body
        elif tp == b"IEND":
            break
    if interlace != 0:
        raise ValueError("interlaced PNG not supported")
    raw = zlib.decompress(idat)
    if depth != 8 and not (ctype in (0, 3) and depth in (1, 2, 4)):
        if depth == 16:
            chans = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
            stride = w * chans * 2
            px = _unfilter(raw, h, stride, chans * 2).reshape(h, w, chans, 2)[..., 0]
            return _expand(px, ctype, plte, trns, w, h)
        raise ValueError("unsupported depth %d" % depth)
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    if depth < 8:
        stride = (w * depth + 7) // 8
        px = _unfilter(raw, h, stride, 1)
        bits = np.unpackbits(px, axis=1)
        bits = bits.reshape(h, -1, depth)
        vals = np.zeros(bits.shape[:2], dtype=np.int32)
        for i in range(depth):
            vals = (vals << 1) | bits[:, :, i]
        vals = vals[:, :w].astype(np.uint8)
        if ctype == 0:
            out = _expand((vals.astype(np.int32) * 255 // ((1 << depth) - 1)).astype(np.uint8)[..., None], ctype,
                          plte, None, w, h)
            if trns is not None and len(trns) >= 2:  # tRNS gray key, in the sample's own bit depth
                out[..., 3][vals == struct.unpack(">H", trns[:2])[0]] = 0
            return out
        return _expand(vals[..., None], ctype, plte, trns, w, h)
    stride = w * chans
    px = _unfilter(raw, h, stride, chans).reshape(h, w, chans)
    return _expand(px, ctype, plte, trns, w, h)


def _expand(px, ctype, plte, trns, w, h):
    out = np.zeros((h, w, 4), dtype=np.uint8)
    if ctype == 6:
        out[:] = px
    elif ctype == 2:
        out[..., :3] = px
        out[..., 3] = 255
        if trns is not None and len(trns) >= 6:
            key = struct.unpack(">HHH", trns[:6])
            m = (px[..., 0] == key[0]) & (px[..., 1] == key[1]) & (px[..., 2] == key[2])
            out[..., 3][m] = 0
    elif ctype == 0:
        out[..., 0] = out[..., 1] = out[..., 2] = px[..., 0]
        out[..., 3] = 255
        if trns is not None and len(trns) >= 2:
            out[..., 3][px[..., 0] == struct.unpack(">H", trns[:2])[0]] = 0
    elif ctype == 4:
        out[..., 0] = out[..., 1] = out[..., 2] = px[..., 0]
        out[..., 3] = px[..., 1]
    elif ctype == 3:
        idx = px[..., 0]
        out[..., :3] = plte[idx]
        alpha = np.full(256, 255, dtype=np.uint8)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, dtype=np.uint8)
        out[..., 3] = alpha[idx]
    return out


def encode_png(rgba: np.ndarray) -> bytes:
    """PNG bytes of an (h, w, 4) uint8 straight-alpha RGBA array."""
    h, w, _ = rgba.shape
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tp, body):
        return struct.pack(">I", len(body)) + tp + body + struct.pack(">I", zlib.crc32(tp + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def write_png(path: str, rgba: np.ndarray) -> None:
    """Writes an (h, w, 4) uint8 straight-alpha RGBA array."""
    with open(path, "wb") as fh:
        fh.write(encode_png(rgba))


def demultiply(premul: np.ndarray) -> np.ndarray:
    """Premultiplied -> straight RGBA, as resvg's test harness does it (f64, +0.5, saturating)."""
    p = premul.astype(np.float64)
    a = p[..., 3:4] / 255.0
    with np.errstate(divide="ignore", invalid="ignore"):
        rgb = p[..., :3] / a + 0.5
    rgb = np.nan_to_num(rgb, nan=0.0, posinf=255.0)
    out = premul.copy()
    out[..., :3] = np.clip(np.floor(rgb), 0, 255).astype(np.uint8)
    return out
