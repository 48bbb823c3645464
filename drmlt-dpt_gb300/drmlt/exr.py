"""OpenEXR images: the writer of the C ABI and a reader for the scene front end.

``write_exr`` is WriteImage (src/image.cpp:45-58) through ``drmlt_write_exr``
(half-float RGB, scanline, uncompressed). ``read_exr`` stands in for
Image3::Image3 (src/image.cpp:5-43) on ``.exr`` files: single-part scanline
images with NONE, RLE, ZIPS or ZIP compression and HALF / FLOAT / UINT
channels; one channel is replicated to RGB, three are returned as R, G, B
(alphabetical otherwise), other counts are rejected like the reference's
"Unsupported number of channels". Tiled, multi-part, deep and PIZ / PXR24 /
B44 / DWA files raise ValueError.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

from . import capi

_COMPRESSION = {0: ("none", 1), 1: ("rle", 1), 2: ("zips", 1), 3: ("zip", 16)}
_PIXEL = {0: np.dtype("<u4"), 1: np.dtype("<f2"), 2: np.dtype("<f4")}


def write_exr(path: str, img: np.ndarray) -> None:
    """H x W x 3 float image (top row first) -> OpenEXR file via the C ABI."""
    img = np.ascontiguousarray(img, np.float32)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("expected an H x W x 3 image")
    h, w, _ = img.shape
    capi.check(capi.lib().drmlt_write_exr(str(path).encode(), w, h, capi.ptr(img)))


def _header(buf: bytes):
    magic, version = struct.unpack_from("<ii", buf, 0)
    if magic != 20000630:
        raise ValueError("not an OpenEXR file")
    if version & 0x1a00:  # tiled, deep, multi-part
        raise ValueError("only single-part scanline OpenEXR files are supported (flags %#x)" % (version & ~0xff))
    pos, attrs = 8, {}
    while buf[pos] != 0:
        e = buf.index(b"\0", pos)
        name = buf[pos:e].decode()
        e2 = buf.index(b"\0", e + 1)
        typ = buf[e + 1:e2].decode()
        size = struct.unpack_from("<i", buf, e2 + 1)[0]
        attrs[name] = (typ, buf[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    return attrs, pos + 1


def _channels(data: bytes):
    out, pos = [], 0
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        ptype, _, xs, ys = struct.unpack_from("<iB3xii", data, e + 1)
        if (xs, ys) != (1, 1):
            raise ValueError("subsampled channels are not supported")
        out.append((data[pos:e].decode(), _PIXEL[ptype]))
        pos = e + 17
    return out


def _unrle(src: bytes, size: int) -> bytes:
    out, i = bytearray(), 0
    while i < len(src) and len(out) < size:
        n = struct.unpack_from("b", src, i)[0]
        i += 1
        if n < 0:
            out += src[i:i - n]
            i -= n
        else:
            out += src[i:i + 1] * (n + 1)
            i += 1
    return bytes(out)


def _unpredict(raw: bytes) -> bytes:
    """Undo the ZIP/RLE byte predictor and the even/odd byte split."""
    t = np.frombuffer(raw, np.uint8).astype(np.int64)
    t = (np.cumsum(t - 128) + 128) & 0xFF  # t[i] = t[i-1] + d[i] - 128, t[0] = d[0]
    t = t.astype(np.uint8)
    half = (len(t) + 1) // 2
    out = np.empty_like(t)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def read_exr(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        buf = f.read()
    attrs, pos = _header(buf)
    chans = _channels(attrs["channels"][1])
    comp = attrs["compression"][1][0]
    if comp not in _COMPRESSION:
        raise ValueError("OpenEXR compression %d is not supported (NONE, RLE, ZIPS, ZIP are)" % comp)
    kind, lines = _COMPRESSION[comp]
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    nblocks = (h + lines - 1) // lines
    offsets = struct.unpack_from("<%dQ" % nblocks, buf, pos)
    planes = {name: np.zeros((h, w), np.float32) for name, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        data = buf[off + 8:off + 8 + size]
        ny = min(lines, y1 - y + 1)
        raw_size = ny * w * sum(dt.itemsize for _, dt in chans)
        if kind != "none" and size < raw_size:
            data = _unpredict(zlib.decompress(data) if kind in ("zip", "zips") else _unrle(data, raw_size))
        if len(data) != raw_size:
            raise ValueError("corrupt OpenEXR block at y=%d" % y)
        p = 0
        for r in range(ny):
            for name, dt in chans:
                row = np.frombuffer(data, dt, w, p)
                planes[name][y - y0 + r] = row.astype(np.float32)
                p += dt.itemsize * w
    names = [n for n, _ in chans]
    if len(names) == 1:
        return np.repeat(planes[names[0]][:, :, None], 3, axis=2)
    if len(names) == 3:
        order = ["R", "G", "B"] if sorted(names) == ["B", "G", "R"] else sorted(names)
        return np.stack([planes[n] for n in order], axis=2)
    raise ValueError("Unsupported number of channels (%d)" % len(names))
