"""Acceptance heatmap of a delayed-rejection render (tools/heatmap.py).

A render with ``acceptanceMap=true`` splats red for every first-stage and green
for every second-stage acceptance (delayed.cpp:244-275). The map is the
second stage's share G / (R + G + eps) per pixel (tools/heatmap.py:13-22),
clipped to [lo, hi] and written as an 8-bit false-colour PNG.

    python -m drmlt.heatmap -t image.exr [-eps 1e-2] [-c 0 1] [-o acceptance-map.png]
"""
from __future__ import annotations

import argparse
import struct
import zlib

import numpy as np

# false-colour ramp: (position, RGB) anchors, linear in between
_RAMP = np.array([[0.0, 0.05, 0.03, 0.35], [0.35, 0.55, 0.05, 0.60], [0.7, 0.93, 0.42, 0.25],
                  [1.0, 0.98, 0.95, 0.20]])


def stage_map(img: np.ndarray, eps: float = 1e-2) -> np.ndarray:
    """Second-stage share of the accepted proposals per pixel."""
    img = np.asarray(img, np.float64)
    return img[:, :, 1] / (img[:, :, 0] + img[:, :, 1] + eps)


def false_colour(v: np.ndarray, clip=(0.0, 1.0)) -> np.ndarray:
    t = np.clip((np.asarray(v, np.float64) - clip[0]) / max(clip[1] - clip[0], 1e-30), 0.0, 1.0)
    rgb = np.stack([np.interp(t, _RAMP[:, 0], _RAMP[:, c]) for c in (1, 2, 3)], axis=-1)
    return np.round(rgb * 255.0).astype(np.uint8)


def write_png(path: str, rgb8: np.ndarray) -> None:
    """8-bit RGB PNG (one IDAT, filter 0 on every row)."""
    h, w, _ = rgb8.shape
    raw = b"".join(b"\0" + rgb8[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def main(argv=None):
    ap = argparse.ArgumentParser(description="Compute delayed rejection acceptance map.")
    ap.add_argument("-t", "--test", required=True, help="acceptance-map render (OpenEXR)")
    ap.add_argument("-eps", "--epsilon", type=float, default=1e-2)
    ap.add_argument("-c", "--clip", nargs=2, type=float, default=[0.0, 1.0])
    ap.add_argument("-o", "--output", default="acceptance-map.png")
    a = ap.parse_args(argv)
    if not a.test.lower().endswith(".exr"):
        raise ValueError("Image must be in OpenEXR format.")
    from .exr import read_exr
    write_png(a.output, false_colour(stage_map(read_exr(a.test), a.epsilon), a.clip))
    return a.output


if __name__ == "__main__":
    main()
