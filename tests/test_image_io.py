"""Image output and input (CPU): the C ABI's OpenEXR writer (WriteImage,
src/image.cpp:45-58), the front end's OpenEXR reader on every compression it
accepts, EXR environment maps, and the acceptance heatmap (tools/heatmap.py).
drmlt_write_exr is host code: it runs without a GPU."""
from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest

import helpers  # noqa: F401  (puts the package on sys.path)
from drmlt import exr, heatmap, scene as dscene


# ---------------------------------------------------------------- a test-side OpenEXR encoder
def _predict(raw: bytes) -> bytes:
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int64)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128) & 0xFF
    return d.astype(np.uint8).tobytes()


def _rle(src: bytes) -> bytes:
    out, i, n = bytearray(), 0, len(src)
    while i < n:
        j = i
        while j < n and j - i < 127 and src[j] == src[i]:
            j += 1
        if j - i >= 3:
            out += struct.pack("b", j - i - 1) + src[i:i + 1]
            i = j
            continue
        j = i
        while j < n and j - i < 127 and not (j + 2 < n and src[j] == src[j + 1] == src[j + 2]):
            j += 1
        out += struct.pack("b", -(j - i)) + src[i:j]
        i = j
    return bytes(out)


def _encode(path, planes: dict, dtypes: dict, compression: int, y0: int = 0, flags: int = 0):
    names = sorted(planes)
    h, w = planes[names[0]].shape
    ptype = {np.dtype("<u4"): 0, np.dtype("<f2"): 1, np.dtype("<f4"): 2}
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", ptype[np.dtype(dtypes[n])], 0, 1, 1) for n in names)
    chl += b"\0"

    def attr(name, typ, data):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data

    win = struct.pack("<iiii", 0, y0, w - 1, y0 + h - 1)
    hdr = struct.pack("<ii", 20000630, 2 | flags) + attr("channels", "chlist", chl)
    hdr += attr("compression", "compression", bytes([compression])) + attr("dataWindow", "box2i", win)
    hdr += attr("displayWindow", "box2i", win) + attr("lineOrder", "lineOrder", b"\0")
    hdr += attr("pixelAspectRatio", "float", struct.pack("<f", 1)) + attr("screenWindowCenter", "v2f", b"\0" * 8)
    hdr += attr("screenWindowWidth", "float", struct.pack("<f", 1)) + b"\0"
    lines = 16 if compression == 3 else 1
    blocks = []
    for b0 in range(0, h, lines):
        raw = b"".join(np.asarray(planes[n][y], dtypes[n]).tobytes() for y in range(b0, min(h, b0 + lines))
                       for n in names)
        if compression in (2, 3):
            data = zlib.compress(_predict(raw))
        elif compression == 1:
            data = _rle(_predict(raw))
        else:
            data = raw
        if len(data) >= len(raw):
            data = raw
        blocks.append(struct.pack("<ii", y0 + b0, len(data)) + data)
    off = len(hdr) + 8 * len(blocks)
    table = b""
    for b in blocks:
        table += struct.pack("<Q", off)
        off += len(b)
    with open(path, "wb") as f:
        f.write(hdr + table + b"".join(blocks))


# ---------------------------------------------------------------- writer (C ABI)
def test_write_exr_rounds_to_half_and_reads_back(built_lib, tmp_path):
    rng = np.random.default_rng(5)
    h, w = 7, 11
    img = (rng.standard_normal((h, w, 3)) * np.exp(rng.uniform(-20, 12, (h, w, 3)))).astype(np.float32)
    special = np.array([0.0, -0.0, 65504.0, 65520.0, 1e9, -1e9, np.inf, -np.inf, np.nan, 6e-8, 2.98e-8,
                        2.9802322e-08, 5.9604645e-08 * 1.5, 1e-30, 0.000061035156, 1.0 + 2 ** -11, 1.0 + 3 * 2 ** -11,
                        -2.5, 3.0e-5, 65519.0, 1.0 / 3.0], np.float32)
    img.reshape(-1)[:len(special)] = special
    fn = str(tmp_path / "img.exr")
    exr.write_exr(fn, img)
    buf = open(fn, "rb").read()
    assert struct.unpack_from("<ii", buf, 0) == (20000630, 2)
    for name in (b"channels\0chlist\0", b"compression\0compression\0", b"dataWindow\0box2i\0",
                 b"displayWindow\0box2i\0", b"lineOrder\0lineOrder\0", b"pixelAspectRatio\0float\0",
                 b"screenWindowCenter\0v2f\0", b"screenWindowWidth\0float\0"):
        assert name in buf
    back = exr.read_exr(fn)
    with np.errstate(over="ignore"):
        want = img.astype(np.float16).astype(np.float32)  # IEEE round to nearest even
    np.testing.assert_array_equal(back, want)
    # header + offset table + per line (y, size, 3 x w halves)
    hdr_end = buf.index(b"screenWindowWidth\0float\0") + len(b"screenWindowWidth\0float\0") + 4 + 4 + 1
    assert len(buf) == hdr_end + 8 * h + h * (8 + 6 * w)


def test_write_exr_errors(built_lib, tmp_path):
    with pytest.raises(ValueError):
        exr.write_exr(str(tmp_path / "x.exr"), np.zeros((4, 4)))
    with pytest.raises(Exception, match="cannot open"):
        exr.write_exr(str(tmp_path / "missing_dir" / "x.exr"), np.zeros((2, 2, 3)))


# ---------------------------------------------------------------- reader
@pytest.mark.parametrize("compression", [0, 1, 2, 3])
@pytest.mark.parametrize("dtype", ["<f2", "<f4"])
def test_read_exr_compressions(tmp_path, compression, dtype):
    rng = np.random.default_rng(compression * 7 + len(dtype))
    h, w = 37, 23
    smooth = np.cumsum(rng.uniform(0, 0.01, (h, w)), axis=1)  # compressible
    planes = {"R": smooth, "G": rng.uniform(0, 4, (h, w)), "B": np.full((h, w), 0.25)}
    fn = str(tmp_path / "c.exr")
    _encode(fn, planes, {k: dtype for k in planes}, compression, y0=3)
    back = exr.read_exr(fn)
    want = np.stack([planes[c].astype(dtype).astype(np.float32) for c in "RGB"], axis=2)
    np.testing.assert_array_equal(back, want)


def test_read_exr_channels(tmp_path):
    y = np.linspace(0, 1, 6 * 5).reshape(6, 5)
    fn = str(tmp_path / "y.exr")
    _encode(fn, {"Y": y}, {"Y": "<f4"}, 3)
    back = exr.read_exr(fn)
    assert back.shape == (6, 5, 3)
    np.testing.assert_array_equal(back[:, :, 2], y.astype(np.float32))
    _encode(fn, {c: y for c in "RGBA"}, {c: "<f2" for c in "RGBA"}, 0)
    with pytest.raises(ValueError, match="Unsupported number of channels"):
        exr.read_exr(fn)
    _encode(fn, {c: y for c in "RGB"}, {c: "<f2" for c in "RGB"}, 0, flags=0x200)
    with pytest.raises(ValueError, match="scanline"):
        exr.read_exr(fn)
    _encode(fn, {c: y for c in "RGB"}, {c: "<u4" for c in "RGB"}, 4)
    with pytest.raises(ValueError, match="compression 4"):
        exr.read_exr(fn)


def test_envmap_exr_matches_pfm(tmp_path):
    """An EXR (float) environment map loads to the same pixels as its PFM."""
    from drmlt import scenegen
    xml = scenegen.config_env(str(tmp_path / "env"))
    sd_pfm = dscene.load_scene(xml)
    img = sd_pfm.env_images[0]
    _encode(str(tmp_path / "env" / "env.exr"), {c: img[:, :, i] for i, c in enumerate("RGB")},
            {c: "<f4" for c in "RGB"}, 3)
    text = open(xml).read()
    assert ".pfm" in text
    xml2 = str(tmp_path / "env" / "scene_exr.xml")
    with open(xml2, "w") as f:
        f.write(text.replace("env.pfm", "env.exr"))
    sd_exr = dscene.load_scene(xml2)
    np.testing.assert_array_equal(sd_exr.env_images[0], img)


# ---------------------------------------------------------------- heatmap
def test_heatmap(tmp_path):
    img = np.zeros((4, 6, 3))
    img[:, :, 0] = np.arange(6)
    img[:, :, 1] = 6 - np.arange(6)
    m = heatmap.stage_map(img, 1e-2)
    np.testing.assert_allclose(m, (6 - np.arange(6)) / (6 + 1e-2) * np.ones((4, 1)))
    rgb = heatmap.false_colour(m)
    assert rgb.shape == (4, 6, 3) and rgb.dtype == np.uint8
    assert (np.diff(rgb[0].astype(int).sum(axis=1)) <= 0).all()  # brighter for larger shares
    fn = str(tmp_path / "m.png")
    heatmap.write_png(fn, rgb)
    data = open(fn, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (6, 4)
    idat = data.index(b"IDAT")
    n = struct.unpack(">I", data[idat - 4:idat])[0]
    raw = zlib.decompress(data[idat + 4:idat + 4 + n])
    rows = np.frombuffer(raw, np.uint8).reshape(4, 1 + 18)
    assert (rows[:, 0] == 0).all()
    np.testing.assert_array_equal(rows[:, 1:].reshape(4, 6, 3), rgb)
