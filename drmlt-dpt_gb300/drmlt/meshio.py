"""Mesh front end: Wavefront OBJ and Mitsuba ``serialized`` meshes -> triangles.

Both loaders return ``(positions, normals)`` as float32 arrays of shape
(triangles, 3 corners, 3) in world space, the per-corner data the device scene
stores. They follow the reference's TriMeshData construction:

* ParseObj (src/parseobj.cpp:148-264): 1-based ``v/vt/vn`` corner indices
  (missing fields -> -1, no negative indices), quads split (0,1,2) (0,2,3),
  vertices deduplicated on the (v, vt, vn) triple, ``vn`` normalised when read
  and transformed by the inverse transpose without renormalisation;
* LoadSerialized (src/loadserialized.cpp:236-317): zlib-compressed meshes of
  format versions 3 and 4, the mesh picked by ``shapeIndex`` through the
  offset table at the end of the file, single or double precision, stored
  normals transformed like OBJ ones but not normalised first;
* ComputeNormal (src/parseobj.cpp:57-91, src/loadserialized.cpp:117-148) when
  a mesh has no normals: angle-weighted vertex normals (Nelson Max, 1999),
  with the reference's angle function as written -- ``(pi - 2) * asin(|u+v|/2)``
  for obtuse corners -- and zero normals where the sum vanishes.

Positions are transformed with the homogeneous divide of XformPoint
(src/transform.h:21-30). Arithmetic is float64, rounded to float32 at the end.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

# ETriMeshFlags (src/loadserialized.cpp:13-21)
HAS_NORMALS = 0x0001
HAS_TEXCOORDS = 0x0002
HAS_COLORS = 0x0008
FACE_NORMALS = 0x0010
SINGLE_PRECISION = 0x1000
DOUBLE_PRECISION = 0x2000
SERIALIZED_MAGIC = 0x041C


def _xform_points(to_world: np.ndarray, P: np.ndarray) -> np.ndarray:
    H = np.c_[P, np.ones(len(P))] @ np.asarray(to_world, np.float64).T
    return H[:, :3] / H[:, 3:4]


def _xform_normals(to_world: np.ndarray, N: np.ndarray) -> np.ndarray:
    """XformNormal with the inverse transform: inv^T n, not renormalised."""
    inv = np.linalg.inv(np.asarray(to_world, np.float64))
    return N @ inv[:3, :3]


def compute_vertex_normals(P: np.ndarray, F: np.ndarray) -> np.ndarray:
    """ComputeNormal: per-vertex sum of unit face normals weighted by the corner
    angle; degenerate faces add nothing; zero sums stay zero."""
    P = np.asarray(P, np.float64)
    F = np.asarray(F, np.int64).reshape(-1, 3)
    out = np.zeros_like(P)
    if len(F) == 0:
        return out
    fn = np.cross(P[F[:, 1]] - P[F[:, 0]], P[F[:, 2]] - P[F[:, 0]])
    fl = np.linalg.norm(fn, axis=1)
    ok = fl != 0
    F, fn = F[ok], fn[ok] / fl[ok, None]
    for i in range(3):
        v0 = P[F[:, i]]
        a = P[F[:, (i + 1) % 3]] - v0
        b = P[F[:, (i + 2) % 3]] - v0
        a /= np.linalg.norm(a, axis=1, keepdims=True)
        b /= np.linalg.norm(b, axis=1, keepdims=True)
        obtuse = np.einsum("ij,ij->i", a, b) < 0
        s_plus = np.clip(0.5 * np.linalg.norm(b + a, axis=1), -1.0, 1.0)
        s_minus = np.clip(0.5 * np.linalg.norm(b - a, axis=1), -1.0, 1.0)
        angle = np.where(obtuse, (np.pi - 2.0) * np.arcsin(s_plus), 2.0 * np.arcsin(s_minus))
        np.add.at(out, F[:, i], fn * angle[:, None])
    length = np.linalg.norm(out, axis=1, keepdims=True)
    return np.where(length != 0, out / np.where(length != 0, length, 1.0), 0.0)


def _per_corner(P: np.ndarray, N: np.ndarray, F: np.ndarray):
    return P[F].astype(np.float32), N[F].astype(np.float32)


# ---------------------------------------------------------------- OBJ
def _corner(tok: str):
    """splitFaceStr + ObjVertex: 'v', 'v/vt', 'v//vn', 'v/vt/vn' -> 0-based
    (v, vt, vn), -1 where absent."""
    ids = [int(p) - 1 if p else -1 for p in tok.split("/")]
    ids += [-1] * (3 - len(ids))
    return ids[:3]


def load_obj(path: str, to_world: np.ndarray):
    pos, nor, corners = [], [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok or tok[0].startswith("#"):
                continue
            if tok[0] == "v":
                w = float(tok[4]) if len(tok) > 4 else 1.0
                pos.append([float(tok[1]) / w, float(tok[2]) / w, float(tok[3]) / w])
            elif tok[0] == "vn":
                n = np.array([float(tok[1]), float(tok[2]), float(tok[3])])
                nor.append(n / np.linalg.norm(n))
            elif tok[0] == "f":
                if len(tok) > 5:
                    raise ValueError("The object file contains n-gon (n>4) that we do not support.")
                c = [_corner(t) for t in tok[1:]]
                corners.append((c[0], c[1], c[2]))
                if len(c) == 4:
                    corners.append((c[0], c[2], c[3]))
    C = np.asarray(corners, np.int64).reshape(-1, 3, 3)
    P = _xform_points(to_world, np.asarray(pos, np.float64).reshape(-1, 3))
    vn = C[:, :, 2]
    if len(C) and (vn >= 0).all():
        N = _xform_normals(to_world, np.asarray(nor, np.float64).reshape(-1, 3))
        return P[C[:, :, 0]].astype(np.float32), N[vn].astype(np.float32)
    if (vn >= 0).any():
        raise ValueError("%s: faces mix corners with and without normals" % path)
    # no normals: the reference's vertices are the distinct (v, vt) corners
    keys, F = np.unique(C[:, :, :2].reshape(-1, 2), axis=0, return_inverse=True)
    F = F.reshape(-1, 3)
    Pv = P[keys[:, 0]]
    return _per_corner(Pv, compute_vertex_normals(Pv, F), F)


# ---------------------------------------------------------------- Mitsuba serialized
def _mesh_offset(data: bytes, version: int, idx: int) -> int:
    """SkipToIdx: the mesh's start from the offset table at the end of the file
    (version 4: uint64 per mesh, version 3: uint32), past its 4-byte header."""
    count = struct.unpack_from("<I", data, len(data) - 4)[0]
    if not 0 <= idx < count:
        raise ValueError("shapeIndex %d out of range (the file holds %d meshes)" % (idx, count))
    if version == 4:
        off = struct.unpack_from("<Q", data, len(data) - 8 * (count - idx) - 4)[0]
    else:
        off = struct.unpack_from("<I", data, len(data) - 4 * (count - idx + 1))[0]
    return off + 4


class _Reader:
    def __init__(self, buf: bytes):
        self.buf, self.pos = buf, 0

    def take(self, dtype, count: int) -> np.ndarray:
        dt = np.dtype(dtype)
        end = self.pos + dt.itemsize * count
        if end > len(self.buf):
            raise ValueError("Read less data than expected")
        a = np.frombuffer(self.buf, dt, count, self.pos)
        self.pos = end
        return a


def load_serialized(path: str, shape_index: int, to_world: np.ndarray):
    with open(path, "rb") as f:
        data = f.read()
    magic, version = struct.unpack_from("<HH", data, 0)
    if magic != SERIALIZED_MAGIC or version not in (3, 4):
        raise ValueError("%s: not a serialized mesh file of version 3 or 4" % path)
    start = _mesh_offset(data, version, shape_index) if shape_index > 0 else 4
    z = zlib.decompressobj(15)
    r = _Reader(z.decompress(data[start:]))
    flags = int(r.take("<u4", 1)[0])
    if version == 4:
        end = r.buf.index(b"\0", r.pos)
        r.pos = end + 1
    nv, nt = (int(x) for x in r.take("<u8", 2))
    real = "<f8" if flags & DOUBLE_PRECISION else "<f4"
    P = _xform_points(to_world, r.take(real, 3 * nv).reshape(nv, 3).astype(np.float64))
    N = None
    if flags & HAS_NORMALS:
        N = _xform_normals(to_world, r.take(real, 3 * nv).reshape(nv, 3).astype(np.float64))
    if flags & HAS_TEXCOORDS:
        r.take(real, 2 * nv)
    if flags & HAS_COLORS:
        r.take("<f8", 3 * nv)  # LoadColor reads doubles whatever the file's precision
    F = r.take("<u4", 3 * nt).reshape(nt, 3).astype(np.int64)
    if nt and F.max() >= nv:
        raise ValueError("%s: triangle index out of range" % path)
    if N is None:
        N = compute_vertex_normals(P, F)
    return _per_corner(P, N, F)


def write_serialized(path: str, meshes: list, version: int = 4, double: bool = False) -> None:
    """Writes meshes in the layout load_serialized reads: per mesh a 4-byte
    header (magic, version) and one zlib stream (flags, [name], counts,
    positions, [normals], [uvs], [colors as float64], uint32 indices), then the
    offset table and the mesh count. Each mesh is a dict with ``positions``
    (V x 3), ``indices`` (T x 3) and optional ``normals``, ``uvs``, ``colors``,
    ``name``."""
    if version not in (3, 4):
        raise ValueError("version must be 3 or 4")
    real = "<f8" if double else "<f4"
    out, offsets = bytearray(), []
    for m in meshes:
        P = np.asarray(m["positions"], np.float64).reshape(-1, 3)
        F = np.asarray(m["indices"], np.int64).reshape(-1, 3)
        flags = DOUBLE_PRECISION if double else SINGLE_PRECISION
        parts = []
        for key, bit, width, dt in (("normals", HAS_NORMALS, 3, real), ("uvs", HAS_TEXCOORDS, 2, real),
                                    ("colors", HAS_COLORS, 3, "<f8")):
            if m.get(key) is not None:
                flags |= bit
                parts.append(np.asarray(m[key], np.float64).reshape(len(P), width).astype(dt).tobytes())
        body = struct.pack("<I", flags)
        if version == 4:
            body += m.get("name", "mesh").encode() + b"\0"
        body += struct.pack("<QQ", len(P), len(F)) + P.astype(real).tobytes() + b"".join(parts)
        body += F.astype("<u4").tobytes()
        offsets.append(len(out))
        out += struct.pack("<HH", SERIALIZED_MAGIC, version) + zlib.compress(body)
    for off in offsets:
        out += struct.pack("<Q" if version == 4 else "<I", off)
    out += struct.pack("<I", len(meshes))
    with open(path, "wb") as f:
        f.write(bytes(out))
