"""Scene front end: the reference's scene XML subset + meshes -> drmlt_scene_desc.

Mirrors ParseScene / ParseSceneNode (src/parsescene.cpp:566-613) for
<sensor type="perspective">, <shape type="obj"|"serialized"> (drmlt/meshio.py)
with diffuse / phong /
roughdielectric / twosided BSDFs and area <emitter>, point and envmap (EXR or
PFM image) <emitter>s, and the <dpt> option block
(ParseDptOptions, src/parsescene.cpp:505-564). Camera matrices follow
Camera::Camera (src/camera.cpp:11-28) and the transform helpers of
src/transform.cpp, computed in double and rounded to float.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .meshio import load_obj, load_serialized  # noqa: F401  (load_obj re-exported)


# ---------------------------------------------------------------- options
@dataclass
class DptOptions:
    """The <dpt> option block with the reference's defaults (src/dptoptions.h:7-38)."""

    integrator: str = "drmlt"
    bidirectional: bool = True
    spp: int = 16
    numInitSamples: int = 100000
    minDepth: int = -1
    maxDepth: int = -1
    directSpp: int = 16
    largeStepProb: float = 0.3
    perturbStdDev: float = 0.01
    roughnessThreshold: float = 0.03
    lensPerturbProb: float = 0.3
    lensPerturbStdDev: float = 0.01
    numChains: int = 1024
    seedOffset: int = 0
    reportIntervalSpp: int = 0
    reportIntervalSeconds: int = 0
    useLightCoordinateSampling: bool = True
    discreteStdDev: float = 0.01
    largeStepMultiplexed: bool = True
    uniformMixingProbability: float = 0.2
    type: str = "green"
    anisoPerturbProb: float = 0.5
    anisoperturbstddev: float = 0.0025
    acceptanceMap: bool = False
    unknown: list = field(default_factory=list)


def parse_dpt_options(node, honour_aniso_stddev: bool = False) -> DptOptions:
    """ParseDptOptions. The reference stores the XML `anisoperturbstddev` into
    lensPerturbStdDev (src/parsescene.cpp:553-554), so its second-stage sigma
    always stays 0.0025; honour_aniso_stddev=True applies the XML value instead."""
    o = DptOptions()
    for ch in node:
        name = ch.get("name", "")
        v = ch.get("value", "")
        b = v == "true"
        if name == "integrator": o.integrator = v
        elif name == "spp": o.spp = int(v)
        elif name == "bidirectional": o.bidirectional = b
        elif name == "numinitsamples": o.numInitSamples = int(v)
        elif name == "largestepprob": o.largeStepProb = float(v)
        elif name == "mindepth": o.minDepth = int(v)
        elif name == "maxdepth": o.maxDepth = int(v)
        elif name == "directspp": o.directSpp = int(v)
        elif name == "perturbstddev": o.perturbStdDev = float(v)
        elif name == "lensperturbstddev": o.lensPerturbStdDev = float(v)
        elif name == "roughnessthreshold": o.roughnessThreshold = float(v)
        elif name == "lensperturbprob": o.lensPerturbProb = float(v)
        elif name == "uniformmixingprobability": o.uniformMixingProbability = float(v)
        elif name == "numchains": o.numChains = int(v)
        elif name == "seedoffset": o.seedOffset = int(v)
        elif name == "reportintervalspp": o.reportIntervalSpp = int(v)
        elif name == "reportintervalseconds": o.reportIntervalSeconds = int(v)
        elif name == "uselightcoordinatesampling": o.useLightCoordinateSampling = b
        elif name == "largestepmultiplexed": o.largeStepMultiplexed = b
        elif name == "type": o.type = v
        elif name == "anisoperturbstddev":
            o.lensPerturbStdDev = float(v)
            if honour_aniso_stddev:
                o.anisoperturbstddev = float(v)
        elif name == "anisoperturbprob": o.anisoPerturbProb = float(v)
        elif name == "acceptanceMap": o.acceptanceMap = b
        else:
            o.unknown.append(name)
    return o


# ---------------------------------------------------------------- transforms
def _scale(x, y, z):
    return np.diag([x, y, z, 1.0])


def _translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = [x, y, z]
    return m


def _rotate(angle, axis):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    s, c = math.sin(math.radians(angle)), math.cos(math.radians(angle))
    m = np.eye(4)
    m[0, :3] = [a[0] * a[0] + (1 - a[0] * a[0]) * c, a[0] * a[1] * (1 - c) - a[2] * s, a[0] * a[2] * (1 - c) + a[1] * s]
    m[1, :3] = [a[0] * a[1] * (1 - c) + a[2] * s, a[1] * a[1] + (1 - a[1] * a[1]) * c, a[1] * a[2] * (1 - c) - a[0] * s]
    m[2, :3] = [a[0] * a[2] * (1 - c) - a[1] * s, a[1] * a[2] * (1 - c) + a[0] * s, a[2] * a[2] + (1 - a[2] * a[2]) * c]
    return m


def _lookat(pos, look, up):
    pos, look, up = (np.asarray(v, np.float64) for v in (pos, look, up))
    d = look - pos
    d /= np.linalg.norm(d)
    upn = up / np.linalg.norm(up)
    left = np.cross(upn, d)
    if np.linalg.norm(left) == 0:
        raise ValueError("lookat: up vector parallel to the view direction")
    left /= np.linalg.norm(left)
    new_up = np.cross(d, left)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = left, new_up, d, pos
    return m


def _perspective(fov, near, far):
    recip = 1.0 / (far - near)
    cot = 1.0 / math.tan(math.radians(fov / 2.0))
    m = np.zeros((4, 4))
    m[0, 0] = m[1, 1] = cot
    m[2, 2] = far * recip
    m[2, 3] = -near * far * recip
    m[3, 2] = 1.0
    return m


def _vec3(s: str):
    parts = [p for p in re.split(r"[, ]+", s.strip()) if p]
    if len(parts) == 1:
        return [float(parts[0])] * 3
    if len(parts) == 3:
        return [float(p) for p in parts]
    raise ValueError("ParseVector3 failed: %r" % s)


def parse_transform(node) -> np.ndarray:
    """ParseTransform (src/parsescene.cpp:83-134): children applied left-multiplied in order."""
    t = np.eye(4)
    for ch in node:
        name = ch.tag.lower()
        g = lambda k, d: float(ch.get(k)) if ch.get(k) is not None else d
        if name == "scale":
            t = _scale(g("x", 1.0), g("y", 1.0), g("z", 1.0)) @ t
        elif name == "translate":
            t = _translate(g("x", 0.0), g("y", 0.0), g("z", 0.0)) @ t
        elif name == "rotate":
            t = _rotate(g("angle", 0.0), (g("x", 0.0), g("y", 0.0), g("z", 0.0))) @ t
        elif name == "lookat":
            t = _lookat(_vec3(ch.get("origin")), _vec3(ch.get("target")), _vec3(ch.get("up"))) @ t
        elif name == "matrix":
            t = np.array([float(v) for v in re.split(r"[, ]+", ch.get("value").strip()) if v]).reshape(4, 4) @ t
    return t


def read_pfm(path: str) -> np.ndarray:
    """A PFM image as H x W x 3 float32, top row first (Image3's layout: the
    file stores rows bottom to top; a one-channel file is replicated to RGB as
    Image3::Image3 does, src/image.cpp:5-43)."""
    with open(path, "rb") as f:
        magic = f.readline().strip()
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        ch = 3 if magic == b"PF" else 1
        data = np.frombuffer(f.read(4 * w * h * ch), "<f4" if scale < 0 else ">f4").reshape(h, w, ch)
    img = np.ascontiguousarray(data[::-1], np.float32)
    return np.repeat(img, 3, axis=2) if ch == 1 else img


def read_image(path: str) -> np.ndarray:
    """Image3::Image3 (src/image.cpp:5-43) for the formats this front end
    reads: OpenEXR (drmlt/exr.py) and PFM; H x W x 3 float32, top row first."""
    low = path.lower()
    if low.endswith(".exr"):
        from .exr import read_exr
        return read_exr(path)
    if low.endswith(".pfm"):
        return read_pfm(path)
    raise ValueError("%s: only .exr and .pfm images are supported" % path)


# ---------------------------------------------------------------- scene
@dataclass
class SceneData:
    positions: np.ndarray          # T x 3 x 3
    normals: np.ndarray            # T x 3 x 3
    shape_first_tri: np.ndarray
    shape_num_tris: np.ndarray
    shape_bsdf: np.ndarray
    shape_light: np.ndarray
    bsdfs: list
    lights: list
    camera: dict
    options: DptOptions
    path: str
    env_images: list = field(default_factory=list)  # keeps the envmap pixels behind drmlt_light.env_rgb

    @property
    def width(self):
        return self.camera["width"]

    @property
    def height(self):
        return self.camera["height"]


def _parse_bsdf(node, two_sided=False):
    t = node.get("type")
    b = capi.Bsdf()
    b.two_sided = 1 if two_sided else 0
    if t == "diffuse":
        b.type = capi.BSDF_LAMBERTIAN
        kd = [0.5, 0.5, 0.5]
        for ch in node:
            if ch.get("name") == "reflectance":
                kd = _vec3(ch.get("value"))
        b.kd[:] = kd
        return b
    if t == "phong":
        b.type = capi.BSDF_PHONG
        kd, ks, e = [0.5] * 3, [0.2] * 3, 30.0
        for ch in node:
            n = ch.get("name")
            if n == "diffuseReflectance": kd = _vec3(ch.get("value"))
            elif n == "specularReflectance": ks = _vec3(ch.get("value"))
            elif n == "exponent": e = float(ch.get("value"))
        b.kd[:] = kd
        b.ks[:] = ks
        b.exponent = e
        return b
    if t == "roughdielectric":
        b.type = capi.BSDF_ROUGHDIELECTRIC
        b.int_ior, b.ext_ior, b.alpha = 1.5046, 1.000277, 0.1
        b.ks[:] = [1.0] * 3
        b.kt[:] = [1.0] * 3
        for ch in node:
            n = ch.get("name")
            if n == "intIOR": b.int_ior = float(ch.get("value"))
            elif n == "extIOR": b.ext_ior = float(ch.get("value"))
            elif n == "alpha": b.alpha = float(ch.get("value"))
        return b
    if t == "twosided":
        for ch in node:
            if ch.tag == "bsdf":
                return _parse_bsdf(ch, True)
    raise ValueError("Unknown BSDF %r" % t)


def load_scene(xml_path: str, honour_aniso_stddev: bool = False) -> SceneData:
    root = ET.parse(xml_path).getroot()
    base = os.path.dirname(os.path.abspath(xml_path))
    options = DptOptions()
    cam = None
    bsdf_map = {}
    bsdfs, lights = [], []
    pos_l, nor_l = [], []
    first, count, sb, sl = [], [], [], []
    env_images = []
    ntri = 0
    for ch in root:
        if ch.tag == "dpt":
            options = parse_dpt_options(ch, honour_aniso_stddev)
        elif ch.tag == "bsdf":
            bsdf_map[ch.get("id")] = _parse_bsdf(ch)
        elif ch.tag == "sensor":
            fov, near, far, W, H = 45.0, 1e-2, 1000.0, 512, 512
            output = os.path.join(base, "image.exr")  # src/parsescene.cpp:574
            to_world = np.eye(4)
            for s in ch:
                n = s.get("name")
                if n == "fov": fov = float(s.get("value"))
                elif n == "nearClip": near = float(s.get("value"))
                elif n == "farClip": far = float(s.get("value"))
                elif n == "toWorld" and s.tag == "transform": to_world = parse_transform(s)
                elif s.tag == "film":
                    for fch in s:
                        if fch.get("name") == "width": W = int(fch.get("value"))
                        elif fch.get("name") == "height": H = int(fch.get("value"))
                        elif fch.get("name") == "filename": output = os.path.join(base, fch.get("value"))
            cam = dict(fov=fov, near=near, far=far, width=W, height=H, to_world=to_world, output=output)
        elif ch.tag == "shape":  # ParseShape (src/parsescene.cpp:190-300)
            kind = ch.get("type")
            if kind not in ("obj", "serialized"):
                raise ValueError("Invalid shape %r (obj and serialized are supported)" % kind)
            bsdf = None
            fname, to_world, shape_index = None, np.eye(4), 0
            emitter = None
            for s in ch:
                if s.tag == "bsdf" and bsdf is None:
                    bsdf = _parse_bsdf(s)
                elif s.tag == "ref" and bsdf is None:
                    bsdf = bsdf_map[s.get("id")]
                elif s.get("name") == "filename":
                    fname = s.get("value")
                elif s.get("name") == "shapeIndex":
                    shape_index = int(s.get("value"))
                elif s.get("name") == "toWorld" and s.tag == "transform":
                    to_world = parse_transform(s)
                elif s.get("name") == "toWorld" and s.tag == "animation":
                    raise ValueError("animated toWorld (motion blur) is not supported")
                elif s.tag == "emitter":
                    emitter = s
            if kind == "obj":
                p, n = load_obj(os.path.join(base, fname), to_world)
            else:
                p, n = load_serialized(os.path.join(base, fname), shape_index, to_world)
            shape_id = len(first)
            first.append(ntri)
            count.append(len(p))
            ntri += len(p)
            pos_l.append(p)
            nor_l.append(n)
            if bsdf is None:
                raise ValueError("shape without bsdf")
            sb.append(len(bsdfs))
            bsdfs.append(bsdf)
            if emitter is not None:
                L = capi.Light()
                L.type = capi.LIGHT_AREA
                L.shape = shape_id
                rad = [1.0, 1.0, 1.0]
                for e in emitter:
                    if e.get("name") == "radiance":
                        rad = _vec3(e.get("value"))
                L.emission[:] = rad
                L.sampling_weight = 1.0
                sl.append(len(lights))
                lights.append(L)
            else:
                sl.append(-1)
        elif ch.tag == "emitter":
            if ch.get("type") == "point":
                L = capi.Light()
                L.type = capi.LIGHT_POINT
                L.shape = -1
                L.sampling_weight = 1.0
                L.emission[:] = [1.0, 1.0, 1.0]
                for e in ch:
                    if e.get("name") == "position":
                        L.pos[:] = [float(e.get(k, 0.0)) for k in ("x", "y", "z")]
                    elif e.get("name") == "intensity":
                        L.emission[:] = _vec3(e.get("value"))
                lights.append(L)
            elif ch.get("type") == "envmap":  # src/parsescene.cpp:477-498
                L = capi.Light()
                L.type = capi.LIGHT_ENV
                L.shape = -1
                L.sampling_weight = 1.0
                to_world = np.eye(4)
                fname = None
                for e in ch:
                    if e.get("name") == "filename":
                        fname = e.get("value")
                    elif e.get("name") == "samplingWeight":
                        L.sampling_weight = float(e.get("value"))
                    elif e.get("name") == "toWorld" and e.tag == "transform":
                        to_world = parse_transform(e)
                if fname is None:
                    raise ValueError("envmap without filename")
                img = read_image(os.path.join(base, fname))
                env_images.append(img)
                L.env_rgb = img.ctypes.data_as(C.POINTER(C.c_float))
                L.env_height, L.env_width = img.shape[0], img.shape[1]
                L.to_world[:] = to_world.astype(np.float32).ravel().tolist()
                lights.append(L)
            else:
                raise ValueError("unsupported emitter %r" % ch.get("type"))
    if cam is None:
        raise ValueError("scene has no sensor")
    return SceneData(np.concatenate(pos_l), np.concatenate(nor_l), np.asarray(first, np.int32),
                     np.asarray(count, np.int32), np.asarray(sb, np.int32), np.asarray(sl, np.int32),
                     bsdfs, lights, cam, options, xml_path, env_images)


def camera_matrices(cam: dict) -> dict:
    """Camera::Camera (src/camera.cpp:11-28): sample<->camera and camera<->world matrices."""
    W, H = cam["width"], cam["height"]
    aspect = W / H
    cam_to_sample = _scale(-0.5, -0.5 * aspect, 1.0) @ _translate(-1.0, -1.0 / aspect, 0.0) @ _perspective(
        cam["fov"], cam["near"], cam["far"])
    sample_to_cam = np.linalg.inv(cam_to_sample)
    c2w = cam["to_world"]
    w2c = np.linalg.inv(c2w)
    dist = W / (2.0 * math.tan((cam["fov"] / 2.0) * (math.pi / 180.0)))
    return dict(sample_to_cam=sample_to_cam, cam_to_sample=cam_to_sample, cam_to_world=c2w, world_to_cam=w2c,
                dist=dist)


class SceneDescHolder:
    """Owns the numpy buffers behind a drmlt_scene_desc for the lifetime of a call."""

    def __init__(self, sd: SceneData):
        self.pos = np.ascontiguousarray(sd.positions, np.float32)
        self.nor = np.ascontiguousarray(sd.normals, np.float32)
        self.first = np.ascontiguousarray(sd.shape_first_tri, np.int32)
        self.count = np.ascontiguousarray(sd.shape_num_tris, np.int32)
        self.sb = np.ascontiguousarray(sd.shape_bsdf, np.int32)
        self.sl = np.ascontiguousarray(sd.shape_light, np.int32)
        self.bsdfs = (capi.Bsdf * len(sd.bsdfs))(*sd.bsdfs)
        self.lights = (capi.Light * len(sd.lights))(*sd.lights)
        d = capi.SceneDesc()
        d.num_tris = len(self.pos)
        d.positions = self.pos.ctypes.data_as(C.POINTER(C.c_float))
        d.normals = self.nor.ctypes.data_as(C.POINTER(C.c_float))
        d.num_shapes = len(self.first)
        d.shape_first_tri = self.first.ctypes.data_as(C.POINTER(C.c_int32))
        d.shape_num_tris = self.count.ctypes.data_as(C.POINTER(C.c_int32))
        d.shape_bsdf = self.sb.ctypes.data_as(C.POINTER(C.c_int32))
        d.shape_light = self.sl.ctypes.data_as(C.POINTER(C.c_int32))
        d.num_bsdfs = len(sd.bsdfs)
        d.bsdfs = self.bsdfs
        d.num_lights = len(sd.lights)
        d.lights = self.lights
        m = camera_matrices(sd.camera)
        d.sample_to_cam[:] = m["sample_to_cam"].astype(np.float32).ravel().tolist()
        d.cam_to_sample[:] = m["cam_to_sample"].astype(np.float32).ravel().tolist()
        d.cam_to_world[:] = m["cam_to_world"].astype(np.float32).ravel().tolist()
        d.world_to_cam[:] = m["world_to_cam"].astype(np.float32).ravel().tolist()
        d.cam_dist = float(np.float32(m["dist"]))
        d.near_clip = sd.camera["near"]
        d.far_clip = sd.camera["far"]
        d.width = sd.camera["width"]
        d.height = sd.camera["height"]
        # BSphere(BBox) (src/bounds.h:30-33) in single precision
        lo = self.pos.reshape(-1, 3).min(0).astype(np.float32)
        hi = self.pos.reshape(-1, 3).max(0).astype(np.float32)
        c = np.float32(0.5) * (lo + hi)
        e = hi - lo
        d.bsphere_center[:] = c.tolist()
        d.bsphere_radius = float(np.float32(0.5) * np.sqrt(np.float32(e[0] * e[0] + e[1] * e[1] + e[2] * e[2])))
        self.sd = sd
        self.desc = d
