"""Seeded synthetic scenes written in the reference's scene-XML + OBJ format.

The same files are read by the reference renderer (src/parsescene.cpp:566-599,
src/parseobj.cpp) and by this library's loader (drmlt/scene.py), so both sides
render identical geometry, materials and options.

Workloads:
  * ``cornell``: Cornell box of 34 triangles (5 wall quads + 2 axis-aligned boxes,
    one OBJ shape each) plus a 0.25 x 0.25 area-light quad (2 triangles) of
    radiance 15. Walls/boxes are Lambertian with reflectance U[0.2, 0.8]^3, or
    Phong (exponent log-U[10, 1000], ks U[0.1, 0.5]) when ``phong=True``.
    Pinhole camera, fov 40 degrees.
  * ``config3``: the Lambertian box plus a rough-dielectric (Beckmann) sphere of
    528 smooth-shaded triangles, alpha U[0.05, 0.5] from the seed, IOR 1.5.
  * ``config_lights``: config 3 with a point light (intensity 3) beside the area light.
  * ``config_env``: config 3 without its ceiling under an 8 x 4 environment map
    (PFM, rotated 30 degrees about y) next to the area light.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

# Quads are (corner, edge_u, edge_v) with the normal = edge_u x edge_v pointing
# into the room; each becomes two triangles (0,1,2) (0,2,3).
_WALLS = {
    "floor": ((-1.0, -1.0, 1.0), (2.0, 0.0, 0.0), (0.0, 0.0, -2.0)),
    "ceiling": ((-1.0, 1.0, -1.0), (2.0, 0.0, 0.0), (0.0, 0.0, 2.0)),
    "back": ((-1.0, -1.0, -1.0), (2.0, 0.0, 0.0), (0.0, 2.0, 0.0)),
    "left": ((-1.0, -1.0, 1.0), (0.0, 0.0, -2.0), (0.0, 2.0, 0.0)),
    "right": ((1.0, -1.0, -1.0), (0.0, 0.0, 2.0), (0.0, 2.0, 0.0)),
}

# Axis-aligned boxes: (min corner, max corner).
_BOXES = {
    "shortbox": ((0.05, -1.0, 0.0), (0.65, -0.4, 0.6)),
    "tallbox": ((-0.65, -1.0, -0.65), (-0.05, 0.2, -0.05)),
}


def _quad_tris(corner, eu, ev):
    c = np.asarray(corner, np.float64)
    eu = np.asarray(eu, np.float64)
    ev = np.asarray(ev, np.float64)
    v = np.stack([c, c + eu, c + eu + ev, c + ev])
    n = np.cross(eu, ev)
    n /= np.linalg.norm(n)
    return v, n


def _box_quads(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    dx, dy, dz = x1 - x0, y1 - y0, z1 - z0
    # outward normals
    return [
        ((x0, y1, z1), (dx, 0, 0), (0, 0, -dz)),   # top (+y)
        ((x0, y0, z0), (dx, 0, 0), (0, 0, dz)),    # bottom (-y)
        ((x0, y0, z1), (dx, 0, 0), (0, dy, 0)),    # front (+z)
        ((x1, y0, z0), (-dx, 0, 0), (0, dy, 0)),   # back (-z)
        ((x1, y0, z1), (0, 0, -dz), (0, dy, 0)),   # right (+x)
        ((x0, y0, z0), (0, 0, dz), (0, dy, 0)),    # left (-x)
    ]


def _write_obj(path, quads):
    lines = []
    vi = 1
    for corner, eu, ev in quads:
        v, n = _quad_tris(corner, eu, ev)
        for p in v:
            lines.append("v %.9g %.9g %.9g" % tuple(p))
        lines.append("vn %.9g %.9g %.9g" % tuple(n))
        ni = len([l for l in lines if l.startswith("vn ")])
        lines.append("f %d//%d %d//%d %d//%d" % (vi, ni, vi + 1, ni, vi + 2, ni))
        lines.append("f %d//%d %d//%d %d//%d" % (vi, ni, vi + 2, ni, vi + 3, ni))
        vi += 4
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _write_sphere_obj(path, center, radius, n_theta=12, n_phi=24):
    """UV sphere with per-vertex normals (outward), triangles wound counter-clockwise seen from outside."""
    c = np.asarray(center, np.float64)
    verts, norms, faces = [], [], []
    for i in range(n_theta + 1):
        th = np.pi * i / n_theta
        for j in range(n_phi):
            ph = 2.0 * np.pi * j / n_phi
            d = np.array([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)])
            verts.append(c + radius * d)
            norms.append(d)
    idx = lambda i, j: i * n_phi + (j % n_phi) + 1
    for i in range(n_theta):
        for j in range(n_phi):
            a, b, cc, d = idx(i, j), idx(i, j + 1), idx(i + 1, j + 1), idx(i + 1, j)
            if i > 0:
                faces.append((a, b, cc))
            if i < n_theta - 1:
                faces.append((a, cc, d))
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in verts]
    lines += ["vn %.9g %.9g %.9g" % tuple(n) for n in norms]
    lines += ["f %d//%d %d//%d %d//%d" % (f[0], f[0], f[1], f[1], f[2], f[2]) for f in faces]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@dataclass
class SceneOptions:
    """The reference's ``<dpt>`` option block (src/dptoptions.h:7-38)."""

    integrator: str = "drmlt"
    type: str = "green"
    spp: int = 64
    numinitsamples: int = 100000
    numchains: int = 4096
    maxdepth: int = 5
    mindepth: int = -1
    directspp: int = 16
    perturbstddev: float = 1.0 / 64.0
    largestepprob: float = 0.3
    anisoperturbprob: float = 0.5
    anisoperturbstddev: float = 0.0025
    acceptanceMap: bool = False
    seedoffset: int = 0
    extra: dict = field(default_factory=dict)

    def xml(self) -> str:
        rows = [
            ("string", "integrator", self.integrator),
            ("string", "type", self.type),
            ("integer", "spp", self.spp),
            ("integer", "numinitsamples", self.numinitsamples),
            ("integer", "numchains", self.numchains),
            ("integer", "maxdepth", self.maxdepth),
            ("integer", "mindepth", self.mindepth),
            ("integer", "directspp", self.directspp),
            ("float", "perturbstddev", "%.9g" % self.perturbstddev),
            ("float", "largestepprob", "%.9g" % self.largestepprob),
            ("float", "anisoperturbprob", "%.9g" % self.anisoperturbprob),
            ("float", "anisoperturbstddev", "%.9g" % self.anisoperturbstddev),
            ("boolean", "acceptanceMap", "true" if self.acceptanceMap else "false"),
            ("integer", "seedoffset", self.seedoffset),
        ]
        for k, v in self.extra.items():
            rows.append(("string", k, v))
        body = "\n".join('    <%s name="%s" value="%s"/>' % r for r in rows)
        return "  <dpt>\n%s\n  </dpt>\n" % body


def write_pfm(path: str, img: np.ndarray) -> None:
    """An H x W x 3 image (top row first) as a little-endian PFM (rows stored bottom to top)."""
    img = np.asarray(img, np.float32)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1\n" % (w, h))
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())


def env_image(width: int = 8, height: int = 4) -> np.ndarray:
    """A sky-like environment map: colours per row band brightening along x.
    Column 0 and the bottom row are black, so the importance sampler never
    picks the last column or row and the reference's unwrapped image lookups
    (src/envlight.cpp:159-160) stay inside the image."""
    bands = np.array([[0.6, 0.8, 1.2], [0.9, 0.9, 0.8], [0.45, 0.4, 0.3], [0.3, 0.3, 0.3]])
    img = np.zeros((height, width, 3), np.float32)
    for y in range(height - 1):
        for x in range(1, width):
            img[y, x] = bands[min(y, len(bands) - 1)] * (0.6 + 0.6 * x / (width - 1))
    return img


def write_cornell(outdir: str, *, seed: int = 1, width: int = 256, height: int = 256,
                  phong: bool = False, options: SceneOptions | None = None,
                  filename: str = "scene.xml", sphere: dict | None = None,
                  point_light: dict | None = None, env: dict | None = None,
                  ceiling: bool = True) -> str:
    """Writes the Cornell-box workload; returns the XML path."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed)
    options = options or SceneOptions()
    shapes = []
    names = [n for n in _WALLS if ceiling or n != "ceiling"] + list(_BOXES)
    for name in names:
        quads = [_WALLS[name]] if name in _WALLS else _box_quads(*_BOXES[name])
        _write_obj(os.path.join(outdir, name + ".obj"), quads)
        kd = rng.uniform(0.2, 0.8, 3)
        if phong:
            expo = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
            ks = float(rng.uniform(0.1, 0.5))
            bsdf = ('<bsdf type="phong"><rgb name="diffuseReflectance" value="%.9g %.9g %.9g"/>'
                    '<rgb name="specularReflectance" value="%.9g %.9g %.9g"/>'
                    '<float name="exponent" value="%.9g"/></bsdf>'
                    % (*kd, ks, ks, ks, expo))
        else:
            bsdf = '<bsdf type="diffuse"><rgb name="reflectance" value="%.9g %.9g %.9g"/></bsdf>' % tuple(kd)
        shapes.append('  <shape type="obj"><string name="filename" value="%s.obj"/>%s</shape>'
                      % (name, bsdf))
    if sphere is not None:
        _write_sphere_obj(os.path.join(outdir, "sphere.obj"), sphere["center"], sphere["radius"])
        shapes.append('  <shape type="obj"><string name="filename" value="sphere.obj"/>'
                      '<bsdf type="roughdielectric"><float name="alpha" value="%.9g"/>'
                      '<float name="intIOR" value="%.9g"/><float name="extIOR" value="1"/></bsdf></shape>'
                      % (sphere["alpha"], sphere["ior"]))
    # Area light: 0.25 x 0.25 quad just below the ceiling, facing down.
    _write_obj(os.path.join(outdir, "light.obj"),
               [((-0.125, 0.999, -0.125), (0.25, 0.0, 0.0), (0.0, 0.0, 0.25))])
    shapes.append('  <shape type="obj"><string name="filename" value="light.obj"/>'
                  '<bsdf type="diffuse"><rgb name="reflectance" value="0 0 0"/></bsdf>'
                  '<emitter type="area"><rgb name="radiance" value="15 15 15"/></emitter></shape>')
    if point_light is not None:
        shapes.append('  <emitter type="point"><point name="position" x="%.9g" y="%.9g" z="%.9g"/>'
                      '<rgb name="intensity" value="%.9g %.9g %.9g"/></emitter>'
                      % (*point_light["pos"], *point_light["intensity"]))
    if env is not None:
        write_pfm(os.path.join(outdir, "env.pfm"), env["image"])
        shapes.append('  <emitter type="envmap"><string name="filename" value="env.pfm"/>'
                      '<transform name="toWorld"><rotate y="1" angle="%.9g"/></transform></emitter>'
                      % env.get("angle", 0.0))
    sensor = ('  <sensor type="perspective">\n'
              '    <float name="fov" value="40"/>\n'
              '    <transform name="toWorld"><lookat origin="0, 0, 3.5" target="0, 0, 0" up="0, 1, 0"/></transform>\n'
              '    <film type="hdrfilm"><integer name="width" value="%d"/><integer name="height" value="%d"/>'
              '<string name="filename" value="image.exr"/></film>\n'
              '  </sensor>\n' % (width, height))
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n<scene version="0.5.0">\n'
           + options.xml() + sensor + "\n".join(shapes) + "\n</scene>\n")
    path = os.path.join(outdir, filename)
    with open(path, "w") as f:
        f.write(xml)
    return path


def config1(outdir: str, spp: int = 64, integrator: str = "drmlt", acceptance_map: bool = False,
            extra: dict | None = None) -> str:
    """Plain DRMLT (green) on the 256x256 Lambertian Cornell box, max depth 5, 4096 chains
    (other integrators / the acceptance map on the same scene for the render tests)."""
    return write_cornell(outdir, seed=1, width=256, height=256, phong=False,
                         options=SceneOptions(maxdepth=5, numchains=4096, spp=spp, type="green", integrator=integrator,
                                              acceptanceMap=acceptance_map, extra=dict(extra or {})))


def config2(outdir: str, dr_type: str = "mira", spp: int = 64) -> str:
    """H2MC second stage on the Phong Cornell box at 1024x1024, max depth 8, 16384 chains."""
    return write_cornell(outdir, seed=2, width=1024, height=1024, phong=True,
                         options=SceneOptions(maxdepth=8, numchains=16384, spp=spp, type=dr_type))


def config3(outdir: str, spp: int = 16, dr_type: str = "green") -> str:
    """The Lambertian Cornell box (seed 3) with a rough-dielectric sphere: alpha
    U[0.05, 0.5] from the seed, IOR 1.5; 256x256, max depth 5, 4096 chains."""
    alpha = float(np.random.default_rng(1003).uniform(0.05, 0.5))
    return write_cornell(outdir, seed=3, width=256, height=256, phong=False,
                         options=SceneOptions(maxdepth=5, numchains=4096, spp=spp, type=dr_type),
                         sphere=dict(center=(-0.45, -0.6, 0.45), radius=0.3, alpha=alpha, ior=1.5))


def config3_deep(outdir: str, spp: int = 16, dr_type: str = "green") -> str:
    """Config 3 at max depth 10: the derivative check batch's scene (the
    Lambertian box with the rough-dielectric sphere, paths of up to 20 primary
    dimensions)."""
    alpha = float(np.random.default_rng(1003).uniform(0.05, 0.5))
    return write_cornell(outdir, seed=3, width=256, height=256, phong=False,
                         options=SceneOptions(maxdepth=10, numchains=4096, spp=spp, type=dr_type),
                         sphere=dict(center=(-0.45, -0.6, 0.45), radius=0.3, alpha=alpha, ior=1.5))


def config_lights(outdir: str, spp: int = 16, dr_type: str = "green") -> str:
    """Config 3 (seed 5) plus a point light of intensity 3 under the ceiling: area
    light, point light and the rough-dielectric sphere together."""
    alpha = float(np.random.default_rng(1005).uniform(0.05, 0.5))
    return write_cornell(outdir, seed=5, width=256, height=256, phong=False,
                         options=SceneOptions(maxdepth=5, numchains=4096, spp=spp, type=dr_type),
                         sphere=dict(center=(-0.45, -0.6, 0.45), radius=0.3, alpha=alpha, ior=1.5),
                         point_light=dict(pos=(0.4, 0.75, 0.3), intensity=(3.0, 3.0, 3.0)))


def config_env(outdir: str, spp: int = 16, dr_type: str = "green") -> str:
    """Config 3 (seed 6) without its ceiling, lit by the area light and an 8 x 4
    environment map rotated 30 degrees about y; the camera sees the map past
    the box's edges."""
    alpha = float(np.random.default_rng(1006).uniform(0.05, 0.5))
    return write_cornell(outdir, seed=6, width=256, height=256, phong=False,
                         options=SceneOptions(maxdepth=5, numchains=4096, spp=spp, type=dr_type),
                         sphere=dict(center=(-0.45, -0.6, 0.45), radius=0.3, alpha=alpha, ior=1.5),
                         env=dict(image=env_image(), angle=30.0), ceiling=False)


def _write_mesh_obj(path, V, F, N):
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in V]
    lines += ["vn %.9g %.9g %.9g" % tuple(n) for n in N]
    lines += ["f %d//%d %d//%d %d//%d" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1) for a, b, c in F]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def config4_small(outdir: str, spp: int = 4, dr_type: str = "mira") -> str:
    """Config 4 in miniature, written as scene XML + OBJ: the displaced geodesic
    sphere at frequency 6 (720 triangles, rough dielectric, alpha from the seed)
    over a 12 x 12 Phong ground grid (288 triangles), the 2 x 1 constant
    environment map and the point light of intensity 50; 256 x 256, max depth
    12 (paths of up to 24 primary dimensions), 4096 chains."""
    from . import procedural as P
    os.makedirs(outdir, exist_ok=True)
    seed = 4
    rng = np.random.default_rng(seed)
    V, F = P.geodesic_sphere(6)
    V = V * (1.0 + 0.05 * P.gradient_noise(3.0 * V, seed))[:, None]
    _write_mesh_obj(os.path.join(outdir, "sphere.obj"), V, F, P._vertex_normals(V, F))
    GV, GF = P._grid(12, 6.0, -1.08)
    _write_mesh_obj(os.path.join(outdir, "ground.obj"), GV, GF, np.tile([0.0, 1.0, 0.0], (len(GV), 1)))
    alpha = float(rng.uniform(0.05, 0.5))
    kd = rng.uniform(0.2, 0.8, 3)
    expo = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
    ks = float(rng.uniform(0.1, 0.5))
    write_pfm(os.path.join(outdir, "env.pfm"), np.ones((1, 2, 3), np.float32))
    options = SceneOptions(maxdepth=12, numchains=4096, spp=spp, type=dr_type)
    shapes = [
        '  <shape type="obj"><string name="filename" value="sphere.obj"/>'
        '<bsdf type="roughdielectric"><float name="alpha" value="%.9g"/>'
        '<float name="intIOR" value="1.5"/><float name="extIOR" value="1"/></bsdf></shape>' % alpha,
        '  <shape type="obj"><string name="filename" value="ground.obj"/>'
        '<bsdf type="phong"><rgb name="diffuseReflectance" value="%.9g %.9g %.9g"/>'
        '<rgb name="specularReflectance" value="%.9g %.9g %.9g"/><float name="exponent" value="%.9g"/></bsdf>'
        '</shape>' % (*kd, ks, ks, ks, expo),
        '  <emitter type="envmap"><string name="filename" value="env.pfm"/></emitter>',
        '  <emitter type="point"><point name="position" x="2" y="4" z="3"/>'
        '<rgb name="intensity" value="50 50 50"/></emitter>',
    ]
    sensor = ('  <sensor type="perspective">\n'
              '    <float name="fov" value="40"/>\n'
              '    <transform name="toWorld"><lookat origin="0, 1.2, 5.5" target="0, -0.2, 0" up="0, 1, 0"/></transform>\n'
              '    <film type="hdrfilm"><integer name="width" value="256"/><integer name="height" value="256"/>'
              '<string name="filename" value="image.exr"/></film>\n'
              '  </sensor>\n')
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n<scene version="0.5.0">\n'
           + options.xml() + sensor + "\n".join(shapes) + "\n</scene>\n")
    path = os.path.join(outdir, "scene.xml")
    with open(path, "w") as f:
        f.write(xml)
    return path


def config_meshes(outdir: str) -> str:
    """Mesh front-end check scene (no render intended): every loader branch of
    the reference's ParseObj / LoadSerialized once, seeded.

    shapes, in order:
      0  OBJ without normals, ``v/vt`` corners with a texture seam, rotated and
         non-uniformly scaled (vertex normals computed; seam vertices split);
      1  OBJ quads with ``vn`` under a non-uniform scale (inverse-transpose
         normals, not renormalised);
      2  serialized v4, single precision, stored normals (shapeIndex 0);
      3  serialized v4, double precision, no normals, uvs + colours, a
         degenerate and obtuse triangles (shapeIndex 1);
      4  serialized v4, single precision, normals + uvs (shapeIndex 2),
         translated;
      5  serialized v3, single precision, no normals (shapeIndex 1)."""
    from . import procedural as P
    from .meshio import write_serialized
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(17)
    V, F = P.geodesic_sphere(3)
    V = V * (1.0 + 0.1 * P.gradient_noise(2.0 * V, 17))[:, None]
    # texture coordinates split along x < 0 / x >= 0: corners of faces that
    # straddle the split get their own vt per side
    side = (V[F].mean(axis=1)[:, 0] >= 0).astype(np.int64)
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in V]
    lines += ["vt %.6g %.6g" % (0.25 + 0.5 * s, 0.5) for s in (0, 1)]
    lines += ["f %d/%d %d/%d %d/%d" % (a + 1, s + 1, b + 1, s + 1, c + 1, s + 1) for (a, b, c), s in zip(F, side)]
    with open(os.path.join(outdir, "noNormals.obj"), "w") as f:
        f.write("\n".join(lines) + "\n")
    qV = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0.2], [0, 1, 0], [2, 0, 0.3], [2, 1, 0]], np.float64)
    qN = rng.normal(size=(6, 3))
    lines = ["v %.9g %.9g %.9g" % tuple(v) for v in qV] + ["vn %.9g %.9g %.9g" % tuple(n) for n in qN]
    lines += ["f 1//1 2//2 3//3 4//4", "f 2//2 5//5 6//6 3//3"]
    with open(os.path.join(outdir, "quads.obj"), "w") as f:
        f.write("\n".join(lines) + "\n")
    gV, gF = P._grid(4, 1.0, 0.0)
    gV = gV + rng.uniform(-0.2, 0.2, gV.shape) * [1, 0, 1]
    gV[:, 1] = rng.uniform(-0.1, 0.1, len(gV))
    gF = np.vstack([gF, [[0, 1, 2]]])  # a degenerate triangle (0, 1, 2 lie on one grid row)
    gV[2] = 2 * gV[1] - gV[0]
    sV, sF = P.geodesic_sphere(2)
    meshes = [dict(positions=sV * 0.5, indices=sF, normals=sV, name="sphere"),
              dict(positions=gV, indices=gF, uvs=gV[:, [0, 2]], colors=rng.uniform(size=gV.shape), name="grid"),
              dict(positions=sV * [0.3, 0.6, 0.3], indices=sF, normals=sV * [2, 1, 2], uvs=sV[:, :2], name="egg")]
    write_serialized(os.path.join(outdir, "meshes_v4_f.serialized"), [meshes[0], meshes[2]], version=4)
    write_serialized(os.path.join(outdir, "meshes_v4_d.serialized"), [meshes[0], meshes[1]], version=4, double=True)
    write_serialized(os.path.join(outdir, "meshes_v4_f3.serialized"), [meshes[1], meshes[1], meshes[2]], version=4)
    write_serialized(os.path.join(outdir, "meshes_v3.serialized"),
                     [meshes[2], dict(positions=gV * 0.7, indices=gF)], version=3)
    diffuse = '<bsdf type="diffuse"><rgb name="reflectance" value="0.5 0.5 0.5"/></bsdf>'
    shapes = [
        ('obj', 'noNormals.obj', None, '<rotate x="0.3" y="1" z="0.2" angle="37"/><scale x="1.5" y="0.7" z="1.1"/>'),
        ('obj', 'quads.obj', None, '<scale x="2" y="0.5" z="1"/><translate x="0.1" y="0" z="-0.3"/>'),
        ('serialized', 'meshes_v4_f.serialized', 0, '<scale x="1" y="2" z="1"/>'),
        ('serialized', 'meshes_v4_d.serialized', 1, '<rotate x="0" y="1" z="0" angle="20"/>'),
        ('serialized', 'meshes_v4_f3.serialized', 2, '<translate x="0.5" y="0.2" z="0.1"/>'),
        ('serialized', 'meshes_v3.serialized', 1, ''),
    ]
    body = []
    for kind, fn, idx, xf in shapes:
        extra = '' if idx is None else '<integer name="shapeIndex" value="%d"/>' % idx
        body.append('  <shape type="%s"><string name="filename" value="%s"/>%s'
                    '<transform name="toWorld">%s</transform>%s</shape>' % (kind, fn, extra, xf, diffuse))
    body.append('  <emitter type="point"><point name="position" x="0" y="3" z="3"/>'
                '<rgb name="intensity" value="10 10 10"/></emitter>')
    sensor = ('  <sensor type="perspective">\n'
              '    <float name="fov" value="40"/>\n'
              '    <transform name="toWorld"><lookat origin="0, 0, 6" target="0, 0, 0" up="0, 1, 0"/></transform>\n'
              '    <film type="hdrfilm"><integer name="width" value="64"/><integer name="height" value="64"/></film>\n'
              '  </sensor>\n')
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n<scene version="0.5.0">\n'
           + SceneOptions(maxdepth=3, numchains=64, spp=1).xml() + sensor + "\n".join(body) + "\n</scene>\n")
    path = os.path.join(outdir, "scene.xml")
    with open(path, "w") as f:
        f.write(xml)
    return path
