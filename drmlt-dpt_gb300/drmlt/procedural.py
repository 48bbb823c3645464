"""Large procedural scenes built in memory (no OBJ files): the multi-million
triangle workloads whose geometry is too large to round-trip through the
reference's text scene format.

  * ``config4``: a displaced geodesic sphere of 1,997,120 triangles (icosahedron
    faces subdivided at frequency 316, radius 1 displaced by 0.05 x gradient
    noise) in rough dielectric (Beckmann, alpha U[0.05, 0.5] from the seed, IOR
    1.5) over a Phong ground grid of 1,002,528 triangles, lit by a constant
    environment map of radiance 1 (a 2 x 1 image) and a point light of
    intensity 50; 1024 x 1024, max depth 12, 65536 chains.
  * ``config5``: an fBm heightfield (6 octaves) of 8,000,000 triangles under a
    glass slab (IOR 1.5, alpha 0.02, below the roughness threshold so its
    vertices use relative parameters) lit by a 0.05 x 0.05 area light of
    radiance 2000; 2048 x 2048, max depth 12, 262144 chains.

Noise: Perlin's improved gradient noise (Perlin, "Improving Noise", SIGGRAPH
2002): a seeded permutation of 0..255, the quintic fade 6t^5 - 15t^4 + 10t^3
and the 12 edge gradients of a cube, restated here in numpy.
"""
from __future__ import annotations

import math

import numpy as np

from . import capi
from .scene import DptOptions, SceneData, _lookat

_GRAD = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                  [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1], [1, 1, 0], [0, -1, 1], [-1, 1, 0], [0, -1, -1]],
                 np.float64)


def gradient_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Improved gradient noise at the points p (N x 3), values in about [-1, 1]."""
    perm = np.random.default_rng(seed).permutation(256)
    perm = np.concatenate([perm, perm])
    fl = np.floor(p)
    i = fl.astype(np.int64) & 255
    f = p - fl
    u = f * f * f * (f * (f * 6.0 - 15.0) + 10.0)
    corners = []
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                h = perm[perm[perm[i[:, 0] + dx] + i[:, 1] + dy] + i[:, 2] + dz] & 15
                g = _GRAD[h]
                corners.append(np.einsum("ij,ij->i", g, f - np.array([dx, dy, dz], np.float64)))
    # trilinear blend with the faded weights: corners are ordered x fastest
    c = corners
    x00 = c[0] + u[:, 0] * (c[1] - c[0])
    x10 = c[2] + u[:, 0] * (c[3] - c[2])
    x01 = c[4] + u[:, 0] * (c[5] - c[4])
    x11 = c[6] + u[:, 0] * (c[7] - c[6])
    y0 = x00 + u[:, 1] * (x10 - x00)
    y1 = x01 + u[:, 1] * (x11 - x01)
    out = y0 + u[:, 2] * (y1 - y0)
    return out


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    return v, f


def geodesic_sphere(freq: int):
    """Unit geodesic sphere: each icosahedron face split into freq^2 triangles
    (counter-clockwise seen from outside). Returns (vertices V x 3, faces F x 3)
    with the vertices shared between faces merged."""
    V, F = _icosahedron()
    ii, jj = np.meshgrid(np.arange(freq + 1), np.arange(freq + 1), indexing="ij")
    keep = ii + jj <= freq
    ii, jj = ii[keep], jj[keep]
    # local index of grid point (i, j) within one face
    lid = -np.ones((freq + 1, freq + 1), np.int64)
    lid[ii, jj] = np.arange(len(ii))
    tri = []
    for i in range(freq):
        for j in range(freq - i):
            tri.append((lid[i, j], lid[i + 1, j], lid[i, j + 1]))
            if i + j < freq - 1:
                tri.append((lid[i + 1, j], lid[i + 1, j + 1], lid[i, j + 1]))
    tri = np.array(tri, np.int64)
    npf = len(ii)
    pts, faces = [], []
    for k, (a, b, c) in enumerate(F):
        A, B, C = V[a], V[b], V[c]
        p = A + np.outer(ii / freq, B - A) + np.outer(jj / freq, C - A)
        pts.append(p / np.linalg.norm(p, axis=1, keepdims=True))
        faces.append(tri + k * npf)
    P = np.concatenate(pts)
    Fc = np.concatenate(faces)
    # merge the copies of the points on shared edges and corners
    key = np.round(P * (1 << 20)).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    return P[first], inv.reshape(-1)[Fc]


def _vertex_normals(V, F):
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    vn = np.zeros_like(V)
    for k in range(3):
        np.add.at(vn, F[:, k], n)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)


def _bsdf(kind, **kw):
    b = capi.Bsdf()
    b.type = kind
    b.two_sided = 0
    for k, v in kw.items():
        if isinstance(v, (list, tuple)):
            getattr(b, k)[:] = list(v)
        else:
            setattr(b, k, v)
    return b


def _options(maxdepth, chains, spp, dr_type):
    o = DptOptions()
    o.maxDepth = maxdepth
    o.numChains = chains
    o.spp = spp
    o.type = dr_type
    o.perturbStdDev = 1.0 / 64.0
    o.numInitSamples = 100000
    return o


def _camera(width, height, origin, target, fov=40.0):
    return dict(fov=fov, near=1e-2, far=1000.0, width=width, height=height,
                to_world=_lookat(np.asarray(origin, np.float64), np.asarray(target, np.float64),
                                 np.array([0.0, 1.0, 0.0])))


def _grid(n, half, y, height=None):
    """(n x n)-cell grid over [-half, half]^2 at height y (+ height(x, z)),
    two triangles per cell, normals up-facing."""
    xs = np.linspace(-half, half, n + 1)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    Y = np.full_like(X, y) if height is None else y + height(X, Z)
    V = np.stack([X, Y, Z], -1).reshape(-1, 3)
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    a, b, c, d = idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]
    F = np.concatenate([np.stack([a, d, c], -1).reshape(-1, 3), np.stack([a, c, b], -1).reshape(-1, 3)])
    return V, F


def _box(lo, hi):
    """Axis-aligned box as 12 triangles with per-face vertices and outward normals."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    V, F, N = [], [], []
    for axis in range(3):
        for side, n in ((lo, -1.0), (hi, 1.0)):
            u, v = (axis + 1) % 3, (axis + 2) % 3
            q = []
            for a, b in ((0, 0), (1, 0), (1, 1), (0, 1)):
                p = np.empty(3)
                p[axis] = side[axis]
                p[u] = (lo, hi)[a][u]
                p[v] = (lo, hi)[b][v]
                q.append(p)
            base = len(V)
            V += q
            nn = np.zeros(3)
            nn[axis] = n
            N += [nn] * 4
            # (u, v) order gives normal +axis; flip for the low side
            F += [(base, base + 1, base + 2), (base, base + 2, base + 3)] if n > 0 else \
                 [(base, base + 2, base + 1), (base, base + 3, base + 2)]
    return np.array(V), np.array(F), np.array(N)


def _assemble(shapes, bsdfs, lights, camera, options, env_images=()):
    """shapes: list of (V, F, N or None, bsdf index, area light index or -1)."""
    pos, nor, first, count, sb, sl = [], [], [], [], [], []
    t = 0
    for V, F, N, b, l in shapes:
        N = _vertex_normals(V, F) if N is None else N
        pos.append(V[F].astype(np.float32))
        nor.append(N[F].astype(np.float32))
        first.append(t)
        count.append(len(F))
        t += len(F)
        sb.append(b)
        sl.append(l)
    return SceneData(np.concatenate(pos), np.concatenate(nor), np.asarray(first, np.int32),
                     np.asarray(count, np.int32), np.asarray(sb, np.int32), np.asarray(sl, np.int32),
                     list(bsdfs), list(lights), camera, options, "<procedural>", list(env_images))


def config4(seed: int = 4, spp: int = 16, dr_type: str = "mira", width: int = 1024, height: int = 1024,
            chains: int = 65536, freq: int = 316, grid: int = 708) -> SceneData:
    rng = np.random.default_rng(seed)
    V, F = geodesic_sphere(freq)
    V = V * (1.0 + 0.05 * gradient_noise(3.0 * V, seed))[:, None]
    alpha = float(rng.uniform(0.05, 0.5))
    GV, GF = _grid(grid, 6.0, -1.08)
    kd = rng.uniform(0.2, 0.8, 3)
    expo = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
    ks = float(rng.uniform(0.1, 0.5))
    bsdfs = [_bsdf(capi.BSDF_ROUGHDIELECTRIC, int_ior=1.5, ext_ior=1.0, alpha=alpha, ks=(1, 1, 1), kt=(1, 1, 1)),
             _bsdf(capi.BSDF_PHONG, kd=tuple(kd), ks=(ks, ks, ks), exponent=expo)]
    env = np.ones((1, 2, 3), np.float32)
    Le = capi.Light()
    Le.type = capi.LIGHT_ENV
    Le.shape = -1
    Le.sampling_weight = 1.0
    Le.env_rgb = env.ctypes.data_as(capi.C.POINTER(capi.C.c_float))
    Le.env_height, Le.env_width = env.shape[0], env.shape[1]
    Le.to_world[:] = np.eye(4, dtype=np.float32).ravel().tolist()
    Lp = capi.Light()
    Lp.type = capi.LIGHT_POINT
    Lp.shape = -1
    Lp.sampling_weight = 1.0
    Lp.emission[:] = [50.0, 50.0, 50.0]
    Lp.pos[:] = [2.0, 4.0, 3.0]
    cam = _camera(width, height, (0.0, 1.2, 5.5), (0.0, -0.2, 0.0))
    return _assemble([(V, F, None, 0, -1), (GV, GF, np.tile([0.0, 1.0, 0.0], (len(GV), 1)), 1, -1)],
                     bsdfs, [Le, Lp], cam, _options(12, chains, spp, dr_type), [env])


def config5(seed: int = 5, spp: int = 16, dr_type: str = "mira", width: int = 2048, height: int = 2048,
            chains: int = 262144, grid: int = 2000, acceptance_map: bool = False) -> SceneData:
    def fbm(X, Z):
        h = np.zeros_like(X)
        amp, freq = 0.12, 1.5
        P = np.stack([X, np.zeros_like(X), Z], -1).reshape(-1, 3)
        for octave in range(6):
            h += amp * gradient_noise(P * freq, seed + octave).reshape(X.shape)
            amp *= 0.5
            freq *= 2.0
        return h
    GV, GF = _grid(grid, 1.0, -0.5, fbm)
    # glass slab 2.2 x 0.1 x 2.2 above the heightfield: 6 flat-shaded faces, outward normals
    SV, SF, SN = _box((-1.1, 0.0, -1.1), (1.1, 0.1, 1.1))
    # area light 0.05 x 0.05 facing down at y = 1.5
    LV = np.array([[-0.025, 1.5, -0.025], [0.025, 1.5, -0.025], [0.025, 1.5, 0.025], [-0.025, 1.5, 0.025]])
    LF = np.array([[0, 1, 2], [0, 2, 3]])
    rng = np.random.default_rng(seed)
    kd = rng.uniform(0.2, 0.8, 3)
    bsdfs = [_bsdf(capi.BSDF_LAMBERTIAN, kd=tuple(kd)),
             _bsdf(capi.BSDF_ROUGHDIELECTRIC, int_ior=1.5, ext_ior=1.0, alpha=0.02, ks=(1, 1, 1), kt=(1, 1, 1)),
             _bsdf(capi.BSDF_LAMBERTIAN, kd=(0.0, 0.0, 0.0))]
    La = capi.Light()
    La.type = capi.LIGHT_AREA
    La.shape = 2
    La.sampling_weight = 1.0
    La.emission[:] = [2000.0, 2000.0, 2000.0]
    flat = lambda V, n: np.tile(n, (len(V), 1))
    cam = _camera(width, height, (0.0, 1.6, 3.2), (0.0, -0.3, 0.0))
    opts = _options(12, chains, spp, dr_type)
    opts.acceptanceMap = acceptance_map
    return _assemble([(GV, GF, None, 0, -1), (SV, SF, SN, 1, -1), (LV, LF, flat(LV, [0.0, -1.0, 0.0]), 2, 0)],
                     bsdfs, [La], cam, opts)


def main(argv=None):
    """Renders a few chain-loop iterations of a procedural scene (and optionally
    one ray-benchmark pass) -- a small driver for profiling runs:
    python -m drmlt.procedural config4 --iterations 4 --lanes 16 --warps 2 --graph 1
    (--wavefront 1 or --persistent 1 --team-sms T select the other schedules;
    --integrator h2mc [--lens-prob P] the h2mc integrator with its lens mutation)"""
    import argparse
    from .integrator import Renderer
    ap = argparse.ArgumentParser()
    ap.add_argument("scene", choices=["config4", "config5"])
    ap.add_argument("--iterations", type=int, default=4)
    ap.add_argument("--lanes", type=int, default=0, help="chains per warp (0: library default)")
    ap.add_argument("--lanes2", type=int, default=0, help="chains per warp of the second-stage kernels")
    ap.add_argument("--warps", type=int, default=0, help="derivative warps per chain (0: library default)")
    ap.add_argument("--graph", type=int, default=0, help="replay iterations as CUDA graphs")
    ap.add_argument("--wavefront", type=int, default=0, help="path tracing in wavefront rounds")
    ap.add_argument("--persistent", type=int, default=0, help="the persistent cooperative schedule")
    ap.add_argument("--team-sms", type=int, default=0, help="persistent schedule: SMs of the team workers")
    ap.add_argument("--rays", default="", choices=["", "primary", "bounce", "shadow"])
    ap.add_argument("--adjoint-min-dim", type=int, default=0,
                    help="derivatives by the reverse-mode adjoint from this path dimension on "
                         "(0: library default, -1: hyper-dual for every path)")
    ap.add_argument("--head-chains", type=int, default=0, help="two-tier stage 1: chains of the head tier")
    ap.add_argument("--head-lanes", type=int, default=0, help="two-tier stage 1: chains per warp of the head tier")
    ap.add_argument("--integrator", default="drmlt", choices=["drmlt", "h2mc", "mcmc"])
    ap.add_argument("--lens-prob", type=float, default=0.3, help="integrator=h2mc: lensperturbprob")
    a = ap.parse_args(argv)
    sd = globals()[a.scene]()
    sd.options.integrator = a.integrator
    sd.options.lensPerturbProb = a.lens_prob
    r = Renderer(sd, seed=77, use_graph=a.graph, stage_lanes=a.lanes, stage2_lanes=a.lanes2, deriv_warps=a.warps,
                 wavefront=a.wavefront, persistent=a.persistent, team_sms=a.team_sms,
                 adjoint_min_dim=a.adjoint_min_dim,
                 head_chains=a.head_chains, head_lanes=a.head_lanes)
    r.prepass()
    r.run(a.iterations)
    st = r.stats()
    out = {"mutations": st["mutations"], "run_ms": r.last_run_ms()}
    if a.integrator == "h2mc":
        out["lens"] = [st["lens"], st["lens_accepted"]]
    if a.rays:
        out["rays"] = r.ray_benchmark(a.rays, 1 << 21, 1)
    r.close()
    print(out)


if __name__ == "__main__":
    main()
