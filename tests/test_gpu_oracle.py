"""CUDA path vs the oracle (oracle/oracle.cpp, itself pinned to the reference by
test_oracle.py) on seeded random inputs, at sizes beyond the golden fixtures.

All CUDA calls go through libdrmlt.so's C ABI. Bars: contributions relative
1e-4; log f relative 1e-4 of the FP64 oracle; gradient and Hessian 1e-3 of the
largest entry against the oracle's FP64 forward-over-reverse derivatives;
ComputeGaussian (FP64 on both sides) 1e-6; ray hits: same triangle on at least
99.99% of rays. The CUDA side computes in FP32 with fused multiply-adds, so a
path whose ray grazes a triangle edge can branch differently; each test bounds
that fraction explicitly.
"""
import os
import sys

import numpy as np
import pytest

from helpers import REPO, scene_xml

sys.path.insert(0, os.path.join(REPO, "oracle"))

pytestmark = pytest.mark.gpu

# cfg4s: config 4 in miniature (displaced rough-dielectric sphere, Phong ground,
# constant environment map, point light) at max depth 12 -- paths of up to 24
# primary dimensions; no reference fixtures (the oracle only)
CFGS = ["cfg1", "cfg2", "cfg3", "cfgL", "cfgE", "cfg4s"]
MAX_DEPTH = {"cfg1": 5, "cfg2": 8, "cfg3": 5, "cfgL": 5, "cfgE": 5, "cfg4s": 12}


@pytest.fixture(scope="module")
def oracles(scene_root):
    import oracle_dr
    from drmlt import scene as dscene
    cache = {}

    def get(cfg):
        if cfg not in cache:
            cache[cfg] = oracle_dr.Oracle(dscene.load_scene(scene_xml(cfg, scene_root)))
        return cache[cfg]

    yield get
    for o in cache.values():
        o.close()


def _random_large_steps(cfg, n, seed):
    """n seeded uniform streams with techniques drawn like the multiplexed large step."""
    rng = np.random.default_rng(seed)
    L = rng.integers(3, MAX_DEPTH[cfg] + 1, n)
    cam = np.array([rng.integers(1, l + 2) for l in L], np.int32)
    lgt = (L + 1 - cam).astype(np.int32)
    tapes = rng.random((n, 64 if MAX_DEPTH[cfg] <= 8 else 128), dtype=np.float32)
    tapes = np.minimum(tapes, np.float32(1.0 - 2 ** -24))
    return tapes, cam, lgt


_CACHE = {}


# random large steps per scene; in the open miniature config 4 under the
# environment map only ~0.7% of random techniques contribute
N_STEPS = {"cfg4s": 1 << 16}
MIN_VALID = {"cfg4s": 1.0 / 400}


def _valid_paths(cfg, renderers, oracles):
    """Random large-step paths traced by both sides; returns the ones both found valid and equal."""
    n = N_STEPS.get(cfg, 4096)
    if cfg in _CACHE:
        return _CACHE[cfg]
    tapes, cam, lgt = _random_large_steps(cfg, n, 17)
    r, o = renderers(cfg), oracles(cfg)
    cg, tg, ctg, pg, sg = r.replay(1, list(tapes), cam, lgt)
    co, to, cto, po, so = o.replay(1, list(tapes), cam, lgt)
    same = (cg == co) & (sg == so)
    keep = np.nonzero(same & (cg == 1))[0]
    _CACHE[cfg] = (tapes, cam, lgt, (cg, ctg, pg, sg), (co, cto, po, so), keep)
    return _CACHE[cfg]


@pytest.mark.parametrize("cfg", CFGS)
def test_random_large_steps_vs_oracle(renderers, oracles, cfg):
    tapes, cam, lgt, g, o, keep = _valid_paths(cfg, renderers, oracles)
    cg, ctg, pg, sg = g
    co, cto, po, so = o
    n = len(tapes)
    bad = int(np.sum((cg != co) | (sg != so)))
    assert len(keep) > n * MIN_VALID.get(cfg, 1.0 / 20)
    for i in keep:
        d = 2 * (pg[i]["c"] + pg[i]["l"] - 1)
        nv = pg[i]["c"] + pg[i]["l"] - 2
        ok = (pg[i]["c"], pg[i]["l"], pg[i]["lgt_light"], pg[i]["lgt_prim"], pg[i]["dl_light"], pg[i]["dl_prim"],
              pg[i]["use_abs"]) == (po[i]["c"], po[i]["l"], po[i]["lgt_light"], po[i]["lgt_prim"], po[i]["dl_light"],
                                    po[i]["dl_prim"], po[i]["use_abs"])
        ok &= np.array_equal(pg[i]["tri"][:nv], po[i]["tri"][:nv])
        ok &= np.allclose(pg[i]["u"][:d], po[i]["u"][:d], atol=1e-5, rtol=0)
        a, b = ctg[i, 0], cto[i, 0]
        ok &= np.allclose(a["rgb"], b["rgb"], rtol=1e-4, atol=1e-12) and abs(a["ss"] - b["ss"]) <= 1e-4 * abs(b["ss"])
        ok &= np.allclose(a["screen"], b["screen"], atol=2e-5, rtol=0)
        bad += 0 if ok else 1
    assert bad <= n // 200, "%d / %d large steps differ" % (bad, n)


@pytest.mark.parametrize("cfg", CFGS)
def test_random_perturbations_vs_oracle(renderers, oracles, cfg):
    """PerturbPathBidir on random valid paths with N(0, sigma) offsets, sigma in {0.01, 0.0025, 0.05}."""
    tapes, cam, lgt, g, o, keep = _valid_paths(cfg, renderers, oracles)
    paths = g[2][keep]
    rng = np.random.default_rng(23)
    sig = rng.choice([0.01, 0.0025, 0.05], len(paths)).astype(np.float32)
    off = (rng.standard_normal((len(paths), 24)) * sig[:, None]).astype(np.float32)
    og, cg = renderers(cfg).perturb(paths, off)
    oo, co = oracles(cfg).perturb(paths, off)
    bad = 0
    for i in range(len(paths)):
        d = 2 * (paths[i]["c"] + paths[i]["l"] - 1)
        ok = bool(cg[i]["valid"]) == bool(co[i]["valid"]) and np.allclose(og[i]["u"][:d], oo[i]["u"][:d], atol=1e-6)
        if ok and co[i]["valid"]:
            ok = abs(cg[i]["ss"] - co[i]["ss"]) <= 1e-4 * abs(co[i]["ss"]) and np.allclose(
                cg[i]["rgb"], co[i]["rgb"], rtol=1e-4, atol=1e-12)
        bad += 0 if ok else 1
    assert bad <= max(2, len(paths) // 200), "%d / %d perturbations differ" % (bad, len(paths))


@pytest.mark.parametrize("cfg", CFGS)
def test_random_derivatives_vs_fp64_oracle(renderers, oracles, cfg):
    """log f, gradient and Hessian (CUDA, FP32 hyper-dual) vs the oracle's FP64
    forward-over-reverse derivatives of the same path function, every technique."""
    tapes, cam, lgt, g, o, keep = _valid_paths(cfg, renderers, oracles)
    paths = g[2][keep]
    ss = g[1][keep, 0]["ss"]
    sel = np.nonzero(ss > 1e-15)[0]
    paths = paths[sel]
    u = np.zeros((len(paths), 24), np.float32)
    for i in range(len(paths)):
        u[i] = paths[i]["u"]
    r, ora = renderers(cfg), oracles(cfg)
    logf = r.path_eval(paths, u)
    gg, hg = r.path_grad_hess(paths, u)
    f64, _, _ = ora.fd_derivs(paths, u.astype(np.float64), 1e-4)
    go, ho = ora.tape_derivs(paths, u)
    bad_f, bad_g, bad_h = [], [], []
    for i in range(len(paths)):
        d = 2 * (paths[i]["c"] + paths[i]["l"] - 1)
        if not np.isfinite(f64[i]):
            continue
        if abs(logf[i] - f64[i]) > 1e-4 * max(1.0, abs(f64[i])):
            bad_f.append(i)
        if np.max(np.abs(gg[i, :d] - go[i, :d])) > 1e-3 * max(np.max(np.abs(go[i, :d])), 1e-6):
            bad_g.append(i)
        if np.max(np.abs(hg[i, :d * d] - ho[i, :d * d])) > 1e-3 * max(np.max(np.abs(ho[i, :d * d])), 1e-6):
            bad_h.append(i)
    n = len(paths)
    assert n > 100
    tol = max(2, n // 100)
    assert len(bad_f) <= tol, "log f: %d / %d" % (len(bad_f), n)
    assert len(bad_g) <= tol, "gradient: %d / %d" % (len(bad_g), n)
    # The Hessians that miss the bar are explained path by path: the
    # single-precision path function is not smooth at the 1e-3 level there
    # (deep paths that graze the tessellated sphere from inside, in the
    # miniature config 4): central differences of the GPU's own FP32 gradient
    # at steps 1e-3 and 2e-3 disagree by more than the bar, while the FP64
    # function's do not. At most 1% of the paths may miss without that reason.
    rough = _fp32_not_smooth(r, ora, paths, u, bad_h)
    unexplained = [i for i in bad_h if not rough[i]]
    assert len(unexplained) <= tol, "Hessian: %d / %d (%d with a non-smooth FP32 gradient)" % (
        len(unexplained), n, len(bad_h) - len(unexplained))
    assert len(bad_h) <= max(2, n // 50), "Hessian: %d / %d" % (len(bad_h), n)


@pytest.mark.parametrize("cfg", CFGS)
def test_random_adjoint_vs_fp64_oracle(renderers, oracles, cfg):
    """The reverse-mode adjoint (drmlt_path_adjoint: forward and backward sweeps
    in Dual numbers, one Hessian row each) on the random paths of the test
    above: against the hyper-dual derivatives of the same FP32 function (1e-3
    of the largest entry; both are exact derivatives, so they differ by FP32
    rounding), and against the oracle's FP64 forward-over-reverse tape with the
    same bars and the same explanation of the misses."""
    tapes, cam, lgt, g, o, keep = _valid_paths(cfg, renderers, oracles)
    paths = g[2][keep]
    ss = g[1][keep, 0]["ss"]
    paths = paths[np.nonzero(ss > 1e-15)[0]]
    u = np.zeros((len(paths), 24), np.float32)
    for i in range(len(paths)):
        u[i] = paths[i]["u"]
    r, ora = renderers(cfg), oracles(cfg)
    ga, ha = r.path_adjoint(paths, u)
    gh, hh = r.path_grad_hess(paths, u)
    go, ho = ora.tape_derivs(paths, u)
    bad_hd, bad_g, bad_h = [], [], []
    for i in range(len(paths)):
        d = 2 * (paths[i]["c"] + paths[i]["l"] - 1)
        H = ha[i, :d * d].reshape(d, d)
        assert np.array_equal(H, H.T), "adjoint Hessian not symmetric"
        if not (np.isfinite(gh[i, :d]).all() and np.isfinite(hh[i, :d * d]).all()):
            continue
        e_g = np.max(np.abs(ga[i, :d] - gh[i, :d])) / max(np.max(np.abs(gh[i, :d])), 1e-6)
        e_h = np.max(np.abs(ha[i, :d * d] - hh[i, :d * d])) / max(np.max(np.abs(hh[i, :d * d])), 1e-6)
        if not (e_g <= 1e-3 and e_h <= 1e-3):
            bad_hd.append(i)
        if np.max(np.abs(ga[i, :d] - go[i, :d])) > 1e-3 * max(np.max(np.abs(go[i, :d])), 1e-6):
            bad_g.append(i)
        if np.max(np.abs(ha[i, :d * d] - ho[i, :d * d])) > 1e-3 * max(np.max(np.abs(ho[i, :d * d])), 1e-6):
            bad_h.append(i)
    n = len(paths)
    assert n > 100
    tol = max(2, n // 100)
    assert len(bad_hd) <= tol, "adjoint vs hyper-dual: %d / %d" % (len(bad_hd), n)
    assert len(bad_g) <= tol, "gradient: %d / %d" % (len(bad_g), n)
    rough = _fp32_not_smooth(r, ora, paths, u, bad_h)
    unexplained = [i for i in bad_h if not rough[i]]
    assert len(unexplained) <= tol, "Hessian: %d / %d (%d with a non-smooth FP32 gradient)" % (
        len(unexplained), n, len(bad_h) - len(unexplained))
    assert len(bad_h) <= max(2, n // 50), "Hessian: %d / %d" % (len(bad_h), n)


def _fp32_not_smooth(r, ora, paths, u, idx, steps=(1e-3, 2e-3)):
    """Whether the FP32 path function of each listed path is not smooth at the
    1e-3 level where the FP64 one is: central-difference Hessians of the GPU's
    FP32 gradient at the two steps disagree by more than 1e-3 of their largest
    entry, while the oracle's FP64 central-difference Hessians at the same
    steps agree to 1e-3."""
    out = {}
    for i in idx:
        d = 2 * (paths[i]["c"] + paths[i]["l"] - 1)
        f32, f64 = [], []
        for h in steps:
            pp = np.repeat(paths[i:i + 1], 2 * d)
            uu = np.repeat(u[i:i + 1], 2 * d, axis=0)
            for j in range(d):
                uu[2 * j, j] += h
                uu[2 * j + 1, j] -= h
            for k in range(2 * d):
                pp[k]["u"] = uu[k]
            gp, _ = r.path_grad_hess(pp, uu)
            f32.append(np.stack([(gp[2 * j, :d] - gp[2 * j + 1, :d]) / (2 * h) for j in range(d)]))
            _, _, h64 = ora.fd_derivs(paths[i:i + 1], u[i:i + 1].astype(np.float64), h)
            f64.append(h64[0, :d * d].reshape(d, d))
        top32 = max(np.max(np.abs(f32[0])), 1e-6)
        top64 = max(np.max(np.abs(f64[0])), 1e-6)
        out[i] = bool(np.max(np.abs(f32[0] - f32[1])) > 1e-3 * top32 and
                      np.max(np.abs(f64[0] - f64[1])) <= 1e-3 * top64)
    return out


@pytest.mark.parametrize("cfg", CFGS)
def test_random_gaussians_vs_fp64_oracle(renderers, oracles, cfg):
    """ComputeGaussian on the GPU (FP32 Jacobi refined to FP64) vs the oracle's sequential FP64 Jacobi."""
    tapes, cam, lgt, g, o, keep = _valid_paths(cfg, renderers, oracles)
    paths = g[2][keep]
    ss = g[1][keep, 0]["ss"].astype(np.float32)
    u = np.stack([p["u"] for p in paths]).astype(np.float32)
    grad, hess = oracles(cfg).tape_derivs(paths, u)
    dims = np.array([2 * (p["c"] + p["l"] - 1) for p in paths], np.int32)
    mg, icg, cvg, ldg = renderers(cfg).compute_gaussian(dims, ss, grad, hess)
    mo, ico, cvo, ldo = oracles(cfg).compute_gaussian(dims, ss, grad, hess)
    worst = []
    for i in range(len(paths)):
        d = dims[i]
        e = [np.max(np.abs(icg[i, :d * d] - ico[i, :d * d])) / max(np.max(np.abs(ico[i, :d * d])), 1e-300),
             np.max(np.abs(cvg[i, :d * d] - cvo[i, :d * d])) / max(np.max(np.abs(cvo[i, :d * d])), 1e-300),
             np.max(np.abs(mg[i, :d] - mo[i, :d])) / max(np.max(np.abs(mo[i, :d])), 1e-3),
             abs(ldg[i] - ldo[i]) / max(1.0, abs(ldo[i]))]
        worst.append(max(e))
    worst = np.array(worst)
    assert np.mean(worst < 1e-6) >= 0.995, "max %g" % worst.max()
    assert np.median(worst) < 1e-10, np.median(worst)


@pytest.mark.parametrize("cfg", ["cfg1"])
def test_ray_hits_vs_oracle(renderers, oracles, cfg):
    """Closest-hit and occlusion casts through the BVH vs brute force over all triangles."""
    rng = np.random.default_rng(5)
    n = 1 << 20
    org = (rng.random((n, 3)) * 1.96 - 0.98).astype(np.float32)
    d = rng.standard_normal((n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r, o = renderers(cfg), oracles(cfg)
    tg, thg = r.trace_rays(org, d)
    to, tho = o.trace_rays(org, d)
    # a different triangle at the same distance is a tie between coplanar
    # triangles (a box's bottom face lies on the floor), not a miss
    tie = (tg != to) & (tg >= 0) & (to >= 0) & (np.abs(thg - tho) <= 1e-5 * np.abs(tho))
    agree = np.mean((tg == to) | tie)
    assert agree >= 0.9999, (agree, np.mean(tie))
    both = (tg == to) & (tg >= 0)
    assert np.allclose(thg[both], tho[both], rtol=1e-5, atol=1e-6)
    og, _ = r.trace_rays(org, d, tmax=1.0, any_hit=True)
    oo, _ = o.trace_rays(org, d, tmax=1.0, any_hit=True)
    assert np.mean((og >= 0) == (oo >= 0)) >= 0.9999


def test_ray_hits_at_scale_vs_oracle_bvh(built_lib):
    """BVH hit parity on the 3.0 M-triangle procedural scene (displaced sphere over a
    ground grid): 2^20 camera-like rays (from the camera position towards random
    points of the scene's box), 2^20 bounce rays (from their hits, random
    directions) and the shadow rays between those hits and random points
    (src/scene.cpp:80-111: closest hit, and occlusion over t in [tmin, tmax]),
    the CUDA BVH (binned SAH, csrc/bvh.cpp) against the oracle's own
    object-median BVH (itself pinned to brute force in tests/test_oracle.py).
    Bar: the same triangle on >= 99.99% of the rays of each kind, where a
    different triangle at the same distance (a tie between triangles sharing
    the hit point: an edge or a vertex of the tessellation) is counted apart."""
    import oracle_dr
    from drmlt import procedural
    from drmlt.integrator import Renderer
    sd = procedural.config4(chains=256)
    assert len(sd.positions) > 2_900_000
    r = Renderer(sd, num_chains=256)
    o = oracle_dr.Oracle(sd)
    try:
        rng = np.random.default_rng(44)
        n = 1 << 20
        P = sd.positions.reshape(-1, 3)
        lo, hi = P.min(0), P.max(0)
        eye = np.array([0.0, 1.2, 5.5], np.float32)
        tgt = lo + rng.random((n, 3)) * (hi - lo)
        d = tgt - eye
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        org = np.broadcast_to(eye, (n, 3)).astype(np.float32)
        report = {}

        def closest(org, d, tmin=1e-3):
            tg, thg = r.trace_rays(org, d, tmin=tmin)
            to, tho = o.trace_rays(org, d, tmin=tmin, mode="bvh")
            tie = (tg != to) & (tg >= 0) & (to >= 0) & (np.abs(thg - tho) <= 1e-5 * np.abs(tho))
            same = tg == to
            both = same & (tg >= 0)
            # same triangle: the same distance up to float rounding of the two
            # Moller-Trumbore evaluations (FMA contraction on the GPU), which
            # grows where the ray grazes the triangle's plane (t is ill-conditioned
            # there: 7 of 458,894 camera-ray hits differ by more than 1e-5)
            rel = np.abs(thg[both] - tho[both]) / np.maximum(np.abs(tho[both]), 1e-6)
            assert np.mean(rel <= 1e-5) >= 0.9999, np.mean(rel <= 1e-5)
            return tg, thg, float(np.mean(same)), float(np.mean(tie)), float(np.mean(to >= 0))

        tg, th, same, tie, hits = closest(org, d)
        report["camera"] = (same, tie, hits)
        assert hits > 0.3 and same + tie >= 0.9999, report
        # bounce rays from the hits (offset back along the ray by tmin's scale)
        h = tg >= 0
        p = (org[h] + th[h, None] * d[h]).astype(np.float32)
        d2 = rng.standard_normal(p.shape)
        d2 = (d2 / np.linalg.norm(d2, axis=1, keepdims=True)).astype(np.float32)
        tg2, th2, same, tie, hits2 = closest(p, d2)
        report["bounce"] = (same, tie, hits2)
        assert hits2 > 0.1 and same + tie >= 0.9999, report
        # shadow rays of length 1 from the hits towards random points of the box
        q = (lo + rng.random(p.shape) * (hi - lo)).astype(np.float32)
        ds = q - p
        ds = (ds / np.linalg.norm(ds, axis=1, keepdims=True)).astype(np.float32)
        og, _ = r.trace_rays(p, ds, tmin=1e-3, tmax=1.0, any_hit=True)
        oo, _ = o.trace_rays(p, ds, tmin=1e-3, tmax=1.0, any_hit=True, mode="bvh")
        agree = float(np.mean((og >= 0) == (oo >= 0)))
        report["shadow"] = (agree, float(np.mean(oo >= 0)))
        assert 0.05 < np.mean(oo >= 0) < 0.95 and agree >= 0.9999, report
        print(report)
    finally:
        r.close()
        o.close()
