"""The derivative check batch: f, gradient and Hessian of log f on the config-3
scene at max depth 10 (the Lambertian box with the rough-dielectric sphere).

* Against the reference's chad library built in FP64 (fixture cfg3d_tech,
  tests/golden/make_golden.py --double): log f relative 1e-4, gradient and
  Hessian 1e-3 of their largest entry, on the technique paths where chad's
  Hessian is the derivative of its own gradient (helpers.chad_hessian_consistent).
* At scale: 2^20 seeded uniform streams, path length L uniform in [2, 10]
  (2L primary coordinates), traced by the multiplexed large step on the GPU;
  every path that contributes is differentiated on the GPU (gradient and
  Hessian finite, Hessian symmetric), and a seeded sample of 4096 of them is
  checked against the oracle's FP64 forward-over-reverse derivatives (1e-3),
  the first 512 also against FP64 central differences of log f with h = 1e-4
  (1e-2: the differences' own truncation and rounding error).

Both derivative methods are held to these bars: the reverse-mode adjoint
(drmlt_path_adjoint) and hyper-dual forward mode (drmlt_path_grad_hess).
"""
import os
import sys

import numpy as np
import pytest

from helpers import REPO, chad_hessian_consistent, golden, path_record  # noqa: I001

sys.path.insert(0, os.path.join(REPO, "oracle"))

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def deep(built_lib, scene_root):
    from drmlt import scenegen
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    import oracle_dr
    sd = dscene.load_scene(scenegen.config3_deep(os.path.join(scene_root, "cfg3d")))
    r = Renderer(sd, num_chains=64)
    o = oracle_dr.Oracle(sd)
    yield sd, r, o
    r.close()
    o.close()


@pytest.mark.parametrize("method", ["adjoint", "hyperdual"])
def test_derivatives_vs_fp64_chad(deep, method):
    recs = golden("cfg3d", "tech")
    if recs is None:
        pytest.skip("no golden fixture cfg3d_tech")
    sd, r, _ = deep
    paths, us = [], []
    for rec in recs:
        c, l = rec["path"]["camDepth"], rec["path"]["lgtDepth"]
        paths.append(path_record(rec["path"], c, l, sd.shape_first_tri, rec["pos"]))
        u = np.zeros(24, np.float32)
        u[:rec["dim"]] = rec["pos"]
        us.append(u)
    paths = np.array(paths)
    logf = r.path_eval(paths, np.array(us))
    g, h = (r.path_adjoint if method == "adjoint" else r.path_grad_hess)(paths, np.array(us))
    bad, n = [], 0
    depths = set()
    for i, rec in enumerate(recs):
        d = rec["dim"]
        if rec.get("logf") is None or not chad_hessian_consistent(rec):
            continue
        n += 1
        depths.add(d // 2)
        gr = np.array(rec["grad"])
        hr = np.array(rec["hess"])
        ok = abs(logf[i] - rec["logf"]) <= 1e-4 * max(1.0, abs(rec["logf"]))
        ok = ok and np.max(np.abs(g[i, :d] - gr)) <= 1e-3 * max(np.max(np.abs(gr)), 1e-6)
        ok = ok and np.max(np.abs(h[i, :d * d] - hr)) <= 1e-3 * max(np.max(np.abs(hr)), 1e-6)
        if not ok:
            bad.append(i)
    assert n >= len(recs) // 3 and max(depths) >= 6, (n, sorted(depths))
    assert len(bad) <= max(2, n // 100), "%d / %d paths differ from FP64 chad" % (len(bad), n)


def test_derivative_batch_of_2e20_vectors(deep):
    sd, r, o = deep
    rng = np.random.default_rng(20)
    n = 1 << 20
    L = rng.integers(2, 11, n)
    cam = np.array([rng.integers(1, l + 2) for l in L], np.int32)
    lgt = (L + 1 - cam).astype(np.int32)
    tapes = np.minimum(rng.random((n, 96), dtype=np.float32), np.float32(1.0 - 2 ** -24))
    cnt, _, ct, pth, _ = r.replay(1, list(tapes), cam, lgt)
    valid = np.nonzero((cnt == 1) & (ct[:, 0]["ss"] > 1e-15))[0]
    assert len(valid) > n // 100
    paths = pth[valid]
    u = np.stack([p["u"] for p in paths]).astype(np.float32)
    dims = 2 * (paths["c"] + paths["l"] - 1)
    assert dims.max() >= 16
    # a seeded sample against the FP64 oracle
    pick = np.sort(np.random.default_rng(21).choice(len(paths), size=min(4096, len(paths)), replace=False))
    go, ho = o.tape_derivs(paths[pick], u[pick])
    # central differences (they also difference the Hessian: d^2 evaluations a path) on the first 512
    nfd = min(512, len(pick))
    _, gfd, hfd = o.fd_derivs(paths[pick[:nfd]], u[pick[:nfd]].astype(np.float64), 1e-4)
    for method in ("adjoint", "hyperdual"):
        g, h = (r.path_adjoint if method == "adjoint" else r.path_grad_hess)(paths, u)
        for i in range(0, len(paths), max(1, len(paths) // 20000)):
            d = dims[i]
            H = h[i, :d * d].reshape(d, d)
            assert np.all(np.isfinite(g[i, :d])) and np.all(np.isfinite(H)), (method, i)
            assert np.array_equal(H, H.T), (method, i)
        bad_g, bad_h, bad_fd = [], [], []
        for k, i in enumerate(pick):
            d = dims[i]
            top_g = max(np.max(np.abs(go[k, :d])), 1e-6)
            top_h = max(np.max(np.abs(ho[k, :d * d])), 1e-6)
            if np.max(np.abs(g[i, :d] - go[k, :d])) > 1e-3 * top_g:
                bad_g.append(i)
            if np.max(np.abs(h[i, :d * d] - ho[k, :d * d])) > 1e-3 * top_h:
                bad_h.append(i)
            if k < nfd and (np.max(np.abs(g[i, :d] - gfd[k, :d])) > 1e-2 * top_g or
                            np.max(np.abs(h[i, :d * d] - hfd[k, :d * d])) > 1e-2 * top_h):
                bad_fd.append(i)
        m = len(pick)
        assert len(bad_g) <= max(2, m // 100), "%s gradient: %d / %d" % (method, len(bad_g), m)
        assert len(bad_h) <= max(2, m // 100), "%s Hessian: %d / %d" % (method, len(bad_h), m)
        assert len(bad_fd) <= max(2, nfd // 50), "%s vs FP64 central differences: %d / %d" % (method, len(bad_fd),
                                                                                            nfd)
        del g, h
