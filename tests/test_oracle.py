"""The oracle (CPU restatement, oracle/oracle.cpp) pinned against the reference's
own outputs (golden fixtures made by tests/golden/make_golden.py from the
reference built from its sources). CPU only."""
import os
import sys

import numpy as np
import pytest

from helpers import REPO, chad_env_defect, chad_hessian_consistent, env_light_index, golden, path_record, scene_xml, ss_rtol

sys.path.insert(0, os.path.join(REPO, "oracle"))

CFGS = ["cfg1", "cfg2", "cfg3", "cfgL", "cfgE"]


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


def lum(c):
    return 0.212671 * c[0] + 0.715160 * c[1] + 0.072169 * c[2]


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_bootstrap_sampler(oracles, cfg):
    """Same techniques, contributions (1e-4) and consumed uniforms as the
    reference; ss to the conditioning of its spherical Jacobians (ss_rtol)."""
    recs = golden(cfg, "bidir")
    o = oracles(cfg)
    cnt, tech, ct, _, cons = o.replay(0, [r["uniforms"] for r in recs])
    for i, rec in enumerate(recs):
        ref = {(c["camDepth"], c["lightDepth"]): c for c in rec["contribs"]}
        mine = {(int(tech[i, k, 0]), int(tech[i, k, 1])): ct[i, k] for k in range(cnt[i])}
        assert cons[i] == rec["consumed"], i
        assert set(ref) == set(mine), i
        for k, c in ref.items():
            np.testing.assert_allclose(mine[k]["rgb"], c["contrib"], rtol=1e-4, atol=1e-12)
            np.testing.assert_allclose(mine[k]["ss"], c["ss"], rtol=ss_rtol(rec["path"]), atol=1e-30)


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_large_step_sampler(oracles, cfg):
    recs = golden(cfg, "subpath")
    o = oracles(cfg)
    cnt, tech, ct, pth, cons = o.replay(1, [r["uniforms"] for r in recs], [r["camLength"] for r in recs],
                                        [r["lgtLength"] for r in recs])
    for i, rec in enumerate(recs):
        assert cons[i] == rec["consumed"] and cnt[i] == len(rec["contribs"]), i
        if cnt[i]:
            np.testing.assert_allclose(ct[i, 0]["ls"], rec["contribs"][0]["ls"], rtol=1e-4)
            exp = path_record(rec["path"], rec["camLength"], rec["lgtLength"], o.scene.shape_first_tri)
            L = rec["camLength"] + rec["lgtLength"] - 1
            np.testing.assert_allclose(pth[i]["u"][:2 * L], exp["u"][:2 * L], atol=2e-5)


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_direct_pass(oracles, cfg):
    recs = golden(cfg, "direct")
    o = oracles(cfg)
    cnt, tech, ct, _, cons = o.replay(2, [r["uniforms"] for r in recs], [r["pixel"][0] for r in recs],
                                      [r["pixel"][1] for r in recs], 8)
    for i, rec in enumerate(recs):
        assert cons[i] == rec["consumed"], i
        assert cnt[i] == len(rec["contribs"]), i
        for k, c in enumerate(rec["contribs"]):
            np.testing.assert_allclose(ct[i, k]["rgb"], c["contrib"], rtol=1e-4, atol=1e-12)


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_perturbation(oracles, cfg):
    recs = golden(cfg, "tech")
    o = oracles(cfg)
    paths, offs, refs = [], [], []
    for rec in recs:
        base = path_record(rec["path"], rec["path"]["camDepth"], rec["path"]["lgtDepth"], o.scene.shape_first_tri,
                           rec["pos"])
        for pt in rec["perturb"]:
            off = np.zeros(24, np.float32)
            off[:rec["dim"]] = pt["offset"]
            paths.append(base)
            offs.append(off)
            refs.append((rec, pt))
    out, ct = o.perturb(np.array(paths), np.array(offs))
    n_early = 0
    for i, (rec, pt) in enumerate(refs):
        if not ct[i]["valid"] and not pt["contribs"] and not np.allclose(out[i]["u"][:rec["dim"]], pt["ypos"], atol=2e-6):
            # both rejected, but stopped at different vertices (the positions of a
            # rejected proposal are never used); bounded below
            n_early += 1
            continue
        np.testing.assert_allclose(out[i]["u"][:rec["dim"]], pt["ypos"], atol=2e-6)
        assert bool(ct[i]["valid"]) == (len(pt["contribs"]) == 1), i
        if ct[i]["valid"]:
            np.testing.assert_allclose(ct[i]["ss"], pt["contribs"][0]["ss"], rtol=ss_rtol(pt["path"]), atol=1e-30)
    assert n_early <= 0.005 * len(refs), n_early


def _deriv_records(cfg, o):
    recs = [r for r in golden(cfg, "tech") if r["haveDerv"] and not r["scrubbed"] and r["contrib"][0]["ss"] > 1e-15]
    P = np.array([path_record(r["path"], r["path"]["camDepth"], r["path"]["lgtDepth"], o.scene.shape_first_tri,
                              r["pos"]) for r in recs])
    U = np.zeros((len(recs), 24))
    for i, r in enumerate(recs):
        U[i, :r["dim"]] = r["pos"]
    return recs, P, U


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_derivatives(oracles, cfg):
    """Forward-over-reverse (FP64 tape) vs chad and vs FP64 central differences (h = 1e-4).

    Gradient vs chad 1e-3 everywhere. Hessian vs chad 1e-3 wherever chad's
    Hessian is the derivative of chad's own gradient (chad_hessian_consistent);
    elsewhere only the check below applies. Hessian vs FP64 differences 1e-3
    on at least 90% of paths (differences straddling a branch of the path
    function are not derivatives).

    Environment light: paths that end on it have f = log of the reference's
    primal ss score (1e-4); chad is compared only where it is the reference's
    primal too (chad_env_defect), the other paths rely on the differences."""
    o = oracles(cfg)
    recs, P, U = _deriv_records(cfg, o)
    env = env_light_index(o.scene)
    f, gfd, hfd = o.fd_derivs(P, U, 1e-4)
    _, gfd6, _ = o.fd_derivs(P, U, 1e-6)  # gradient differences closer in (Tent's kink at 0.5)
    g, h = o.tape_derivs(P, U.astype(np.float32))
    n_fd_ok = n_defect = 0
    for i, r in enumerate(recs):
        d = r["dim"]
        p = r["path"]
        if env >= 0 and p["lgtDepth"] == 0 and p["camSurf"][-1]["shape"] < 0:
            assert abs(f[i] - np.log(r["contrib"][0]["ss"])) <= 1e-4 * max(1.0, abs(f[i])), i
        if np.max(np.abs(h[i, :d * d] - hfd[i, :d * d])) <= 1e-3 * np.max(np.abs(hfd[i, :d * d])):
            n_fd_ok += 1
        if chad_env_defect(r, env):
            n_defect += 1
            assert np.max(np.abs(g[i, :d] - gfd6[i, :d])) <= 1e-3 * np.max(np.abs(gfd6[i, :d])), i
            continue
        assert abs(f[i] - r["logf"]) <= 1e-4 * max(1.0, abs(r["logf"])), i
        assert np.max(np.abs(g[i, :d] - r["grad"])) <= 1e-3 * np.max(np.abs(r["grad"])), i
        hr = np.array(r["hess"])
        if chad_hessian_consistent(r):
            assert np.max(np.abs(h[i, :d * d] - hr)) <= 1e-3 * np.max(np.abs(hr)), i
    assert n_fd_ok >= 0.9 * len(recs), (n_fd_ok, len(recs))
    assert n_defect <= 0.2 * len(recs), n_defect


def test_oracle_derivatives_vs_fp64_chad(oracles):
    """The oracle's FP64 derivatives against the reference's chad library built in
    FP64 (fixture cfg3d_tech: config 3 at max depth 10, paths of up to 20
    primary coordinates): log f to 1e-5 relative, gradient and Hessian to 1e-4
    of their largest entry (wherever chad's Hessian is the derivative of its
    own gradient) -- ten times tighter than against the single-precision chad
    (measured: log f median 1.3e-7, max 2.7e-6; gradient max 3.3e-5; Hessian
    max 4.1e-5);
    what is left is the scene itself (the FP64 reference reads the mesh files'
    9-digit coordinates in double, the oracle in float) and the fixture's 9
    printed digits."""
    if golden("cfg3d", "tech") is None:
        pytest.skip("no golden fixture cfg3d_tech")
    o = oracles("cfg3d")
    recs, P, U = _deriv_records("cfg3d", o)
    f, _, _ = o.fd_derivs(P, U, 1e-4)
    g, h = o.tape_derivs(P, U.astype(np.float32))
    n = 0
    for i, r in enumerate(recs):
        d = r["dim"]
        assert abs(f[i] - r["logf"]) <= 1e-5 * max(1.0, abs(r["logf"])), (i, f[i], r["logf"])
        assert np.max(np.abs(g[i, :d] - r["grad"])) <= 1e-4 * np.max(np.abs(r["grad"])), i
        if chad_hessian_consistent(r):
            n += 1
            hr = np.array(r["hess"])
            assert np.max(np.abs(h[i, :d * d] - hr)) <= 1e-4 * np.max(np.abs(hr)), i
    assert n >= len(recs) // 2 and max(r["dim"] for r in recs) == 20, (n, len(recs))


@pytest.mark.parametrize("cfg", CFGS)
def test_oracle_gaussian(oracles, cfg):
    recs = golden(cfg, "tech")
    o = oracles(cfg)
    n = len(recs)
    dims = np.array([r["dim"] for r in recs])
    ss = np.array([r["contrib"][0]["ss"] for r in recs], np.float32)
    G = np.zeros((n, 24), np.float32)
    H = np.zeros((n, 576), np.float32)
    for i, r in enumerate(recs):
        G[i, :r["dim"]] = r["grad"]
        H[i, :r["dim"] ** 2] = r["hess"]
    mean, ic, cv, ld = o.compute_gaussian(dims, ss, G, H)
    ok = 0
    for i, r in enumerate(recs):
        d = r["dim"]
        icr = np.array(r["gauss"]["invCov"]).reshape(d, d).T
        e = np.max(np.abs(ic[i, :d * d].reshape(d, d) - icr)) / np.max(np.abs(icr))
        ok += e < 1e-3 and abs(ld[i] - r["gauss"]["logDet"]) <= 1e-3 * max(1.0, abs(r["gauss"]["logDet"]))
    assert ok >= 0.98 * n


def test_oracle_dr_loop_runs(oracles):
    """A short CPU chain loop: finite film, counters consistent with the reference's loop."""
    o = oracles("cfg1")
    r = o.dr_run(num_chains=64, iterations=20, threads=2, num_init=2000)
    st = r["stats"]
    assert r["mutations"] == 64 * 20 == st[8]
    assert st[0] + st[2] == st[8]            # every iteration is a large step or a stage-1 small step
    assert st[4] + st[6] <= st[2] - st[3]    # second stages only after rejected small steps
    assert np.isfinite(r["film"]).all() and r["film"].sum() > 0


def test_oracle_bvh_matches_brute_force():
    """The oracle's own BVH (object-median splits, used above 1024 triangles,
    e.g. for the 3.0 M-triangle config-4 scene) returns the brute-force
    answer: the same closest triangle and distance for every ray, the same
    occlusion answer for every shadow ray (src/scene.cpp:80-111 semantics)."""
    import oracle_dr
    from drmlt import procedural
    sd = procedural.config4(freq=24, grid=48, chains=256)  # 16,128 triangles, same construction as config 4
    o = oracle_dr.Oracle(sd)
    rng = np.random.default_rng(3)
    n = 20000
    org = (rng.random((n, 3)) * 4 - 2).astype(np.float32)
    d = rng.standard_normal((n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    # rays from surface points along the normal-ish direction, the bounce-ray case
    tb, thb = o.trace_rays(org, d, mode="brute")
    tv, thv = o.trace_rays(org, d, mode="bvh")
    assert (tb >= 0).mean() > 0.3
    assert np.array_equal(tb, tv)
    assert np.array_equal(thb, thv)
    hit = tb >= 0
    p = org[hit] + thb[hit, None] * d[hit]
    d2 = rng.standard_normal(p.shape)
    d2 = (d2 / np.linalg.norm(d2, axis=1, keepdims=True)).astype(np.float32)
    p = p.astype(np.float32)
    tb2, _ = o.trace_rays(p, d2, mode="brute")
    tv2, _ = o.trace_rays(p, d2, mode="bvh")
    assert np.array_equal(tb2, tv2)
    ab, _ = o.trace_rays(org, d, tmax=1.0, any_hit=True, mode="brute")
    av, _ = o.trace_rays(org, d, tmax=1.0, any_hit=True, mode="bvh")
    assert np.array_equal(ab >= 0, av >= 0)
    o.close()
