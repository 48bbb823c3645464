"""integrator=h2mc's lens mutation vs the reference's own outputs
(tests/golden/<cfg>_lens.jsonl.gz, ref_harness mode lens).

Per technique path: the lens score (SubpathContrib::lensScore), the lens
vertex position, the chad lens-mode log f with its gradient and Hessian w.r.t.
the screen position, the 2-D Gaussian of the integrator's ComputeGaussian; per
perturbation: PerturbLensBidir's path, contribution and lens score.

Tolerances: scores and contributions 1e-4 relative (lens scores 1e-3: the
walk re-evaluates the BSDFs the sampler evaluated); log f 1e-4 absolute;
gradient and Hessian 1e-3 relative to the largest entry of the reference's.
Where chad's lens Hessian is not symmetric to 1e-3 it is not the derivative
of chad's own gradient (some paths ending on or lit by the environment), and
the CUDA Hessian is compared with the central differences of chad's gradient
(fixture field fdHess, h = 1e-4) at 2e-2 instead; paths emitted by the
environment light in the half of its disc where the generated
SampleConcentricDisc takes another branch (helpers.chad_env_defect) have no
chad reference and are left out. The Gaussian (FP64 here, FP32 Eigen in the
reference): 1e-3 relative. As in
the other parity tests, a small fraction of records may take another branch
(a grazing ray resolves differently in the float BVH than in the reference's
intersector); each test bounds that fraction.
"""
import numpy as np
import pytest

from helpers import chad_env_defect, env_light_index, golden, path_record, rel_err, ss_rtol

pytestmark = pytest.mark.gpu

CFGS = ["cfg1", "cfg3", "cfgL", "cfgE"]


def _need(cfg):
    g = golden(cfg, "lens")
    if g is None:
        pytest.skip("no golden fixture %s_lens" % cfg)
    return g


def _inputs(r, recs):
    first = r.scene.shape_first_tri
    paths, screen, ss = [], [], []
    for rec in recs:
        c, l = rec["path"]["camDepth"], rec["path"]["lgtDepth"]
        paths.append(path_record(rec["path"], c, l, first, rec["pos"]))
        screen.append(rec["contrib"][0]["screen"])
        ss.append(rec["contrib"][0]["ss"])
    return np.array(paths), np.array(screen, np.float32), np.array(ss, np.float32)


@pytest.mark.parametrize("cfg", CFGS)
def test_lens_scores_and_derivatives_vs_reference(renderers, cfg):
    recs = _need(cfg)
    r = renderers(cfg)
    paths, screen, ss = _inputs(r, recs)
    sigma = r.scene.options.lensPerturbStdDev
    out = r.lens_eval(paths, screen, ss, lens_sigma=sigma, max_derivative_depth=5)
    env = env_light_index(r.scene)
    bad_score = bad_der = bad_gauss = nder = 0
    for i, rec in enumerate(recs):
        p = rec["path"]
        emitted_by_env = p["lgtDepth"] >= 2 and p["lgtLight"] == env
        chad_ok = not (emitted_by_env and chad_env_defect(rec, env))
        ref = rec["contrib"][0]["lens"]
        if not (rel_err(out["score"][i], ref, 1e-20) < 1e-3 or (ref == 0 and out["score"][i] == 0)):
            bad_score += 1
            continue
        c = rec["path"]["camDepth"]
        if c >= 3 and not np.allclose(out["pos"][i], rec["lensPos"], atol=1e-4, rtol=1e-5):
            bad_score += 1
        if rec["haveDerv"] and ref > 1e-15 and not rec["scrubbed"] and chad_ok:
            nder += 1
            g_ref = np.array(rec["grad"], np.float64)
            h_ref = np.array(rec["hess"], np.float64)
            gs = max(np.abs(g_ref).max(), 1e-6)
            hs = max(np.abs(h_ref).max(), 1e-6)
            good = abs(out["logf"][i] - rec["logf"]) < 1e-4 * max(1.0, abs(rec["logf"]))
            good = good and np.abs(out["grad"][i] - g_ref).max() <= 1e-3 * gs
            if abs(h_ref[1] - h_ref[2]) <= 1e-3 * hs:
                good = good and np.abs(out["hess"][i] - h_ref).max() <= 1e-3 * hs
            else:
                fd = np.array(rec["fdHess"], np.float64)
                good = good and np.abs(out["hess"][i] - fd).max() <= 2e-2 * max(np.abs(fd).max(), 1e-6)
            bad_der += 0 if good else 1
        if not chad_ok:
            continue
        g = rec["gauss"]
        good = np.allclose(out["mean"][i], g["mean"], rtol=1e-3, atol=1e-3 * max(1e-8, np.abs(g["mean"]).max()))
        ic = np.array(g["invCov"], np.float64)
        good = good and np.abs(out["inv_cov"][i] - ic).max() <= 1e-3 * np.abs(ic).max()
        good = good and abs(out["log_det"][i] - g["logDet"]) <= 1e-3 * max(1.0, abs(g["logDet"]))
        bad_gauss += 0 if good else 1
    n = len(recs)
    assert nder > n // 2
    assert bad_score <= max(1, n // 50), "%d / %d lens scores differ" % (bad_score, n)
    assert bad_der <= max(1, nder // 50), "%d / %d lens derivatives differ" % (bad_der, nder)
    assert bad_gauss <= max(1, n // 50), "%d / %d lens Gaussians differ" % (bad_gauss, n)


@pytest.mark.parametrize("cfg", CFGS)
def test_lens_perturbation_vs_reference(renderers, cfg):
    """PerturbLensBidir: same primary vector, hit triangles, contribution and lens score."""
    recs = _need(cfg)
    r = renderers(cfg)
    first = r.scene.shape_first_tri
    paths, scr, lpos, refs = [], [], [], []
    for rec in recs:
        c, l = rec["path"]["camDepth"], rec["path"]["lgtDepth"]
        base = path_record(rec["path"], c, l, first, rec["pos"])
        for pt in rec["perturb"]:
            paths.append(base)
            scr.append(pt["screen"])
            lpos.append(rec["lensPos"])
            refs.append((rec, pt))
    if not refs:
        pytest.skip("no lens perturbations in the fixture")
    out, ct, score = r.lens_perturb(np.array(paths), np.array(scr, np.float32), np.array(lpos, np.float32))
    bad = nvalid = 0
    for i, (rec, pt) in enumerate(refs):
        dim = rec["dim"]
        c, l = rec["path"]["camDepth"], rec["path"]["lgtDepth"]
        valid = len(pt["contribs"]) == 1
        good = bool(ct[i]["valid"]) == valid
        if good and valid:
            nvalid += 1
            ref = pt["contribs"][0]
            good = np.allclose(out[i]["u"][:dim], pt["ypos"], atol=2e-5)
            good = good and np.allclose(ct[i]["screen"], ref["screen"], atol=2e-5, rtol=0)
            good = good and bool(np.all(rel_err(ct[i]["rgb"], ref["contrib"], 1e-12) < 1e-4) or
                                 np.allclose(ct[i]["rgb"], ref["contrib"], rtol=1e-4, atol=1e-9))
            good = good and rel_err(ct[i]["ls"], ref["ls"], 1e-12) < 1e-4
            good = good and rel_err(ct[i]["ss"], ref["ss"], 1e-12) < max(1e-3, ss_rtol(pt["path"]))
            good = good and (rel_err(score[i], ref["lens"], 1e-20) < 1e-3 or (ref["lens"] == 0 and score[i] == 0))
            exp = path_record(pt["path"], c, l, first)
            nv = (l - 1 if l > 1 else 0) + c - 1
            good = good and np.array_equal(out[i]["tri"][:nv], exp["tri"][:nv])
            good = good and int(out[i]["use_abs"]) >> 31 == 1
        bad += 0 if good else 1
    assert nvalid > len(refs) // 2
    assert bad <= max(1, len(refs) // 50), "%d / %d lens perturbations differ" % (bad, len(refs))


IDENTITY_DEPTH = {"cfg3": 5, "cfgE": 5, "cfg4s": 12}
IDENTITY_STEPS = {"cfg3": 4096, "cfgE": 4096, "cfg4s": 1 << 16}


@pytest.mark.parametrize("cfg", ["cfg3", "cfgE", "cfg4s"])
def test_lens_perturbation_to_the_own_screen_position_is_the_identity(renderers, cfg):
    """A property that holds at any size, on random valid paths up to depth 12
    (the miniature config 4): PerturbLensBidir of a state with a positive lens
    score to its own screen position, aimed at its own lens vertex, gives the
    state back as PerturbPathBidir with zero offsets re-traces it (both
    evaluate the BSDF at the absolute-parameter vertices; the sampler that made
    the state sampled them, whose pdfs can differ) -- the same hit triangles
    and, for c >= 2, the same contribution (1e-3: the first camera vertex's
    direction is recomputed toward the lens vertex) and lens score. For c = 1
    the contribution differs by design: PerturbLensLastVertex multiplies the
    throughput by its shading-normal factor with wi and wo swapped
    (src/path.cpp:1862-1866), which differs from BSDFSampling's on
    smooth-shaded vertices."""
    r = renderers(cfg)
    rng = np.random.default_rng(23)
    n = IDENTITY_STEPS[cfg]
    L = rng.integers(3, IDENTITY_DEPTH[cfg] + 1, n)
    cam = np.array([rng.integers(1, x + 2) for x in L], np.int32)
    lgt = (L + 1 - cam).astype(np.int32)
    tapes = rng.random((n, 64 if IDENTITY_DEPTH[cfg] <= 8 else 128), dtype=np.float32)
    tapes = np.minimum(tapes, np.float32(1.0 - 2 ** -24))
    cnt, _, ct, pth, _ = r.replay(1, list(tapes), cam, lgt)
    keep = np.nonzero(cnt == 1)[0]
    paths, contrib = pth[keep], ct[keep, 0]
    screen = np.ascontiguousarray(contrib["screen"], np.float32)
    ev = r.lens_eval(paths, screen, contrib["ss"], lens_sigma=0.01, max_derivative_depth=IDENTITY_DEPTH[cfg])
    sel = np.nonzero(ev["score"] > 0)[0]
    assert len(sel) > 50
    p0, c0 = r.perturb(paths[sel], np.zeros((len(sel), 24), np.float32))
    out, c2, s2 = r.lens_perturb(paths[sel], screen[sel], ev["pos"][sel])
    bad = 0
    for j, i in enumerate(sel):
        c, l = int(paths[i]["c"]), int(paths[i]["l"])
        nv = (l - 1 if l > 1 else 0) + c - 1
        good = bool(c2[j]["valid"]) and bool(c0[j]["valid"])
        good = good and np.array_equal(out[j]["tri"][:nv], p0[j]["tri"][:nv])
        if c >= 2:
            good = good and rel_err(c2[j]["ls"], c0[j]["ls"], 1e-20) < 1e-3
            good = good and np.allclose(c2[j]["rgb"], c0[j]["rgb"], rtol=1e-3, atol=1e-12)
            good = good and rel_err(s2[j], ev["score"][i], 1e-20) < 1e-3
        bad += 0 if good else 1
    assert bad <= max(2, len(sel) // 100), "%d / %d identity lens perturbations differ" % (bad, len(sel))
