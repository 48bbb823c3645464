"""The lens-mutation fixtures of the reference (tests/golden/<cfg>_lens.jsonl.gz),
checked on the CPU: the properties of the reference that the CUDA lens code
mirrors, and the 2-D ComputeGaussian (src/integrators/h2mc.cpp:14-83,
607-640) restated in numpy against the reference's Eigen output.

* chad's lens-mode log f is log lensScore on every technique but (3, 1), where
  the AD DirectLighting keeps x2's adjoint factor in a local copy
  (src/path.cpp:2857-2868): there log f - log lensScore is that factor's
  negative log, so the two differ; and but light paths connected to the
  camera (c = 1) through a smooth-shaded vertex, where the lens-mode
  function takes PerturbLensLastVertex's shading-normal factor with wi and wo
  swapped (src/path.cpp:1862-1866) against the sampler's score (on the flat
  Cornell box, cfg1, the two agree for c = 1 as well).
* PerturbLensBidir puts the camera subpath of c >= 2 at the requested screen
  position.
"""
import math

import numpy as np
import pytest

from helpers import chad_env_defect, env_light_index, golden, scene_xml

CFGS = ["cfg1", "cfg3", "cfgL", "cfgE"]
L = math.pi / 2.0


def _need(cfg):
    g = golden(cfg, "lens")
    if g is None:
        pytest.skip("no golden fixture %s_lens" % cfg)
    return g


def lens_gaussian(sigma, ss, g, h):
    """ComputeGaussian for dimension 2 in FP64 (mean, inverse covariance, log det)."""
    f32 = np.float32
    pos_scale = float(f32(0.5) * (f32(math.exp(L)) - f32(math.exp(-L))) * f32(0.5) * (f32(math.exp(L)) - f32(math.exp(-L))))
    pos_off = float(f32(0.5) * (f32(math.exp(L)) + f32(math.exp(-L)) - f32(1.0)))
    neg_scale = float(f32(math.sin(L)) * f32(math.sin(L)))
    neg_off = float(-(f32(math.cos(L)) - f32(1.0)))
    inv = 1.0 / (sigma * sigma)
    H = np.array(h, np.float64).reshape(2, 2)
    if ss <= 1e-15 or np.linalg.norm(H) < 0.5 / (sigma * sigma):
        return np.zeros(2), np.eye(2) * inv, 2.0 * math.log(inv)
    A = np.array([[H[0, 0], H[0, 1]], [H[0, 1], H[1, 1]]])  # the upper triangle, as the solver reads it
    lam, V = np.linalg.eigh(A)
    p = np.zeros(2)
    mc = np.zeros(2)
    for k in range(2):
        vg = V[:, k] @ np.array(g, np.float64)
        eb = 1.0 / abs(lam[k]) if abs(lam[k]) > 1e-10 else 0.0
        ob = eb * vg
        if abs(lam[k]) > 1e-10:
            s2, o = (pos_scale, ob * pos_off) if lam[k] > 0 else (neg_scale, ob * neg_off)
        else:
            s2, o = L * L, 0.5 * ob * L * L
        eb *= s2
        eb = 1.0 / eb if eb > 1e-10 else 0.0
        p[k] = eb + inv
        mc[k] = eb / p[k] * o
    return V @ mc, V @ np.diag(p) @ V.T, float(np.log(p).sum())


@pytest.mark.parametrize("cfg", CFGS)
def test_chad_lens_function_is_log_lens_score_but_on_direct_lighting_at_x2(cfg, scene_root):
    """(Paths emitted by the environment light in the half of its disc where
    the generated SampleConcentricDisc takes another branch have no chad
    reference: helpers.chad_env_defect.)"""
    from drmlt import scene as dscene
    recs = _need(cfg)
    env = env_light_index(dscene.load_scene(scene_xml(cfg, scene_root)))
    same = differ = 0
    for r in recs:
        ls = r["contrib"][0]["lens"]
        if not (r["haveDerv"] and ls > 1e-15):
            continue
        p = r["path"]
        if p["lgtDepth"] >= 2 and p["lgtLight"] == env and chad_env_defect(r, env):
            continue
        d = abs(r["logf"] - math.log(ls))
        if (r["path"]["camDepth"], r["path"]["lgtDepth"]) == (3, 1):
            differ += d > 1e-2
        elif r["path"]["camDepth"] == 1 and cfg != "cfg1":
            continue
        else:
            assert d < 1e-4 * max(1.0, abs(r["logf"])), (r["path"]["camDepth"], r["path"]["lgtDepth"], d)
            same += 1
    assert same > 50 and differ > 0


@pytest.mark.parametrize("cfg", CFGS)
def test_lens_perturbation_lands_on_the_requested_screen_position(cfg):
    recs = _need(cfg)
    n = 0
    for r in recs:
        if r["path"]["camDepth"] < 2:
            continue
        for pt in r["perturb"]:
            if pt["contribs"]:
                assert np.allclose(pt["contribs"][0]["screen"], pt["screen"], atol=1e-6)
                n += 1
    assert n > 100


@pytest.mark.parametrize("cfg", CFGS)
def test_two_dimensional_gaussian_restated(cfg):
    """The restated 2-D ComputeGaussian against the reference's (FP32 Eigen):
    mean, inverse covariance and log det within 1e-3 relative."""
    recs = _need(cfg)
    aniso = 0
    # sigma is the scene's lensPerturbStdDev: read back from an isotropic record
    iso = [x for x in recs if x["gauss"]["mean"] == [0, 0] and x["gauss"]["invCov"][1] == 0]
    sigma = math.sqrt(1.0 / iso[0]["gauss"]["invCov"][0])
    for r in recs:
        if not r["haveDerv"]:
            continue
        mean, ic, ld = lens_gaussian(sigma, r["contrib"][0]["ss"], r["grad"], r["hess"])
        g = r["gauss"]
        ric = np.array(g["invCov"]).reshape(2, 2)
        assert np.abs(ic - ric).max() <= 1e-3 * np.abs(ric).max()
        assert np.abs(mean - np.array(g["mean"])).max() <= 1e-3 * max(np.abs(g["mean"]).max(), 1e-8) + 1e-12
        assert abs(ld - g["logDet"]) <= 1e-3 * max(1.0, abs(g["logDet"]))
        aniso += g["mean"] != [0, 0]
    assert aniso > 3
