"""Per-stage acceptance probabilities against the reference's own mutation code.

Fixtures (tests/golden/<cfg>_accept.jsonl.gz, made by the reference harness
from the reference's LargeStep / SmallStep / PH2MCSmallStep objects on fixed
current states with recorded draws) hold, per state x: a large step on a
recorded uniform stream (src/mutation.cpp:7-120) with its a1; the isotropic
first stage y = PerturbPathBidir(x, o1) and its a1 (mutation.cpp:126-166); two
second stages from the same x -- isotropic z (mutation.cpp:167-208) and H2MC z
(drsmallstep.cpp:113-212) -- each with a2, the H2MC log-density ratio
log N_z(-o2) - log N_x(o2) (gaussian.cpp:18-34), Green's y* acceptance
(mutation.cpp:210-238), Mira's isotropic kernel ratio and the Green / Mira
second-stage acceptances (delayed.cpp:466-541).

The CUDA side evaluates the same quantities through drmlt_dr_eval and
drmlt_large_step_eval (the chain loop's own device code). Bars:
  * probabilities and scores: 1e-4 (relative for ss, absolute for values in
    [0, 1]);
  * the H2MC log ratio: 2e-3 absolute (the reference's Gaussians are FP32 Eigen
    eigensolves of FP32 Hessians, here FP64; the FP64 side is checked against
    the FP64 oracle in tests/test_gpu_oracle.py), a2 relative 2e-3;
  * a small fraction of states may take a different branch: the reference's
    perturbations jitter the discrete BSDF choice by N(0, 0.01)
    (PerturbPathBidir), the evaluation here does not, and a grazing ray can
    resolve differently in float vs double intersection. Each test bounds that
    fraction.
H2MC ratios are compared only where chad's derivatives are the derivatives of
the reference's own primal (not for light paths connected to the camera,
technique c = 1, nor for paths touching the environment light; see
tests/helpers.py:chad_env_defect and chad_hessian_consistent for the two
defects of the generated code).
"""
import numpy as np
import pytest

from helpers import golden, path_record, ss_rtol  # noqa: I001 (puts the package on sys.path)
from drmlt import capi

pytestmark = pytest.mark.gpu

CFGS = ["cfg1", "cfg3", "cfgL", "cfgE"]


def _need(cfg):
    g = golden(cfg, "accept")
    if g is None:
        pytest.skip("no golden fixture %s_accept" % cfg)
    return g


def _contrib(c):
    ct = np.zeros((), capi.CONTRIB_DTYPE)
    ct["screen"] = c["screen"]
    ct["rgb"] = c["contrib"]
    ct["ls"] = c["ls"]
    ct["ss"] = c["ss"]
    ct["valid"] = 1
    return ct


def _states(r, recs):
    paths, cts = [], []
    for rec in recs:
        p = rec["path"]
        c = rec["contrib"][0]
        paths.append(path_record(p, c["camDepth"], c["lightDepth"], r.scene.shape_first_tri, rec["pos"]))
        cts.append(_contrib(c))
    return np.array(paths), np.array(cts)


def _offsets(recs, key):
    o = np.zeros((len(recs), capi.MAX_DIM), np.float32)
    for i, rec in enumerate(recs):
        o[i, :rec["dim"]] = rec[key]["offset"]
    return o


def _close(a, b, tol):
    a, b = float(a), float(b)
    if np.isnan(a) or np.isnan(b):
        return np.isnan(a) and np.isnan(b)
    return abs(a - b) <= tol * max(1.0, abs(b))


def _rel(a, b, tol):
    a, b = float(a), float(b)
    return abs(a - b) <= tol * max(abs(b), 1e-30) or (a == 0 and b == 0)


@pytest.mark.parametrize("cfg", CFGS)
def test_large_step_acceptance(renderers, cfg):
    """LargeStep::Mutate on the reference's recorded stream: same proposal technique,
    contribution, uniforms consumed and first-stage acceptance a1."""
    recs = _need(cfg)
    r = renderers(cfg)
    x, xc = _states(r, recs)
    tapes = [rec["large"]["uniforms"] for rec in recs]
    lf = recs[0]["lengthFunc"]
    assert all(rec["lengthFunc"] == lf for rec in recs)
    a1, tech, ct, cons = r.large_step_eval(tapes, x, xc, lf)
    bad, nvalid = [], 0
    for i, rec in enumerate(recs):
        L = rec["large"]
        good = cons[i] == L["consumed"] and _close(a1[i], L["a1"], 1e-4)
        if L["contribs"]:
            c = L["contribs"][0]
            good = good and (tech[i, 0], tech[i, 1]) == (c["camDepth"], c["lightDepth"])
            good = good and _rel(ct[i]["ss"], c["ss"], 1e-4) and _rel(ct[i]["ls"], c["ls"], 1e-4)
            nvalid += 1
        else:
            good = good and (tech[i, 0], tech[i, 1]) == (0, 0)
        if not good:
            bad.append((i, float(a1[i]), L["a1"], int(cons[i]), L["consumed"]))
    assert nvalid >= 5  # proposals that contribute (9 of 80 on the environment scene, 22-25 elsewhere)
    assert len(bad) <= max(1, len(recs) // 40), "%d / %d large steps differ: %s" % (len(bad), len(recs), bad[:5])


def _dr(r, recs, kind):
    x, xc = _states(r, recs)
    o1 = _offsets(recs, "small")
    o2 = _offsets(recs, kind)
    an = np.full(len(recs), 1 if kind == "h2mc" else 0, np.int32)
    return r.dr_eval(x, xc, o1, o2, an)


@pytest.mark.parametrize("cfg", CFGS)
def test_first_stage_acceptance(renderers, cfg):
    """SmallStep::Mutate (sigma1): the perturbed state y, its validity, ss(y) and a1."""
    recs = _need(cfg)
    r = renderers(cfg)
    out, y, _ = _dr(r, recs, "iso")
    bad, nvalid = [], 0
    for i, rec in enumerate(recs):
        s = rec["small"]
        dim = rec["dim"]
        good = np.allclose(y[i]["u"][:dim], s["ypos"], atol=2e-6)
        good = good and bool(out[i]["valid_y"]) == bool(s["valid"])
        if good and s["valid"]:
            nvalid += 1
            good = _rel(out[i]["ss_y"], s["ss"], ss_rtol(rec["path"]))
        good = good and _close(out[i]["a1"], s["a1"], 1e-4)
        if not good:
            bad.append((i, float(out[i]["a1"]), s["a1"], float(out[i]["ss_y"]), s["ss"]))
    assert nvalid >= len(recs) // 4
    assert len(bad) <= max(1, len(recs) // 40), "%d / %d first stages differ: %s" % (len(bad), len(recs), bad[:5])


@pytest.mark.parametrize("cfg", CFGS)
def test_isotropic_second_stage_acceptance(renderers, cfg):
    """Isotropic second stage (sigma2): a2, Green's y* acceptance and alpha2, Mira's
    kernel ratio Q1(z, y) / Q1(x, y) (FP64 log domain here) and alpha2."""
    recs = _need(cfg)
    r = renderers(cfg)
    out, _, z = _dr(r, recs, "iso")
    bad, nvalid, nstar, nmira = [], 0, 0, 0
    for i, rec in enumerate(recs):
        s = rec["iso"]
        dim = rec["dim"]
        o = out[i]
        good = np.allclose(z[i]["u"][:dim], s["zpos"], atol=2e-6)
        good = good and bool(o["valid_z"]) == bool(s["valid"])
        good = good and _close(o["a2"], s["a2"], 1e-4)
        if s["valid"]:
            nvalid += 1
            good = good and _rel(o["ss_z"], s["ss"], ss_rtol(rec["path"]))
            good = good and _close(o["a_star_green"], s["aStar"], 1e-4)
            nstar += 0 < s["aStar"] < 1
        good = good and _close(o["alpha2_green"], s["alphaGreen"], 1e-4)
        good = good and _close(o["alpha2_mira"], s["alphaMira"], 1e-4)
        if s["transRatio"] > 0:
            nmira += 1
            good = good and _rel(np.exp(o["log_q_mira"]), s["transRatio"], 1e-4)
        if not good:
            bad.append((i, [float(o[k]) for k in ("a2", "a_star_green", "alpha2_green", "alpha2_mira")],
                        [s[k] for k in ("a2", "aStar", "alphaGreen", "alphaMira")]))
    assert nvalid >= len(recs) // 4 and nmira > 0
    assert len(bad) <= max(1, len(recs) // 40), "%d / %d iso second stages differ: %s" % (len(bad), len(recs),
                                                                                         bad[:5])


def _chad_exact(rec, sd):
    """Techniques whose chad derivatives are those of the reference's primal
    (see the module docstring)."""
    c = rec["contrib"][0]
    if c["camDepth"] == 1:
        return False
    from helpers import env_light_index
    env = env_light_index(sd)
    if env < 0:
        return True
    p = rec["path"]
    escapes = c["lightDepth"] == 0 and p["camSurf"] and p["camSurf"][c["camDepth"] - 2]["shape"] < 0
    return not escapes and p["lgtLight"] != env and all(v.get("dlLight", -1) != env for v in p["camSurf"])


@pytest.mark.parametrize("cfg", CFGS)
def test_h2mc_second_stage_acceptance(renderers, cfg):
    """PH2MCSmallStep::Mutate: z for the reference's offset, the Gaussian log-density
    ratio log N_z(-o) - log N_x(o), the unclamped a2 = exp(ratio) ss(z) / ss(x), and
    the Green / Mira second-stage acceptances built on it."""
    recs = _need(cfg)
    r = renderers(cfg)
    out, _, z = _dr(r, recs, "h2mc")
    bad, n_cmp, n_aniso = [], 0, 0
    for i, rec in enumerate(recs):
        s = rec["h2mc"]
        dim = rec["dim"]
        o = out[i]
        good = np.allclose(z[i]["u"][:dim], s["zpos"], atol=2e-6)
        good = good and bool(o["valid_z"]) == bool(s["valid"])
        if good and s["valid"] and _chad_exact(rec, r.scene):
            n_cmp += 1
            n_aniso += s["logRatio"] != 0
            good = abs(o["log_ratio"] - s["logRatio"]) <= 2e-3
            good = good and _rel(o["a2"], s["a2"], 2e-3)
            good = good and _close(o["alpha2_green"], s["alphaGreen"], 2e-3)
            good = good and _close(o["alpha2_mira"], s["alphaMira"], 2e-3)
        if not good:
            bad.append((i, float(o["log_ratio"]), s["logRatio"], float(o["a2"]), s["a2"]))
    assert n_cmp >= 10 and n_aniso > 0
    assert len(bad) <= max(2, len(recs) // 20), "%d / %d H2MC second stages differ: %s" % (len(bad), len(recs),
                                                                                          bad[:5])
