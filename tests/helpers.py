"""Shared test helpers: golden fixtures, scenes and record conversion."""
from __future__ import annotations

import functools
import gzip
import json
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "drmlt-dpt_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

from drmlt import capi, scenegen  # noqa: E402
from drmlt import scene as dscene  # noqa: E402

SCENE_WRITERS = {
    "cfg1": scenegen.config1,
    "cfg2": lambda d: scenegen.config2(d, "green"),
    "cfg3": lambda d: scenegen.config3(d),
    "cfgL": lambda d: scenegen.config_lights(d),
    "cfgE": lambda d: scenegen.config_env(d),
    "cfg4s": lambda d: scenegen.config4_small(d),
    "cfg3d": lambda d: scenegen.config3_deep(d),
}


@functools.lru_cache(maxsize=None)
def golden(cfg: str, mode: str):
    path = os.path.join(GOLDEN, "%s_%s.jsonl.gz" % (cfg, mode))
    if not os.path.exists(path):
        return None
    with gzip.open(path, "rt") as f:
        return [json.loads(line) for line in f]


_SCENE_CACHE = {}


def scene_xml(cfg: str, tmp_root: str) -> str:
    if cfg not in _SCENE_CACHE:
        _SCENE_CACHE[cfg] = SCENE_WRITERS[cfg](os.path.join(tmp_root, cfg))
    return _SCENE_CACHE[cfg]


def path_u(p: dict, c: int, l: int) -> list:
    """GetPathPos (src/path.cpp:2393-2439) of a reference path dump for technique (c, l)."""
    nl = l - 1 if l > 1 else 0
    nc = c - 1
    u = []
    if l > 1:
        u += p["lgtPos"] + p["lgtDir"]
        for i in range(nl - 1):
            u += p["lgtSurf"][i]["bsdfRnd"]
    if c > 1:
        u += p["screen"]
        for i in range(nc - 1):
            u += p["camSurf"][i]["bsdfRnd"]
        if l == 1:
            u += p["camSurf"][nc - 1]["dlRnd"]
    return u


def path_record(p: dict, c: int, l: int, first_tri: np.ndarray, u=None) -> np.ndarray:
    """A reference path dump as a drmlt_path record for technique (c, l)."""
    rec = np.zeros((), capi.PATH_DTYPE)
    nl = l - 1 if l > 1 else 0
    nc = c - 1
    rec["c"], rec["l"] = c, l
    rec["lgt_light"], rec["lgt_prim"] = p["lgtLight"], p["lgtPrim"]
    last = p["camSurf"][nc - 1] if nc > 0 else None
    rec["dl_light"] = last["dlLight"] if last else -1
    rec["dl_prim"] = last["dlPrim"] if last else -1
    verts = p["lgtSurf"][:nl] + p["camSurf"][:nc]
    use_abs = 0
    for i, v in enumerate(verts):
        rec["tri"][i] = first_tri[v["shape"]] + v["prim"] if v["shape"] >= 0 else -1
        rec["disc"][i] = v["disc"]
        rec["rr"][i] = v["rr"] if v["rr"] is not None else 0.0
        if v["useAbs"]:
            use_abs |= 1 << i
    rec["use_abs"] = use_abs
    uu = path_u(p, c, l) if u is None else u
    rec["u"][:len(uu)] = uu
    return rec


def rel_err(a, b, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def ss_rtol(p: dict, base: float = 1e-4) -> float:
    """Tolerance for a contribution's ss score (ls times the primary-sample
    Jacobian). An absolute-parameter vertex contributes |sin(pi u1)| of its
    direction's spherical coordinates (src/path.cpp:623-642); near the poles
    that factor amplifies the last-ulp differences of a float direction by
    about 1 / sin^2, so the tolerance widens with it."""
    s = [abs(np.sin(np.pi * v["bsdfRnd"][1])) for v in p["lgtSurf"] + p["camSurf"] if v["useAbs"]]
    m = min(s) if s else 1.0
    return max(base, 1e-6 / max(m * m, 1e-12))


def env_light_index(sd) -> int:
    for i, L in enumerate(sd.lights):
        if L.type == capi.LIGHT_ENV:
            return i
    return -1


def chad_env_defect(rec: dict, env: int) -> bool:
    """Technique paths where the chad-generated function is not the reference's
    own primal on the environment light, so chad's f and derivatives are not
    a reference for them:
      * paths ending on the environment light whose chad log f differs from
        the log of the reference's primal ss score: EmissionEnvLight
        (src/envlight.cpp:330-357) takes the cell coordinates of the wrapped
        pixel index, which are off by the image width or height wherever the
        unwrapped column or row is negative;
      * paths emitted by the environment light whose disc sample falls in the
        |2 u0 - 1| > |2 u1 - 1| half: the generated SampleConcentricDisc
        (src/sampling.h:70-97) evaluates its last branch there.
    """
    p = rec["path"]
    if env < 0:
        return False
    if p["lgtDepth"] == 0 and p["camSurf"] and p["camSurf"][-1]["shape"] < 0:
        lf = rec["logf"]
        return lf is None or abs(lf - np.log(rec["contrib"][0]["ss"])) > 1e-4 * max(1.0, abs(lf))
    if p["lgtDepth"] >= 2 and p["lgtLight"] == env:
        r1, r2 = 2.0 * p["lgtPos"][0] - 1.0, 2.0 * p["lgtPos"][1] - 1.0
        return r1 != 0.0 and r2 != 0.0 and r1 * r1 > r2 * r2
    return False


def chad_hessian_consistent(rec: dict) -> bool:
    """Whether chad's Hessian is the derivative of chad's own gradient: within
    2% of the central differences of that gradient (fixture field `fdHess`,
    h = 1e-3, itself accurate to a few 0.1%) and symmetric to 1e-3. It is not
    for light paths connected to the camera (c = 1), for some rough-dielectric
    paths, and on the direction rows of some environment-emitted paths."""
    d = rec["dim"]
    hr = np.array(rec["hess"]).reshape(d, d)
    hfd = np.array(rec["fdHess"]).reshape(d, d)
    top = max(np.max(np.abs(hfd)), 1e-6)
    return (rec["path"]["camDepth"] != 1 and np.max(np.abs(hr - hfd)) <= 2e-2 * top
            and np.max(np.abs(hr - hr.T)) <= 1e-3 * max(np.max(np.abs(hr)), 1e-6))
