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
