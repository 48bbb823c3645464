"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference harness (oracle/ref/ref_harness.cpp, built from the
reference's own sources by oracle/ref/Makefile into oracle/_ref/) on the seeded
synthetic Cornell-box scenes of drmlt/scenegen.py and writes gzipped JSON lines:

  <cfg>_camera.jsonl.gz   the reference camera matrices and bounding sphere
  <cfg>_bidir.jsonl.gz    GeneratePathBidir: recorded uniform stream -> path + contributions
  <cfg>_subpath.jsonl.gz  GenerateSubpath (large step): stream + technique -> path + contribution
  <cfg>_direct.jsonl.gz   GeneratePath direct-lighting pass: stream + pixel -> contributions
  <cfg>_tech.jsonl.gz     technique paths with chad log f, gradient, Hessian,
                          ComputeGaussian output and PerturbPathBidir results
  <cfg>_accept.jsonl.gz   per-stage acceptances of one DR iteration from the
                          reference's own mutations on fixed states: LargeStep::Mutate
                          on a recorded stream, SmallStep::Mutate (both sigmas),
                          PH2MCSmallStep::Mutate, SmallStep::Trace (Green's y*), with
                          their offsets, and Green / Mira second-stage acceptances
  <cfg>_lens.jsonl.gz     the lens mutation of integrator=h2mc on technique paths:
                          lens scores, chad lens-mode log f / gradient / Hessian
                          w.r.t. the screen position, the 2-D Gaussian and
                          PerturbLensBidir results
  cfg3d_tech.jsonl.gz     technique paths of config 3 at max depth 10 with the FP64
                          chad library's log f, gradient and Hessian
  <cfg>_render*.json.gz   a full `dpt -d` render of the scene (the reference's
                          DRIntegrator::Render): its printed acceptance counters
                          and the final image averaged over 16 x 16 blocks
  cfgM_mesh.jsonl.gz      every shape of drmlt/scenegen.py:config_meshes as the
                          reference's ParseObj / LoadSerialized load it

usage (in a container that has the reference at /root/reference):
  python tests/golden/make_golden.py [--render] [cfg1] [cfg2]   (--render: only the renders)
  python tests/golden/make_golden.py --mesh                     (only cfgM_mesh)
  python tests/golden/make_golden.py --accept [cfg1] ...        (only the acceptance fixtures)
  python tests/golden/make_golden.py --lens [cfg1] ...          (only the lens-mutation fixtures)
  python tests/golden/make_golden.py --render-only cfg1 render_h2mc_lens   (named renders only)
  python tests/golden/make_golden.py --double                    (cfg3d_tech: FP64 chad, depth 10)
"""
from __future__ import annotations

import gzip
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "drmlt-dpt_gb300"))

from drmlt import scenegen  # noqa: E402

REF_DIR = os.path.join(REPO, "oracle", "_ref", "single")
HARNESS = os.path.join(REF_DIR, "ref_harness")
DPT = os.path.join(REF_DIR, "dpt")

CONFIGS = {
    # name: (scene writer, derivative depth, counts)
    "cfg1": (scenegen.config1, 5, dict(bidir=200, subpath=300, direct=200, tech=150, perturb=6)),
    "cfg2": (lambda d: scenegen.config2(d, "green"), 8, dict(bidir=100, subpath=200, direct=100, tech=100, perturb=6)),
    "cfg3": (lambda d: scenegen.config3(d), 5, dict(bidir=200, subpath=300, direct=200, tech=200, perturb=6)),
    "cfgL": (lambda d: scenegen.config_lights(d), 5, dict(bidir=200, subpath=300, direct=200, tech=200, perturb=6)),
    "cfgE": (lambda d: scenegen.config_env(d), 5, dict(bidir=200, subpath=300, direct=200, tech=250, perturb=6)),
}

# full renders: (output suffix, scene writer with the render's spp, derivative depth)
NO_LENS = {"lensperturbprob": "0"}  # h2mc / mcmc without the lens mutation (render_h2mc_lens has it)
RENDERS = {
    "cfg1": [("render", lambda d: scenegen.config1(d, spp=16), 5),
             ("render_h2mc", lambda d: scenegen.config1(d, spp=16, integrator="h2mc", extra=NO_LENS), 5),
             ("render_h2mc_lens", lambda d: scenegen.config1(d, spp=16, integrator="h2mc"), 5),
             ("render_mcmc", lambda d: scenegen.config1(d, spp=16, integrator="mcmc", extra=NO_LENS), 5),
             ("render_accmap", lambda d: scenegen.config1(d, spp=16, acceptance_map=True), 5)],
    "cfg3": [("render", lambda d: scenegen.config3(d, spp=16), 5)],
    "cfgL": [("render", lambda d: scenegen.config_lights(d, spp=16), 5)],
    "cfgE": [("render", lambda d: scenegen.config_env(d, spp=16), 5)],
    "cfg2": [("render_mira", lambda d: scenegen.config2(d, "mira", spp=1), 8),
             ("render_green", lambda d: scenegen.config2(d, "green", spp=1), 8)],
}


def read_pfm(path):
    import numpy as np
    with open(path, "rb") as f:
        magic = f.readline().strip()
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        ch = 3 if magic == b"PF" else 1
        data = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(h, w, ch)
    return data[::-1].astype(np.float64)


def _stats(log: str) -> dict:
    """The last 'Rendering Statistics' block. DRMLT (delayed.cpp:312-320) prints
    the H2MC ratio under the 'isotropic' label and vice versa; undone here.
    H2MC / MCMC (h2mc.cpp:139-149, mcmc.cpp:76-86) print large, small and lens."""
    block = log[log.rindex("Rendering Statistics"):]
    vals = [[float(a) if a not in ("nan", "-nan") else None, int(b)]
            for a, b in re.findall(r":\s*(-?nan|[-0-9.e]+)\s*\((\d+)\)", block)]
    if "First stage" in block:
        return dict(large=vals[0], stage1=vals[1], stage2_h2mc=vals[2], stage2_iso=vals[3])
    return dict(large=vals[0], small=vals[1], lens=vals[2])


def render(cfg: str, blocks: int = 16, only=None):
    import numpy as np
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"], stdout=subprocess.DEVNULL)
    for name, writer, depth in RENDERS[cfg]:
        if only and name not in only:
            continue
        tmp = tempfile.mkdtemp()
        try:
            xml = writer(os.path.join(tmp, "scene"))
            wd = os.path.dirname(xml)
            shutil.copy(os.path.join(REF_DIR, "lib_d%d" % depth, "pathlibbidir.so"), wd)
            out = subprocess.run([DPT, os.path.basename(xml), "-d", "--z", "--p=8", "--max-derivatives-depth=%d" % depth],
                                 cwd=wd, check=True, capture_output=True, text=True).stdout
            img = read_pfm(os.path.join(wd, "image.pfm"))
            H, W, _ = img.shape
            blk = img.reshape(blocks, H // blocks, blocks, W // blocks, 3).mean(axis=(1, 3))
            rec = dict(stats=_stats(out), mean=img.mean(axis=(0, 1)).tolist(), blocks=blk.round(8).tolist(),
                       width=W, height=H)
            dst = os.path.join(HERE, "%s_%s.json.gz" % (cfg, name))
            with open(dst, "wb") as raw:
                with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                    g.write(json.dumps(rec).encode())
            print(dst, rec["stats"], rec["mean"])
        finally:
            shutil.rmtree(tmp)


def run(cfg: str):
    writer, depth, n = CONFIGS[cfg]
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"], stdout=subprocess.DEVNULL)
    libdir = os.path.join(REF_DIR, "lib_d%d" % depth)
    os.makedirs(libdir, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        xml = writer(os.path.join(tmp, "scene"))
        jobs = [("camera", 0, 0, 0), ("bidir", 1, n["bidir"], 0), ("subpath", 1, n["subpath"], 0),
                ("direct", 1, n["direct"], 0), ("tech", 1, n["tech"], n["perturb"])]
        for mode, seed, count, extra in jobs:
            out = os.path.join(tmp, mode + ".jsonl")
            subprocess.check_call([HARNESS, xml, libdir, str(depth), out, mode, str(seed), str(count), str(extra)],
                                  stdout=subprocess.DEVNULL)
            dst = os.path.join(HERE, "%s_%s.jsonl.gz" % (cfg, mode))
            with open(out, "rb") as f, open(dst, "wb") as raw:
                with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                    shutil.copyfileobj(f, g)
            print(dst, os.path.getsize(dst))
    finally:
        shutil.rmtree(tmp)


ACCEPT_COUNT = 80


def accept(cfg: str):
    writer, depth, _ = CONFIGS[cfg]
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"], stdout=subprocess.DEVNULL)
    libdir = os.path.join(REF_DIR, "lib_d%d" % depth)
    os.makedirs(libdir, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        xml = writer(os.path.join(tmp, "scene"))
        out = os.path.join(tmp, "accept.jsonl")
        subprocess.check_call([HARNESS, xml, libdir, str(depth), out, "accept", "11", str(ACCEPT_COUNT), "0"],
                              stdout=subprocess.DEVNULL)
        dst = os.path.join(HERE, "%s_accept.jsonl.gz" % cfg)
        with open(out, "rb") as f, open(dst, "wb") as raw:
            with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                shutil.copyfileobj(f, g)
        print(dst, os.path.getsize(dst))
    finally:
        shutil.rmtree(tmp)


LENS_COUNT = 120
LENS_PERTURB = 4


def lens(cfg: str):
    """<cfg>_lens.jsonl.gz: the lens mutation of integrator=h2mc on technique
    paths -- lens scores, chad lens-mode derivatives, the 2-D Gaussian and
    PerturbLensBidir results (ref_harness mode lens)."""
    writer, depth, _ = CONFIGS[cfg]
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"], stdout=subprocess.DEVNULL)
    libdir = os.path.join(REF_DIR, "lib_d%d" % depth)
    os.makedirs(libdir, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        xml = writer(os.path.join(tmp, "scene"))
        out = os.path.join(tmp, "lens.jsonl")
        subprocess.check_call([HARNESS, xml, libdir, str(depth), out, "lens", "21", str(LENS_COUNT), str(LENS_PERTURB)],
                              stdout=subprocess.DEVNULL)
        dst = os.path.join(HERE, "%s_lens.jsonl.gz" % cfg)
        with open(out, "rb") as f, open(dst, "wb") as raw:
            with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                shutil.copyfileobj(f, g)
        print(dst, os.path.getsize(dst))
    finally:
        shutil.rmtree(tmp)


DEEP_COUNT = 240


def double_tech():
    """cfg3d_tech: technique paths of the depth-10 config-3 scene with the FP64
    chad library's log f, gradient and Hessian (the reference built with
    PREC=DOUBLE, commondef.h:54-60, chad.h:41-46) and central differences of
    that gradient."""
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "PREC=DOUBLE", "-j8"],
                          stdout=subprocess.DEVNULL)
    ref_double = os.path.join(REPO, "oracle", "_ref", "double")
    libdir = os.path.join(ref_double, "lib_d10")
    os.makedirs(libdir, exist_ok=True)
    tmp = tempfile.mkdtemp()
    try:
        xml = scenegen.config3_deep(os.path.join(tmp, "scene"))
        out = os.path.join(tmp, "tech.jsonl")
        subprocess.check_call([os.path.join(ref_double, "ref_harness"), xml, libdir, "10", out, "tech", "1",
                               str(DEEP_COUNT), "0"], stdout=subprocess.DEVNULL)
        dst = os.path.join(HERE, "cfg3d_tech.jsonl.gz")
        with open(out, "rb") as f, open(dst, "wb") as raw:
            with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                shutil.copyfileobj(f, g)
        print(dst, os.path.getsize(dst))
    finally:
        shutil.rmtree(tmp)


def mesh():
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"], stdout=subprocess.DEVNULL)
    tmp = tempfile.mkdtemp()
    try:
        xml = scenegen.config_meshes(os.path.join(tmp, "scene"))
        out = os.path.join(tmp, "mesh.jsonl")
        subprocess.check_call([HARNESS, xml, tmp, "5", out, "mesh", "0", "0"], stdout=subprocess.DEVNULL)
        dst = os.path.join(HERE, "cfgM_mesh.jsonl.gz")
        with open(out, "rb") as f, open(dst, "wb") as raw:
            with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as g:
                shutil.copyfileobj(f, g)
        print(dst, os.path.getsize(dst))
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--mesh" in args:
        mesh()
        sys.exit(0)
    if "--double" in args:
        double_tech()
        sys.exit(0)
    if "--lens" in args:
        for c in [a for a in args if not a.startswith("--")] or ["cfg1", "cfg3", "cfgL", "cfgE"]:
            lens(c)
        sys.exit(0)
    if "--accept" in args:
        for c in [a for a in args if not a.startswith("--")] or list(CONFIGS):
            accept(c)
        sys.exit(0)
    if "--render-only" in args:  # --render-only cfg name ...: single renders
        rest = [a for a in args if not a.startswith("--")]
        render(rest[0], only=set(rest[1:]))
        sys.exit(0)
    only_render = "--render" in args
    for c in [a for a in args if not a.startswith("--")] or ["cfg1"]:
        if not only_render:
            run(c)
        render(c)
