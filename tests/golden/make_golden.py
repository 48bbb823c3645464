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

usage (in a container that has the reference at /root/reference):
  python tests/golden/make_golden.py [cfg1] [cfg2]
"""
from __future__ import annotations

import gzip
import os
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

CONFIGS = {
    # name: (scene writer, derivative depth, counts)
    "cfg1": (scenegen.config1, 5, dict(bidir=200, subpath=300, direct=200, tech=150, perturb=6)),
    "cfg2": (lambda d: scenegen.config2(d, "green"), 8, dict(bidir=100, subpath=200, direct=100, tech=100, perturb=6)),
}


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


if __name__ == "__main__":
    for c in (sys.argv[1:] or ["cfg1"]):
        run(c)
