"""Calibrates the CPU baseline: the reference's own DR chain loop (the `dpt`
binary built by this directory's Makefile) against the oracle's restatement of
it, on the same scene and the same host threads.

The reference prints no time for its chain loop alone, so it is measured as a
difference: two `dpt -d` renders of the config-2 scene (Phong Cornell box,
1024 x 1024, depth 8, 16384 chains, mira) that differ only in spp (1 and 3)
run the same prepass and direct-lighting pass, and their wall-time difference
is the chain loop of 2 x 1024 x 1024 mutations. The oracle's chain loop
(oracle/oracle_dr.py) then runs a bounded sample of the same scene on the same
number of threads. Prints one JSON line with both rates and their ratio.

Needs the reference sources (for the `dpt` build and its chad library); run
where they are, e.g.
    python oracle/ref/calibrate_cpu.py [threads]
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "drmlt-dpt_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from drmlt import scenegen  # noqa: E402

REF_OUT = os.path.join(REPO, "oracle", "_ref")
DPT = os.path.join(REF_OUT, "single", "dpt")
DEPTH = 8


def _scene(root: str, spp: int) -> str:
    return scenegen.write_cornell(root, seed=2, width=1024, height=1024, phong=True,
                                  options=scenegen.SceneOptions(maxdepth=DEPTH, numchains=16384, spp=spp,
                                                                type="mira"))


def _dpt_seconds(spp: int, threads: int, lib: str) -> float:
    tmp = tempfile.mkdtemp()
    try:
        xml = _scene(os.path.join(tmp, "s"), spp)
        wd = os.path.dirname(xml)
        shutil.copy(lib, wd)
        t0 = time.perf_counter()
        subprocess.run([DPT, os.path.basename(xml), "-d", "--z", "--p=%d" % threads,
                        "--max-derivatives-depth=%d" % DEPTH], cwd=wd, check=True, capture_output=True)
        return time.perf_counter() - t0
    finally:
        shutil.rmtree(tmp)


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    lib = os.path.join(REF_OUT, "single", "lib_d%d" % DEPTH, "pathlibbidir.so")
    if not (os.path.exists(DPT) and os.path.exists(lib)):
        sys.exit("build the reference first: make -C oracle/ref, and its depth-%d chad library "
                 "(tests/golden/make_golden.py cfg2)" % DEPTH)
    t1 = min(_dpt_seconds(1, threads, lib) for _ in range(2))
    t3 = min(_dpt_seconds(3, threads, lib) for _ in range(2))
    mut = 2 * 1024 * 1024
    ref_rate = mut / (t3 - t1)
    import oracle_dr
    tmp = tempfile.mkdtemp()
    try:
        port = oracle_dr.cpu_throughput(_scene(os.path.join(tmp, "s"), 1), seconds=15.0, threads=threads)
    finally:
        shutil.rmtree(tmp)
    print(json.dumps({"threads": threads, "dpt_spp1_s": round(t1, 3), "dpt_spp3_s": round(t3, 3),
                      "reference_loop_mutations_per_s": ref_rate, "port_mutations_per_s": port["value"],
                      "port_over_reference": port["value"] / ref_rate, "port_sample": port["sample"]}))


if __name__ == "__main__":
    main()
