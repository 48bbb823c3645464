"""Builds libdrmlt.so in-tree for sm_103a (nvcc: the chain-loop translation unit, the
persistent-schedule translation unit, the path-derivative translation unit, the host
BVH builder and the host image writer, compiled in parallel as relocatable device code
and device-linked into the library).

usage: python drmlt-dpt_gb300/build.py [--force]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libdrmlt.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I" + os.path.join(REPO, "include")]
# The derivative kernel is instruction-fetch bound on its long hyper-dual code;
# fast-math intrinsics keep the transcendental calls short. Its outputs are
# derivatives (checked to 1e-3) and never a path contribution. The persistent
# kernel (persist.cu, compiled without fast math like the path code) calls the
# same derivative code compiled with the same flags in derivs_dev.cu: those two
# are relocatable device code (device-linked into the library), held to the
# 128 registers of the kernel; the other translation units are whole-program
# code (relocatable code changes their register allocation: k_gauss 56 -> 95).
FAST = ["--use_fast_math"]
TU_FLAGS = {"derivs.cu": FAST, "derivs_dev.cu": FAST + ["-rdc=true", "-maxrregcount=128"],
            "persist.cu": ["-rdc=true"]}
SOURCES = ("drmlt.cu", "persist.cu", "derivs.cu", "derivs_dev.cu", "bvh.cpp", "image_io.cpp")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [os.path.join(REPO, "include", "drmlt_capi.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objs = []
    jobs = []
    for src in SOURCES:
        obj = os.path.join(LIBDIR, src + ".o")
        cmd = [NVCC] + ARCH + FLAGS + TU_FLAGS.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [NVCC] + ARCH + FLAGS + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
        objs.append(obj)
    for j in jobs:
        out, _ = j.communicate()
        if j.returncode != 0:
            sys.stderr.write(out.decode())
            raise RuntimeError("nvcc failed")
        if verbose:
            sys.stderr.write(out.decode())
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        sys.stderr.write(r.stdout.decode())
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
