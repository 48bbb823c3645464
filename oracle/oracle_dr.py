"""ORACLE (test infrastructure): ctypes wrapper of oracle/_build/liboracle.so.

The oracle is the CPU restatement of the reference's hot path in oracle.cpp. It
is used by the tests as the checker and by bench.py as the timed CPU baseline;
the GPU product never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")
sys.path.insert(0, os.path.join(REPO, "drmlt-dpt_gb300"))

from drmlt import capi  # noqa: E402  (record layouts and option structs only; no GPU library load)
from drmlt import scene as dscene  # noqa: E402

_lib = None
V = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.check_call(["make", "-C", HERE, "-s"])
        l = C.CDLL(LIB)
        l.ora_create.restype = V
        l.ora_create.argtypes = [C.POINTER(capi.SceneDesc), C.POINTER(capi.Options)]
        l.ora_destroy.argtypes = [V]
        l.ora_perturb.argtypes = [V, V, V, C.c_int, V, V]
        l.ora_replay.argtypes = [V, C.c_int, V, V, C.c_int, C.c_int, V, V, C.c_int, V, V, V, V, V]
        l.ora_fd_derivs.argtypes = [V, V, V, C.c_int, C.c_double, V, V, V]
        l.ora_tape_derivs.argtypes = [V, V, V, C.c_int, V, V]
        l.ora_compute_gaussian.argtypes = [V, V, V, V, C.c_int, C.c_float, V, V, V, V]
        l.ora_trace_rays.argtypes = [V, V, V, C.c_float, C.c_float, C.c_int, C.c_int, V, V]
        l.ora_trace_rays_ex.argtypes = [V, V, V, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, V, V]
        l.ora_dr_run.restype = C.c_longlong
        l.ora_dr_run.argtypes = [V, C.c_int, C.c_int, C.c_longlong, C.c_double, C.c_int, C.c_uint64, V, V, V, V]
        _lib = l
    return _lib


def _p(a):
    return a.ctypes.data_as(V)


def default_options_py() -> capi.Options:
    """drmlt_options with the reference's DptOptions defaults (no GPU library needed)."""
    o = capi.Options()
    o.integrator, o.dr_type = 0, 0
    o.aniso_perturb_prob, o.aniso_perturb_stddev = 0.5, 0.0025
    o.perturb_stddev, o.large_step_prob, o.roughness_threshold = 0.01, 0.3, 0.03
    o.discrete_stddev, o.uniform_mixing_prob = 0.01, 0.2
    o.num_chains, o.num_init_samples, o.spp, o.direct_spp = 1024, 100000, 16, 16
    o.min_depth, o.max_depth, o.use_light_coordinate_sampling, o.max_derivative_depth = -1, -1, 1, 9
    o.seed = 0x1234ABCD
    return o


def options_from_scene(sd) -> capi.Options:
    d = sd.options
    o = default_options_py()
    o.dr_type = 1 if d.type == "mira" else 0
    o.aniso_perturb_prob = d.anisoPerturbProb
    o.aniso_perturb_stddev = d.anisoperturbstddev
    o.acceptance_map = int(d.acceptanceMap)
    o.perturb_stddev = d.perturbStdDev
    o.large_step_prob = d.largeStepProb
    o.roughness_threshold = d.roughnessThreshold
    o.discrete_stddev = d.discreteStdDev
    o.num_chains = d.numChains
    o.num_init_samples = d.numInitSamples
    o.spp = d.spp
    o.direct_spp = d.directSpp
    o.min_depth = d.minDepth
    o.max_depth = d.maxDepth
    o.use_light_coordinate_sampling = int(d.useLightCoordinateSampling)
    return o


class Oracle:
    def __init__(self, sd, options: capi.Options | None = None):
        self.scene = sd
        self.options = options or options_from_scene(sd)
        self._desc = dscene.SceneDescHolder(sd)
        self.h = lib().ora_create(C.byref(self._desc.desc), C.byref(self.options))

    def close(self):
        if self.h:
            lib().ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def perturb(self, paths, offsets):
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        off = np.ascontiguousarray(offsets, np.float32).reshape(n, capi.MAX_DIM)
        out = np.zeros(n, capi.PATH_DTYPE)
        ct = np.zeros(n, capi.CONTRIB_DTYPE)
        lib().ora_perturb(self.h, _p(paths), _p(off), n, _p(out), _p(ct))
        return out, ct

    def replay(self, mode, tapes, cam_len=None, lgt_len=None, max_contribs=64):
        n = len(tapes)
        stride = max(1, max(len(t) for t in tapes))
        T = np.zeros((n, stride), np.float32)
        lens = np.zeros(n, np.int32)
        for i, t in enumerate(tapes):
            T[i, :len(t)] = t
            lens[i] = len(t)
        mc = max_contribs if mode != 1 else 1
        cnt = np.zeros(n, np.int32)
        tech = np.zeros((n, mc, 2), np.int32)
        ct = np.zeros((n, mc), capi.CONTRIB_DTYPE)
        pth = np.zeros(n, capi.PATH_DTYPE)
        cons = np.zeros(n, np.int32)
        cl = np.ascontiguousarray(cam_len if cam_len is not None else np.zeros(n), np.int32)
        ll = np.ascontiguousarray(lgt_len if lgt_len is not None else np.zeros(n), np.int32)
        lib().ora_replay(self.h, mode, _p(T), _p(lens), stride, n, _p(cl), _p(ll), mc, _p(cnt), _p(tech), _p(ct),
                         _p(pth), _p(cons))
        return cnt, tech, ct, pth, cons

    def fd_derivs(self, paths, u, step=1e-4):
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        u = np.ascontiguousarray(u, np.float64).reshape(n, capi.MAX_DIM)
        f = np.zeros(n)
        g = np.zeros((n, capi.MAX_DIM))
        h = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM))
        lib().ora_fd_derivs(self.h, _p(paths), _p(u), n, step, _p(f), _p(g), _p(h))
        return f, g, h

    def tape_derivs(self, paths, u):
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        u = np.ascontiguousarray(u, np.float32).reshape(n, capi.MAX_DIM)
        g = np.zeros((n, capi.MAX_DIM), np.float32)
        h = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM), np.float32)
        lib().ora_tape_derivs(self.h, _p(paths), _p(u), n, _p(g), _p(h))
        return g, h

    def compute_gaussian(self, dims, ss, grad, hess):
        n = len(dims)
        dims = np.ascontiguousarray(dims, np.int32)
        ss = np.ascontiguousarray(ss, np.float32)
        grad = np.ascontiguousarray(grad, np.float32).reshape(n, capi.MAX_DIM)
        hess = np.ascontiguousarray(hess, np.float32).reshape(n, capi.MAX_DIM ** 2)
        mean = np.zeros((n, capi.MAX_DIM))
        ic = np.zeros((n, capi.MAX_DIM ** 2))
        cv = np.zeros((n, capi.MAX_DIM ** 2))
        ld = np.zeros(n)
        lib().ora_compute_gaussian(_p(dims), _p(ss), _p(grad), _p(hess), n, self.options.perturb_stddev, _p(mean),
                                   _p(ic), _p(cv), _p(ld))
        return mean, ic, cv, ld

    def trace_rays(self, org, dirs, tmin=1e-3, tmax=float("inf"), any_hit=False, mode="auto"):
        """Closest-hit (or any-hit) casts; mode "auto" (brute force below 1024
        triangles, the oracle's BVH above), "brute" or "bvh"."""
        org = np.ascontiguousarray(org, np.float32).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = len(org)
        tri = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        m = {"auto": 0, "brute": 1, "bvh": 2}[mode]
        lib().ora_trace_rays_ex(self.h, _p(org), _p(dirs), tmin, tmax, n, int(any_hit), m, _p(tri), _p(t))
        return tri, t

    def dr_run(self, num_chains, iterations, seconds=0.0, threads=None, num_init=None, seed=0x1234):
        threads = threads or os.cpu_count() or 1
        num_init = num_init or self.options.num_init_samples
        W, H = self.scene.width, self.scene.height
        film = np.zeros((H, W, 3), np.float32)
        stats = np.zeros(9, np.int64)
        el = C.c_double()
        b = C.c_float()
        n = lib().ora_dr_run(self.h, int(num_chains), int(num_init), int(iterations), float(seconds), int(threads),
                             int(seed), _p(film), _p(stats), C.byref(el), C.byref(b))
        return {"mutations": int(n), "seconds": el.value, "film": film, "stats": stats, "b": b.value}


class CpuChainLoop:
    """The oracle's DR chain loop on this host's threads over one scene, kept
    open so that several bounded samples share one scene set-up (and, on large
    scenes, one BVH build)."""

    def __init__(self, sd, threads: int | None = None, chains: int | None = None, num_init: int = 20000):
        self.threads = threads or os.cpu_count() or 1
        self.chains = chains or min(sd.options.numChains, 64 * self.threads)
        self.num_init = num_init
        self.oracle = Oracle(sd)
        self.seed = 0x1234

    def sample(self, seconds: float):
        self.seed += 1
        r = self.oracle.dr_run(self.chains, iterations=1 << 40, seconds=seconds, threads=self.threads,
                               num_init=self.num_init, seed=self.seed)
        return {"value": r["mutations"] / r["seconds"], "unit": "mutations/s", "cores": self.threads, "kind": "port",
                "sample": "%d chains, %.1f s of the chain loop (prepass of %d bootstrap paths excluded), %d mutations"
                          % (self.chains, r["seconds"], self.num_init, r["mutations"])}

    def close(self):
        self.oracle.close()


def cpu_throughput_scene(sd, seconds: float = 15.0, threads: int | None = None, chains: int | None = None):
    """Mutations/s of the oracle's DR chain loop on this host: a bounded sample of
    the workload (its scene, options and derivative path), prepass excluded."""
    loop = CpuChainLoop(sd, threads, chains)
    try:
        return loop.sample(seconds)
    finally:
        loop.close()


def cpu_throughput(xml: str, seconds: float = 15.0, threads: int | None = None, chains: int | None = None):
    """cpu_throughput_scene on a scene XML file."""
    return cpu_throughput_scene(dscene.load_scene(xml), seconds, threads, chains)
