"""Host-side integrator surface over libdrmlt.so.

Mirrors the reference's plugin interface: ``Integrator`` with ``Render()`` and
``PrePass()`` (src/integrator.h:9-22), constructed from a parsed scene, with
``output_name`` / ``verbose`` / ``deterministic`` attributes, dispatched on the
scene's ``integrator`` option like main() (src/main.cpp:104-120). The work runs
on the GPU through the C ABI; this module only marshals arguments.
"""
from __future__ import annotations

import os
import time

import ctypes as C

import numpy as np

from . import capi
from .scene import SceneData, SceneDescHolder, load_scene

_INTEGRATORS = {"drmlt": capi.INTEGRATOR_DRMLT, "h2mc": capi.INTEGRATOR_H2MC, "mcmc": capi.INTEGRATOR_MCMC}


def make_options(sd: SceneData, *, seed: int = 0x1234ABCD, device: int = 0,
                 max_derivative_depth: int = 9, **override) -> capi.Options:
    """drmlt_options from the scene's <dpt> block (unknown DR type -> green, delayed.cpp:352-362)."""
    o = capi.default_options()
    d = sd.options
    if d.integrator not in _INTEGRATORS:
        raise ValueError("Unknown integrator %r" % d.integrator)
    o.integrator = _INTEGRATORS[d.integrator]
    # mcmc's SmallStep never proposes a lens mutation (mutation.cpp:126-166); only
    # H2MCSmallStep does (h2mc.cpp:466-532): the options are read for integrator=h2mc
    o.lens_perturb_prob = d.lensPerturbProb
    o.lens_perturb_stddev = d.lensPerturbStdDev
    o.dr_type = capi.DR_MIRA if d.type == "mira" else capi.DR_GREEN
    o.aniso_perturb_prob = d.anisoPerturbProb
    o.aniso_perturb_stddev = d.anisoperturbstddev
    o.acceptance_map = int(d.acceptanceMap)
    o.perturb_stddev = d.perturbStdDev
    o.large_step_prob = d.largeStepProb
    o.roughness_threshold = d.roughnessThreshold
    o.discrete_stddev = d.discreteStdDev
    o.uniform_mixing_prob = d.uniformMixingProbability
    o.num_chains = d.numChains
    o.num_init_samples = d.numInitSamples
    o.spp = d.spp
    o.direct_spp = d.directSpp
    o.min_depth = d.minDepth
    o.max_depth = d.maxDepth
    o.seed_offset = d.seedOffset
    o.use_light_coordinate_sampling = int(d.useLightCoordinateSampling)
    o.max_derivative_depth = max_derivative_depth
    o.seed = (seed + d.seedOffset) & 0xFFFFFFFFFFFFFFFF
    o.device = device
    for k, v in override.items():
        setattr(o, k, v)
    return o


class Renderer:
    """Owns one libdrmlt handle (scene on the device + chain state + film)."""

    def __init__(self, sd: SceneData, options: capi.Options | None = None, **kw):
        self.scene = sd
        self.options = options if options is not None else make_options(sd, **kw)
        self._desc = SceneDescHolder(sd)
        h = C.c_void_p()
        capi.check(capi.lib().drmlt_create(C.byref(self._desc.desc), C.byref(self.options), C.byref(h)))
        self.handle = h
        self.b = None

    def close(self):
        if self.handle:
            capi.lib().drmlt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def prepass(self) -> float:
        b = C.c_float()
        capi.check(capi.lib().drmlt_prepass(self.handle, C.byref(b)))
        self.b = b.value
        return self.b

    def direct(self):
        capi.check(capi.lib().drmlt_direct(self.handle))

    def run(self, iterations: int) -> int:
        done = C.c_int64()
        capi.check(capi.lib().drmlt_run(self.handle, int(iterations), C.byref(done)))
        return done.value

    def run_async(self, iterations: int, slot: int) -> int:
        """drmlt_run_async: enqueues the iterations and a copy of the statistics
        into pinned slot `slot` (0 or 1) without waiting; returns the mutations."""
        done = C.c_int64()
        capi.check(capi.lib().drmlt_run_async(self.handle, int(iterations), int(slot), C.byref(done)))
        return done.value

    def wait_stats(self, slot: int) -> dict:
        """drmlt_wait_stats: the statistics copied by the run_async call on `slot`."""
        s = capi.Stats()
        capi.check(capi.lib().drmlt_wait_stats(self.handle, int(slot), C.byref(s)))
        return {k: getattr(s, k) for k, _ in capi.Stats._fields_}

    def render(self):
        capi.check(capi.lib().drmlt_render(self.handle))

    def last_run_ms(self) -> float:
        ms = C.c_float()
        capi.check(capi.lib().drmlt_last_run_ms(self.handle, C.byref(ms)))
        return ms.value

    def kernel_launches(self) -> int:
        n = C.c_int64()
        capi.check(capi.lib().drmlt_kernel_launches(self.handle, C.byref(n)))
        return n.value

    def autotune(self, iterations_per_candidate: int = 8):
        """drmlt_autotune: (chains per warp, derivative warps) it settled on."""
        lanes, warps = C.c_int(), C.c_int()
        capi.check(capi.lib().drmlt_autotune(self.handle, int(iterations_per_candidate), C.byref(lanes),
                                             C.byref(warps)))
        return lanes.value, warps.value

    RAY_KINDS = ("primary", "bounce", "shadow")

    def ray_benchmark(self, kind: str, n_rays: int = 1 << 20, repeats: int = 10) -> dict:
        """drmlt_ray_benchmark: ms per pass, rays traced, nodes fetched, triangles tested."""
        ms = C.c_float()
        counts = np.zeros(3, np.float64)
        capi.check(capi.lib().drmlt_ray_benchmark(self.handle, self.RAY_KINDS.index(kind), int(n_rays), int(repeats),
                                                  C.byref(ms), counts.ctypes.data))
        return {"ms": ms.value, "rays": counts[0], "nodes": counts[1], "tris": counts[2]}

    def launch_shape(self) -> dict:
        """drmlt_get_launch_shape: the shape the next run uses."""
        v = [C.c_int() for _ in range(4)]
        capi.check(capi.lib().drmlt_get_launch_shape(self.handle, *(C.byref(x) for x in v)))
        shape = dict(zip(("chains_per_warp", "stage2_chains_per_warp", "derivative_warps", "graph_iterations"),
                         (x.value for x in v)))
        w = C.c_int()
        capi.check(capi.lib().drmlt_get_wavefront(self.handle, C.byref(w)))
        shape["wavefront"] = w.value
        hc, hl = C.c_int(), C.c_int()
        capi.check(capi.lib().drmlt_get_head_tier(self.handle, C.byref(hc), C.byref(hl)))
        shape["head_chains"] = hc.value
        shape["head_lanes"] = hl.value
        a = C.c_int()
        capi.check(capi.lib().drmlt_get_adjoint_min_dim(self.handle, C.byref(a)))
        shape["adjoint_min_dim"] = a.value
        return shape

    def fma_benchmark(self, fp64: bool = False, iterations: int | None = None) -> dict:
        """drmlt_fma_benchmark: the device's FP32 or FP64 FMA throughput."""
        ms, flops = C.c_float(), C.c_double()
        it = iterations or (4000 if fp64 else 200000)
        capi.check(capi.lib().drmlt_fma_benchmark(self.handle, int(fp64), int(it), C.byref(ms), C.byref(flops)))
        return {"ms": ms.value, "flops": flops.value, "tflops": flops.value / (ms.value * 1e-3) / 1e12}

    STAGES = ("stage1", "derivs_x", "gauss_x", "stage2", "derivs_z", "gauss_z", "finish")

    def profile(self, iterations: int):
        ms = np.zeros(len(self.STAGES), np.float32)
        done = C.c_int64()
        capi.check(capi.lib().drmlt_profile(self.handle, int(iterations), capi.ptr(ms), C.byref(done)))
        return dict(zip(self.STAGES, ms.tolist())), done.value

    def total_iterations(self) -> int:
        n = C.c_int64()
        capi.check(capi.lib().drmlt_total_iterations(self.handle, C.byref(n)))
        return n.value

    def film(self) -> np.ndarray:
        out = np.zeros((self.scene.height, self.scene.width, 3), np.float32)
        capi.check(capi.lib().drmlt_get_film(self.handle, capi.ptr(out)))
        return out

    def partial_film(self) -> np.ndarray:
        """The indirect film scaled by pixels / mutations so far (the reference's
        intermediate images, delayed.cpp:612-637)."""
        out = np.zeros((self.scene.height, self.scene.width, 3), np.float32)
        capi.check(capi.lib().drmlt_get_partial_film(self.handle, capi.ptr(out)))
        return out

    def stats(self) -> dict:
        s = capi.Stats()
        capi.check(capi.lib().drmlt_get_stats(self.handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in capi.Stats._fields_}

    # ---- per-path entry points
    def path_eval(self, paths: np.ndarray, u: np.ndarray) -> np.ndarray:
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        u = np.ascontiguousarray(u, np.float32).reshape(len(paths), capi.MAX_DIM)
        out = np.zeros(len(paths), np.float32)
        capi.check(capi.lib().drmlt_path_eval(self.handle, capi.ptr(paths), capi.ptr(u), len(paths), capi.ptr(out)))
        return out

    def path_grad_hess(self, paths: np.ndarray, u: np.ndarray):
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        u = np.ascontiguousarray(u, np.float32).reshape(n, capi.MAX_DIM)
        g = np.zeros((n, capi.MAX_DIM), np.float32)
        h = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM), np.float32)
        capi.check(capi.lib().drmlt_path_grad_hess(self.handle, capi.ptr(paths), capi.ptr(u), n, capi.ptr(g),
                                                    capi.ptr(h)))
        return g, h

    def path_adjoint(self, paths: np.ndarray, u: np.ndarray):
        """Gradient and Hessian of log f by the reverse-mode adjoint (drmlt_path_adjoint)."""
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        u = np.ascontiguousarray(u, np.float32).reshape(n, capi.MAX_DIM)
        g = np.zeros((n, capi.MAX_DIM), np.float32)
        h = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM), np.float32)
        capi.check(capi.lib().drmlt_path_adjoint(self.handle, capi.ptr(paths), capi.ptr(u), n, capi.ptr(g),
                                                  capi.ptr(h)))
        return g, h

    def perturb(self, paths: np.ndarray, offsets: np.ndarray):
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        off = np.ascontiguousarray(offsets, np.float32).reshape(n, capi.MAX_DIM)
        out = np.zeros(n, capi.PATH_DTYPE)
        ct = np.zeros(n, capi.CONTRIB_DTYPE)
        capi.check(capi.lib().drmlt_perturb(self.handle, capi.ptr(paths), capi.ptr(off), n, capi.ptr(out),
                                             capi.ptr(ct)))
        return out, ct

    def lens_eval(self, paths: np.ndarray, screen: np.ndarray, ss: np.ndarray, lens_sigma: float = 0.01,
                  max_derivative_depth: int = 9):
        """integrator=h2mc's lens quantities of each path (drmlt_lens_eval): lens
        score, lens vertex position, lens-mode log f, its gradient and Hessian
        w.r.t. the screen position, and the 2-D Gaussian (mean, inverse
        covariance, log det)."""
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        screen = np.ascontiguousarray(screen, np.float32).reshape(n, 2)
        ss = np.ascontiguousarray(ss, np.float32).reshape(n)
        score = np.zeros(n, np.float32)
        pos = np.zeros((n, 3), np.float32)
        logf = np.zeros(n, np.float32)
        g = np.zeros((n, 2), np.float32)
        h = np.zeros((n, 4), np.float32)
        gauss = np.zeros((n, 7), np.float64)
        capi.check(capi.lib().drmlt_lens_eval(self.handle, capi.ptr(paths), capi.ptr(screen), capi.ptr(ss), n,
                                               float(lens_sigma), int(max_derivative_depth), capi.ptr(score),
                                               capi.ptr(pos), capi.ptr(logf), capi.ptr(g), capi.ptr(h),
                                               capi.ptr(gauss)))
        return dict(score=score, pos=pos, logf=logf, grad=g, hess=h, mean=gauss[:, :2], inv_cov=gauss[:, 2:6],
                    log_det=gauss[:, 6])

    def lens_perturb(self, paths: np.ndarray, screen_new: np.ndarray, lens_pos: np.ndarray):
        """PerturbLensBidir of each path (drmlt_lens_perturb): perturbed paths,
        contributions and lens scores."""
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        scr = np.ascontiguousarray(screen_new, np.float32).reshape(n, 2)
        lp = np.ascontiguousarray(lens_pos, np.float32).reshape(n, 3)
        out = np.zeros(n, capi.PATH_DTYPE)
        ct = np.zeros(n, capi.CONTRIB_DTYPE)
        score = np.zeros(n, np.float32)
        capi.check(capi.lib().drmlt_lens_perturb(self.handle, capi.ptr(paths), capi.ptr(scr), capi.ptr(lp), n,
                                                  capi.ptr(out), capi.ptr(ct), capi.ptr(score)))
        return out, ct, score

    def replay(self, mode: int, tapes: list, cam_len=None, lgt_len=None, max_contribs: int = 64):
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
        capi.check(capi.lib().drmlt_replay(self.handle, mode, capi.ptr(T), capi.ptr(lens), stride, n, capi.ptr(cl),
                                            capi.ptr(ll), mc, capi.ptr(cnt), capi.ptr(tech), capi.ptr(ct),
                                            capi.ptr(pth), capi.ptr(cons)))
        return cnt, tech, ct, pth, cons

    def dr_eval(self, paths, contribs, offset1, offset2, aniso):
        """drmlt_dr_eval: per-stage acceptances of one DR iteration from states
        `paths` (with contributions) for given first / second-stage offsets.
        Returns (results, y paths, z paths)."""
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        contribs = np.ascontiguousarray(contribs, capi.CONTRIB_DTYPE)
        o1 = np.ascontiguousarray(offset1, np.float32).reshape(n, capi.MAX_DIM)
        o2 = np.ascontiguousarray(offset2, np.float32).reshape(n, capi.MAX_DIM)
        an = np.ascontiguousarray(aniso, np.int32)
        out = np.zeros(n, capi.DR_RESULT_DTYPE)
        y = np.zeros(n, capi.PATH_DTYPE)
        z = np.zeros(n, capi.PATH_DTYPE)
        capi.check(capi.lib().drmlt_dr_eval(self.handle, n, capi.ptr(paths), capi.ptr(contribs), capi.ptr(o1),
                                            capi.ptr(o2), capi.ptr(an), capi.ptr(out), capi.ptr(y), capi.ptr(z)))
        return out, y, z

    def large_step_eval(self, tapes, paths, contribs, length_func):
        """drmlt_large_step_eval: (a1, technique (n x 2), contributions, uniforms consumed)."""
        paths = np.ascontiguousarray(paths, capi.PATH_DTYPE)
        n = len(paths)
        stride = max(1, max(len(t) for t in tapes))
        T = np.zeros((n, stride), np.float32)
        lens = np.zeros(n, np.int32)
        for i, t in enumerate(tapes):
            T[i, :len(t)] = t
            lens[i] = len(t)
        contribs = np.ascontiguousarray(contribs, capi.CONTRIB_DTYPE)
        lf = np.ascontiguousarray(length_func, np.float32)
        a1 = np.zeros(n, np.float32)
        tech = np.zeros((n, 2), np.int32)
        ct = np.zeros(n, capi.CONTRIB_DTYPE)
        cons = np.zeros(n, np.int32)
        capi.check(capi.lib().drmlt_large_step_eval(self.handle, n, capi.ptr(T), capi.ptr(lens), stride,
                                                    capi.ptr(paths), capi.ptr(contribs), capi.ptr(lf), len(lf),
                                                    capi.ptr(a1), capi.ptr(tech), capi.ptr(ct), capi.ptr(cons)))
        return a1, tech, ct, cons

    def trace_rays(self, org, dirs, tmin=1e-3, tmax=float("inf"), any_hit=False):
        org = np.ascontiguousarray(org, np.float32).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = len(org)
        tri = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        capi.check(capi.lib().drmlt_trace_rays(self.handle, capi.ptr(org), capi.ptr(dirs), tmin, tmax, n,
                                                int(any_hit), capi.ptr(tri), capi.ptr(t)))
        return tri, t

    def compute_gaussian(self, dims, ss, grad, hess):
        n = len(dims)
        dims = np.ascontiguousarray(dims, np.int32)
        ss = np.ascontiguousarray(ss, np.float32)
        grad = np.ascontiguousarray(grad, np.float32).reshape(n, capi.MAX_DIM)
        hess = np.ascontiguousarray(hess, np.float32).reshape(n, capi.MAX_DIM * capi.MAX_DIM)
        mean = np.zeros((n, capi.MAX_DIM))
        ic = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM))
        cv = np.zeros((n, capi.MAX_DIM * capi.MAX_DIM))
        ld = np.zeros(n)
        capi.check(capi.lib().drmlt_compute_gaussian(self.handle, capi.ptr(dims), capi.ptr(ss), capi.ptr(grad),
                                                      capi.ptr(hess), n, capi.ptr(mean), capi.ptr(ic),
                                                      capi.ptr(cv), capi.ptr(ld)))
        return mean, ic, cv, ld


class Integrator:
    """src/integrator.h:9-22: Render() writes the film; PrePass() returns b."""

    def __init__(self, scene: SceneData, **kw):
        self.scene = scene
        self.output_name = ""
        self.verbose = True
        self.deterministic = False
        self.renderer = Renderer(scene, **kw)

    def PrePass(self) -> float:
        return self.renderer.prepass()

    def Render(self) -> np.ndarray:
        """The whole render (drmlt_render). With reportintervalseconds > 0 the
        chain loop runs in slices and, like delayed.cpp:612-637, writes the
        partial film to <partial dir>/<name>_<k>.exr once k intervals have
        passed since the prepass, appending the elapsed seconds to
        <name>_time.csv; the partial dir is <integrator>_partial (or
        <output_name>_partial) beside the scene's output image."""
        interval = self.scene.options.reportIntervalSeconds
        r = self.renderer
        if interval <= 0:
            r.render()
            return r.film()
        r.direct()
        r.prepass()
        if r.options.autotune and r.total_iterations() >= 1024:
            r.autotune(8)
        base = self.output_name or self.scene.options.integrator
        partial = os.path.join(os.path.dirname(self.output_path()), base + "_partial")
        os.makedirs(partial, exist_ok=True)
        t0, image_id, step = time.perf_counter(), 1, 8
        while True:
            t = time.perf_counter()
            if r.run(step) == 0:
                break
            # slices of about a tenth of the interval keep the write times close to it
            step = max(1, min(4 * step, int(step * 0.1 * interval / max(time.perf_counter() - t, 1e-6))))
            elapsed = time.perf_counter() - t0
            if elapsed >= interval * image_id:
                write_image(os.path.join(partial, "%s_%d.exr" % (base, image_id)), r.partial_film())
                with open(os.path.join(partial, base + "_time.csv"), "w" if image_id == 1 else "a") as f:
                    f.write("%g,\n" % elapsed)
                image_id += 1
        return r.film()

    def output_path(self) -> str:
        """The scene's output image (the film's filename, default image.exr
        beside the scene file, src/parsescene.cpp:149-160, 574)."""
        return self.scene.camera.get("output") or os.path.join(os.path.dirname(os.path.abspath(self.scene.path)),
                                                               "image.exr")

    def write_image(self, path: str | None = None) -> str:
        """WriteImage of the final film (src/main.cpp:130) to path or output_path()."""
        path = path or self.output_path()
        write_image(path, self.renderer.film())
        return path


def write_image(path: str, img: np.ndarray) -> None:
    """WriteImage (src/image.cpp:45-58): .exr through the C ABI, .pfm as float PFM."""
    if path.lower().endswith(".exr"):
        from .exr import write_exr
        write_exr(path, img)
    elif path.lower().endswith(".pfm"):
        from .scenegen import write_pfm
        write_pfm(path, img)
    else:
        raise ValueError("%s: only .exr and .pfm output is supported" % path)


class DRIntegrator(Integrator):
    """Delayed-rejection MLT (src/integrators/delayed/delayed.cpp)."""


class H2MCIntegrator(Integrator):
    """H2MC (src/integrators/h2mc.cpp), with its lens mutation."""


class MCMCIntegrator(Integrator):
    """Plain MMLT (src/integrators/mcmc.cpp) without its lens mutation."""


_CLASSES = {"drmlt": DRIntegrator, "h2mc": H2MCIntegrator, "mcmc": MCMCIntegrator}


def make_integrator(xml_path: str, **kw) -> Integrator:
    """main()'s dispatch on the scene's integrator (src/main.cpp:104-120); the
    reference's `mc` path tracer is not part of this library."""
    sd = load_scene(xml_path)
    if sd.options.integrator not in _CLASSES:
        raise ValueError("Unknown integrator %r" % sd.options.integrator)
    return _CLASSES[sd.options.integrator](sd, **kw)
