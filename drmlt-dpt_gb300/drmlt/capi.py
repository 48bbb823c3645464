"""ctypes binding of libdrmlt.so (include/drmlt_capi.h).

The library is built in-tree by ``drmlt-dpt_gb300/build.py``; importing this
module loads it and raises if it is missing, so no caller can silently run
without the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libdrmlt.so")

MAX_LEN = 12
MAX_DIM = 24

BSDF_LAMBERTIAN, BSDF_PHONG, BSDF_ROUGHDIELECTRIC = 0, 1, 2
LIGHT_POINT, LIGHT_AREA, LIGHT_ENV = 0, 1, 2
INTEGRATOR_DRMLT, INTEGRATOR_H2MC, INTEGRATOR_MCMC = 0, 1, 2
DR_GREEN, DR_MIRA = 0, 1

F3 = C.c_float * 3
F16 = C.c_float * 16


class Bsdf(C.Structure):
    _fields_ = [("type", C.c_int32), ("two_sided", C.c_int32), ("kd", F3), ("ks", F3),
                ("exponent", C.c_float), ("int_ior", C.c_float), ("ext_ior", C.c_float),
                ("alpha", C.c_float), ("kt", F3)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("shape", C.c_int32), ("emission", F3), ("pos", F3),
                ("sampling_weight", C.c_float), ("env_rgb", C.POINTER(C.c_float)),
                ("env_width", C.c_int32), ("env_height", C.c_int32), ("to_world", F16)]


class SceneDesc(C.Structure):
    _fields_ = [("num_tris", C.c_int32), ("positions", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("num_shapes", C.c_int32),
                ("shape_first_tri", C.POINTER(C.c_int32)), ("shape_num_tris", C.POINTER(C.c_int32)),
                ("shape_bsdf", C.POINTER(C.c_int32)), ("shape_light", C.POINTER(C.c_int32)),
                ("num_bsdfs", C.c_int32), ("bsdfs", C.POINTER(Bsdf)), ("num_lights", C.c_int32),
                ("lights", C.POINTER(Light)), ("sample_to_cam", F16), ("cam_to_sample", F16),
                ("cam_to_world", F16), ("world_to_cam", F16), ("cam_dist", C.c_float),
                ("near_clip", C.c_float), ("far_clip", C.c_float), ("width", C.c_int32),
                ("height", C.c_int32), ("bsphere_center", F3), ("bsphere_radius", C.c_float)]


class Options(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("dr_type", C.c_int32), ("aniso_perturb_prob", C.c_float),
                ("aniso_perturb_stddev", C.c_float), ("acceptance_map", C.c_int32),
                ("perturb_stddev", C.c_float), ("large_step_prob", C.c_float),
                ("roughness_threshold", C.c_float), ("discrete_stddev", C.c_float),
                ("uniform_mixing_prob", C.c_float), ("num_chains", C.c_int32),
                ("num_init_samples", C.c_int32), ("spp", C.c_int32), ("direct_spp", C.c_int32),
                ("min_depth", C.c_int32), ("max_depth", C.c_int32), ("seed_offset", C.c_int32),
                ("use_light_coordinate_sampling", C.c_int32), ("max_derivative_depth", C.c_int32),
                ("seed", C.c_uint64), ("device", C.c_int32), ("use_graph", C.c_int32),
                ("chain_groups", C.c_int32), ("stage_lanes", C.c_int32), ("deriv_warps", C.c_int32),
                ("smem_carveout", C.c_int32), ("autotune", C.c_int32), ("stage2_lanes", C.c_int32),
                ("graph_iters", C.c_int32), ("wavefront", C.c_int32), ("head_chains", C.c_int32),
                ("head_lanes", C.c_int32), ("persistent", C.c_int32),
                ("team_sms", C.c_int32), ("wait_limit", C.c_int32), ("adjoint_min_dim", C.c_int32),
                ("lens_perturb_prob", C.c_float), ("lens_perturb_stddev", C.c_float)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "large_step", "large_step_accepted", "stage1", "stage1_accepted", "stage2_iso",
        "stage2_iso_accepted", "stage2_h2mc", "stage2_h2mc_accepted", "mutations", "gaussians",
        "gaussians_fp64_fallback", "lens", "lens_accepted")]


class Path(C.Structure):
    _fields_ = [("c", C.c_int32), ("l", C.c_int32), ("lgt_light", C.c_int32), ("lgt_prim", C.c_int32),
                ("dl_light", C.c_int32), ("dl_prim", C.c_int32), ("use_abs", C.c_uint32),
                ("u", C.c_float * MAX_DIM), ("tri", C.c_int32 * MAX_LEN),
                ("disc", C.c_float * MAX_LEN), ("rr", C.c_float * MAX_LEN)]


class Contrib(C.Structure):
    _fields_ = [("screen", C.c_float * 2), ("rgb", F3), ("ls", C.c_float), ("ss", C.c_float),
                ("valid", C.c_int32)]


# numpy views of the record structs (same layout)
PATH_DTYPE = np.dtype([("c", "<i4"), ("l", "<i4"), ("lgt_light", "<i4"), ("lgt_prim", "<i4"),
                       ("dl_light", "<i4"), ("dl_prim", "<i4"), ("use_abs", "<u4"),
                       ("u", "<f4", (MAX_DIM,)), ("tri", "<i4", (MAX_LEN,)),
                       ("disc", "<f4", (MAX_LEN,)), ("rr", "<f4", (MAX_LEN,))])
CONTRIB_DTYPE = np.dtype([("screen", "<f4", (2,)), ("rgb", "<f4", (3,)), ("ls", "<f4"),
                          ("ss", "<f4"), ("valid", "<i4")])
DR_RESULT_DTYPE = np.dtype([("a1", "<f4"), ("ss_y", "<f4"), ("ss_z", "<f4"), ("valid_y", "<i4"), ("valid_z", "<i4"),
                            ("a2", "<f4"), ("log_ratio", "<f8"), ("a_star_green", "<f4"), ("alpha2_green", "<f4"),
                            ("alpha2_mira", "<f4"), ("pad", "<i4"), ("log_q_mira", "<f8")])
assert DR_RESULT_DTYPE.itemsize == 56
assert PATH_DTYPE.itemsize == C.sizeof(Path)
assert CONTRIB_DTYPE.itemsize == C.sizeof(Contrib)

# Every entry point the header declares, with its argument types.
_SIGS = {
    "drmlt_default_options": (None, [C.POINTER(Options)]),
    "drmlt_last_error": (C.c_char_p, []),
    "drmlt_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "drmlt_destroy": (C.c_int, [C.c_void_p]),
    "drmlt_prepass": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "drmlt_direct": (C.c_int, [C.c_void_p]),
    "drmlt_run": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "drmlt_run_async": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_int64)]),
    "drmlt_wait_stats": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "drmlt_render": (C.c_int, [C.c_void_p]),
    "drmlt_get_film": (C.c_int, [C.c_void_p, C.c_void_p]),
    "drmlt_get_launch_shape": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
    "drmlt_get_partial_film": (C.c_int, [C.c_void_p, C.c_void_p]),
    "drmlt_get_wavefront": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "drmlt_get_head_tier": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "drmlt_get_adjoint_min_dim": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "drmlt_write_exr": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_void_p]),
    "drmlt_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "drmlt_last_run_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "drmlt_kernel_launches": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "drmlt_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "drmlt_fma_benchmark": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "drmlt_ray_benchmark": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_void_p]),
    "drmlt_profile": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(C.c_int64)]),
    "drmlt_total_iterations": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "drmlt_path_eval": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "drmlt_path_grad_hess": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "drmlt_path_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "drmlt_perturb": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "drmlt_lens_eval": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "drmlt_lens_perturb": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    "drmlt_replay": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                               C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "drmlt_dr_eval": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p]),
    "drmlt_large_step_eval": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "drmlt_trace_rays": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_int, C.c_int,
                                   C.c_void_p, C.c_void_p]),
    "drmlt_compute_gaussian": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "drmlt_compute_gaussian_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


class DrmltError(RuntimeError):
    """A libdrmlt call failed: `code` is its DRMLT_E_* return value."""

    def __init__(self, msg: str, code: int = 0):
        super().__init__(msg)
        self.code = code


def lib():
    """Loads libdrmlt.so (once); raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DrmltError("libdrmlt.so not built: run drmlt-dpt_gb300/build.py (%s missing)" % LIB_PATH)
        l = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(rc: int):
    if rc != 0:
        raise DrmltError("libdrmlt error %d: %s" % (rc, lib().drmlt_last_error().decode()), rc)


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def default_options() -> Options:
    o = Options()
    lib().drmlt_default_options(C.byref(o))
    return o
