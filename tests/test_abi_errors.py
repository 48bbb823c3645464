"""Error behaviour of the C ABI: every entry point returns a negative
DRMLT_E_* code with a message instead of crashing or falling back, like the
reference's Error() throws (src/flexception.h). The argument checks that run
before any device call are tested on the CPU; the rest on the GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import helpers  # noqa: F401  (puts the package on sys.path)
from drmlt import capi

E_ARG, E_STATE = -1, -3


def _scene_desc(built_lib, scene_root):
    from drmlt import scene as dscene, scenegen
    import os
    sd = dscene.load_scene(scenegen.config1(os.path.join(scene_root, "abi_errors"), spp=1))
    return sd, dscene.SceneDescHolder(sd)


def _create(holder, opt):
    h = C.c_void_p()
    rc = capi.lib().drmlt_create(C.byref(holder.desc), C.byref(opt), C.byref(h))
    return rc, h


@pytest.mark.parametrize("field,value,msg", [("max_depth", 13, "max_depth"), ("max_depth", 2, "max_depth"),
                                             ("num_chains", 0, "num_chains")])
def test_create_rejects_bad_options_before_any_device_call(built_lib, scene_root, field, value, msg):
    sd, holder = _scene_desc(built_lib, scene_root)
    from drmlt.integrator import make_options
    opt = make_options(sd)
    setattr(opt, field, value)
    rc, h = _create(holder, opt)
    assert rc == E_ARG and not h.value
    assert msg in capi.lib().drmlt_last_error().decode()


def test_create_rejects_an_empty_scene(built_lib, scene_root):
    sd, holder = _scene_desc(built_lib, scene_root)
    from drmlt.integrator import make_options
    holder.desc.num_lights = 0
    rc, h = _create(holder, make_options(sd))
    assert rc == E_ARG and "light" in capi.lib().drmlt_last_error().decode()


def test_null_handles_are_rejected(built_lib):
    l = capi.lib()
    buf = np.zeros(12, np.float32)
    n = C.c_int64()
    assert l.drmlt_prepass(None, None) == E_ARG
    assert l.drmlt_run(None, 1, C.byref(n)) == E_ARG
    assert l.drmlt_render(None) == E_ARG
    assert l.drmlt_get_film(None, capi.ptr(buf)) == E_ARG
    assert l.drmlt_get_partial_film(None, capi.ptr(buf)) == E_ARG
    assert l.drmlt_fma_benchmark(None, 0, 1, None, None) == E_ARG
    assert l.drmlt_write_exr(None, 1, 1, capi.ptr(buf)) == E_ARG
    assert l.drmlt_write_exr(b"x.exr", 0, 1, capi.ptr(buf)) == E_ARG


@pytest.mark.gpu
def test_device_side_argument_and_state_errors(built_lib, scene_root):
    from drmlt.integrator import Renderer, make_options
    sd, holder = _scene_desc(built_lib, scene_root)
    # a shape pointing at a BSDF that does not exist
    bad = holder.sb.copy()
    bad[0] = 99
    holder.desc.shape_bsdf = bad.ctypes.data_as(C.POINTER(C.c_int32))
    rc, h = _create(holder, make_options(sd, num_chains=256))
    assert rc == E_ARG and "bsdf" in capi.lib().drmlt_last_error().decode()
    with Renderer(sd, num_chains=256) as r:
        n = C.c_int64()
        assert capi.lib().drmlt_run(r.handle, 1, C.byref(n)) == E_STATE
        assert "before prepass" in capi.lib().drmlt_last_error().decode()
        lanes, warps = C.c_int(), C.c_int()
        assert capi.lib().drmlt_autotune(r.handle, 1, C.byref(lanes), C.byref(warps)) == E_STATE
        ms, cnt = C.c_float(), np.zeros(3)
        assert capi.lib().drmlt_ray_benchmark(r.handle, 3, 16, 1, C.byref(ms), cnt.ctypes.data) == E_ARG
        fl = C.c_double()
        assert capi.lib().drmlt_fma_benchmark(r.handle, 0, 0, C.byref(ms), C.byref(fl)) == E_ARG
        dims = np.array([3], np.int32)  # odd dimension
        z = np.zeros(24 * 24)
        assert capi.lib().drmlt_compute_gaussian(r.handle, capi.ptr(dims), capi.ptr(np.ones(1, np.float32)),
                                                 capi.ptr(np.zeros(24, np.float32)),
                                                 capi.ptr(np.zeros(576, np.float32)), 1, capi.ptr(np.zeros(24)),
                                                 capi.ptr(z), capi.ptr(z.copy()), capi.ptr(np.zeros(1))) == E_ARG
        # the handle still works after the rejected calls
        r.prepass()
        assert r.run(2) == 2 * 256
