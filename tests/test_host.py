"""Host-side checks that need no GPU: the scene front-end against the reference's
camera matrices, the dpt option parser, and the C-ABI library's exports."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import REPO, golden, scene_xml
from drmlt import scene as dscene

HEADER = os.path.join(REPO, "include", "drmlt_capi.h")


@pytest.mark.parametrize("cfg", ["cfg1", "cfg2"])
def test_camera_matrices_match_reference(scene_root, cfg):
    ref = golden(cfg, "camera")[0]
    sd = dscene.load_scene(scene_xml(cfg, scene_root))
    m = dscene.camera_matrices(sd.camera)
    for mine, key in (("sample_to_cam", "sampleToCam"), ("cam_to_sample", "camToSample"),
                      ("cam_to_world", "camToWorld"), ("world_to_cam", "worldToCam")):
        np.testing.assert_allclose(m[mine], np.array(ref[key]).reshape(4, 4), rtol=1e-5, atol=1e-5, err_msg=key)
    assert abs(m["dist"] - ref["dist"]) <= 1e-4 * ref["dist"]


def test_dpt_option_defaults_and_parse(scene_root):
    sd = dscene.load_scene(scene_xml("cfg2", scene_root))
    o = sd.options
    assert o.type == "green" and o.maxDepth == 8 and o.numChains == 16384
    assert o.largeStepProb == pytest.approx(0.3) and o.roughnessThreshold == pytest.approx(0.03)
    d = dscene.DptOptions()
    # DptOptions defaults (src/dptoptions.h)
    assert (d.perturbStdDev, d.largeStepProb, d.anisoPerturbProb) == (0.01, 0.3, 0.5)
    assert d.useLightCoordinateSampling and d.minDepth == -1 and d.maxDepth == -1


def _declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(drmlt_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = _declared_symbols()
    for n in ("drmlt_create", "drmlt_prepass", "drmlt_run", "drmlt_get_film", "drmlt_path_grad_hess",
              "drmlt_path_eval", "drmlt_path_adjoint", "drmlt_compute_gaussian", "drmlt_compute_gaussian_noalloc",
              "drmlt_lens_eval", "drmlt_lens_perturb"):
        assert n in names


def test_library_loads_and_exports_every_declared_symbol(built_lib):
    so = ctypes.CDLL(built_lib.LIB_PATH)
    missing = [n for n in _declared_symbols() if not hasattr(so, n)]
    assert not missing, missing
    # every symbol the ctypes layer binds is declared in the header
    assert set(built_lib._SIGS) <= set(_declared_symbols())


def test_default_options_and_error_path_without_device(built_lib):
    """drmlt_default_options is host-only; on a machine without a GPU, create
    fails with DRMLT_E_CUDA and a readable message (no silent CPU path)."""
    o = built_lib.default_options()
    assert o.large_step_prob == pytest.approx(0.3) and o.perturb_stddev == pytest.approx(0.01)
    # lensPerturbProb / lensPerturbStdDev defaults (src/dptoptions.h:20-21)
    assert o.lens_perturb_prob == pytest.approx(0.3) and o.lens_perturb_stddev == pytest.approx(0.01)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    l = built_lib.lib()
    h = ctypes.c_void_p()
    desc = built_lib.SceneDesc()
    rc = l.drmlt_create(ctypes.byref(desc), ctypes.byref(o), ctypes.byref(h))
    assert rc != 0 and not h.value
    assert l.drmlt_last_error().decode()
