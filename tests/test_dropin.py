"""The C++ drop-in (drmlt-dpt_gb300/dropin): the reference's own scene parser
feeding the GPU integrator.

`dpt_gpu` is built by oracle/ref/Makefile (target dropin) from the reference's
sources and the drop-in's GpuDRIntegrator, and linked with libdrmlt.so. Its
--dump-desc mode writes the drmlt_scene_desc and drmlt_options that
BuildSceneDesc / BuildOptions make from the reference's parsed Scene; they are
compared field by field with what the Python host (drmlt/scene.py,
drmlt/integrator.py) makes from the same XML. Without a GPU, rendering fails
with the library's DRMLT_E_CUDA error. Runs where the reference sources are
present (the drop-in compiles against them); skipped elsewhere.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from helpers import REPO, SCENE_WRITERS  # noqa: I001 (puts the package on sys.path)
from drmlt import capi
from drmlt import scene as dscene
from drmlt.integrator import make_options

DPT_GPU = os.path.join(REPO, "oracle", "_ref", "single", "dpt_gpu")


@pytest.fixture(scope="module")
def dpt_gpu(built_lib):
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-s", "-j8", "dropin-if-present"], check=True,
                   capture_output=True)
    if not os.path.exists(DPT_GPU):
        pytest.skip("the drop-in needs the reference sources")
    return DPT_GPU


def _c(arr, n):
    return np.array([arr[i] for i in range(n)], np.float64)


@pytest.mark.parametrize("cfg", ["cfg1", "cfg2", "cfg3", "cfgL", "cfgE"])
def test_dropin_scene_descriptor_matches_the_python_host(dpt_gpu, scene_root, cfg):
    xml = SCENE_WRITERS[cfg](os.path.join(scene_root, "dropin_" + cfg))
    wd = os.path.dirname(xml)
    out = os.path.join(wd, "desc.json")
    subprocess.run([dpt_gpu, "--dump-desc", out, "--max-derivatives-depth=9", os.path.basename(xml)], cwd=wd,
                   check=True, capture_output=True)
    cpp = json.load(open(out))
    sd = dscene.load_scene(xml)
    h = dscene.SceneDescHolder(sd)
    d = h.desc
    T = d.num_tris
    assert cpp["num_tris"] == T
    np.testing.assert_allclose(np.array(cpp["positions"]), h.pos.ravel(), rtol=0, atol=2e-6)
    np.testing.assert_allclose(np.array(cpp["normals"]), h.nor.ravel(), rtol=0, atol=1e-5)
    for k, a in (("shape_first_tri", h.first), ("shape_num_tris", h.count), ("shape_bsdf", h.sb),
                 ("shape_light", h.sl)):
        assert cpp[k] == a.tolist(), k
    assert len(cpp["bsdfs"]) == d.num_bsdfs
    for b, mine in zip(cpp["bsdfs"], sd.bsdfs):
        assert b["type"] == mine.type
        np.testing.assert_allclose(b["kd"], _c(mine.kd, 3), rtol=1e-6)
        np.testing.assert_allclose(b["ks"], _c(mine.ks, 3), rtol=1e-6)
        if mine.type == capi.BSDF_ROUGHDIELECTRIC:
            np.testing.assert_allclose(b["kt"], _c(mine.kt, 3), rtol=1e-6)
            assert b["eta"] == pytest.approx(mine.int_ior / mine.ext_ior, rel=1e-6)
            assert b["alpha"] == pytest.approx(mine.alpha, rel=1e-6)
        else:
            assert b["two_sided"] == mine.two_sided
        if mine.type == capi.BSDF_PHONG:
            assert b["exponent"] == pytest.approx(mine.exponent, rel=1e-6)
    assert len(cpp["lights"]) == d.num_lights
    for L, mine in zip(cpp["lights"], sd.lights):
        assert (L["type"], L["shape"]) == (mine.type, mine.shape)
        assert L["sampling_weight"] == pytest.approx(mine.sampling_weight)
        np.testing.assert_allclose(L["emission"], _c(mine.emission, 3), rtol=1e-6)
        if mine.type == capi.LIGHT_POINT:
            np.testing.assert_allclose(L["pos"], _c(mine.pos, 3), rtol=1e-6)
        if mine.type == capi.LIGHT_ENV:
            assert (L["env_width"], L["env_height"]) == (mine.env_width, mine.env_height)
            n = mine.env_width * mine.env_height * 3
            np.testing.assert_allclose(L["env_rgb"], _c(mine.env_rgb, n), rtol=1e-6)
            np.testing.assert_allclose(L["to_world"], _c(mine.to_world, 16), rtol=1e-5, atol=1e-6)
    for k in ("sample_to_cam", "cam_to_sample", "cam_to_world", "world_to_cam"):
        np.testing.assert_allclose(cpp[k], _c(getattr(d, k), 16), rtol=1e-5, atol=1e-5, err_msg=k)
    assert cpp["cam_dist"] == pytest.approx(d.cam_dist, rel=1e-6)
    assert (cpp["near_clip"], cpp["far_clip"]) == pytest.approx((d.near_clip, d.far_clip), rel=1e-6)
    assert (cpp["width"], cpp["height"]) == (d.width, d.height)
    np.testing.assert_allclose(cpp["bsphere_center"], _c(d.bsphere_center, 3), rtol=1e-6, atol=1e-6)
    assert cpp["bsphere_radius"] == pytest.approx(d.bsphere_radius, rel=1e-6)
    o = make_options(sd, max_derivative_depth=9)
    for k, v in cpp["options"].items():
        assert getattr(o, k) == pytest.approx(v, rel=1e-6), k


def test_dropin_reports_the_library_error_without_a_gpu(dpt_gpu, scene_root):
    """On a machine without a CUDA device the drop-in's Render() throws the
    library's DRMLT_E_CUDA error, which main() prints before exiting 1."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    xml = SCENE_WRITERS["cfg1"](os.path.join(scene_root, "dropin_err"))
    r = subprocess.run([dpt_gpu, os.path.basename(xml)], cwd=os.path.dirname(xml), capture_output=True, text=True)
    assert r.returncode == 1
    assert "libdrmlt error %d" % -2 in r.stderr, r.stderr
