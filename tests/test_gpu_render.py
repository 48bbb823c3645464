"""Whole renders on the GPU vs full renders of the reference (`dpt -d`, fixtures
<cfg>_render*.json.gz made by tests/golden/make_golden.py): same scene, same
options, same number of mutations, different random streams, so the checks are
statistical.

Bars. Acceptance ratios: within 0.006 (large step, stage 1) and 0.012 (second
stages) of the reference's -- two `dpt` runs of the 16-spp Cornell box with
different seeds differ by up to 0.0035 on the second stages. The H2MC
(anisotropic) second stage on the Phong box is the exception: the oracle's CPU
chain loop and this GPU path agree with each other there (0.105 / 0.321 for
mira / green on the Phong box; 0.334 / 0.323 green on the rough-dielectric
scenes) but sit above the reference (0.097 / 0.282; 0.293 / 0.274). The
reference's chad Hessian is not the exact Hessian for light-tracing techniques
(camDepth = 1) and for some rough-dielectric paths (it disagrees with central
differences of chad's own gradient) while this build's is, so its anisotropic
proposals differ there; bars 0.015 (mira) and 0.06 (green).
Image: per-channel mean within 2%, 8 x 8 block means within 6% on average."""
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu

RENDERS = [("cfg1", "render", "green"), ("cfg2", "render_mira", "mira"), ("cfg2", "render_green", "green"),
           ("cfg1", "render_accmap", "green"), ("cfg3", "render", "green"), ("cfgL", "render", "green")]
SINGLE_STAGE = [("cfg1", "render_h2mc", "h2mc"), ("cfg1", "render_mcmc", "mcmc")]


def _fixture(cfg, name):
    import gzip
    import json
    p = os.path.join(GOLDEN, "%s_%s.json.gz" % (cfg, name))
    with gzip.open(p, "rt") as f:
        return json.load(f)


def _scene(cfg, dr_type, root, name="render"):
    from drmlt import scenegen
    d = os.path.join(root, "%s_%s_%s" % (cfg, dr_type, name))
    if name == "render_accmap":
        return scenegen.config1(d, spp=16, acceptance_map=True)
    if dr_type in ("h2mc", "mcmc"):
        return scenegen.config1(d, spp=16, integrator=dr_type, extra={"lensperturbprob": "0"})
    if cfg == "cfg1":
        return scenegen.config1(d, spp=16)
    if cfg == "cfg3":
        return scenegen.config3(d, spp=16)
    if cfg == "cfgL":
        return scenegen.config_lights(d, spp=16)
    return scenegen.config2(d, dr_type, spp=1)


@pytest.mark.parametrize("cfg,name,dr_type", RENDERS)
def test_render_statistics_match_reference(built_lib, scene_root, cfg, name, dr_type):
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    ref = _fixture(cfg, name)
    sd = dscene.load_scene(_scene(cfg, dr_type, scene_root, name))
    with Renderer(sd) as r:
        r.render()
        img = r.film().astype(np.float64)
        st = r.stats()
    # the reference's loop runs numSamplesPerChain % numChains extra samples
    # (chainsNeedExtraSamples, delayed.cpp:209-210,339), so the total is within one
    # sample per chain of spp * W * H
    assert abs(st["mutations"] - sd.options.spp * sd.width * sd.height) <= sd.options.numChains
    mine = dict(large=st["large_step_accepted"] / st["large_step"],
                stage1=st["stage1_accepted"] / st["stage1"],
                stage2_iso=st["stage2_iso_accepted"] / st["stage2_iso"],
                stage2_h2mc=st["stage2_h2mc_accepted"] / st["stage2_h2mc"])
    tol = dict(large=0.006, stage1=0.006, stage2_iso=0.012, stage2_h2mc=0.015 if dr_type == "mira" else 0.06)
    for k, t in tol.items():
        assert abs(mine[k] - ref["stats"][k][0]) <= t, (k, mine[k], ref["stats"][k][0])
    mean = img.mean(axis=(0, 1))
    np.testing.assert_allclose(mean, ref["mean"], rtol=0.02)
    blk = np.array(ref["blocks"])
    rb = blk.reshape(8, 2, 8, 2, 3).mean(axis=(1, 3))
    H, W, _ = img.shape
    mb = img.reshape(8, H // 8, 8, W // 8, 3).mean(axis=(1, 3))
    rel = np.abs(mb - rb) / np.maximum(rb, 1e-3)
    assert rel.mean() < 0.06, rel.mean()


def test_tuning_parameters_do_not_change_the_chains(built_lib, scene_root):
    """Graph replay, chain groups, chains per warp and derivative-team size only
    change the scheduling: the chains take the same steps (integer counters identical,
    film equal up to the order of the floating-point splat additions)."""
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    sd = dscene.load_scene(_scene("cfg2", "mira", scene_root))
    out = []
    for kw in (dict(), dict(use_graph=0), dict(chain_groups=4, stage_lanes=4, deriv_warps=1),
               dict(chain_groups=3, stage_lanes=32, deriv_warps=4, use_graph=0)):
        with Renderer(sd, num_chains=4096, **kw) as r:
            r.prepass()
            r.run(12)
            out.append((r.stats(), r.film().astype(np.float64)))
    for st, film in out[1:]:
        assert st == out[0][0]
        np.testing.assert_allclose(film, out[0][1], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("cfg,name,integrator", SINGLE_STAGE)
def test_single_stage_integrators_match_reference(built_lib, scene_root, cfg, name, integrator):
    """integrator=h2mc (H2MC small step with uniform mixing, h2mc.cpp:200-240,
    448-606) and integrator=mcmc (mcmc.cpp) against `dpt -d` renders of the
    same scene, with lensperturbprob = 0 (the lens mutation is not part of this
    build). Small-step ratio within 0.012, large step 0.006, image as above."""
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    ref = _fixture(cfg, name)
    sd = dscene.load_scene(_scene(cfg, integrator, scene_root, name))
    with Renderer(sd) as r:
        r.render()
        img = r.film().astype(np.float64)
        st = r.stats()
    assert st["stage2_iso"] == 0 and (integrator == "h2mc") == (st["stage2_h2mc"] > 0)
    large = st["large_step_accepted"] / st["large_step"]
    small = (st["stage1_accepted"] + st["stage2_h2mc_accepted"]) / (st["stage1"] + st["stage2_h2mc"])
    assert abs(large - ref["stats"]["large"][0]) <= 0.006, (large, ref["stats"]["large"])
    assert abs(small - ref["stats"]["small"][0]) <= 0.012, (small, ref["stats"]["small"])
    np.testing.assert_allclose(img.mean(axis=(0, 1)), ref["mean"], rtol=0.02)
    rb = np.array(ref["blocks"]).reshape(8, 2, 8, 2, 3).mean(axis=(1, 3))
    H, W, _ = img.shape
    mb = img.reshape(8, H // 8, 8, W // 8, 3).mean(axis=(1, 3))
    assert (np.abs(mb - rb) / np.maximum(rb, 1e-3)).mean() < 0.06
