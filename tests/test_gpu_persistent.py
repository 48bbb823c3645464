"""The persistent chain-loop schedule (persist.cu) against the staged one.

Under the persistent schedule one cooperative kernel runs every chain through
its iterations with work queues between path tracing and the H2MC derivative /
Gaussian workers, and no barrier between stages or iterations. The chains'
random streams are keyed by (seed, chain, iteration, stage), so the chains must
take exactly the staged schedule's steps: integer counters identical, film
equal up to the order of the floating-point splat additions. Every device-side
wait of the schedule is bounded; a run whose wait limit runs out returns
DRMLT_E_TIMEOUT instead of hanging (tested on a tiny case with a limit of one
poll, after which the device stays usable).
"""
import os

import numpy as np
import pytest

from helpers import scene_xml  # noqa: I001 (puts the package on sys.path)
from drmlt import capi

pytestmark = pytest.mark.gpu

DRMLT_E_TIMEOUT = -6


def _scene(cfg, dr_type, root):
    from drmlt import scenegen
    from drmlt import scene as dscene
    if cfg == "cfg4s":
        xml = scenegen.config4_small(os.path.join(root, "persist_cfg4s_" + dr_type), dr_type=dr_type)
    elif cfg == "cfg2":
        xml = scenegen.config2(os.path.join(root, "persist_cfg2_" + dr_type), dr_type)
    else:
        xml = scene_xml(cfg, root)
    return dscene.load_scene(xml)


@pytest.mark.parametrize("cfg,dr_type", [("cfg2", "mira"), ("cfg2", "green"), ("cfg3", "green"), ("cfgE", "green"),
                                         ("cfg4s", "mira"), ("cfg4s", "green")])
def test_persistent_takes_the_staged_steps(built_lib, scene_root, cfg, dr_type):
    """Two persistent runs (4 + 7 iterations) against staged launches of the same
    11 iterations, on scenes with Phong and rough-dielectric BSDFs, the
    environment light, Green's y* and depth-12 paths (cfg4s). The persistent
    schedule takes hyper-dual derivatives for every path, so the staged run
    does too (adjoint_min_dim=-1: the adjoint rounds differently)."""
    from drmlt.integrator import Renderer
    sd = _scene(cfg, dr_type, scene_root)
    out = []
    for kw in (dict(persistent=1), dict(persistent=1, team_sms=3, stage_lanes=32),
               dict(persistent=0, adjoint_min_dim=-1)):
        with Renderer(sd, num_chains=4096, **kw) as r:
            r.prepass()
            assert r.run(4) == 4 * 4096
            assert r.run(7) == 7 * 4096
            out.append((r.stats(), r.film().astype(np.float64)))
    ref_stats, ref_film = out[-1]
    assert ref_stats["stage2_h2mc"] > 0 and ref_stats["large_step_accepted"] > 0
    for st, film in out[:-1]:
        assert st == ref_stats
        np.testing.assert_allclose(film, ref_film, rtol=1e-4, atol=1e-6)


def test_persistent_extra_samples_and_run_end(built_lib, scene_root):
    """The reference's chainsNeedExtraSamples rule (delayed.cpp:205-210) under
    the persistent schedule: 5041 chains on the 256 x 256 box at 1 spp get 13
    samples each and 13 of them a 14th; a run past the end stops there."""
    from drmlt import scenegen
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    sd = dscene.load_scene(scenegen.config1(os.path.join(scene_root, "persist_extra"), spp=1))
    out = []
    for kw in (dict(persistent=1), dict(persistent=0, adjoint_min_dim=-1)):
        with Renderer(sd, num_chains=5041, **kw) as r:
            assert r.total_iterations() == 14
            r.prepass()
            assert r.run(9) == 9 * 5041
            assert r.run(20) == 4 * 5041 + 13
            assert r.run(3) == 0
            out.append((r.stats(), r.film().astype(np.float64)))
    assert out[0][0] == out[1][0]
    assert out[0][0]["mutations"] == 13 * 5041 + 13
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-4, atol=1e-6)


def test_persistent_wait_limit_returns_an_error(built_lib, scene_root):
    """With a wait limit of one poll, idle workers give up at once: the run
    returns DRMLT_E_TIMEOUT (the kernel returns; nothing traps or hangs) and the
    device stays usable for a new handle."""
    from drmlt.integrator import Renderer
    sd = _scene("cfg1", "green", scene_root)
    with Renderer(sd, num_chains=256, persistent=1, wait_limit=1) as r:
        r.prepass()
        with pytest.raises(capi.DrmltError) as e:
            r.run(4)
        assert e.value.code == DRMLT_E_TIMEOUT, str(e.value)
    with Renderer(sd, num_chains=256, persistent=1) as r:
        r.prepass()
        assert r.run(2) == 2 * 256
