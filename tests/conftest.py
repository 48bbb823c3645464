import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


@pytest.fixture(scope="session")
def scene_root(tmp_path_factory):
    return str(tmp_path_factory.mktemp("scenes"))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Builds libdrmlt.so if needed; GPU tests fail (not skip) when it cannot load."""
    from helpers import PKG
    sys.path.insert(0, PKG)
    import build as drmlt_build
    drmlt_build.build()
    from drmlt import capi
    capi.lib()
    return capi


@pytest.fixture(scope="session")
def renderers(built_lib, scene_root):
    """One renderer per golden scene (cfg1 / cfg2), small chain count."""
    from helpers import scene_xml
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer
    cache = {}

    def get(cfg):
        if cfg not in cache:
            sd = dscene.load_scene(scene_xml(cfg, scene_root))
            cache[cfg] = Renderer(sd, num_chains=64)
        return cache[cfg]

    yield get
    for r in cache.values():
        r.close()
