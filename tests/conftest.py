import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU visible")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    import build_oracle
    build_oracle.build()
    import orc as _orc
    return _orc


@pytest.fixture(scope="session")
def gpda_lib():
    """libgpda.so, built in-tree on first use (nvcc cross-compiles without a GPU)."""
    from gsmfretda_gb300 import build
    build.build()
    from gsmfretda_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def engine(gpda_lib):
    from gsmfretda_gb300.api import Engine
    eng = Engine(0)
    yield eng
    eng.close()


def model_kw():
    from gsmfretda_gb300.synth import MODEL_DEFAULTS
    return dict(MODEL_DEFAULTS)


@pytest.fixture
def rng():
    return np.random.default_rng(12345)
