"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs
on the CPU (oracle, host algorithms of the library through a host-only
context, symbol exports)."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def vlib():
    from vrad_gb300 import _lib

    return _lib.load(build=True)


@pytest.fixture(scope="session")
def host_ctx(vlib):
    from vrad_gb300.environment import Context

    return Context(-1)


@pytest.fixture(scope="session")
def gpu_ctx(vlib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from vrad_gb300.environment import Context

    return Context(0)


@pytest.fixture(scope="session")
def anyhit_scene():
    from vrad_gb300 import scenes

    return scenes.anyhit_scene(0)


@pytest.fixture(scope="session")
def lit_scene():
    from vrad_gb300 import scenes

    return scenes.lit_scene(0)


def small_lit_scene(n_faces=96, seed=3):
    from vrad_gb300 import scenes

    return scenes.lit_scene(seed, n_faces=n_faces, n_point=12, n_spot=4)


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
