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


def rel_error_stats(got, ref, floor_frac=1e-3):
    """Per-value error of a device result against the oracle: the share of
    bit-identical values, the max and p99 relative error |got-ref|/|ref|
    over values with ref != 0, how many ref == 0 values are not exactly 0 on
    the device, and how many values lie under floor_frac x the largest |ref|
    (where a relative figure is dominated by rounding of tiny numbers; they
    are still inside the max above)."""
    g = np.ascontiguousarray(got, dtype=np.float32).ravel()
    r = np.ascontiguousarray(ref, dtype=np.float32).ravel()
    g64, r64 = g.astype(np.float64), r.astype(np.float64)
    nz = r64 != 0.0
    rel = np.abs(g64[nz] - r64[nz]) / np.abs(r64[nz])
    return {
        "n": int(g.size),
        "bit_identical": float(np.mean(g.view(np.uint32) == r.view(np.uint32))) if g.size else 1.0,
        "max_rel": float(rel.max()) if rel.size else 0.0,
        "p99_rel": float(np.percentile(rel, 99)) if rel.size else 0.0,
        "zero_ref_nonzero": int(np.count_nonzero(g64[~nz])),
        "under_floor": int(np.count_nonzero(np.abs(r64) < floor_frac * (np.abs(r64).max() if r64.size else 0.0))),
    }
