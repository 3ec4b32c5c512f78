"""The oracle against the committed golden fixtures (no GPU).

``trace_geometry.npz`` answers shadow lines by float64 geometry that shares
no code with the oracle; ``pipeline_small.npz`` holds the oracle's own
outputs for a small lit scene.  Both are made by tests/golden/make_golden.py."""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import bits_equal

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

import make_golden as mg  # noqa: E402


@pytest.fixture(scope="module")
def geom():
    return dict(np.load(GOLDEN / "trace_geometry.npz"))


@pytest.fixture(scope="module")
def pipe():
    return dict(np.load(GOLDEN / "pipeline_small.npz"))


def check_against_geometry(g, k, hit, t, mask=None, frac=None):
    """hit/t: closest-hit index and distance per line; mask: occlusion bits;
    frac: fractionVisible.  Only lines the geometry decided are compared."""
    want = g[f"hit{k}"]
    dec = want != mg.UNDECIDED_HIT
    assert dec.mean() > 0.99
    assert np.array_equal(hit[dec], want[dec]), np.nonzero(dec & (hit != want))[0][:10]
    has = dec & (want >= 0)
    seg = np.linalg.norm(g["stops"].astype(np.float64) - g["starts"], axis=1)
    assert np.all(np.abs(t[has] - g[f"t{k}"][has]) <= 1e-4 * (seg[has] + 1.0))
    occ = g[f"occ{k}"]
    if mask is not None:
        bits = (mask[np.arange(len(occ)) >> 5] >> (np.arange(len(occ)) & 31)) & 1
        assert np.array_equal(bits[dec], occ[dec].astype(np.uint32))
    if frac is not None:
        assert np.array_equal(frac[dec], (1 - occ[dec]).astype(np.float32))


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_lines_match_float64_geometry(oracle, geom, k):
    g = geom
    skip = int(g["skip_ids"][k])
    s = oracle.Scene(g["xyz"], g["ids"])
    mask, hit, t = s.occlusion_mask(g["starts"], g["stops"], skip=skip, closest=True)
    check_against_geometry(g, k, hit, t, mask=mask)
    frac = s.test_lines(g["starts"], g["stops"], skip=skip, brute=True)
    check_against_geometry(g, k, hit, t, frac=frac)


def test_fixture_matches_the_scene_generator(pipe):
    assert str(pipe["inputs"]) == mg.pipeline_inputs_digest(mg.pipeline_scene())


def test_oracle_pipeline_matches_fixture(oracle, pipe):
    now = mg.oracle_pipeline(oracle, threads=4)
    assert bits_equal(now["luxel_rgb"], pipe["luxel_rgb"])
    assert int(now["rays"]) == int(pipe["rays"])
    for k in ("patches", "transfers"):
        assert now[k] == str(pipe[k]), k
    assert int(now["nnz"]) == int(pipe["nnz"]) and int(now["n_leaves"]) == int(pipe["n_leaves"])
    assert bits_equal(now["patch_direct"], pipe["patch_direct"])
    assert int(now["bounce_iters"]) == int(pipe["bounce_iters"])
    np.testing.assert_allclose(now["bounce_total"], pipe["bounce_total"], rtol=1e-12, atol=0)


def test_library_patches_match_fixture(host_ctx, pipe):
    from vrad_gb300.environment import Environment

    lit = mg.pipeline_scene()
    env = Environment(host_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    P = env.make_patches()
    assert mg.patch_digest(P) == str(pipe["patches"])
    assert P["n_leaves"] == int(pipe["n_leaves"])
