"""Transparent shadows on the device against the oracle: Trace4Rays with a
coverage-counting transparency callback (raytracer/environment.go:140-142,
raytracer/types/coverageCount.go:27-41) and TestLineDoesHitSky with texture
shadows (raytracer/trace/testline.go:29-33,53-55).  Hits are taken in
ascending (t, triangle index), so the coverage sums are the same floats in
the same order: recorded hits, t, coverage and fractions visible must be
bit-identical."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu

TRANSPARENT = 1


def _scene(seed, n_boxes=160):
    """A box room (sky ceiling) whose boxes are a mix of opaque, transparent
    (coverage 0.05-0.7 from the colour's x) and static-prop ones."""
    from vrad_gb300 import scenes

    sc = scenes.anyhit_scene(seed, n_boxes=n_boxes, n_rays=16)
    xyz, ids = sc.xyz.copy(), sc.ids.copy()
    n = len(ids)
    rng = np.random.default_rng(seed)
    box = np.arange(n) // 12
    kind = rng.integers(0, 4, box.max() + 1)[box]
    flags = np.where((kind >= 2) & (np.arange(n) >= 12), TRANSPARENT, 0).astype(np.uint8)
    cover = rng.uniform(0.05, 0.7, box.max() + 1).astype(np.float32)[box]
    colours = np.zeros((n, 3), np.float32)
    colours[:, 0] = cover
    ids[(kind == 1) & (np.arange(n) >= 12)] = 0x04000003  # static props with id 3
    ids[:2] = 0x01000000  # the room's far wall is sky
    return xyz, ids, flags, colours


@pytest.fixture(scope="module")
def cov_env(gpu_ctx):
    from vrad_gb300.environment import Environment

    xyz, ids, flags, colours = _scene(5)
    env = Environment(gpu_ctx)
    env.add_triangles(xyz, ids)
    env.set_triangle_flags(0, flags, colours)
    env.SetupAccelerationStructure()
    return env, xyz, ids, flags, colours


def test_trace_coverage_matches_oracle(cov_env, oracle):
    env, xyz, ids, flags, colours = cov_env
    s = oracle.Scene(xyz, ids, flags=flags)
    rng = np.random.default_rng(11)
    n = 20000
    o = rng.uniform(1, 4095, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.sqrt((d * d).sum(1, keepdims=True)).astype(np.float32)
    tmax = rng.uniform(10, 6000, n).astype(np.float32)
    hit, t, cov = env.trace_coverage(o, d, 0.0, tmax)
    rh, rt, rc = s.trace_coverage(colours[:, 0], o, d, 0.0, tmax, threads=16)
    assert np.array_equal(hit, rh)
    assert bits_equal(t, rt) and bits_equal(cov, rc)
    # the cases are all there: partial coverage, saturated coverage on a
    # transparent triangle, opaque hits behind transparent ones, misses
    tr = flags[np.maximum(hit, 0)] == TRANSPARENT
    assert ((cov > 0) & (cov < 1)).sum() > 100
    assert ((hit >= 0) & tr & (cov == 1)).sum() > 10
    assert ((hit >= 0) & ~tr & (cov > 0)).sum() > 100
    assert (hit < 0).sum() > 10
    # skip id
    hit2, t2, cov2 = env.trace_coverage(o[:4000], d[:4000], 0.0, tmax[:4000], skip_id=0x04000003)
    rh2, rt2, rc2 = s.trace_coverage(colours[:, 0], o[:4000], d[:4000], 0.0, tmax[:4000],
                                     skip=0x04000003, threads=16)
    assert np.array_equal(hit2, rh2) and bits_equal(t2, rt2) and bits_equal(cov2, rc2)


def test_line_coverage_matches_oracle(cov_env, oracle):
    env, xyz, ids, flags, colours = cov_env
    s = oracle.Scene(xyz, ids, flags=flags)
    rng = np.random.default_rng(12)
    n = 20000
    a = rng.uniform(1, 4095, (n, 3)).astype(np.float32)
    b = rng.uniform(1, 4095, (n, 3)).astype(np.float32)
    b[: n // 3, 2] = 60000.0  # out through the sky wall
    b[-10:] = a[-10:]  # zero length: visible
    for skip in (-1, 3):
        frac = env.test_line_coverage(a, b, static_prop_to_skip=skip)
        ref = s.test_lines_coverage(colours[:, 0], a, b, skip=0x04000000 | skip, threads=16)
        assert bits_equal(frac, ref)
    assert ((frac > 0) & (frac < 1)).sum() > 100 and (frac == 1).sum() > 10
    # without transparency every line is 0 or 1, as TestLineDoesHitSky gives;
    # transparent occluders let part of the light through
    plain = env.test_line_does_hit_sky(a, b, 3)
    assert set(np.unique(plain)) <= {0.0, 1.0}
    assert ((plain == 0) & (frac > 0)).sum() > 100
    assert not ((plain == 1) & (frac < 1)).any()
