"""Lightmap samples on the device (vrg_env_get_lightmap): bit-identical to the
oracle fed the same bake (luxel direct light and leaf bounced light), on a
small scene, on the 4,096-face bake and on faces too large for the kernel's
shared copy of a face's patch tree; face offsets; call-order errors."""
import numpy as np
import pytest

from conftest import small_lit_scene

pytestmark = pytest.mark.gpu


def _face_root(P, n_faces):
    root = np.full(n_faces, -1, np.int32)
    for i in range(len(P["face"]) - 1, -1, -1):
        if P["parent"][i] < 0:
            root[P["face"][i]] = i
    return root


def _baked(ctx, lit, k=128, max_bounces=8):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    env = Environment(ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    P["face_root"] = _face_root(P, lit.n_faces)
    env.make_transfers(scenes.transfer_directions(k))
    env.bake(supersamples=4, seed=5, max_bounces=max_bounces, rel_tol=0.0)
    return env, P


@pytest.mark.parametrize("which", ["small", "full"])
def test_lightmap_matches_oracle(gpu_ctx, oracle, lit_scene, which):
    lit = small_lit_scene(96, seed=21) if which == "small" else lit_scene
    env, P = _baked(gpu_ctx, lit)
    res = env.get_bake(P["n_leaves"])
    assert np.abs(res["patch_total"]).max() > 0  # the bounce term is exercised
    samples, offsets = env.get_lightmap()
    assert samples.shape == (lit.n_luxels, 4)
    assert np.array_equal(offsets, 4 * lit.luxel_offset())
    want = oracle.lightmap(lit, P, res["luxels"], res["patch_total"])
    assert np.array_equal(samples.view("<u4").ravel(), want)


def test_lightmap_large_faces_match_oracle(gpu_ctx, oracle):
    # faces of up to 2,400 units at 32-unit luxels split into more than 128
    # leaf patches (over 256 tree nodes), more than the kernel's shared copy
    # holds: those faces are walked in global memory, beside faces that fit
    from vrad_gb300 import scenes

    lit = scenes.lit_scene(5, n_faces=18, spacing=32.0, n_point=6, n_spot=2, edge=(300.0, 2400.0))
    env, P = _baked(gpu_ctx, lit, k=64, max_bounces=4)
    leaves = np.bincount(np.asarray(P["face"])[np.asarray(P["leaf_index"]) >= 0], minlength=lit.n_faces)
    assert leaves.max() > 128 and leaves.min() <= 128  # both paths run
    res = env.get_bake(P["n_leaves"])
    samples, _ = env.get_lightmap()
    want = oracle.lightmap(lit, P, res["luxels"], res["patch_total"])
    assert np.array_equal(samples.view("<u4").ravel(), want)


def test_lightmap_call_order(gpu_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    lit = small_lit_scene(24, seed=4)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    with pytest.raises(VrgError, match="out of order"):
        env.get_lightmap()  # no bake yet
    env2, _ = _baked(gpu_ctx, lit, max_bounces=2)
    env2.get_lightmap()
    env2.make_patches(8.0, 8.0)  # new leaves: the old bounced light no longer fits
    with pytest.raises(VrgError, match="out of order"):
        env2.get_lightmap()
