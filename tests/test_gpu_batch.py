"""Whole bakes: the one-scene path (vrg_env_bake) against the oracle, and the
batched path (vrg_batch_bake: one persistent direct launch over every
scene, block-diagonal bounce with per-scene stops) against the one-scene
path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _make_env(ctx, lit, k=128):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    env = Environment(ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    env.make_transfers(scenes.transfer_directions(k))
    return env, P["n_leaves"]


@pytest.fixture(scope="module")
def small_batch(gpu_ctx):
    from vrad_gb300 import scenes

    lits = [scenes.lit_scene(40 + i, n_faces=n, spacing=24.0, n_point=10, n_spot=3)
            for i, n in enumerate([12, 90, 31, 64, 7])]
    envs = [_make_env(gpu_ctx, lit) for lit in lits]
    return lits, envs


def test_plain_bake_matches_oracle(small_batch, oracle):
    lits, envs = small_batch
    lit, (env, nl) = lits[1], envs[1]
    rays = env.bake(supersamples=4, seed=3, max_bounces=6, rel_tol=0.0)
    res = env.get_bake(nl)
    s = oracle.Scene(lit.xyz, lit.ids)
    lights = oracle.make_lights(lit.lights)
    ref, rrays = oracle.gather_luxels(s, lights, len(lit.lights), lit, 0, lit.n_faces, ss=4,
                                      seed=3, threads=16)
    err = np.abs(res["luxels"] - ref) / np.maximum(np.abs(ref), 1e-3 * ref.max())
    assert err.max() <= 1e-4
    assert rays > rrays  # luxel rays plus the patch-centre rays
    assert res["bounces"] == 6


@pytest.mark.parametrize("tol,max_b", [(0.0, 5), (1e-3, 60)])
def test_batched_bake_equals_plain(small_batch, gpu_ctx, tol, max_b):
    from vrad_gb300.environment import Batch

    lits, envs = small_batch
    plain = []
    plain_rays = 0
    for env, nl in envs:
        plain_rays += env.bake(4, 7, max_b, tol)
        plain.append(env.get_bake(nl))
    batch = Batch(gpu_ctx)
    for env, _ in envs:
        batch.add(env)
    rays = batch.bake(4, 7, max_b, tol)
    assert rays == plain_rays
    for (env, nl), p in zip(envs, plain):
        b = env.get_bake(nl)
        assert np.array_equal(b["luxels"], p["luxels"])
        assert np.array_equal(b["patch_direct"], p["patch_direct"])
        if tol == 0.0:
            assert b["bounces"] == p["bounces"] == max_b
            assert np.array_equal(b["patch_total"], p["patch_total"])
        else:
            assert abs(b["bounces"] - p["bounces"]) <= 1
            scale = max(np.abs(p["patch_total"]).max(), 1e-30)
            err = np.abs(b["patch_total"] - p["patch_total"]) / np.maximum(
                np.abs(p["patch_total"]), 1e-6 * scale)
            assert err.max() <= 1e-3


def test_batch_rejects_unprepared_scene(gpu_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Batch, Environment

    env = Environment(gpu_ctx)
    env.AddAxisAlignedRectangularSolid(0x02000000, (0, 0, 0), (1, 1, 1))
    env.SetupAccelerationStructure()
    batch = Batch(gpu_ctx)
    batch.add(env)
    with pytest.raises(VrgError, match="call out of order"):
        batch.bake()


def test_batch_gather_variants_identical(small_batch, gpu_ctx, tmp_path):
    # the register walk and the walk with its constants in shared memory give
    # the same luxels, leaf-point light and shadow-ray count
    from vrad_gb300.environment import Batch, Context

    lits, envs = small_batch
    tris = sum(env.num_triangles() for env, _ in envs)
    items = sum(env.num_luxels() * 4 + nl for env, nl in envs)
    key = Context.tune_key("batch_gather", tris, items)
    outs = []
    for v in range(3):
        p = tmp_path / f"tune_batch_{v}.txt"
        p.write_text(f"{key} {v}\n")
        gpu_ctx.autotune_load(str(p))
        assert gpu_ctx.autotune_choice(key)[0] == v
        batch = Batch(gpu_ctx)
        for env, _ in envs:
            batch.add(env)
        rays = batch.bake(4, 11, 3, 0.0)
        outs.append((rays, [env.get_bake(nl) for env, nl in envs]))
    r0, b0 = outs[0]
    assert r0 > 0
    for r1, b1 in outs[1:]:
        assert r1 == r0
        for x, y in zip(b0, b1):
            assert np.array_equal(x["luxels"], y["luxels"])
            assert np.array_equal(x["patch_direct"], y["patch_direct"])
            assert np.array_equal(x["patch_total"], y["patch_total"])
