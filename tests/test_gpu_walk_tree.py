"""The walk tree built on the GPU (binned SAH): every triangle in a leaf,
depth within the traversal stack, and the answers of the reference's tree --
checked by the oracle walking the device-built tree and by the device
walking it against the host-built one."""
import numpy as np
import pytest

from conftest import bits_equal, small_lit_scene

pytestmark = pytest.mark.gpu


def _scene(which, anyhit_scene, lit_scene):
    if which == "anyhit":
        return anyhit_scene.xyz, anyhit_scene.ids, anyhit_scene.starts[:200000], \
            anyhit_scene.stops[:200000]
    if which == "lit":
        rng = np.random.default_rng(3)
        a = rng.uniform(1, 4095, (100000, 3)).astype(np.float32)
        b = (a + rng.normal(0, 1500, (100000, 3))).astype(np.float32)
        b[::3, 2] = 4146.0
        return lit_scene.xyz, lit_scene.ids, a, b
    rng = np.random.default_rng(5)  # overlapping, non axis-aligned, coplanar duplicates
    c = rng.uniform(0, 1000, (3000, 1, 3))
    xyz = (c + rng.normal(0, 30, (3000, 3, 3))).reshape(-1, 9).astype(np.float32)
    xyz[1::7] = xyz[::7][: len(xyz[1::7])]
    ids = np.full(3000, 0x02000000, np.int32)
    a = rng.uniform(-50, 1050, (50000, 3)).astype(np.float32)
    b = rng.uniform(-50, 1050, (50000, 3)).astype(np.float32)
    return xyz, ids, a, b


@pytest.mark.parametrize("which", ["anyhit", "lit", "random"])
def test_device_built_walk_tree(gpu_ctx, oracle, anyhit_scene, lit_scene, which):
    from vrad_gb300.environment import Environment

    xyz, ids, a, b = _scene(which, anyhit_scene, lit_scene)
    envs = {}
    for on_device in (True, False):
        env = Environment(gpu_ctx)
        env.set_walk_tree_builder(on_device)
        env.add_triangles(xyz, ids)
        env.SetupAccelerationStructure()
        envs[on_device] = env
    ch, sp, refs, height = envs[True].walk_tree()
    assert height < 32
    assert np.array_equal(np.unique(refs), np.arange(len(ids)))
    # the oracle walking the device-built tree answers as the reference's tree
    ref = oracle.Scene(xyz, ids)
    walk = oracle.Scene(xyz, ids)
    walk.set_tree(ch, sp, refs)
    n = min(len(a), 60000)
    m0, h0, t0 = ref.occlusion_mask(a[:n], b[:n], threads=16, closest=True)
    m1, h1, t1 = walk.occlusion_mask(a[:n], b[:n], threads=16, closest=True)
    assert np.array_equal(m0, m1) and np.array_equal(h0, h1) and bits_equal(t0, t1)
    # the device on either tree: the same masks, hits and distances
    md, hd, td = envs[True].occlusion_mask(a, b, closest=True)
    mh, hh, th = envs[False].occlusion_mask(a, b, closest=True)
    assert np.array_equal(md, mh) and np.array_equal(hd, hh) and bits_equal(td, th)
    assert np.array_equal(md[: n // 32], m0[: n // 32])


@pytest.mark.parametrize("n", [0, 1, 2, 3, 7, 25, 300])
def test_device_built_walk_tree_small(gpu_ctx, oracle, n):
    from vrad_gb300.environment import Environment

    rng = np.random.default_rng(n)
    xyz = rng.uniform(0, 10, (n, 9)).astype(np.float32)
    if n >= 3:
        xyz[0, 2::3] = 1.0
        xyz[1] = xyz[1, :3].tolist() * 3
    ids = np.full(n, 0x02000000, np.int32)
    env = Environment(gpu_ctx)
    env.set_walk_tree_builder(1)
    env.add_triangles(xyz, ids)
    env.SetupAccelerationStructure()
    ch, sp, refs, height = env.walk_tree()
    assert len(ch) >= 1 and height < 32
    if n:
        assert np.array_equal(np.unique(refs), np.arange(n))
        a = rng.uniform(-1, 11, (5000, 3)).astype(np.float32)
        b = rng.uniform(-1, 11, (5000, 3)).astype(np.float32)
        m, h, t = env.occlusion_mask(a, b, closest=True)
        rm, rh, rt = oracle.Scene(xyz, ids).occlusion_mask(a, b, threads=4, closest=True)
        assert np.array_equal(m, rm) and np.array_equal(h, rh) and bits_equal(t, rt)


def test_direct_light_on_device_built_tree(gpu_ctx):
    from vrad_gb300.environment import Environment

    lit = small_lit_scene(96, seed=12)
    out = {}
    for on_device in (True, False):
        env = Environment(gpu_ctx)
        env.set_walk_tree_builder(on_device)
        env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        env.set_faces(lit)
        env.set_lights(lit.lights)
        out[on_device] = env.gather_direct_light(supersamples=4, seed=2)
    assert out[True][1] == out[False][1]
    assert bits_equal(out[True][0], out[False][0])


def test_large_scene_builds_on_the_gpu_by_default(gpu_ctx, oracle):
    # 72,012 triangles through the default builder (the GPU's)
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    sc = scenes.anyhit_scene(3, n_boxes=6000, n_rays=30000)
    env = Environment(gpu_ctx)
    env.add_triangles(sc.xyz, sc.ids)
    env.SetupAccelerationStructure()
    ch, sp, refs, height = env.walk_tree()
    assert height < 32 and np.array_equal(np.unique(refs), np.arange(len(sc.ids)))
    m, h, t = env.occlusion_mask(sc.starts, sc.stops, closest=True)
    rm, rh, rt = oracle.Scene(sc.xyz, sc.ids).occlusion_mask(sc.starts, sc.stops, threads=16,
                                                             closest=True)
    assert np.array_equal(m, rm) and np.array_equal(h, rh) and bits_equal(t, rt)
