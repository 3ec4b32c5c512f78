"""Edge cases through the C ABI on the GPU: empty batches, ragged sizes
around the 32-line mask words and warp claims, lines starting on a
triangle's plane (also through every tuned walk variant, with lines along
the axes), and a relight that changes nothing."""
import numpy as np
import pytest

from conftest import bits_equal, small_lit_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env_and_oracle(gpu_ctx, oracle, anyhit_scene):
    from vrad_gb300.environment import Environment

    env = Environment(gpu_ctx)
    env.add_triangles(anyhit_scene.xyz, anyhit_scene.ids)
    env.SetupAccelerationStructure()
    return env, oracle.Scene(anyhit_scene.xyz, anyhit_scene.ids)


def test_empty_batches(env_and_oracle):
    env, _ = env_and_oracle
    z = np.zeros((0, 3), np.float32)
    assert env.occlusion_mask(z, z).shape == (0,)
    m, h, t = env.occlusion_mask(z, z, closest=True)
    assert m.shape == h.shape == t.shape == (0,)
    h, t = env.trace_closest(z, z, 0.0, 1.0)
    assert h.shape == (0,)
    assert env.test_line_does_hit_sky(z, z).shape == (0,)


@pytest.mark.parametrize("n", [1, 31, 32, 33, 127, 4097, 100003])
def test_ragged_line_counts(env_and_oracle, anyhit_scene, n):
    env, osc = env_and_oracle
    a, b = anyhit_scene.starts[:n], anyhit_scene.stops[:n]
    mask, hit, t = env.occlusion_mask(a, b, closest=True)
    rmask, rhit, rt = osc.occlusion_mask(a, b, threads=16, closest=True)
    assert np.array_equal(mask, rmask)
    assert np.array_equal(hit, rhit) and bits_equal(t, rt)


def test_lines_from_triangle_planes(env_and_oracle, anyhit_scene):
    # lines that start exactly on a box face (t = 0 hits) and lines that
    # end exactly on one (t = len, excluded by tmin <= t < tmax)
    env, osc = env_and_oracle
    xyz = anyhit_scene.xyz.reshape(-1, 3, 3)
    rng = np.random.default_rng(5)
    pick = rng.choice(len(xyz), size=4000, replace=False)
    on = xyz[pick].mean(axis=1).astype(np.float32)  # centroids lie on their triangles
    far = rng.uniform(1, 4095, (4000, 3)).astype(np.float32)
    for a, b in ((on, far), (far, on)):
        mask = env.occlusion_mask(a, b)
        assert np.array_equal(mask, osc.occlusion_mask(a, b, threads=16))


def test_every_walk_variant_on_plane_and_axis_lines(gpu_ctx, oracle, anyhit_scene, tmp_path):
    # each tuned form of the shadow-line walk, forced in turn, on lines that
    # start or end on a triangle's plane and on lines along the axes (zero
    # direction components, walked through the reciprocal guard): the mask,
    # hit indices and t equal the oracle's
    from vrad_gb300.environment import Context, Environment

    xyz = anyhit_scene.xyz.reshape(-1, 3, 3)
    rng = np.random.default_rng(9)
    on = xyz[rng.choice(len(xyz), size=1500, replace=False)].mean(axis=1).astype(np.float32)
    far = rng.uniform(1, 4095, (1500, 3)).astype(np.float32)
    o = rng.uniform(1, 4095, (1500, 3)).astype(np.float32)
    ax = o.copy()
    for i in range(1500):
        ax[i, i % 3] = np.float32(4095.0 - o[i, i % 3])  # the other two coordinates kept
    a = np.concatenate([on, far, o])
    b = np.concatenate([far, on, ax])
    env = Environment(gpu_ctx)
    env.add_triangles(anyhit_scene.xyz, anyhit_scene.ids)
    env.SetupAccelerationStructure()
    osc = oracle.Scene(anyhit_scene.xyz, anyhit_scene.ids)
    rmask = osc.occlusion_mask(a, b, threads=16)
    _, rhit, rt = osc.occlusion_mask(a, b, threads=16, closest=True)
    for closest in (False, True):
        key = Context.tune_key("trace_mask_hit" if closest else "trace_mask", env.num_triangles(), len(a))
        for v in range(20):
            p = tmp_path / f"tune_{closest}_{v}.txt"
            p.write_text(f"{key} {v}\n")
            gpu_ctx.autotune_load(str(p))
            if closest:
                m, h, t = env.occlusion_mask(a, b, closest=True)
                assert np.array_equal(h, rhit) and bits_equal(t, rt), v
            else:
                m = env.occlusion_mask(a, b)
            assert np.array_equal(m, rmask), (closest, v)


def test_relight_without_change_keeps_the_bake(gpu_ctx):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment, make_light

    lit = small_lit_scene(48, seed=21)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    env.make_transfers(scenes.transfer_directions(128))
    env.relight_prepare(4, 3, 100, 1e-4)
    before = env.get_bake(P["n_leaves"])
    li = lit.lights[0]
    same = make_light(li.type, li.origin, li.intensity, li.normal, **li.keys)
    env.relight([], max_iters=50, rel_tol=1e-4)
    env.relight([(0, same)], max_iters=50, rel_tol=1e-4)  # an edit to the same values
    after = env.get_bake(P["n_leaves"])
    assert np.array_equal(before["luxels"], after["luxels"])
    assert np.array_equal(before["patch_direct"], after["patch_direct"])
    scale = max(np.abs(before["patch_total"]).max(), 1e-30)
    err = np.abs(after["patch_total"] - before["patch_total"]) / np.maximum(
        np.abs(before["patch_total"]), 1e-6 * scale)
    assert err.max() <= 1e-3


def test_page_locked_inputs_are_read_in_place(env_and_oracle, anyhit_scene):
    # page-locked end points go to the walk without a copy; the answers are
    # those of pageable inputs (which are copied first)
    import ctypes as C

    import torch

    env, _ = env_and_oracle
    n = 50000
    a, b = anyhit_scene.starts[:n], anyhit_scene.stops[:n]
    want = env.occlusion_mask(a, b, closest=True)
    ha = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hb = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
    mask = np.zeros((n + 31) // 32, np.uint32)
    hit = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    rc = env.lib.vrg_env_occlusion_mask(env.h, C.c_void_p(ha.data_ptr()), C.c_void_p(hb.data_ptr()), n,
                                        -1, mask.ctypes.data, hit.ctypes.data, t.ctypes.data)
    assert rc == 0
    assert np.array_equal(mask, want[0]) and np.array_equal(hit, want[1]) and bits_equal(t, want[2])


def test_page_locked_rays_and_lines(env_and_oracle, anyhit_scene):
    import ctypes as C

    import torch

    env, _ = env_and_oracle
    n = 20000
    a, b = anyhit_scene.starts[:n], anyhit_scene.stops[:n]
    d = (b - a).astype(np.float32)
    ln = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
    dn = (d * (np.float32(1.0) / ln)[:, None]).astype(np.float32)
    want_h, want_t = env.trace_closest(a, dn, 0.0, ln)
    want_f = env.test_line_does_hit_sky(a, b)
    pin = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
           for x in (a, dn, np.zeros(n, np.float32), ln, b)]
    hit = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    frac = np.empty(n, np.float32)
    p = [C.c_void_p(x.data_ptr()) for x in pin]
    assert env.lib.vrg_env_trace_closest(env.h, p[0], p[1], p[2], p[3], n, -1, hit.ctypes.data,
                                         t.ctypes.data) == 0
    assert env.lib.vrg_env_test_line_does_hit_sky(env.h, p[0], p[4], n, -1, frac.ctypes.data) == 0
    assert np.array_equal(hit, want_h) and bits_equal(t, want_t)
    assert np.array_equal(frac, want_f)


def test_wall_slots_respect_the_skip_id(gpu_ctx, oracle):
    # a room whose walls are one static prop: skipping that prop lets lines
    # through the walls (the wall test must skip them as the walk does)
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    prop = scenes.TRACE_ID_STATICPROP | 5
    soup = scenes.TriangleSoup()
    soup.add_box(prop, (0.0, 0.0, 0.0), (scenes.ROOM,) * 3, ceiling_id=scenes.TRACE_ID_SKY)
    soup.add_box(scenes.TRACE_ID_OPAQUE, (1000.0, 1000.0, 1000.0), (1500.0, 1500.0, 1500.0))
    xyz, ids = soup.arrays()
    env = Environment(gpu_ctx)
    env.add_triangles(xyz, ids)
    env.SetupAccelerationStructure()
    tris, counts = env.wall_slots()
    assert counts[:5].tolist() == [2, 2, 2, 2, 2] and counts[5] == 0
    rng = np.random.default_rng(8)
    a = rng.uniform(1, 4095, (20000, 3)).astype(np.float32)
    b = (a + rng.normal(0, 8000, (20000, 3))).astype(np.float32)  # most leave the room
    s = oracle.Scene(xyz, ids)
    for skip_prop in (-1, 5):
        got = env.test_line_does_hit_sky(a, b, skip_prop)
        want = s.test_lines(a, b, skip=(prop if skip_prop == 5 else -1), threads=16)
        assert np.array_equal(got, want)
    assert (env.test_line_does_hit_sky(a, b, 5) == 1.0).mean() > 0.5
