"""Host algorithms of libvradgpu.so (no GPU: host-only context) against the
oracle: kd tree, intersection records, light parameters, patch subdivision,
and the C ABI's exported symbols."""
import ctypes as C

import numpy as np
import pytest

from conftest import bits_equal, small_lit_scene


def _env(host_ctx, xyz, ids):
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    env.add_triangles(xyz, ids)
    env.SetupAccelerationStructure()
    return env


def test_every_header_symbol_is_exported(vlib):
    from vrad_gb300 import _lib

    names = _lib.header_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(vlib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_header_is_plain_c(tmp_path):
    """The boundary header compiles as C99 and C11 with -pedantic, as a cgo
    preamble or a C caller includes it."""
    import shutil
    import subprocess
    from pathlib import Path

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = Path(__file__).resolve().parent.parent / "include"
    src = tmp_path / "use.c"
    src.write_text('#include "vradgpu.h"\n'
                   "int main(void) { vrg_bsp_world w = {0}; vrg_light l = {0};\n"
                   "  (void)w; (void)l; return VRG_OK; }\n")
    for std in ("c99", "c11"):
        r = subprocess.run([cc, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                            str(inc), "-c", str(src), "-o", str(tmp_path / "use.o")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("which", ["anyhit", "lit", "random"])
def test_kd_tree_matches_oracle(oracle, host_ctx, which, anyhit_scene, lit_scene):
    if which == "anyhit":
        xyz, ids = anyhit_scene.xyz, anyhit_scene.ids
    elif which == "lit":
        xyz, ids = lit_scene.xyz, lit_scene.ids
    else:  # arbitrary (non axis-aligned, overlapping) triangles
        rng = np.random.default_rng(5)
        c = rng.uniform(0, 1000, (3000, 1, 3))
        xyz = (c + rng.normal(0, 30, (3000, 3, 3))).reshape(-1, 9).astype(np.float32)
        ids = np.full(3000, 0x02000000, np.int32)
    env = _env(host_ctx, xyz, ids)
    ch, sp, refs, height = env.tree()
    s = oracle.Scene(xyz, ids)
    och, osp, orefs = s.tree()
    assert np.array_equal(ch, och)
    assert bits_equal(sp, osp)
    assert np.array_equal(refs, orefs)
    assert height < 32
    assert np.array_equal(env.triangle_records(), s.tri_records())


def _walk_tree_scene(which, anyhit_scene, lit_scene):
    rng = np.random.default_rng(11)
    if which == "anyhit":
        return anyhit_scene.xyz, anyhit_scene.ids, anyhit_scene.starts[:40000], \
            anyhit_scene.stops[:40000]
    if which == "lit":  # sky ceiling; lines from face points up and across
        xyz, ids = lit_scene.xyz, lit_scene.ids
        a = rng.uniform(1, 4095, (30000, 3)).astype(np.float32)
        b = a + rng.normal(0, 1500, (30000, 3)).astype(np.float32)
        b[::3, 2] = 4096.0 + 50.0  # through the sky ceiling
        return xyz, ids, a, b.astype(np.float32)
    # overlapping, non axis-aligned triangles and coplanar duplicates
    c = rng.uniform(0, 1000, (3000, 1, 3))
    xyz = (c + rng.normal(0, 30, (3000, 3, 3))).reshape(-1, 9).astype(np.float32)
    xyz[1::7] = xyz[::7][: len(xyz[1::7])]
    ids = np.full(3000, 0x02000000, np.int32)
    a = rng.uniform(-50, 1050, (30000, 3)).astype(np.float32)
    b = rng.uniform(-50, 1050, (30000, 3)).astype(np.float32)
    return xyz, ids, a, b


@pytest.mark.parametrize("which", ["anyhit", "lit", "random"])
def test_walk_tree_gives_the_reference_trees_answers(oracle, host_ctx, which, anyhit_scene,
                                                     lit_scene):
    # the device walks its own tree; the oracle's walk over that tree must
    # give the answers of the reference's tree and of brute force
    xyz, ids, a, b = _walk_tree_scene(which, anyhit_scene, lit_scene)
    env = _env(host_ctx, xyz, ids)
    ch, sp, refs, height = env.walk_tree()
    assert height < 32
    assert np.array_equal(np.unique(refs), np.arange(len(ids)))  # every triangle in a leaf
    ref = oracle.Scene(xyz, ids)
    walk = oracle.Scene(xyz, ids)
    walk.set_tree(ch, sp, refs)
    m0, h0, t0 = ref.occlusion_mask(a, b, threads=16, closest=True)
    m1, h1, t1 = walk.occlusion_mask(a, b, threads=16, closest=True)
    assert np.array_equal(m0, m1) and np.array_equal(h0, h1) and bits_equal(t0, t1)
    d = (b - a).astype(np.float32)
    o = a[:4000]
    hb, tb = ref.trace_closest(o, d[:4000], 0.0, 1.0, brute=True, threads=16)
    hw, tw = walk.trace_closest(o, d[:4000], 0.0, 1.0, threads=16)
    assert np.array_equal(hb, hw) and bits_equal(tb, tw)
    assert np.array_equal(walk.test_lines(a, b, threads=16), ref.test_lines(a, b, threads=16))
    # the walk that never enters leaves without triangles: same answers and
    # fewer nodes on average (a far child it descends into directly skips
    # the closest-hit pruning a pop applies, so a few lines visit more)
    _, _, _, st0 = walk.occlusion_mask(a, b, threads=16, closest=True, stats=True)
    walk.set_skip_empty(True)
    m2, h2, t2, st2 = walk.occlusion_mask(a, b, threads=16, closest=True, stats=True)
    assert np.array_equal(m0, m2) and np.array_equal(h0, h2) and bits_equal(t0, t2)
    assert st2[:, 0].mean() < st0[:, 0].mean()
    assert np.mean(st2[:, 0] > st0[:, 0]) < 0.01


@pytest.mark.parametrize("n", [0, 1, 2, 3, 7, 25])
def test_walk_tree_small_and_degenerate(oracle, host_ctx, n):
    rng = np.random.default_rng(n)
    xyz = rng.uniform(0, 10, (n, 9)).astype(np.float32)
    if n >= 3:
        xyz[0, 2::3] = 1.0
        xyz[1] = xyz[1, :3].tolist() * 3
    ids = np.full(n, 0x02000000, np.int32)
    env = _env(host_ctx, xyz, ids)
    ch, sp, refs, height = env.walk_tree()
    assert len(ch) >= 1 and height < 32
    if n:
        assert np.array_equal(np.unique(refs), np.arange(n))
        walk = oracle.Scene(xyz, ids)
        walk.set_tree(ch, sp, refs)
        a = rng.uniform(-1, 11, (2000, 3)).astype(np.float32)
        b = rng.uniform(-1, 11, (2000, 3)).astype(np.float32)
        ref = oracle.Scene(xyz, ids)
        _, h0, t0 = ref.occlusion_mask(a, b, threads=4, closest=True)
        _, h1, t1 = walk.occlusion_mask(a, b, threads=4, closest=True)
        assert np.array_equal(h0, h1) and bits_equal(t0, t1)


def test_walk_tree_costs_are_checked(host_ctx, anyhit_scene):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    with pytest.raises(VrgError):
        env.set_walk_tree_costs(max_depth=32)
    with pytest.raises(VrgError):
        env.set_walk_tree_costs(empty_bonus=1.5)
    with pytest.raises(VrgError):
        env.set_walk_tree_builder(2)
    env.set_walk_tree_builder(1)  # a host-only context still builds on the host
    env.set_walk_tree_costs(1.0, 1.5, 0.9, 20)
    env.add_triangles(anyhit_scene.xyz[:600], anyhit_scene.ids[:600])
    env.SetupAccelerationStructure()
    assert env.walk_tree()[3] <= 20
    with pytest.raises(VrgError):
        env.set_walk_tree_costs()


@pytest.mark.parametrize("n", [0, 1, 2, 3, 7, 25])
def test_kd_tree_small_and_degenerate(oracle, host_ctx, n):
    rng = np.random.default_rng(n)
    xyz = rng.uniform(0, 10, (n, 9)).astype(np.float32)
    if n >= 3:
        xyz[0, 2::3] = 1.0  # a triangle flat in z
        xyz[1] = xyz[1, :3].tolist() * 3  # a degenerate (point) triangle
    ids = np.full(n, 0x02000000, np.int32)
    env = _env(host_ctx, xyz, ids)
    ch, sp, refs, _ = env.tree()
    och, osp, orefs = oracle.Scene(xyz, ids).tree()
    assert np.array_equal(ch, och) and bits_equal(sp, osp) and np.array_equal(refs, orefs)


def test_axis_aligned_solid_and_quad_match_soup(host_ctx):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    env.AddAxisAlignedRectangularSolid(0x02000000, (1, 2, 3), (4, 6, 9))
    env.AddQuad(0x01000000, (0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    env.SetupAccelerationStructure()
    soup = scenes.TriangleSoup()
    soup.add_box(0x02000000, (1, 2, 3), (4, 6, 9))
    soup.add_quad(0x01000000, (0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0))
    xyz, ids = soup.arrays()
    recs = env.triangle_records()
    assert env.num_triangles() == 14
    assert recs[:, 4].view(np.int32).tolist() == ids.tolist()


def test_lights_match_oracle(oracle, lit_scene):
    from vrad_gb300.environment import light_array
    from vrad_gb300.scenes import Light

    extra = [Light(1, (1, 2, 3), (10, 20, 30), keys=dict(fifty_percent_distance=120.0,
                                                         zero_percent_distance=500.0)),
             Light(1, (1, 2, 3), (10, 20, 30), keys=dict(fifty_percent_distance=120.0,
                                                         zero_percent_distance=500.0,
                                                         hard_falloff=1)),
             Light(1, (1, 2, 3), (10, 20, 30), keys=dict(constant_attn=1.0, linear_attn=0.5)),
             Light(2, (1, 2, 3), (1, 1, 1), (0, 0, -1), keys=dict(inner_cone=120.0, cone=150.0))]
    lights = lit_scene.lights + extra
    mine = light_array(lights)
    ref = oracle.make_lights(lights)
    n = len(lights)
    assert bytes(mine)[: 80 * n] == bytes(ref)[: 80 * n]


def test_patches_match_oracle(oracle, host_ctx):
    lit = small_lit_scene(240)
    env = _env(host_ctx, lit.xyz, lit.ids)
    env.set_faces(lit)
    P = env.make_patches()
    O = oracle.make_patches(lit)
    for k in ("mins", "maxs", "center", "area", "split_dist"):
        assert bits_equal(P[k], O[k]), k
    for k in ("face", "parent", "child1", "child2", "split_axis", "leaf_index"):
        assert np.array_equal(P[k], O[k]), k
    assert P["n_leaves"] == int((O["leaf_index"] >= 0).sum())
    # every leaf spans < 4 luxels (64 units at 16-unit luxels) on each axis
    leaf = O["leaf_index"] >= 0
    ext = (O["maxs"] - O["mins"])[leaf] / 16.0
    assert (ext < 4.0).all()


def test_device_calls_refused_on_host_context(host_ctx, anyhit_scene):
    from vrad_gb300._lib import VrgError

    env = _env(host_ctx, anyhit_scene.xyz[:100], anyhit_scene.ids[:100])
    with pytest.raises(VrgError, match="call out of order"):
        env.occlusion_mask(anyhit_scene.starts[:4], anyhit_scene.stops[:4])


def test_bad_inputs_are_rejected(host_ctx, vlib):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    env.AddTriangle(1, (0, 0, 0), (1, 0, 0), (0, 1, 0))
    # tracing before SetupAccelerationStructure
    with pytest.raises(VrgError):
        env.occlusion_mask(np.zeros((1, 3)), np.ones((1, 3)))
    env.SetupAccelerationStructure()
    # adding triangles after the build
    with pytest.raises(VrgError, match="call out of order"):
        env.AddTriangle(1, (0, 0, 0), (1, 0, 0), (0, 1, 0))
    # null pointers
    assert vlib.vrg_env_add_triangle(env.h, 1, None, None, None, None, 0, 0) == -1
    h = C.c_void_p()
    assert vlib.vrg_ctx_create(0, None) == -1
    assert vlib.vrg_env_create(None, C.byref(h)) == -1


def test_wall_slots_and_their_shortcut_keep_the_verdicts(oracle, host_ctx):
    # the room's opaque walls and floor fill the wall slots (the sky ceiling
    # does not); shadow lines that test them before walking get the same
    # verdicts, bit for bit, with fewer nodes walked
    from vrad_gb300 import scenes

    lit = small_lit_scene(96, seed=7)
    env = _env(host_ctx, lit.xyz, lit.ids)
    env.set_faces(lit)
    tris, counts = env.wall_slots()
    assert counts.tolist() == [2, 2, 2, 2, 2, 0]  # x min/max, y min/max, z min (floor), z max (sky)
    for f in range(5):
        a, side = divmod(f, 2)
        for t in tris[f, :2]:
            v = lit.xyz[t].reshape(3, 3)
            assert (v[:, a] == (scenes.ROOM if side else 0.0)).all()
            assert lit.ids[t] & scenes.TRACE_ID_SKY == 0
    s = oracle.Scene(lit.xyz, lit.ids)
    lights = oracle.make_lights(lit.lights)
    ref, rays, st0 = oracle.gather_luxels(s, lights, len(lit.lights), lit, 0, lit.n_faces, ss=4,
                                          seed=3, threads=16, stats=True)
    s.set_walls(tris, counts)
    got, rays2, st1 = oracle.gather_luxels(s, lights, len(lit.lights), lit, 0, lit.n_faces, ss=4,
                                           seed=3, threads=16, stats=True)
    assert rays == rays2 and bits_equal(got, ref)
    assert st1[1] < 0.8 * st0[1]  # kd nodes
    # arbitrary lines through the room, through its walls and out of it
    rng = np.random.default_rng(4)
    a = rng.uniform(1, 4095, (20000, 3)).astype(np.float32)
    b = (a + rng.normal(0, 6000, (20000, 3))).astype(np.float32)
    f_walls = s.test_lines(a, b, threads=16)
    s.set_walls()
    assert np.array_equal(f_walls, s.test_lines(a, b, threads=16))


def test_set_triangle_flags_errors(host_ctx):
    from vrad_gb300 import scenes
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    sc = scenes.anyhit_scene(1, n_boxes=4, n_rays=16)
    xyz, ids = sc.xyz, sc.ids
    flags = np.zeros(len(ids), np.uint8)
    flags[12:] = 1
    colours = np.full((len(ids), 3), 0.5, np.float32)
    env = Environment(host_ctx)
    env.add_triangles(xyz, ids)
    with pytest.raises(VrgError):
        env.set_triangle_flags(len(ids) - 2, flags[:4])  # past the last triangle
    env.set_triangle_flags(0, flags, colours)
    env.SetupAccelerationStructure()
    with pytest.raises(VrgError, match="out of order"):
        env.set_triangle_flags(0, flags)  # after the build
