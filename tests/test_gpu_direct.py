"""GPU parity of direct-light gathering: luxel RGB within 1e-4 relative of
the oracle (the arithmetic is the same float32 sequence, so most luxels are
bit-identical; powf is the one library call whose last bit may differ)."""
import numpy as np
import pytest

from conftest import small_lit_scene

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def _rel_err(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    den = np.maximum(np.abs(b), 1e-3 * max(np.abs(b).max(), 1e-30))
    return np.abs(a - b) / den


@pytest.fixture(scope="module")
def lit_env(gpu_ctx, lit_scene):
    from vrad_gb300.environment import Environment

    env = Environment(gpu_ctx)
    env.add_triangles(lit_scene.xyz, lit_scene.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit_scene)
    env.set_lights(lit_scene.lights)
    return env


def test_direct_luxels_config_subset(lit_env, lit_scene, oracle):
    # the full 4,096-face bake on the GPU, compared on a slice of faces
    rgb, rays = lit_env.gather_direct_light(supersamples=4, seed=0)
    assert rgb.shape == (lit_scene.n_luxels, 3)
    assert np.isfinite(rgb).all() and (rgb >= 0).all()
    s = oracle.Scene(lit_scene.xyz, lit_scene.ids)
    lights = oracle.make_lights(lit_scene.lights)
    off = lit_scene.luxel_offset()
    for f0, f1 in ((0, 24), (2000, 2016), (4080, 4096)):
        ref, _ = oracle.gather_luxels(s, lights, len(lit_scene.lights), lit_scene, f0, f1, ss=4,
                                      seed=0, threads=16)
        got = rgb[off[f0]:off[f1]]
        err = _rel_err(got, ref)
        assert err.max() <= RTOL, f"faces {f0}-{f1}: max rel err {err.max():.3g}"
    assert rays > 100 * lit_scene.n_luxels  # ~86 shadow rays per sample


def test_direct_small_scene_every_luxel_and_ray_count(gpu_ctx, oracle):
    from vrad_gb300.environment import Environment

    lit = small_lit_scene(96)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    for ss in (1, 4):
        rgb, rays = env.gather_direct_light(supersamples=ss, seed=5)
        s = oracle.Scene(lit.xyz, lit.ids)
        lights = oracle.make_lights(lit.lights)
        ref, rrays = oracle.gather_luxels(s, lights, len(lit.lights), lit, 0, lit.n_faces, ss=ss,
                                          seed=5, threads=16)
        assert rays == rrays
        assert _rel_err(rgb, ref).max() <= RTOL
        exact = np.mean(rgb.view(np.uint32) == ref.view(np.uint32))
        assert exact > 0.99


def test_gather_points_with_fades_and_exponent(gpu_ctx, oracle, lit_scene):
    # lights that exercise the 50%-distance curve, hard falloff, a sun and a
    # spot exponent that goes through powf
    from vrad_gb300.environment import Environment
    from vrad_gb300.scenes import Light

    lights = [Light(1, (2000, 2000, 2000), (300, 200, 100),
                    keys=dict(fifty_percent_distance=300.0, zero_percent_distance=900.0)),
              Light(1, (1000, 3000, 2500), (300, 200, 100),
                    keys=dict(fifty_percent_distance=300.0, zero_percent_distance=900.0,
                              hard_falloff=1)),
              Light(2, (2000, 1000, 3000), (500, 500, 500), (0.0, 0.6, -0.8),
                    keys=dict(inner_cone=20.0, cone=60.0, exponent=2.5, quadratic_attn=1.0)),
              Light(3, (0, 0, 0), (5, 5, 5), (0.3, 0.2, -0.93)),
              Light(5, (0, 0, 0), (40, 50, 70))]
    env = Environment(gpu_ctx)
    env.add_triangles(lit_scene.xyz, lit_scene.ids)
    env.SetupAccelerationStructure()
    env.set_lights(lights)
    rng = np.random.default_rng(4)
    pts = rng.uniform(1, 4095, (4096, 3)).astype(np.float32)
    nrm = rng.normal(size=(4096, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    got, rays = env.gather_points(pts, nrm)
    s = oracle.Scene(lit_scene.xyz, lit_scene.ids)
    ref, rrays = oracle.gather_points(s, oracle.make_lights(lights), len(lights), pts, nrm,
                                      threads=16)
    assert rays == rrays
    assert _rel_err(got, ref).max() <= RTOL


def test_wall_cells_holding_more_triangles_than_they_list(gpu_ctx, oracle):
    # room faces cut into 80 x 80 tiles under a 32 x 32 grid: a cell overlaps
    # up to 9 tiles (18 triangles) and lists the 8 largest, so many lines
    # miss the listed ones and are walked; the luxels are the oracle's all
    # the same, with the cells on or off
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = scenes.lit_scene(8, n_faces=64, n_point=10, n_spot=3, wall_tiles=80)
    outs = []
    for cells in (True, False):
        env = Environment(gpu_ctx)
        env.set_wall_slots(cells)
        env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        counts = env.wall_slots()[1]
        assert (counts == 4).sum() == (5 if cells else 0)  # walls and floor, the sky face has none
        env.set_faces(lit)
        env.set_lights(lit.lights)
        outs.append(env.gather_direct_light(supersamples=4, seed=2))
    assert outs[0][1] == outs[1][1] and np.array_equal(outs[0][0].view(np.uint32),
                                                       outs[1][0].view(np.uint32))
    ref, rays = oracle.gather_luxels(oracle.Scene(lit.xyz, lit.ids),
                                     oracle.make_lights(lit.lights), len(lit.lights), lit, 0,
                                     lit.n_faces, ss=4, seed=2, threads=16)
    assert rays == outs[0][1]
    assert _rel_err(outs[0][0], ref).max() <= RTOL


def test_tiled_room_with_and_without_wall_slots(gpu_ctx, oracle):
    # walls split into tiles (as brush sides make them): the gather with the
    # wall slots, without them, and the oracle give the same luxels
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = scenes.lit_scene(6, n_faces=96, n_point=12, n_spot=4, wall_tiles=8)
    outs = []
    for slots in (True, False):
        env = Environment(gpu_ctx)
        env.set_wall_slots(slots)
        env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        assert (env.wall_slots()[1] > 0).any() == slots
        env.set_faces(lit)
        env.set_lights(lit.lights)
        outs.append(env.gather_direct_light(supersamples=4, seed=1))
    assert outs[0][1] == outs[1][1] and np.array_equal(outs[0][0].view(np.uint32),
                                                       outs[1][0].view(np.uint32))
    ref, rays = oracle.gather_luxels(oracle.Scene(lit.xyz, lit.ids),
                                     oracle.make_lights(lit.lights), len(lit.lights), lit, 0,
                                     lit.n_faces, ss=4, seed=1, threads=16)
    assert rays == outs[0][1]
    assert _rel_err(outs[0][0], ref).max() <= RTOL
