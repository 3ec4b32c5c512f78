"""A brush world ingested through vrg_env_add_bsp_world (the reference's
addBrushesForRayTrace) feeds the device scene: shadow lines and closest hits
on the GPU equal the oracle's on the same triangles."""
import numpy as np
import pytest

from test_bsp_ingest import World

pytestmark = pytest.mark.gpu


def brush_room(seed=1, n_boxes=60, n_convex=12):
    """A 2048-unit room of wall brushes with an open roof closed by a sky
    face, box brushes and random convex brushes inside."""
    rng = np.random.default_rng(seed)
    w = World()
    t = 16.0
    L = 2048.0
    w.box((-t, -t, -t), (L + t, L + t, 0))  # floor
    w.box((-t, -t, 0), (0, L + t, L))
    w.box((L, -t, 0), (L + t, L + t, L))
    w.box((0, -t, 0), (L, 0, L))
    w.box((0, L, 0), (L, L + t, L))
    w.face([(0, 0, L), (L, 0, L), (L, L, L), (0, L, L)], texinfo=1)  # sky over the room
    for _ in range(n_boxes):
        c = rng.uniform(100, L - 100, 3)
        e = rng.uniform(10, 120, 3)
        w.box(c - e, c + e)
    for _ in range(n_convex):
        c = rng.uniform(300, L - 300, 3)
        r = rng.uniform(30, 150)
        n = rng.normal(size=(8, 3))
        n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
        planes = [(n[i], float(np.float32(n[i].astype(np.float64) @ c + r))) for i in range(8)]
        for a in range(3):
            e = np.zeros(3, np.float32)
            e[a] = 1
            planes += [(e, float(c[a] + 1.5 * r)), (-e, float(-(c[a] - 1.5 * r)))]
        w.brush(planes)
    return w.lumps()


def test_brush_world_traces_like_the_oracle(gpu_ctx, oracle):
    from vrad_gb300.environment import Environment

    lumps = brush_room()
    env = Environment(gpu_ctx)
    nb, ns = env.add_bsp_world(lumps)
    assert nb > 0 and ns == 2
    env.SetupAccelerationStructure()
    xyz, ids = env.get_triangle_vertices()
    rng = np.random.default_rng(2)
    a = rng.uniform(1, 2047, (40000, 3)).astype(np.float32)
    b = rng.uniform(1, 2047, (40000, 3)).astype(np.float32)
    b[::4, 2] = 3000.0  # a quarter of the lines leave through the sky face
    m, h, t = env.occlusion_mask(a, b, closest=True)
    rm, rh, rt = oracle.Scene(xyz, ids).occlusion_mask(a, b, threads=16, closest=True)
    assert np.array_equal(m, rm) and np.array_equal(h, rh)
    assert np.array_equal(t.view(np.uint32), rt.view(np.uint32))
    frac = env.test_line_does_hit_sky(a[::4], b[::4])
    rfrac = oracle.Scene(xyz, ids).test_lines(a[::4], b[::4], threads=16)
    assert np.array_equal(frac, rfrac) and 0 < frac.mean() < 1


def test_can_leaf_trace_to_sky_like_the_oracle(gpu_ctx, oracle):
    from vrad_gb300.environment import Environment, leaf_sky_lines

    env = Environment(gpu_ctx)
    env.add_bsp_world(brush_room(seed=3))
    env.SetupAccelerationStructure()
    xyz, ids = env.get_triangle_vertices()
    rng = np.random.default_rng(4)
    mins = rng.integers(20, 1900, (300, 3)).astype(np.int32)
    maxs = (mins + rng.integers(1, 120, (300, 3))).astype(np.int32)
    mins[:20, 2], maxs[:20, 2] = -12, -4  # centres inside the solid floor: every line is stopped
    got = env.CanLeafTraceToSky(mins, maxs)
    a, b = leaf_sky_lines(mins, maxs)
    frac = oracle.Scene(xyz, ids).test_lines(a, b, skip=-1, threads=16)
    want = (frac.reshape(-1, 162) > 0).any(axis=1)
    assert np.array_equal(got, want) and not want[:20].any() and want[20:].mean() > 0.5


def test_direct_light_on_a_brush_world_like_the_oracle(gpu_ctx, oracle):
    # the direct-light gather over boxes and walls ingested as brushes, with
    # the wall cells on and off: every luxel bit-identical to the oracle's
    from conftest import bits_equal
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lumps, lit = scenes.lit_brush_world(3, n_faces=384)
    ref = None
    for walls in (True, False):
        env = Environment(gpu_ctx)
        env.set_wall_slots(walls)
        env.add_bsp_world(lumps)
        env.SetupAccelerationStructure()
        env.set_faces(lit)
        env.set_lights(lit.lights)
        rgb, rays = env.gather_direct_light(supersamples=4, seed=5)
        if ref is None:
            xyz, ids = env.get_triangle_vertices()
            ref, rrays = oracle.gather_luxels(oracle.Scene(xyz, ids), oracle.make_lights(lit.lights),
                                              len(lit.lights), lit, 0, lit.n_faces, ss=4, seed=5,
                                              threads=16)
            assert rays == rrays and np.abs(ref).max() > 0
        assert bits_equal(rgb, ref)
        env.close()
