"""Brush ingest on the CPU (host-only context): addBrushesForRayTrace /
addBrushToRaytraceEnvironment (cmd/tasks/loadbsp/main.go:241-340) and the
winding helpers (vmath/polygon/winding.go) of the library against the
oracle bit for bit, against closed-form box surfaces and against scipy's
half-space intersection for random convex brushes; the flags (opaque
contents, sky and displacement sides, bevels), the brush order of the BSP
walk, sky faces through signed surfedges, and rejected input."""
import numpy as np
import pytest

SKY, OPAQUE = 0x01000000, 0x02000000
SURF_SKY, CONTENTS_SOLID, CONTENTS_WATER = 0x4, 0x1, 0x20


from vrad_gb300.scenes import BrushMap as World  # noqa: E402  (the lump writer)


def _ingest(host_ctx, lumps, **kw):
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    nb, ns = env.add_bsp_world(lumps, **kw)
    xyz, ids = env.get_triangle_vertices()
    return env, xyz, ids, nb, ns


def _area(xyz):
    t = xyz.reshape(-1, 3, 3).astype(np.float64)
    return 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1).sum()


def test_base_winding_and_chop_match_oracle(vlib, oracle):
    from vrad_gb300.environment import base_winding_for_plane, chop_winding

    rng = np.random.default_rng(4)
    axes = [np.eye(3)[a] * s for a in range(3) for s in (1, -1)]
    normals = axes + list(rng.normal(size=(300, 3)))
    for n in normals:
        n = (np.asarray(n) / np.linalg.norm(n)).astype(np.float32)
        d = np.float32(rng.uniform(-3000, 3000))
        w = base_winding_for_plane(n, d)
        assert np.array_equal(w, oracle.base_winding(n, d))
        assert np.allclose(w @ n.astype(np.float64), d, atol=0.05)  # on the plane
        for _ in range(3):
            m = rng.normal(size=3)
            m = (m / np.linalg.norm(m)).astype(np.float32)
            e = np.float32(rng.uniform(-2000, 2000))
            c = chop_winding(w, m, e)
            assert np.array_equal(c, oracle.chop_winding(w, m, e))
            if len(c):
                assert np.all(c.astype(np.float64) @ m - e >= -0.05)
            w = c if len(c) >= 3 else w


def test_chop_keeps_on_points_and_uses_exact_axis_planes(vlib):
    from vrad_gb300.environment import chop_winding

    sq = np.array([[0, 0, 0], [10, 0, 0], [10, 10, 0], [0, 10, 0]], np.float32)
    assert np.array_equal(chop_winding(sq, [0, 0, 1], 5), np.zeros((0, 3)))  # all behind
    assert np.array_equal(chop_winding(sq, [0, 0, 1], -5), sq)  # all in front
    assert np.array_equal(chop_winding(sq, [1, 0, 0], 0), sq)  # an edge on the plane
    half = chop_winding(sq, [1, 0, 0], 3.3)
    assert np.all(half[:, 0] >= np.float32(3.3)) and set(half[:, 0]) == {np.float32(3.3), 10}


def test_box_brushes_give_their_surface(vlib, host_ctx, oracle):
    w = World()
    boxes = [((0, 0, 0), (64, 32, 16)), ((-100.5, 7.25, 3), (-20, 90, 40.75))]
    for mn, mx in boxes:
        w.box(mn, mx)
    lumps = w.lumps()
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps)
    assert (nb, ns) == (24, 0) and np.all(ids == OPAQUE)
    rx, rids, rnb = oracle.bsp_world_triangles(lumps)
    assert np.array_equal(xyz, rx) and np.array_equal(ids, rids) and rnb == nb
    # every vertex is a box corner, exactly (axis planes take the plane's distance)
    for k, (mn, mx) in enumerate(boxes):
        v = xyz[12 * k:12 * (k + 1)].reshape(-1, 3)
        for a in range(3):
            assert set(v[:, a]) == {np.float32(mn[a]), np.float32(mx[a])}
        e = np.subtract(mx, mn, dtype=np.float64)
        assert _area(xyz[12 * k:12 * (k + 1)]) == pytest.approx(2 * (e[0] * e[1] + e[1] * e[2] + e[0] * e[2]))


def test_random_convex_brushes_match_halfspace_intersection(vlib, host_ctx, oracle):
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(8)
    w = World()
    hulls = []
    for _ in range(20):
        c = rng.uniform(-2000, 2000, 3)
        r = rng.uniform(20, 300)
        n = rng.normal(size=(int(rng.integers(5, 14)), 3))
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        n = n.astype(np.float32)
        d = (n.astype(np.float64) @ c + r * rng.uniform(1.0, 1.6, len(n))).astype(np.float32)
        # close it with an axis box around the sphere's bounds
        planes = [(n[i], float(d[i])) for i in range(len(n))]
        for a in range(3):
            e = np.zeros(3, np.float32)
            e[a] = 1
            planes += [(e, float(c[a] + 1.8 * r)), (-e, float(-(c[a] - 1.8 * r)))]
        w.brush(planes)
        hs = np.array([[*p[0], -p[1]] for p in planes], np.float64)
        hulls.append(spatial.ConvexHull(spatial.HalfspaceIntersection(hs, c).intersections).area)
    lumps = w.lumps()
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps)
    rx, rids, rnb = oracle.bsp_world_triangles(lumps)
    assert np.array_equal(xyz, rx) and np.array_equal(ids, rids)
    # per brush area: triangles of brush k are consecutive; split by the oracle per brush
    start = 0
    for k in range(len(hulls)):
        one = World()
        one.planes, one.sides = w.planes, w.sides
        one.brushes = [w.brushes[k]]
        bx, _, bn = oracle.bsp_world_triangles(one.lumps())
        assert np.array_equal(xyz[start:start + bn], bx)
        assert _area(bx) == pytest.approx(hulls[k], rel=1e-3)
        start += bn
    assert start == nb


def test_flags_and_order(vlib, host_ctx, oracle):
    w = World()
    b0 = w.box((0, 0, 0), (10, 10, 10))
    b1 = w.box((20, 0, 0), (30, 10, 10), contents=CONTENTS_WATER)  # not opaque
    b2 = w.box((40, 0, 0), (50, 10, 10), texinfo={0: 1})  # +x side is sky
    b3 = w.box((60, 0, 0), (70, 10, 10), disp={2: 7})  # +y side is a displacement
    cut = np.array([1, 1, 0], np.float32) / np.float32(np.sqrt(2))
    b4 = w.box((80, 0, 0), (90, 10, 10))
    w.sides.append([w.plane(cut, float(np.float32(90 / np.sqrt(2)))), 0, 0, 1])  # bevel x + y = 90
    w.brushes[b4][1] += 1
    w.face([(0, 0, 100), (100, 0, 100), (100, 100, 100), (0, 100, 100)], texinfo=1)  # sky
    w.face([(0, 0, 0), (1, 0, 0), (1, 1, 0)], texinfo=0)  # not sky
    w.face([(0, 0, 50), (5, 0, 50), (9, 4, 50), (5, 9, 50), (0, 5, 50)], texinfo=1, flip_every=3)
    # leaves [b4], [b0], [b0, b2, b1], [b3, b4] -> walk order b4, b0, b2, b1, b3
    lumps = w.lumps(leaves=[[b4], [b0], [b0, b2, b1], [b3, b4]])
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps)
    rx, rids, rnb = oracle.bsp_world_triangles(lumps)
    assert np.array_equal(xyz, rx) and np.array_equal(ids, rids) and rnb == nb
    # b4: 12 box triangles unchanged by the bevel + the bevel's own cross-section
    # b0: 12; b2: 10 (sky side left out); b1: none; b3: 10
    assert nb == (12 + 2) + 12 + 10 + 10 and ns == 2 + 3
    assert np.all(ids[:nb] == OPAQUE) and np.all(ids[nb:] == SKY)
    plain = World()
    plain.box((80, 0, 0), (90, 10, 10))
    px, _, _ = oracle.bsp_world_triangles(plain.lumps())
    assert np.array_equal(xyz[:12], px)  # the bevel chops no other side
    assert np.all(xyz[14:26].reshape(-1, 3)[:, 0] <= 10)  # then b0
    sky = xyz[nb:].reshape(-1, 3, 3)
    assert np.array_equal(sky[0], np.float32([(0, 0, 100), (100, 0, 100), (100, 100, 100)]))
    assert np.array_equal(sky[4], np.float32([(0, 0, 50), (5, 9, 50), (0, 5, 50)]))


def test_first_face_range_and_empty_world(vlib, host_ctx, oracle):
    w = World()
    for z in (10, 20, 30):
        w.face([(0, 0, z), (1, 0, z), (1, 1, z)], texinfo=1)
    lumps = w.lumps(leaves=[])
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps, first_face=1, num_model_faces=1)
    assert (nb, ns) == (0, 1) and np.all(xyz.reshape(3, 3)[:, 2] == 20)
    env, xyz, ids, nb, ns = _ingest(host_ctx, {})
    assert (nb, ns) == (0, 0) and len(ids) == 0


def test_rejected_input_adds_nothing(vlib, host_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    w = World()
    w.box((0, 0, 0), (1, 1, 1))
    w.face([(0, 0, 5), (1, 0, 5), (1, 1, 5)])
    good = w.lumps()
    bad = []
    l1 = dict(good, brush_sides=np.array(good["brush_sides"]) + [[100, 0, 0, 0]])
    bad.append(l1)  # plane out of range
    bad.append(dict(good, node_children=[[0, -1]]))  # node 0 is its own child
    bad.append(dict(good, leaf_brush_ranges=[[0, 5]]))  # past the leaf-brush lump
    bad.append(dict(good, surf_edges=[1, -2, 99]))  # edge out of range
    pl = np.array(good["planes"], np.float32)
    pl[3, 1] = np.nan
    bad.append(dict(good, planes=pl))
    for lumps in bad:
        env = Environment(host_ctx)
        with pytest.raises(VrgError):
            env.add_bsp_world(lumps)
        assert env.num_triangles() == 0
    env = Environment(host_ctx)
    with pytest.raises(VrgError):
        env.add_bsp_world(good, first_face=0, num_model_faces=5)
    env.add_bsp_world(good)
    env.SetupAccelerationStructure()
    with pytest.raises(VrgError):  # after the build
        env.add_bsp_world(good)


def test_many_brushes_keep_the_reference_order(vlib, host_ctx, oracle):
    """Enough brushes for the ingest to split the list over threads: the
    triangles still come out in the BSP walk's order, bit for bit."""
    rng = np.random.default_rng(12)
    w = World()
    for k in range(3000):
        c = rng.uniform(0, 8000, 3)
        if k % 7 == 0:
            n = rng.normal(size=(6, 3))
            n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
            planes = [(n[i], float(np.float32(n[i].astype(np.float64) @ c + 40))) for i in range(6)]
            for a in range(3):
                e = np.zeros(3, np.float32)
                e[a] = 1
                planes += [(e, float(c[a] + 60)), (-e, float(-(c[a] - 60)))]
            w.brush(planes, contents=CONTENTS_SOLID if k % 11 else CONTENTS_WATER)
        else:
            e = rng.uniform(4, 100, 3)
            w.box(c - e, c + e, texinfo={int(k % 6): 1} if k % 5 == 0 else None)
    order = rng.permutation(3000)
    leaves = [list(order[i:i + 37]) for i in range(0, 3000, 37)]
    lumps = w.lumps(leaves=leaves)
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps)
    rx, rids, rnb = oracle.bsp_world_triangles(lumps)
    assert nb == rnb > 30000 and np.array_equal(xyz, rx) and np.array_equal(ids, rids)


def test_lit_brush_world_faces_follow_the_ingest(host_ctx):
    # the brush world of the direct-light bench: every triangle its tri_face
    # maps to a lit face lies in that face's rectangle, the room's brushes and
    # the sky face map to none, and its walls are ingested brush sides
    from vrad_gb300 import scenes

    lumps, lit = scenes.lit_brush_world(0, n_faces=600)
    env, xyz, ids, nb, ns = _ingest(host_ctx, lumps)
    assert ns == 2 and len(lit.tri_face) == len(ids) == nb + 2 == 12 * (5 + 100) + 2
    f = lit.tri_face
    assert (f[:60] == -1).all() and (f[-2:] == -1).all() and (ids[-2:] & SKY).all()
    m = f >= 0
    assert np.array_equal(np.unique(f[m]), np.arange(600))
    v = xyz[m].reshape(-1, 3, 3).astype(np.float64)
    c, u, w, n = (a[f[m]][:, None, :].astype(np.float64) for a in (lit.corner, lit.u, lit.v, lit.normal))
    assert np.abs(((v - c) * n).sum(-1)).max() < 1e-3
    for e in (u, w):
        s = ((v - c) * e).sum(-1) / (e * e).sum(-1)
        assert s.min() > -1e-6 and s.max() < 1 + 1e-6
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    tris, counts = env.wall_slots()
    assert counts.tolist() == [4, 4, 4, 4, 2, 4]  # the outer sides of wall and floor brushes
