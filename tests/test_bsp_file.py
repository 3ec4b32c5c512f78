"""The BSP reader (vrg_bsp_open): a compiled map written here from a test
world in the Source BSP record layouts decodes back to the same lumps, and
ingesting the file gives the same triangles as ingesting the lumps; both
leaf lump versions; texinfo lightmap vectors; malformed files rejected.
No real map is part of the project, so the layouts are pinned only by this
writer, which follows the published format independently of the reader."""
import struct

import numpy as np
import pytest

from test_bsp_ingest import World

PLANES, VERTEXES, NODES, TEXINFO, FACES, LEAFS = 1, 3, 5, 6, 7, 10
EDGES, SURFEDGES, MODELS, LEAFBRUSHES, BRUSHES, BRUSHSIDES = 12, 13, 14, 17, 18, 19
FACES_HDR = 58


def write_bsp(lumps, headnode=0, first_face=0, num_faces=None, version=20, leaf_version=1,
              lightmap_vecs=None, compressed=(), faces_hdr=None):
    """Bytes of a BSP file holding the given lump arrays (other lumps empty)."""
    a = {k: np.asarray(v) for k, v in lumps.items()}
    n_faces = len(a["faces"]) if num_faces is None else num_faces
    body = {}
    body[PLANES] = b"".join(struct.pack("<4fi", *p[:4], 0) for p in a["planes"].reshape(-1, 4))
    body[VERTEXES] = a["vertexes"].astype("<f4").tobytes()
    body[NODES] = b"".join(struct.pack("<3i6h4h", 0, int(c[0]), int(c[1]), *([0] * 6), 0, 0, 0, 0)
                           for c in a["node_children"].reshape(-1, 2))
    ntex = len(a["texinfo_flags"])
    vecs = (np.zeros((ntex, 2, 4)) if lightmap_vecs is None else np.asarray(lightmap_vecs))
    body[TEXINFO] = b"".join(struct.pack("<8f8f2i", *([0.25] * 8), *vecs[t].ravel(),
                                         int(a["texinfo_flags"][t]), 0) for t in range(ntex))
    def face_lump(faces):
        return b"".join(struct.pack("<HBBihhhh4BifiiiiiHHI", 0, 0, 0, int(f[0]), int(f[1]), int(f[2]),
                                    -1, 0, 0, 255, 255, 255, 0, 1.0, 0, 0, 4, 4, -1, 0, 0, 0)
                        for f in np.asarray(faces).reshape(-1, 3))

    body[FACES] = face_lump(a["faces"])
    if faces_hdr is not None:
        body[FACES_HDR] = face_lump(faces_hdr)
    leaves = []
    for first, n in a["leaf_brush_ranges"].reshape(-1, 2):
        rec = struct.pack("<ihh6h4Hh", 1, 0, 0, *([0] * 6), 0, 0, int(first), int(n), -1)
        rec += b"\0\0" if leaf_version == 1 else b"\x07" * 24 + b"\0\0"
        leaves.append(rec)
    body[LEAFS] = b"".join(leaves)
    body[EDGES] = a["edges"].astype("<u2").tobytes()
    body[SURFEDGES] = a["surf_edges"].astype("<i4").tobytes()
    body[MODELS] = struct.pack("<9f3i", *([0.0] * 9), headnode, first_face, n_faces)
    body[LEAFBRUSHES] = a["leaf_brushes"].astype("<u2").tobytes()
    body[BRUSHES] = a["brushes"].astype("<i4").tobytes()
    body[BRUSHSIDES] = b"".join(struct.pack("<Hhhbb", int(s[0]), int(s[1]), int(s[2]), int(s[3]), 0)
                                for s in a["brush_sides"].reshape(-1, 4))
    header_len = 8 + 16 * 64 + 4
    out = bytearray(header_len)
    struct.pack_into("<4si", out, 0, b"VBSP", version)
    for i in range(64):
        data = body.get(i, b"")
        ofs = len(out) if data else 0
        lump_version = leaf_version if i == LEAFS else 0
        fourcc = len(data) if i in compressed else 0
        struct.pack_into("<3ii", out, 8 + 16 * i, ofs, len(data), lump_version, fourcc)
        out += data
        out += b"\0" * (-len(out) % 4)
    struct.pack_into("<i", out, 8 + 16 * 64, 1)
    return bytes(out)


def _world():
    w = World()
    b0 = w.box((0, 0, 0), (64, 32, 16))
    b1 = w.box((100, 0, 0), (140, 50, 30), texinfo={4: 1})
    b2 = w.box((-50, -50, -8), (200, 200, 0), bevel={1: 1})
    w.face([(0, 0, 300), (300, 0, 300), (300, 300, 300), (0, 300, 300)], texinfo=1)
    w.face([(0, 0, 0), (1, 0, 0), (1, 1, 0)], texinfo=0)
    w.face([(0, 0, 250), (5, 0, 250), (9, 4, 250), (5, 9, 250), (0, 5, 250)], texinfo=1, flip_every=3)
    return w.lumps(leaves=[[b2], [b0, b1], [b1, b2]])


@pytest.mark.parametrize("leaf_version", [0, 1])
def test_file_decodes_to_its_lumps(vlib, leaf_version):
    from vrad_gb300.environment import BspWorld, read_bsp

    lumps = _world()
    vecs = np.arange(2 * 8, dtype=np.float32).reshape(2, 2, 4) / 16
    m = read_bsp(write_bsp(lumps, leaf_version=leaf_version, lightmap_vecs=vecs))
    assert m["version"] == 20 and (m["headnode"], m["first_face"], m["num_model_faces"]) == (0, 0, 3)
    for name, dt, per in BspWorld.LUMPS:
        want = np.asarray(lumps[name], dt).reshape(-1, per)
        assert np.array_equal(m["lumps"][name], want), name
    assert np.array_equal(m["lightmap_vecs"], vecs)


def test_file_ingest_equals_lump_ingest(vlib, host_ctx):
    from vrad_gb300.environment import Environment

    lumps = _world()
    a = Environment(host_ctx)
    counts_a = a.add_bsp_world(lumps)
    b = Environment(host_ctx)
    counts_b = b.add_bsp_file(write_bsp(lumps))
    assert counts_a == counts_b and counts_a[0] > 0 and counts_a[1] == 5
    xa, ia = a.get_triangle_vertices()
    xb, ib = b.get_triangle_vertices()
    assert np.array_equal(xa, xb) and np.array_equal(ia, ib)
    # model 0 covering only the second face: no sky triangles
    c = Environment(host_ctx)
    assert c.add_bsp_file(write_bsp(lumps, first_face=1, num_faces=1))[1] == 0


def test_lightmap_vecs_feed_face_extents(vlib, oracle):
    from vrad_gb300.environment import calc_face_extents, read_bsp

    lumps = _world()
    vecs = np.array([[[1 / 16, 0, 0, 0], [0, 1 / 16, 0, 0]], [[0, 1 / 8, 0, 3], [0, 0, 1 / 8, -2]]],
                    np.float32)
    m = read_bsp(write_bsp(lumps, lightmap_vecs=vecs))
    verts = np.float32([(0, 0, 300), (300, 0, 300), (300, 300, 300), (0, 300, 300)])
    for t in range(2):
        got = calc_face_extents(verts, m["lightmap_vecs"][t])
        assert got == oracle.calc_face_extents(verts, vecs[t])
    assert calc_face_extents(verts, m["lightmap_vecs"][0]) == ((0, 0), (19, 19), False)


def test_malformed_files_are_rejected(vlib):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import read_bsp

    good = write_bsp(_world())
    read_bsp(good)
    bad = [b"", good[:100], b"XBSP" + good[4:], write_bsp(_world(), version=18),
           write_bsp(_world(), compressed=(BRUSHES,))]
    past = bytearray(good)
    struct.pack_into("<i", past, 8 + 16 * BRUSHES + 4, len(good))  # brushes run past the end
    bad.append(bytes(past))
    ragged = bytearray(good)
    ofs, n = struct.unpack_from("<2i", good, 8 + 16 * BRUSHSIDES)
    struct.pack_into("<i", ragged, 8 + 16 * BRUSHSIDES + 4, n - 3)  # not whole records
    bad.append(bytes(ragged))
    for data in bad:
        with pytest.raises(VrgError):
            read_bsp(data)


def test_hdr_faces(vlib, host_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment, read_bsp

    lumps = _world()
    faces = np.asarray(lumps["faces"])
    # the HDR lump holds only the pentagon; model 0 has one face
    data = write_bsp(lumps, num_faces=1, faces_hdr=faces[2:3])
    assert np.array_equal(read_bsp(data, hdr=True)["lumps"]["faces"], faces[2:3])
    assert np.array_equal(read_bsp(data)["lumps"]["faces"], faces)
    env = Environment(host_ctx)
    assert env.add_bsp_file(data, hdr=True)[1] == 3  # the pentagon's fan
    env = Environment(host_ctx)
    assert env.add_bsp_file(data)[1] == 2  # LDR face 0: the square's fan
    env = Environment(host_ctx)  # no HDR lump for model 0's face range: refused
    with pytest.raises(VrgError):
        env.add_bsp_file(write_bsp(lumps, num_faces=1), hdr=True)
    assert env.num_triangles() == 0
