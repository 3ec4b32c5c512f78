"""Lightmap output on the CPU: the shared-exponent sample encoding of the
oracle against an independent numpy restatement and known answers, face
extents (CalcFaceExtents, rad/world/face.go:14-90) of the library's host
entry point against the oracle, and the oracle's luxel -> leaf patch lookup
against the patch boxes."""
import numpy as np
import pytest

FLT_MAX = np.float32(3.4028234663852886e38)


def np_encode(rgb):
    """floor(c * 2^-x) with x from frexp of the largest channel, float64 scaling."""
    rgb = np.asarray(rgb, np.float32).reshape(-1, 3)
    with np.errstate(invalid="ignore"):
        c = np.where(rgb > 0, rgb, np.float32(0))
    c = np.minimum(c, FLT_MAX)
    m = c.max(axis=1)
    _, e = np.frexp(m)
    x = np.maximum(e.astype(np.int64) - 8, -128)
    b = np.floor(np.ldexp(c.astype(np.float64), -x[:, None]))
    b = np.minimum(b, 255).astype(np.uint32)
    w = b[:, 0] | (b[:, 1] << 8) | (b[:, 2] << 16) | ((x & 255).astype(np.uint32) << 24)
    w[m == 0] = 0
    return w


def decode(w):
    w = np.asarray(w, np.uint32)
    x = (w >> 24).astype(np.uint8).view(np.int8).astype(np.int64)
    b = np.stack([(w >> (8 * a)) & 255 for a in range(3)], axis=-1).astype(np.float64)
    return np.ldexp(b, x[..., None]), x


def _values(n, seed):
    rng = np.random.default_rng(seed)
    tiny = np.float32(1.4e-45)
    special = np.array([0.0, -0.0, -1.0, np.nan, np.inf, -np.inf, tiny, 2 * tiny, 1.1754942e-38,
                        1.1754944e-38, 1.0, np.nextafter(np.float32(1), np.float32(0)), 255.0,
                        255.99998, 256.0, 0.5, 2.0 ** -120, 2.0 ** -121, 2.0 ** -127, 2.0 ** 120,
                        FLT_MAX, 3.0e38], np.float32)
    logu = np.exp2(rng.uniform(-150, 128, n)).astype(np.float32)
    rgb = np.stack([logu, logu * rng.uniform(0, 1, n).astype(np.float32),
                    rng.uniform(0, 1000, n).astype(np.float32)], axis=1)
    rng.shuffle(rgb, axis=1)
    picks = rng.integers(0, len(special), (3000, 3))
    return np.concatenate([rgb, special[picks], np.stack([special] * 3, axis=1)]).astype(np.float32)


def test_encode_known_answers(oracle):
    assert oracle.encode_sample(0, 0, 0) == 0
    assert oracle.encode_sample(-1, np.nan, -np.inf) == 0
    # 1.0 = 0.5 * 2^1 -> x = -7, bytes 128
    assert oracle.encode_sample(1, 1, 1) == 0x80 | 0x80 << 8 | 0x80 << 16 | 0xF9 << 24
    assert oracle.encode_sample(255, 0, 0) == 255
    assert oracle.encode_sample(256, 1, 0) == 128 | 0 << 8 | 1 << 24  # 1 * 2^-1 floors to 0
    assert oracle.encode_sample(0, 0, 3.0) == 192 << 16 | 0xFA << 24  # 3 * 2^6 = 192
    # +inf clamps to FLT_MAX = (2 - 2^-23) * 2^127: x = 120, byte 255
    assert oracle.encode_sample(np.inf, 0, 0) == 255 | 120 << 24
    # the smallest denormal: x clamps to -128, 2^-149 * 2^128 floors to 0
    assert oracle.encode_sample(1.4e-45, 0, 0) == 0x80 << 24


def test_encode_matches_numpy_restatement(oracle):
    v = _values(20000, 7)
    got = np.array([oracle.encode_sample(*t) for t in v], np.uint32)
    assert np.array_equal(got, np_encode(v))


def test_encode_decode_bounds(oracle):
    v = _values(5000, 9)
    w = np.array([oracle.encode_sample(*t) for t in v], np.uint32)
    dec, x = decode(w)
    c = np.minimum(np.where(np.nan_to_num(v, nan=-1.0) > 0, v, 0), FLT_MAX).astype(np.float64)
    assert np.all(dec <= c)
    assert np.all(c - dec < np.ldexp(1.0, x)[:, None])
    m = c.max(axis=1)
    big = (m > 0) & (x > -128)
    top = ((w >> 0) & 255, (w >> 8) & 255, (w >> 16) & 255)
    assert np.all(np.maximum.reduce(top)[big] >= 128)  # the largest channel keeps 8 bits


# ---- face extents ----

def _vecs(s, t, so=0.0, to=0.0):
    return np.array([[*s, so], [*t, to]], np.float32)


def test_face_extents_known_answers(vlib, oracle):
    from vrad_gb300.environment import calc_face_extents

    quad = np.array([[0, 0, 0], [64, 0, 0], [64, 64, 0], [0, 64, 0]], np.float32)
    cases = [
        (quad, _vecs((1 / 16, 0, 0), (0, 1 / 16, 0)), ((0, 0), (4, 4), False)),
        (quad, _vecs((1 / 16, 0, 0), (0, 1 / 16, 0), 0.5, 0.5), ((0, 0), (5, 5), False)),
        (quad - 8, _vecs((1 / 16, 0, 0), (0, 1 / 16, 0)), ((-1, -1), (5, 5), False)),  # -0.5 .. 3.5
        (quad * [126 / 4, 1, 1], _vecs((1 / 16, 0, 0), (0, 1 / 16, 0)), ((0, 0), (126, 4), False)),
        (quad * [127 / 4, 1, 1], _vecs((1 / 16, 0, 0), (0, 1 / 16, 0)), ((0, 0), (127, 4), True)),
        # a wall (x = const) mapped with the y and z axes
        (np.array([[5, 0, 0], [5, 32, 0], [5, 32, 48]], np.float32),
         _vecs((0, 1 / 16, 0), (0, 0, -1 / 16)), ((0, -3), (2, 3), False)),
    ]
    for verts, vecs, want in cases:
        assert calc_face_extents(verts, vecs) == want
        assert oracle.calc_face_extents(verts, vecs) == want


def test_face_extents_random_faces(vlib, oracle):
    from vrad_gb300.environment import calc_face_extents

    rng = np.random.default_rng(11)
    for i in range(400):
        n = int(rng.integers(1, 9))
        verts = rng.uniform(-8192, 8192, (n, 3)).astype(np.float32)
        vecs = rng.normal(0, 0.1, (2, 4)).astype(np.float32)
        vecs[:, 3] = rng.uniform(-300, 300, 2)
        assert calc_face_extents(verts, vecs) == oracle.calc_face_extents(verts, vecs)


def test_face_extents_errors(vlib, oracle):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import calc_face_extents

    vecs = _vecs((1.0, 0, 0), (0, 1.0, 0))
    with pytest.raises(VrgError):
        calc_face_extents(np.zeros((0, 3), np.float32), vecs)
    with pytest.raises(VrgError):
        calc_face_extents(np.array([[np.inf, 0, 0]], np.float32), vecs)
    with pytest.raises(VrgError):  # beyond int32
        calc_face_extents(np.array([[0, 0, 0], [3e9, 0, 0]], np.float32), vecs)
    assert oracle.calc_face_extents(np.zeros((0, 3), np.float32), vecs) is None
    assert oracle.calc_face_extents(np.array([[0, 0, 0], [3e9, 0, 0]], np.float32), vecs) is None


# ---- luxel -> leaf patch ----

def test_oracle_lightmap_finds_the_leaf_under_each_luxel(oracle):
    """Bounced light tagged with its leaf number (every channel in [128, 255], so
    the sample holds it exactly) comes back on luxels whose centres the leaf's
    box contains; with no bounced light the sample is the direct light's."""
    from vrad_gb300 import scenes

    lit = scenes.lit_scene(5, n_faces=60, spacing=16.0, n_point=4, n_spot=1)
    P = oracle.make_patches(lit)
    nleaf = int((P["leaf_index"] >= 0).sum())
    ids = np.arange(nleaf)
    total = np.stack([128 + (ids & 127), 128 + ((ids >> 7) & 127), 128 + ((ids >> 14) & 127)],
                     axis=1).astype(np.float32)
    nlux = lit.n_luxels
    words = oracle.lightmap(lit, P, np.zeros((nlux, 3), np.float32), total)
    dec, x = decode(words)
    assert np.all(x == 0)
    leaf = (dec[:, 0] - 128) + 128 * (dec[:, 1] - 128) + 16384 * (dec[:, 2] - 128)
    leaf = leaf.astype(np.int64)
    patch_of_leaf = np.nonzero(P["leaf_index"] >= 0)[0][np.argsort(P["leaf_index"][P["leaf_index"] >= 0])]
    off = lit.luxel_offset()
    for f in range(lit.n_faces):
        pts = oracle.luxel_samples(lit, f, ss=1)
        p = patch_of_leaf[leaf[off[f]:off[f + 1]]]
        assert np.all(P["face"][p] == f)
        nax = int(np.argmax(np.abs(lit.normal[f])))
        for a in range(3):
            if a != nax:
                assert np.all(pts[:, a] >= P["mins"][p, a]) and np.all(pts[:, a] <= P["maxs"][p, a])
    rng = np.random.default_rng(2)
    direct = rng.uniform(0, 50, (nlux, 3)).astype(np.float32)
    plain = oracle.lightmap(lit, P, direct, np.zeros_like(total))
    assert np.array_equal(plain, np_encode(direct))
