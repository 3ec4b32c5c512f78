"""Seeded synthetic scenes for the radiosity hot path.

The reference's own inputs are BSP maps (``cmd/args.go:53``) that are not part
of the project; these generators stand in for them with box rooms built the
way ``raytracer/environment.go:77-117`` (``AddAxisAlignedRectangularSolid``)
builds a box: six quads in the order far (z max), near (z min), left (x min),
right (x max), top (y max), bottom (y min); each quad ``(v1,v2,v3,v4)``
becomes triangles ``(v1,v2,v3)`` and ``(v1,v3,v4)`` with ids ``id`` and
``id+1`` (``AddQuad``, ``environment.go:71-75``).

All randomness is SplitMix64 (Steele, Lea & Flood 2014) over a counter, one
stream per purpose, so the same seed gives the same float32 arrays on any
machine.  No transcendental function touches a value that reaches a kernel
except the transfer direction table, which is built once in float64 and
handed to both the GPU path and the oracle as an input.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

TRACE_ID_SKY = 0x01000000
TRACE_ID_OPAQUE = 0x02000000
TRACE_ID_STATICPROP = 0x04000000

EMIT_SURFACE, EMIT_POINT, EMIT_SPOTLIGHT, EMIT_SKYLIGHT, EMIT_QUAKELIGHT, EMIT_SKYAMBIENT = range(6)

# BSP flags a written map uses (texinfo surface flag, brush contents)
SURF_SKY, CONTENTS_SOLID = 0x4, 0x1

ROOM = 4096.0
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# stream ids
S_BOXES, S_RAYS, S_LIGHTS, S_REFL, S_SPOTDIR = 1, 2, 3, 4, 5


def splitmix(seed: int, idx: np.ndarray) -> np.ndarray:
    """SplitMix64 output for state ``seed + (idx+1)*gamma`` (wrapping)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (idx.astype(np.uint64) + np.uint64(1)) * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Stream:
    """Counter-based uniform stream: u = (h >> 40) * 2^-24 in [0, 1)."""

    def __init__(self, seed: int, stream: int):
        self.base = int(splitmix(seed, np.array([stream], dtype=np.uint64))[0])
        self.pos = 0

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        h = splitmix(self.base, np.arange(self.pos, self.pos + n, dtype=np.uint64))
        self.pos += n
        u = (h >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)
        return np.float32(lo) + np.float32(hi - lo) * u


def box_quads(mins, maxs):
    """Six quads (4 x xyz) of an axis-aligned box, in the reference's order,
    with each face's outward normal."""
    x0, y0, z0 = (float(c) for c in mins)
    x1, y1, z1 = (float(c) for c in maxs)
    quads = [
        ((x0, y1, z1), (x1, y1, z1), (x1, y0, z1), (x0, y0, z1)),  # far
        ((x0, y1, z0), (x1, y1, z0), (x1, y0, z0), (x0, y0, z0)),  # near
        ((x0, y1, z1), (x0, y1, z0), (x0, y0, z0), (x0, y0, z1)),  # left
        ((x1, y1, z1), (x1, y1, z0), (x1, y0, z0), (x1, y0, z1)),  # right
        ((x0, y1, z1), (x1, y1, z1), (x1, y1, z0), (x0, y1, z0)),  # top
        ((x0, y0, z1), (x1, y0, z1), (x1, y0, z0), (x0, y0, z0)),  # bottom
    ]
    normals = [(0, 0, 1), (0, 0, -1), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, -1, 0)]
    return quads, normals


@dataclass
class TriangleSoup:
    """What ``Environment.AddTriangle`` receives: 9 floats and an id per triangle."""

    xyz: list = field(default_factory=list)
    ids: list = field(default_factory=list)

    def add_triangle(self, tid, v1, v2, v3):
        self.xyz.append((*v1, *v2, *v3))
        self.ids.append(tid)

    def add_quad(self, tid, v1, v2, v3, v4):
        self.add_triangle(tid, v1, v2, v3)
        self.add_triangle(tid + 1, v1, v3, v4)

    def add_box(self, tid, mins, maxs, ceiling_id=None):
        quads, _ = box_quads(mins, maxs)
        for k, q in enumerate(quads):
            self.add_quad(ceiling_id if (k == 0 and ceiling_id is not None) else tid, *q)

    def arrays(self):
        xyz = np.asarray(self.xyz, dtype=np.float32).reshape(-1, 9)
        ids = np.asarray(self.ids, dtype=np.int64).astype(np.int32)
        return np.ascontiguousarray(xyz), np.ascontiguousarray(ids)


def _random_boxes(rng: Stream, n: int, edge_lo: float, edge_hi: float):
    c = rng.uniform(3 * n, 0.0, ROOM).reshape(n, 3)
    e = rng.uniform(3 * n, edge_lo, edge_hi).reshape(n, 3)
    half = e * np.float32(0.5)
    mins = np.maximum(c - half, np.float32(1.0))
    maxs = np.minimum(c + half, np.float32(ROOM - 1.0))
    return mins.astype(np.float32), maxs.astype(np.float32)


@dataclass
class TraceScene:
    xyz: np.ndarray  # (N, 9) float32
    ids: np.ndarray  # (N,) int32
    starts: np.ndarray  # (R, 3) float32
    stops: np.ndarray  # (R, 3) float32


def anyhit_scene(seed: int = 0, n_boxes: int = 1024, n_rays: int = 1 << 20,
                 edge=(8.0, 128.0)) -> TraceScene:
    """Box room (12 triangles) + ``n_boxes`` boxes of 12 triangles (12,300 for
    1,024 boxes); ``n_rays`` shadow lines with both ends uniform inside the
    room.  Every triangle is TRACE_ID_OPAQUE."""
    soup = TriangleSoup()
    soup.add_box(TRACE_ID_OPAQUE, (0.0, 0.0, 0.0), (ROOM, ROOM, ROOM))
    mins, maxs = _random_boxes(Stream(seed, S_BOXES), n_boxes, *edge)
    for b in range(n_boxes):
        soup.add_box(TRACE_ID_OPAQUE, mins[b], maxs[b])
    xyz, ids = soup.arrays()
    rr = Stream(seed, S_RAYS)
    starts = rr.uniform(3 * n_rays, 1.0, ROOM - 1.0).reshape(n_rays, 3)
    stops = rr.uniform(3 * n_rays, 1.0, ROOM - 1.0).reshape(n_rays, 3)
    return TraceScene(xyz, ids, np.ascontiguousarray(starts), np.ascontiguousarray(stops))


@dataclass
class Light:
    type: int
    origin: tuple
    intensity: tuple
    normal: tuple = (0.0, 0.0, -1.0)
    keys: dict = field(default_factory=dict)


@dataclass
class LitScene:
    xyz: np.ndarray
    ids: np.ndarray
    tri_face: np.ndarray  # (N,) int32 face of each triangle, -1 if not a lit face
    corner: np.ndarray  # (F, 3)
    u: np.ndarray  # (F, 3)
    v: np.ndarray  # (F, 3)
    normal: np.ndarray  # (F, 3)
    nu: np.ndarray  # (F,) int32
    nv: np.ndarray  # (F,) int32
    luxscale: np.ndarray  # (F,) float32 luxels per world unit
    refl: np.ndarray  # (F, 3) float32, clamped to 0.99
    lights: list

    @property
    def n_faces(self):
        return int(self.corner.shape[0])

    @property
    def n_luxels(self):
        return int((self.nu.astype(np.int64) * self.nv).sum())

    def luxel_offset(self):
        off = np.zeros(self.n_faces + 1, dtype=np.int64)
        np.cumsum(self.nu.astype(np.int64) * self.nv, out=off[1:])
        return off


def _face_record(quad, normal, spacing):
    p = np.asarray(quad, dtype=np.float32)
    mn, mx = p.min(axis=0), p.max(axis=0)
    nax = int(np.argmax(np.abs(normal)))
    a, b = (nax + 1) % 3, (nax + 2) % 3
    corner = mn.copy()
    u = np.zeros(3, np.float32)
    v = np.zeros(3, np.float32)
    u[a] = mx[a] - mn[a]
    v[b] = mx[b] - mn[b]
    nu = max(1, int(np.ceil(float(u[a]) / spacing)))
    nv = max(1, int(np.ceil(float(v[b]) / spacing)))
    return corner, u, v, np.asarray(normal, np.float32), nu, nv


def _unit_vectors(rng: Stream, n: int) -> np.ndarray:
    """Uniform directions by rejection from the cube, normalised in float32."""
    out = []
    while len(out) < n:
        x, y, z = (float(c) for c in rng.uniform(3, -1.0, 1.0))
        r2 = np.float32(np.float32(x * x) + np.float32(y * y)) + np.float32(z * z)
        if 0.0 < r2 <= 1.0:
            inv = np.float32(1.0) / np.sqrt(np.float32(r2))
            out.append((np.float32(x) * inv, np.float32(y) * inv, np.float32(z) * inv))
    return np.asarray(out, dtype=np.float32)


def _tiled_room(soup: TriangleSoup, tiles: int, sky: bool) -> int:
    """The room's six faces, each split into tiles x tiles quads in its plane
    (the way a map's walls arrive as many brush sides), in the box's face
    order; returns the triangle count."""
    quads, _ = box_quads((0.0, 0.0, 0.0), (ROOM, ROOM, ROOM))
    for k, (v1, v2, _v3, v4) in enumerate(quads):
        a, b, d = (np.asarray(v, np.float64) for v in (v1, v2, v4))
        tid = TRACE_ID_SKY if (k == 0 and sky) else TRACE_ID_OPAQUE
        for i in range(tiles):
            for j in range(tiles):
                def at(s, t):
                    return tuple(float(c) for c in (a + (b - a) * (s / tiles) + (d - a) * (t / tiles)))
                soup.add_quad(tid, at(i, j), at(i + 1, j), at(i + 1, j + 1), at(i, j + 1))
    return 12 * tiles * tiles


def lit_scene(seed: int = 0, n_faces: int = 4096, spacing: float = 16.0, n_point: int = 64,
              n_spot: int = 8, sky: bool = True, edge=(64.0, 512.0), wall_tiles: int = 1) -> LitScene:
    """Direct-lighting scene: ``ceil(n_faces/6)`` boxes (edges U(64,512))
    whose first ``n_faces`` faces carry lightmaps at ``spacing`` units per
    luxel; the room ceiling (z = 4096) is TRACE_ID_SKY.  Lights: point lights
    with RGB U(50,500), quadratic attenuation, radius 1,024; spotlights with a
    30/45 degree cone; one sky-ambient light over the 162 sky directions.
    ``wall_tiles`` > 1 splits each room face into that many tiles per side
    (same planes, same lit boxes and lights)."""
    n_boxes = (n_faces + 5) // 6
    soup = TriangleSoup()
    if wall_tiles > 1:
        n_room = _tiled_room(soup, wall_tiles, sky)
    else:
        soup.add_box(TRACE_ID_OPAQUE, (0.0, 0.0, 0.0), (ROOM, ROOM, ROOM),
                     ceiling_id=TRACE_ID_SKY if sky else None)
        n_room = 12
    mins, maxs = _random_boxes(Stream(seed, S_BOXES), n_boxes, *edge)
    faces = []
    tri_face = [-1] * n_room
    for b in range(n_boxes):
        quads, normals = box_quads(mins[b], maxs[b])
        for k, q in enumerate(quads):
            soup.add_quad(TRACE_ID_OPAQUE, *q)
            f = 6 * b + k
            if f < n_faces:
                faces.append(_face_record(q, normals[k], spacing))
                tri_face += [f, f]
            else:
                tri_face += [-1, -1]
    xyz, ids = soup.arrays()
    corner = np.array([f[0] for f in faces], np.float32).reshape(-1, 3)
    u = np.array([f[1] for f in faces], np.float32).reshape(-1, 3)
    v = np.array([f[2] for f in faces], np.float32).reshape(-1, 3)
    nrm = np.array([f[3] for f in faces], np.float32).reshape(-1, 3)
    nu = np.array([f[4] for f in faces], np.int32)
    nv = np.array([f[5] for f in faces], np.int32)
    refl = np.minimum(Stream(seed, S_REFL).uniform(3 * len(faces), 0.1, 0.8).reshape(-1, 3),
                      np.float32(0.99))

    lr = Stream(seed, S_LIGHTS)
    lights = []
    for _ in range(n_point):
        o = tuple(float(c) for c in lr.uniform(3, 1.0, ROOM - 1.0))
        it = tuple(float(c) for c in lr.uniform(3, 50.0, 500.0))
        lights.append(Light(EMIT_POINT, o, it, keys=dict(quadratic_attn=1.0, distance=1024.0)))
    dirs = _unit_vectors(Stream(seed, S_SPOTDIR), n_spot)
    for i in range(n_spot):
        o = tuple(float(c) for c in lr.uniform(3, 1.0, ROOM - 1.0))
        it = tuple(float(c) for c in lr.uniform(3, 50.0, 500.0))
        lights.append(Light(EMIT_SPOTLIGHT, o, it, tuple(float(c) for c in dirs[i]),
                            keys=dict(quadratic_attn=1.0, distance=1024.0, inner_cone=30.0,
                                      cone=45.0, exponent=1.0)))
    if sky:
        lights.append(Light(EMIT_SKYAMBIENT, (0.0, 0.0, 0.0), (40.0, 50.0, 70.0)))
    return LitScene(xyz, ids, np.asarray(tri_face, np.int32), corner, u, v, nrm, nu, nv,
                    np.full(len(faces), np.float32(1.0 / spacing), np.float32),
                    np.ascontiguousarray(refl, dtype=np.float32), lights)


class BrushMap:
    """Lump arrays of a compiled map, written the way a BSP lays them out
    (the arrays ``Environment.add_bsp_world`` takes): planes in pairs (p ^ 1
    faces the other way), brushes over brush sides, leaves over leaf
    brushes, faces over signed surfedges.  Texinfo 0 is plain, 1 is sky."""

    def __init__(self):
        self.planes, self.sides, self.brushes = [], [], []
        self.texinfo = [0, SURF_SKY]  # texinfo 0 plain, 1 sky
        self.verts, self.edges, self.surf, self.faces = [], [[0, 0]], [], []

    def plane(self, n, d):
        n = np.asarray(n, np.float32)
        self.planes += [[*n, d], [*(-n), -d]]
        return len(self.planes) - 2

    def brush(self, planes, contents=CONTENTS_SOLID, texinfo=None, disp=None, bevel=None):
        first = len(self.sides)
        for i, (n, d) in enumerate(planes):
            self.sides.append([self.plane(n, d), (texinfo or {}).get(i, 0), (disp or {}).get(i, 0),
                               (bevel or {}).get(i, 0)])
        self.brushes.append([first, len(planes), contents])
        return len(self.brushes) - 1

    def box(self, mn, mx, **kw):
        planes = []
        for a in range(3):
            e = np.zeros(3, np.float32)
            e[a] = 1
            planes += [(e, float(mx[a])), (-e, -float(mn[a]))]
        return self.brush(planes, **kw)

    def face(self, pts, texinfo=1, flip_every=2):
        first = len(self.surf)
        base = len(self.verts)
        self.verts += [list(p) for p in pts]
        n = len(pts)
        for j in range(n):
            a, b = base + j, base + (j + 1) % n
            if j % flip_every == 1:  # stored the other way round: read through -edge
                self.edges.append([b, a])
                self.surf.append(-(len(self.edges) - 1))
            else:
                self.edges.append([a, b])
                self.surf.append(len(self.edges) - 1)
        self.faces.append([first, n, texinfo])

    def lumps(self, leaves=None):
        """leaves: brush lists of the leaves, which a chain of nodes visits in
        order (node k: leaf k in front, node k + 1 behind; the last node has
        the last two leaves; one leaf sits on both sides of node 0)."""
        leaves = leaves if leaves is not None else [list(range(len(self.brushes)))]
        ranges, lb = [], []
        for L in leaves:
            ranges.append([len(lb), len(L)])
            lb += L
        nl = len(leaves)
        if nl == 0:
            children = np.zeros((0, 2))
        elif nl == 1:
            children = [[-1, -1]]
        else:
            children = [[-1 - k, k + 1] for k in range(nl - 2)] + [[-1 - (nl - 2), -nl]]
        return dict(planes=self.planes, node_children=children, leaf_brush_ranges=ranges,
                    leaf_brushes=lb, brushes=self.brushes, brush_sides=self.sides,
                    texinfo_flags=self.texinfo, vertexes=self.verts or np.zeros((0, 3)),
                    edges=self.edges, surf_edges=self.surf or np.zeros(0),
                    faces=self.faces or np.zeros((0, 3)))


def lit_brush_world(seed: int = 0, n_faces: int = 4096, spacing: float = 16.0,
                    thick: float = 16.0):
    """The scene of ``lit_scene(seed, n_faces, spacing)`` -- its lit box faces
    and its lights -- with the room and the boxes written as brushes of a
    compiled map: a floor and four walls ``thick`` units thick around the
    same 4096-unit room, a sky face closing its top, and one box brush per
    box.  Returns (lumps, lit): the triangles are what ``add_bsp_world``
    makes of the lumps (``lit.xyz`` / ``lit.ids`` are empty), and
    ``lit.tri_face`` follows their order -- the room's five brushes, then
    each box's six sides in plane order (+x, -x, +y, -y, +z, -z, two
    triangles each), then the sky face."""
    lit = lit_scene(seed, n_faces=n_faces, spacing=spacing)
    n_boxes = (n_faces + 5) // 6
    mins, maxs = _random_boxes(Stream(seed, S_BOXES), n_boxes, 64.0, 512.0)
    w = BrushMap()
    t, L = float(thick), ROOM
    w.box((-t, -t, -t), (L + t, L + t, 0.0))  # floor
    w.box((-t, -t, 0.0), (0.0, L + t, L))
    w.box((L, -t, 0.0), (L + t, L + t, L))
    w.box((0.0, -t, 0.0), (L, 0.0, L))
    w.box((0.0, L, 0.0), (L, L + t, L))
    w.face([(0.0, 0.0, L), (L, 0.0, L), (L, L, L), (0.0, L, L)], texinfo=1)
    for b in range(n_boxes):
        w.box(tuple(float(c) for c in mins[b]), tuple(float(c) for c in maxs[b]))
    # box_quads' face order is z max, z min, x min, x max, y max, y min
    side_face = (3, 2, 4, 5, 0, 1)
    tri_face = [-1] * (5 * 12)
    for b in range(n_boxes):
        for s in range(6):
            f = 6 * b + side_face[s]
            tri_face += [f, f] if f < n_faces else [-1, -1]
    tri_face += [-1, -1]  # the sky face's two triangles
    lit.xyz = np.zeros((0, 9), np.float32)
    lit.ids = np.zeros(0, np.int32)
    lit.tri_face = np.asarray(tri_face, np.int32)
    return w.lumps(), lit


def transfer_directions(k: int) -> np.ndarray:
    """K cosine-weighted directions in a local frame (x, y tangent; z normal):
    a Fibonacci lattice on the unit disk lifted by Malley's method.  Built in
    float64 and rounded once to float32; callers pass the same table to the
    GPU path and to the oracle."""
    i = np.arange(k, dtype=np.float64)
    u1 = (i + 0.5) / k
    u2 = np.mod(i * 0.6180339887498949, 1.0)
    r = np.sqrt(u1)
    phi = 2.0 * np.pi * u2
    d = np.stack([r * np.cos(phi), r * np.sin(phi), np.sqrt(1.0 - u1)], axis=1)
    return np.ascontiguousarray(d.astype(np.float32))


S_BATCH = 6


def batch_face_counts(seed: int = 0, n_scenes: int = 256, lo: int = 64, hi: int = 4096):
    """Face counts log-uniform in [lo, hi] (uneven scene sizes)."""
    u = Stream(seed, S_BATCH).uniform(n_scenes).astype(np.float64)
    return np.rint(np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))).astype(np.int64)


def batch_scenes(seed: int = 0, n_scenes: int = 256, lo: int = 64, hi: int = 4096,
                 spacing: float = 48.0, n_point: int = 64, n_spot: int = 8):
    """Scenes built like the direct-light scene, with log-uniform face
    counts; scene i uses seed 1000*seed + i + 1."""
    counts = batch_face_counts(seed, n_scenes, lo, hi)
    return [lit_scene(1000 * seed + i + 1, n_faces=int(c), spacing=spacing, n_point=n_point,
                      n_spot=n_spot) for i, c in enumerate(counts)]
