"""Python face of the C ABI, named after the reference's Go API.

``Environment`` mirrors ``raytracer.Environment`` (raytracer/environment.go):
AddTriangle, AddQuad, AddAxisAlignedRectangularSolid,
SetupAccelerationStructure, Trace4Rays, GetTriangle and the ray stream;
``test_line_does_hit_sky`` mirrors ``trace.TestLineDoesHitSky``
(raytracer/trace/testline.go:18).  The radiosity stages the reference lacks
(gather, transfers, bounce) are methods on the same object.  Every call goes
through libvradgpu.so; nothing here computes a result itself.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

TRACE_ID_SKY = 0x01000000
TRACE_ID_OPAQUE = 0x02000000
TRACE_ID_STATICPROP = 0x04000000


class Light(C.Structure):
    """vrg_light (include/vradgpu.h)."""

    _fields_ = [("type", C.c_int32), ("origin", C.c_float * 3), ("intensity", C.c_float * 3),
                ("normal", C.c_float * 3), ("stopdot", C.c_float), ("stopdot2", C.c_float),
                ("exponent", C.c_float), ("constant_attn", C.c_float), ("linear_attn", C.c_float),
                ("quadratic_attn", C.c_float), ("radius", C.c_float), ("start_fade", C.c_float),
                ("end_fade", C.c_float), ("cap_distance", C.c_float)]


class LightKeys(C.Structure):
    _fields_ = [("fifty_percent_distance", C.c_float), ("zero_percent_distance", C.c_float),
                ("hard_falloff", C.c_int32), ("constant_attn", C.c_float),
                ("linear_attn", C.c_float), ("quadratic_attn", C.c_float), ("distance", C.c_float),
                ("inner_cone", C.c_float), ("cone", C.c_float), ("exponent", C.c_float)]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if shape is None else a.reshape(shape)


class Context:
    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.vrg_ctx_create(device, C.byref(h)), None, "vrg_ctx_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.vrg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream_ptr: int | None):
        check(self.lib.vrg_ctx_set_stream(self.h, C.c_void_p(stream_ptr or 0)), self.h, "set_stream")

    def synchronize(self):
        check(self.lib.vrg_ctx_synchronize(self.h), self.h, "synchronize")

    def set_timing(self, on: bool):
        check(self.lib.vrg_ctx_set_timing(self.h, int(on)), self.h, "set_timing")

    def kernel_stats(self, name: str):
        ms = C.c_double()
        n = C.c_int64()
        check(self.lib.vrg_ctx_kernel_stats(self.h, name.encode(), C.byref(ms), C.byref(n)),
              self.h, "kernel_stats")
        return ms.value, n.value

    def reset_stats(self):
        check(self.lib.vrg_ctx_reset_stats(self.h), self.h, "reset_stats")

    def launch_count(self) -> int:
        return int(self.lib.vrg_ctx_launch_count(self.h))

    def set_transfer_table_limit(self, limit: int):
        check(self.lib.vrg_ctx_set_transfer_table_limit(self.h, int(limit)), self.h,
              "set_transfer_table_limit")

    def set_hbm_reserve(self, nbytes: int):
        """Device memory that relight admission keeps free (default 1 GiB)."""
        check(self.lib.vrg_ctx_set_hbm_reserve(self.h, int(nbytes)), self.h, "set_hbm_reserve")

    def set_autotune(self, on: bool):
        check(self.lib.vrg_ctx_set_autotune(self.h, int(on)), self.h, "set_autotune")

    def autotune_choice(self, key: str):
        """(variant, per-variant ms) of a tuned bucket; variant -1 if untuned."""
        v = C.c_int32(-1)
        ms = (C.c_double * 32)()  # a launch site has at most 32 variants
        check(self.lib.vrg_ctx_autotune_choice(self.h, key.encode(), C.byref(v), ms, 32),
              self.h, "autotune_choice")
        return v.value, [x for x in ms if x > 0.0]

    def autotune_save(self, path: str):
        check(self.lib.vrg_ctx_autotune_save(self.h, str(path).encode()), self.h, "autotune_save")

    def autotune_load(self, path: str):
        check(self.lib.vrg_ctx_autotune_load(self.h, str(path).encode()), self.h, "autotune_load")

    @staticmethod
    def tune_key(site: str, triangles: int, work: int) -> str:
        """Bucket key of a tuned launch site (floor log2 of both sizes)."""
        lg = lambda v: int(v).bit_length() - 1 if v > 0 else 0
        return f"{site}/t{lg(triangles)}/n{lg(work)}"


def make_light(type_, origin, intensity, normal=(0.0, 0.0, -1.0), **keys) -> Light:
    """Builds one light the way CreateDirectLights does for an entity:
    ParseLightSpot / ParseLightPoint (rad/lightmap/lights.go:210-257,417-426)
    for spot and point lights."""
    lib = _lib.load()
    li = Light()
    li.type = type_
    li.origin[:] = origin
    li.intensity[:] = intensity
    li.normal[:] = normal
    li.start_fade, li.end_fade, li.cap_distance = 0.0, -1.0, 1.0e22
    k = LightKeys()
    for name, val in keys.items():
        setattr(k, name, val)
    if type_ == 2:
        check(lib.vrg_light_parse_spot(C.byref(k), C.byref(li)), None, "parse_spot")
    elif type_ == 1:
        check(lib.vrg_light_parse_point(C.byref(k), C.byref(li)), None, "parse_point")
    return li


class BspWorld(C.Structure):
    """vrg_bsp_world: the lump arrays addBrushesForRayTrace reads."""

    _fields_ = [("planes", C.c_void_p), ("num_planes", C.c_int32),
                ("node_children", C.c_void_p), ("num_nodes", C.c_int32),
                ("leaf_brush_ranges", C.c_void_p), ("num_leafs", C.c_int32),
                ("leaf_brushes", C.c_void_p), ("num_leaf_brushes", C.c_int32),
                ("brushes", C.c_void_p), ("num_brushes", C.c_int32),
                ("brush_sides", C.c_void_p), ("num_brush_sides", C.c_int32),
                ("texinfo_flags", C.c_void_p), ("num_texinfo", C.c_int32),
                ("vertexes", C.c_void_p), ("num_vertexes", C.c_int32),
                ("edges", C.c_void_p), ("num_edges", C.c_int32),
                ("surf_edges", C.c_void_p), ("num_surf_edges", C.c_int32),
                ("faces", C.c_void_p), ("num_faces", C.c_int32),
                ("headnode", C.c_int32), ("first_face", C.c_int32),
                ("num_model_faces", C.c_int32)]

    # (field, dtype, values per record)
    LUMPS = [("planes", np.float32, 4), ("node_children", np.int32, 2),
             ("leaf_brush_ranges", np.int32, 2), ("leaf_brushes", np.int32, 1),
             ("brushes", np.int32, 3), ("brush_sides", np.int32, 4),
             ("texinfo_flags", np.int32, 1), ("vertexes", np.float32, 3), ("edges", np.int32, 2),
             ("surf_edges", np.int32, 1), ("faces", np.int32, 3)]
    COUNTS = {"planes": "num_planes", "node_children": "num_nodes",
              "leaf_brush_ranges": "num_leafs", "leaf_brushes": "num_leaf_brushes",
              "brushes": "num_brushes", "brush_sides": "num_brush_sides",
              "texinfo_flags": "num_texinfo", "vertexes": "num_vertexes", "edges": "num_edges",
              "surf_edges": "num_surf_edges", "faces": "num_faces"}

    @classmethod
    def from_arrays(cls, lumps: dict, headnode: int = 0, first_face: int = 0,
                    num_model_faces: int | None = None):
        """lumps maps each field name to an array of records; returns the
        structure and the contiguous arrays it points into (keep them alive)."""
        w = cls()
        keep = []
        for name, dt, per in cls.LUMPS:
            a = np.ascontiguousarray(lumps.get(name, np.zeros((0, per))), dtype=dt).reshape(-1, per)
            keep.append(a)
            setattr(w, name, a.ctypes.data if a.size else None)
            setattr(w, cls.COUNTS[name], a.shape[0])
        w.headnode = headnode
        w.first_face = first_face
        w.num_model_faces = w.num_faces - first_face if num_model_faces is None else num_model_faces
        return w, keep


def read_bsp(data: bytes, hdr: bool = False):
    """Decodes a compiled map (vrg_bsp_open): the lump arrays the brush ingest
    reads, keyed as BspWorld.from_arrays takes them, plus model 0's headnode and
    face range, the BSP version and the texinfos' lightmap vectors."""
    lib = _lib.load()
    buf = np.frombuffer(data, np.uint8)
    h = C.c_void_p()
    check(lib.vrg_bsp_open(_p(buf) if buf.size else None, buf.size, C.byref(h)), None, "bsp_open")
    try:
        check(lib.vrg_bsp_use_hdr_faces(h, int(hdr)), None, "bsp_use_hdr_faces")
        w = BspWorld()
        check(lib.vrg_bsp_get_world(h, C.byref(w)), None, "bsp_get_world")
        out = {}
        for name, dt, per in BspWorld.LUMPS:
            n = getattr(w, BspWorld.COUNTS[name]) * per
            ptr = getattr(w, name)
            ct = C.c_float if dt == np.float32 else C.c_int32
            a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), (n,)).copy() if n else np.zeros(0, dt)
            out[name] = a.reshape(-1, per)
        version, ntex, vecs = C.c_int32(), C.c_int32(), C.POINTER(C.c_float)()
        check(lib.vrg_bsp_info(h, C.byref(version), C.byref(ntex), C.byref(vecs)), None, "bsp_info")
        lm = (np.ctypeslib.as_array(vecs, (ntex.value * 8,)).copy() if ntex.value
              else np.zeros(0, np.float32)).reshape(-1, 2, 4)
        return dict(lumps=out, headnode=w.headnode, first_face=w.first_face,
                    num_model_faces=w.num_model_faces, version=version.value, lightmap_vecs=lm)
    finally:
        lib.vrg_bsp_close(h)


def leaf_sky_lines(leaf_mins, leaf_maxs):
    """The (n * 162) start and stop points CanLeafTraceToSky traces for each leaf."""
    lib = _lib.load()
    mn = np.ascontiguousarray(leaf_mins, np.int32).reshape(-1, 3)
    mx = np.ascontiguousarray(leaf_maxs, np.int32).reshape(-1, 3)
    n = mn.shape[0]
    a = np.zeros((n * 162, 3), np.float32)
    b = np.zeros((n * 162, 3), np.float32)
    check(lib.vrg_leaf_sky_lines(_p(mn), _p(mx), n, _p(a), _p(b)), None, "leaf_sky_lines")
    return a, b


def base_winding_for_plane(normal, dist):
    """BaseWindingForPlane (vmath/polygon/winding.go:25-83): 4 x 3 float32."""
    lib = _lib.load()
    out = np.zeros((4, 3), np.float32)
    check(lib.vrg_base_winding_for_plane(_p(_f32(normal, (3,))), float(dist), _p(out)), None,
          "base_winding_for_plane")
    return out


def chop_winding(points, normal, dist, epsilon=0.0):
    """ChopWindingInPlace (winding.go:85-170): the part in front of the plane."""
    lib = _lib.load()
    pts = _f32(points, (-1, 3))
    out = np.zeros((pts.shape[0] + 4, 3), np.float32)
    n = np.zeros(1, np.int32)
    check(lib.vrg_chop_winding(_p(pts), pts.shape[0], _p(_f32(normal, (3,))), float(dist),
                               float(epsilon), _p(out), _p(n)), None, "chop_winding")
    return out[: n[0]]


def calc_face_extents(vertices, lightmap_vecs):
    """CalcFaceExtents (rad/world/face.go:14-90): LightmapTextureMinsInLuxels,
    LightmapTextureSizeInLuxels and whether the face is too big for a lightmap,
    from the face's vertices (winding order) and LightmapVecsLuxelsPerWorldUnits."""
    lib = _lib.load()
    v = _f32(vertices, (-1, 3))
    vecs = _f32(lightmap_vecs, (2, 4))
    mins, size, big = np.zeros(2, np.int32), np.zeros(2, np.int32), np.zeros(1, np.int32)
    check(lib.vrg_calc_face_extents(_p(v), v.shape[0], _p(vecs), _p(mins), _p(size), _p(big)),
          None, "calc_face_extents")
    return (int(mins[0]), int(mins[1])), (int(size[0]), int(size[1])), bool(big[0])


def light_array(lights) -> "C.Array":
    arr = (Light * max(len(lights), 1))()
    for i, li in enumerate(lights):
        arr[i] = li if isinstance(li, Light) else make_light(li.type, li.origin, li.intensity,
                                                             li.normal, **li.keys)
    return arr


class Environment:
    """raytracer.Environment on the GPU."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        check(self.lib.vrg_env_create(ctx.h, C.byref(h)), ctx.h, "vrg_env_create")
        self.h = h
        self.n_lights = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.vrg_env_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc, what):
        check(rc, self.ctx.h, what)

    # --- triangle soup (environment.go:41-117) ---
    def AddTriangle(self, tid, v1, v2, v3, colour=None, flags=0, material=0):
        vs = [_f32(v, 3) for v in (v1, v2, v3)]
        col = None if colour is None else _f32(colour, 3)
        self._chk(self.lib.vrg_env_add_triangle(self.h, tid, *[_p(v) for v in vs], _p(col), flags,
                                                material), "AddTriangle")

    def AddQuad(self, tid, v1, v2, v3, v4, colour=None):
        vs = [_f32(v, 3) for v in (v1, v2, v3, v4)]
        col = None if colour is None else _f32(colour, 3)
        self._chk(self.lib.vrg_env_add_quad(self.h, tid, *[_p(v) for v in vs], _p(col)), "AddQuad")

    def AddAxisAlignedRectangularSolid(self, tid, mins, maxs, colour=None):
        a, b = _f32(mins, 3), _f32(maxs, 3)
        col = None if colour is None else _f32(colour, 3)
        self._chk(self.lib.vrg_env_add_axis_aligned_rectangular_solid(self.h, tid, _p(a), _p(b),
                                                                      _p(col)),
                  "AddAxisAlignedRectangularSolid")

    def add_triangles(self, xyz, ids):
        xyz = _f32(xyz, (-1, 9))
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        self._chk(self.lib.vrg_env_add_triangles(self.h, _p(xyz), _p(ids), xyz.shape[0]),
                  "add_triangles")

    def SetupAccelerationStructure(self):
        self._chk(self.lib.vrg_env_setup_acceleration_structure(self.h),
                  "SetupAccelerationStructure")

    def add_bsp_world(self, lumps: dict, headnode: int = 0, first_face: int = 0,
                      num_model_faces: int | None = None):
        """addBrushesForRayTrace (cmd/tasks/loadbsp/main.go:283-340): the world's
        opaque brushes and sky faces as triangles; returns (brush, sky) counts."""
        w, keep = BspWorld.from_arrays(lumps, headnode, first_face, num_model_faces)
        nb, ns = C.c_int64(), C.c_int64()
        self._chk(self.lib.vrg_env_add_bsp_world(self.h, C.byref(w), C.byref(nb), C.byref(ns)),
                  "add_bsp_world")
        del keep
        return nb.value, ns.value

    def add_bsp_file(self, data: bytes, hdr: bool = False):
        """A compiled map's brushes and sky faces (vrg_bsp_open + vrg_env_add_bsp_world);
        hdr takes the world's faces from the HDR face lump, as loadbsp does with -hdr."""
        m = read_bsp(data, hdr)
        return self.add_bsp_world(m["lumps"], m["headnode"], m["first_face"], m["num_model_faces"])

    def get_triangle_vertices(self, first: int = 0, n: int | None = None):
        """(n, 9) vertices and (n,) ids of the triangles added so far."""
        n = self.num_triangles() - first if n is None else n
        xyz = np.zeros((n, 9), np.float32)
        ids = np.zeros(n, np.int32)
        self._chk(self.lib.vrg_env_get_triangle_vertices(self.h, first, n, _p(xyz), _p(ids)),
                  "get_triangle_vertices")
        return xyz, ids

    def num_triangles(self) -> int:
        return int(self.lib.vrg_env_num_triangles(self.h))

    def tree(self):
        nn, nr, ht = C.c_int64(), C.c_int64(), C.c_int32()
        self._chk(self.lib.vrg_env_tree_info(self.h, C.byref(nn), C.byref(nr), C.byref(ht)),
                  "tree_info")
        ch = np.zeros(nn.value, np.uint32)
        sp = np.zeros(nn.value, np.float32)
        refs = np.zeros(max(nr.value, 1), np.int32)
        self._chk(self.lib.vrg_env_get_tree(self.h, _p(ch), _p(sp), _p(refs)), "get_tree")
        return ch, sp, refs[: nr.value], ht.value

    def set_walk_tree_costs(self, traversal=1.0, intersection=1.2, empty_bonus=0.9,
                            max_depth=28):
        self._chk(self.lib.vrg_env_set_walk_tree_costs(self.h, traversal, intersection,
                                                       empty_bonus, max_depth),
                  "set_walk_tree_costs")

    def set_walk_tree_builder(self, mode):
        """0 / False: host, 1 / True or -1 (the default): the context's GPU."""
        self._chk(self.lib.vrg_env_set_walk_tree_builder(self.h, int(mode)),
                  "set_walk_tree_builder")

    def walk_tree(self):
        """The tree the device walks: (children, split, refs, height)."""
        nn, nr, ht = C.c_int64(), C.c_int64(), C.c_int32()
        self._chk(self.lib.vrg_env_walk_tree_info(self.h, C.byref(nn), C.byref(nr),
                                                  C.byref(ht)), "walk_tree_info")
        ch = np.zeros(nn.value, np.uint32)
        sp = np.zeros(nn.value, np.float32)
        refs = np.zeros(max(nr.value, 1), np.int32)
        self._chk(self.lib.vrg_env_get_walk_tree(self.h, _p(ch), _p(sp), _p(refs)),
                  "get_walk_tree")
        return ch, sp, refs[: nr.value], ht.value

    def set_wall_slots(self, enable: bool):
        """Wall slots on (default) or off; before SetupAccelerationStructure."""
        self._chk(self.lib.vrg_env_set_wall_slots(self.h, int(bool(enable))), "set_wall_slots")

    def wall_slots(self):
        """(tris (6, 4), counts (6,)): the opaque triangles in each scene-box
        face that shadow lines test before walking."""
        tris = np.zeros(24, np.int32)
        counts = np.zeros(6, np.int32)
        self._chk(self.lib.vrg_env_wall_slots(self.h, _p(tris), _p(counts)), "wall_slots")
        return tris.reshape(6, 4), counts

    def GetTriangle(self, index) -> bytes:
        buf = (C.c_uint8 * 48)()
        self._chk(self.lib.vrg_env_get_triangle(self.h, index, buf), "GetTriangle")
        return bytes(buf)

    def triangle_records(self) -> np.ndarray:
        n = self.num_triangles()
        return np.frombuffer(b"".join(self.GetTriangle(i) for i in range(n)),
                             dtype=np.uint32).reshape(n, 12)

    # --- trace (environment.go:140, testline.go:18) ---
    def Trace4Rays(self, origin, direction, tmin, tmax, skip_id=-1):
        """FourRays in SoA order (x x x x y y y y z z z z)."""
        o, d = _f32(origin, 12), _f32(direction, 12)
        t0, t1 = _f32(tmin, 4), _f32(tmax, 4)
        hit = np.zeros(4, np.int32)
        dist = np.zeros(4, np.float32)
        nrm = np.zeros(12, np.float32)
        self._chk(self.lib.vrg_env_trace4_rays(self.h, _p(o), _p(d), _p(t0), _p(t1), skip_id,
                                               _p(hit), _p(dist), _p(nrm)), "Trace4Rays")
        return hit, dist, nrm

    def trace_closest(self, origin, direction, tmin, tmax, skip_id=-1):
        o, d = _f32(origin, (-1, 3)), _f32(direction, (-1, 3))
        n = o.shape[0]
        t0 = _f32(np.broadcast_to(np.float32(tmin) if np.isscalar(tmin) else tmin, (n,)))
        t1 = _f32(np.broadcast_to(np.float32(tmax) if np.isscalar(tmax) else tmax, (n,)))
        hit = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        self._chk(self.lib.vrg_env_trace_closest(self.h, _p(o), _p(d), _p(t0), _p(t1), n, skip_id,
                                                 _p(hit), _p(t)), "trace_closest")
        return hit, t

    def set_triangle_flags(self, first, flags, colours=None):
        """Flags (VRG_TRIFLAG_TRANSPARENT = 1) and colours of triangles
        [first, first + len(flags)); colour x is a transparent triangle's
        coverage."""
        fl = np.ascontiguousarray(flags, np.uint8)
        col = None if colours is None else _f32(colours, (-1, 3))
        self._chk(self.lib.vrg_env_set_triangle_flags(self.h, int(first), fl.size, _p(fl),
                                                      _p(col)), "set_triangle_flags")

    def trace_coverage(self, origin, direction, tmin, tmax, skip_id=-1):
        """Trace4Rays with a coverage-counting transparency callback: per ray
        the recorded hit, its t and the coverage."""
        o, d = _f32(origin, (-1, 3)), _f32(direction, (-1, 3))
        n = o.shape[0]
        t0 = _f32(np.broadcast_to(np.float32(tmin) if np.isscalar(tmin) else tmin, (n,)))
        t1 = _f32(np.broadcast_to(np.float32(tmax) if np.isscalar(tmax) else tmax, (n,)))
        hit, t, cov = np.empty(n, np.int32), np.empty(n, np.float32), np.empty(n, np.float32)
        self._chk(self.lib.vrg_env_trace_coverage(self.h, _p(o), _p(d), _p(t0), _p(t1), n, skip_id,
                                                  _p(hit), _p(t), _p(cov)), "trace_coverage")
        return hit, t, cov

    def test_line_coverage(self, start, stop, static_prop_to_skip=-1):
        """TestLineDoesHitSky with texture shadows (transparent coverage)."""
        a, b = _f32(start, (-1, 3)), _f32(stop, (-1, 3))
        out = np.empty(a.shape[0], np.float32)
        self._chk(self.lib.vrg_env_test_line_coverage(self.h, _p(a), _p(b), a.shape[0],
                                                      static_prop_to_skip, _p(out)),
                  "test_line_coverage")
        return out

    def test_line_does_hit_sky(self, start, stop, static_prop_to_skip=-1):
        a, b = _f32(start, (-1, 3)), _f32(stop, (-1, 3))
        out = np.empty(a.shape[0], np.float32)
        self._chk(self.lib.vrg_env_test_line_does_hit_sky(self.h, _p(a), _p(b), a.shape[0],
                                                          static_prop_to_skip, _p(out)),
                  "TestLineDoesHitSky")
        return out

    def CanLeafTraceToSky(self, leaf_mins, leaf_maxs):
        """rad/lightmap/lightmap.go:425-451 for every leaf: bool per leaf."""
        mn = np.ascontiguousarray(leaf_mins, np.int32).reshape(-1, 3)
        mx = np.ascontiguousarray(leaf_maxs, np.int32).reshape(-1, 3)
        out = np.zeros(mn.shape[0], np.uint8)
        self._chk(self.lib.vrg_env_can_leaf_trace_to_sky(self.h, _p(mn), _p(mx), mn.shape[0],
                                                         _p(out)), "CanLeafTraceToSky")
        return out.astype(bool)

    def occlusion_mask(self, start, stop, skip_id=-1, closest=False):
        a, b = _f32(start, (-1, 3)), _f32(stop, (-1, 3))
        n = a.shape[0]
        mask = np.zeros((n + 31) // 32, np.uint32)
        hit = np.empty(n, np.int32) if closest else None
        t = np.empty(n, np.float32) if closest else None
        self._chk(self.lib.vrg_env_occlusion_mask(self.h, _p(a), _p(b), n, skip_id, _p(mask),
                                                  _p(hit), _p(t)), "occlusion_mask")
        return (mask, hit, t) if closest else mask

    def AddToRayStream(self, start, stop, skip_id=-1):
        a, b = _f32(start, 3), _f32(stop, 3)
        self._chk(self.lib.vrg_env_add_to_ray_stream(self.h, _p(a), _p(b), skip_id),
                  "AddToRayStream")

    def FlushStreamEntry(self):
        self._chk(self.lib.vrg_env_flush_stream_entry(self.h), "FlushStreamEntry")

    def FinishRayStream(self, capacity):
        out = np.empty(max(capacity, 1), np.float32)
        cnt = C.c_int64()
        self._chk(self.lib.vrg_env_finish_ray_stream(self.h, _p(out), capacity, C.byref(cnt)),
                  "FinishRayStream")
        return out[: cnt.value]

    # --- lights / faces / gather ---
    def set_lights(self, lights):
        arr = light_array(lights)
        self.n_lights = len(lights)
        self._chk(self.lib.vrg_env_set_lights(self.h, arr, len(lights)), "set_lights")
        return arr

    def set_faces(self, lit):
        self._faces = dict(corner=_f32(lit.corner), u=_f32(lit.u), v=_f32(lit.v),
                           normal=_f32(lit.normal), nu=np.ascontiguousarray(lit.nu, np.int32),
                           nv=np.ascontiguousarray(lit.nv, np.int32),
                           luxscale=_f32(lit.luxscale), refl=_f32(lit.refl),
                           tri_face=np.ascontiguousarray(lit.tri_face, np.int32))
        f = self._faces
        self._chk(self.lib.vrg_env_set_faces(self.h, lit.n_faces, _p(f["corner"]), _p(f["u"]),
                                             _p(f["v"]), _p(f["normal"]), _p(f["nu"]),
                                             _p(f["nv"]), _p(f["luxscale"]), _p(f["refl"]), None,
                                             _p(f["tri_face"])), "set_faces")

    def num_luxels(self) -> int:
        return int(self.lib.vrg_env_num_luxels(self.h))

    def gather_direct_light(self, supersamples=4, seed=0):
        out = np.empty((self.num_luxels(), 3), np.float32)
        rays = C.c_uint64()
        self._chk(self.lib.vrg_env_gather_direct_light(self.h, supersamples, seed, _p(out),
                                                       C.byref(rays)), "gather_direct_light")
        return out, rays.value

    def gather_points(self, pts, nrm):
        pts, nrm = _f32(pts, (-1, 3)), _f32(nrm, (-1, 3))
        out = np.empty_like(pts)
        rays = C.c_uint64()
        self._chk(self.lib.vrg_env_gather_points(self.h, _p(pts), _p(nrm), pts.shape[0], _p(out),
                                                 C.byref(rays)), "gather_points")
        return out, rays.value

    # --- patches / transfers / bounce ---
    def make_patches(self, max_chop=4.0, min_chop=4.0):
        npch, nl = C.c_int64(), C.c_int64()
        self._chk(self.lib.vrg_env_make_patches(self.h, max_chop, min_chop, C.byref(npch),
                                                C.byref(nl)), "make_patches")
        n = npch.value
        P = dict(mins=np.zeros((n, 3), np.float32), maxs=np.zeros((n, 3), np.float32),
                 center=np.zeros((n, 3), np.float32), area=np.zeros(n, np.float32),
                 face=np.zeros(n, np.int32), parent=np.zeros(n, np.int32),
                 child1=np.zeros(n, np.int32), child2=np.zeros(n, np.int32),
                 split_axis=np.zeros(n, np.int32), split_dist=np.zeros(n, np.float32),
                 leaf_index=np.zeros(n, np.int32))
        self._chk(self.lib.vrg_env_get_patches(self.h, *[_p(P[k]) for k in (
            "mins", "maxs", "center", "area", "face", "parent", "child1", "child2", "split_axis",
            "split_dist", "leaf_index")]), "get_patches")
        P["n_leaves"] = nl.value
        return P

    def make_transfers(self, dirs_local):
        d = _f32(dirs_local, (-1, 3))
        nnz = C.c_int64()
        self._chk(self.lib.vrg_env_make_transfers(self.h, _p(d), d.shape[0], C.byref(nnz)),
                  "make_transfers")
        return nnz.value

    def transfer_info(self):
        """(k, nnz, rows past the shared-memory row table) of the last build."""
        k, nnz, ovf = C.c_int32(), C.c_int64(), C.c_int64()
        self._chk(self.lib.vrg_env_transfer_info(self.h, C.byref(k), C.byref(nnz), C.byref(ovf)),
                  "transfer_info")
        return k.value, nnz.value, ovf.value

    def get_transfers(self, n_leaves, nnz):
        row_ptr = np.zeros(n_leaves + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int32)
        w = np.zeros(max(nnz, 1), np.float32)
        self._chk(self.lib.vrg_env_get_transfers(self.h, _p(row_ptr), _p(col), _p(w)),
                  "get_transfers")
        return row_ptr, col[:nnz], w[:nnz]

    def gather_patch_direct(self, n_leaves):
        out = np.empty((n_leaves, 3), np.float32)
        self._chk(self.lib.vrg_env_gather_patch_direct(self.h, _p(out)), "gather_patch_direct")
        return out

    def bake(self, supersamples=4, seed=0, max_bounces=100, rel_tol=1e-3):
        """Direct light + bounce of this scene (the one-scene-per-launch path)."""
        rays = C.c_uint64()
        self._chk(self.lib.vrg_env_bake(self.h, supersamples, seed, max_bounces, rel_tol,
                                        C.byref(rays)), "bake")
        return rays.value

    def relight_prepare(self, supersamples=4, seed=0, max_bounces=100, rel_tol=1e-3):
        self._chk(self.lib.vrg_env_relight_prepare(self.h, supersamples, seed, max_bounces,
                                                   rel_tol), "relight_prepare")

    def relight(self, edits, max_iters=32, rel_tol=1e-3):
        """edits: [(light index, Light)]; returns (bounces, delta)."""
        arr = edit_array(edits)
        b, d = C.c_int32(), C.c_float()
        self._chk(self.lib.vrg_env_relight(self.h, arr, len(edits), max_iters, rel_tol,
                                           C.byref(b), C.byref(d)), "relight")
        return b.value, d.value

    def get_bake(self, n_leaves):
        lux = np.empty((self.num_luxels(), 3), np.float32)
        direct = np.empty((n_leaves, 3), np.float32)
        total = np.empty((n_leaves, 3), np.float32)
        b, d = C.c_int32(), C.c_float()
        self._chk(self.lib.vrg_env_get_bake(self.h, _p(lux), _p(direct), _p(total), C.byref(b),
                                            C.byref(d)), "get_bake")
        return dict(luxels=lux, patch_direct=direct, patch_total=total, bounces=b.value,
                    delta=d.value)

    def get_lightmap(self):
        """Lightmap samples of the last bake: (num_luxels, 4) uint8 shared-exponent
        samples (r, g, b, signed exponent) and the nfaces + 1 byte offsets of each
        face's first sample."""
        samples = np.empty((self.num_luxels(), 4), np.uint8)
        nf = len(self._faces["nu"]) if hasattr(self, "_faces") else 0
        offsets = np.empty(nf + 1, np.int64)
        self._chk(self.lib.vrg_env_get_lightmap(self.h, _p(samples), _p(offsets)), "get_lightmap")
        return samples, offsets

    def bounce_light(self, n_leaves, max_bounces=100, rel_tol=1e-3):
        total = np.empty((n_leaves, 3), np.float32)
        b = C.c_int32()
        d = C.c_float()
        self._chk(self.lib.vrg_env_bounce_light(self.h, max_bounces, rel_tol, _p(total),
                                                C.byref(b), C.byref(d)), "bounce_light")
        return total, b.value, d.value


class LightEdit(C.Structure):
    """vrg_light_edit: replace light `index` with `light`."""

    _fields_ = [("index", C.c_int32), ("light", Light)]


def edit_array(edits) -> "C.Array":
    arr = (LightEdit * max(len(edits), 1))()
    for i, (idx, li) in enumerate(edits):
        arr[i].index = idx
        arr[i].light = li if isinstance(li, Light) else make_light(li.type, li.origin,
                                                                   li.intensity, li.normal,
                                                                   **li.keys)
    return arr


class Server:
    """Relight server (vrg_server_*): slots requests in flight at once, one
    CUDA stream each, admitted as slots and scenes free up."""

    def __init__(self, ctx: Context, slots=8, max_iters=32, rel_tol=1e-3):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        check(self.lib.vrg_server_create(ctx.h, slots, max_iters, rel_tol, C.byref(h)), ctx.h,
              "vrg_server_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.vrg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_scene(self, env: Environment) -> int:
        sid = C.c_int32()
        check(self.lib.vrg_server_add_scene(self.h, env.h, C.byref(sid)), self.ctx.h, "add_scene")
        return sid.value

    def submit(self, scene: int, edits) -> int:
        arr = edit_array(edits)
        t = C.c_int64()
        check(self.lib.vrg_server_submit(self.h, scene, arr, len(edits), C.byref(t)), self.ctx.h,
              "submit")
        return t.value

    def wait(self, ticket: int, timeout=60.0) -> int:
        return int(self.lib.vrg_server_wait(self.h, ticket, timeout))

    def drain(self, timeout=600.0):
        check(self.lib.vrg_server_drain(self.h, timeout), self.ctx.h, "drain")

    def result(self, ticket: int) -> dict:
        st, b, d = C.c_int32(), C.c_int32(), C.c_float()
        times = (C.c_double * 3)()
        dig = (C.c_double * 2)()
        check(self.lib.vrg_server_result(self.h, ticket, C.byref(st), C.byref(b), C.byref(d), times,
                                         dig), self.ctx.h, "result")
        return dict(status=st.value, bounces=b.value, delta=d.value, submit=times[0],
                    start=times[1], done=times[2], digest=(dig[0], dig[1]))


class Batch:
    """Resident scenes baked together (vrg_batch_*): one persistent direct
    launch over all scenes and one block-diagonal bounce loop."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        check(self.lib.vrg_batch_create(ctx.h, C.byref(h)), ctx.h, "vrg_batch_create")
        self.h = h
        self.envs = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.vrg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add(self, env: Environment):
        check(self.lib.vrg_batch_add(self.h, env.h), self.ctx.h, "vrg_batch_add")
        self.envs.append(env)

    def bake(self, supersamples=4, seed=0, max_bounces=100, rel_tol=1e-3):
        rays = C.c_uint64()
        check(self.lib.vrg_batch_bake(self.h, supersamples, seed, max_bounces, rel_tol,
                                      C.byref(rays)), self.ctx.h, "vrg_batch_bake")
        return rays.value
