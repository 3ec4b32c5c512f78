"""ctypes view of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product library never does.  ``build()`` compiles
``vrad_oracle.c`` with gcc into ``oracle/_build/liboracle.so``.
"""
from __future__ import annotations

import ctypes as C  # noqa: N812
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

FIXED, LITERAL = 0, 1


def build(force: bool = False) -> Path:
    src = HERE / "vrad_oracle.c"
    deps = [src, HERE / "vrad_oracle.h", HERE.parent / "vrad_gb300" / "csrc" / "anorms_table.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-std=c11", "-shared",
           "-pthread", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class OTri(C.Structure):
    _fields_ = [("nx", C.c_float), ("ny", C.c_float), ("nz", C.c_float), ("d", C.c_float),
                ("id", C.c_int32), ("e", C.c_float * 6), ("cs0", C.c_uint8), ("cs1", C.c_uint8),
                ("flags", C.c_uint8), ("unused", C.c_uint8)]


class OLight(C.Structure):
    _fields_ = [("type", C.c_int32), ("origin", C.c_float * 3), ("intensity", C.c_float * 3),
                ("normal", C.c_float * 3), ("stopdot", C.c_float), ("stopdot2", C.c_float),
                ("exponent", C.c_float), ("constant_attn", C.c_float), ("linear_attn", C.c_float),
                ("quadratic_attn", C.c_float), ("radius", C.c_float), ("start_fade", C.c_float),
                ("end_fade", C.c_float), ("cap_distance", C.c_float)]


class OKeys(C.Structure):
    _fields_ = [("fifty_percent_distance", C.c_float), ("zero_percent_distance", C.c_float),
                ("hard_falloff", C.c_int32), ("constant_attn", C.c_float),
                ("linear_attn", C.c_float), ("quadratic_attn", C.c_float), ("distance", C.c_float),
                ("inner_cone", C.c_float), ("cone", C.c_float), ("exponent", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.orc_scene_new.restype = C.c_void_p
        _lib.orc_scene_new.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int]
        _lib.orc_scene_free.argtypes = [C.c_void_p]
        for f in ("orc_scene_num_nodes", "orc_scene_num_refs"):
            getattr(_lib, f).restype = C.c_int64
            getattr(_lib, f).argtypes = [C.c_void_p]
        _lib.orc_scene_depth.argtypes = [C.c_void_p]
        _lib.orc_make_patches.restype = C.c_int64
        _lib.orc_make_transfers.restype = C.c_int64
        _lib.orc_bounce_f64.restype = C.c_int
        _lib.orc_encode_sample.restype = C.c_uint32
        _lib.orc_encode_sample.argtypes = [C.c_float, C.c_float, C.c_float]
        _lib.orc_calc_face_extents.restype = C.c_int
        _lib.orc_calc_face_extents.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Scene:
    """Oracle triangle soup + kd tree (``SetupAccelerationStructure``)."""

    def __init__(self, xyz, ids, flags=None, mode=FIXED):
        L = lib()
        self.xyz = f32(xyz).reshape(-1, 9)
        self.ids = np.ascontiguousarray(ids, dtype=np.int32)
        self.n = self.xyz.shape[0]
        fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
        self.h = L.orc_scene_new(_p(self.xyz), _p(self.ids), _p(fl), self.n, mode)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_free(C.c_void_p(self.h))
            self.h = None

    def tree(self):
        L = lib()
        nn = L.orc_scene_num_nodes(self.h)
        nr = L.orc_scene_num_refs(self.h)
        ch = np.zeros(nn, np.uint32)
        sp = np.zeros(nn, np.float32)
        refs = np.zeros(max(nr, 1), np.int32)
        L.orc_scene_get_tree(C.c_void_p(self.h), _p(ch), _p(sp), _p(refs))
        return ch, sp, refs[:nr]

    def set_tree(self, children, split, refs):
        """Walk another tree of the same format (e.g. the library's walk tree)."""
        ch = np.ascontiguousarray(children, np.uint32)
        sp = np.ascontiguousarray(split, np.float32)
        rf = np.ascontiguousarray(refs, np.int32)
        rc = lib().orc_scene_set_tree(C.c_void_p(self.h), _p(ch), _p(sp), C.c_int64(ch.size),
                                      _p(rf), C.c_int64(rf.size))
        if rc != 0:
            raise RuntimeError("orc_scene_set_tree failed")

    def set_skip_empty(self, on: bool):
        """Walk as the library's kOptSkip variants do (for node counts)."""
        lib().orc_scene_set_skip_empty(C.c_void_p(self.h), int(bool(on)))

    def set_walls(self, tris=None, counts=None):
        """Test each shadow line's exit-face wall triangles first, as the
        library does (tris: 6 x 4 triangle indices, counts: 6); None: off."""
        if tris is None:
            lib().orc_scene_set_walls(C.c_void_p(self.h), None, None)
            return
        t = np.ascontiguousarray(tris, np.int32).reshape(24)
        c = np.ascontiguousarray(counts, np.int32).reshape(6)
        lib().orc_scene_set_walls(C.c_void_p(self.h), _p(t), _p(c))

    def tris(self):
        out = (OTri * max(self.n, 1))()
        lib().orc_scene_get_tris(C.c_void_p(self.h), out)
        return out

    def tri_records(self) -> np.ndarray:
        """(N, 12) uint32 view of the 48-byte intersection records."""
        t = self.tris()
        return np.frombuffer(bytes(t), dtype=np.uint32).reshape(-1, 12)[: self.n].copy()

    def bounds(self):
        mn = np.zeros(3, np.float32)
        mx = np.zeros(3, np.float32)
        lib().orc_scene_bounds(C.c_void_p(self.h), _p(mn), _p(mx))
        return mn, mx

    def trace_closest(self, o, d, tmin, tmax, skip=-1, brute=False, threads=8, stats=False):
        o, d = f32(o).reshape(-1, 3), f32(d).reshape(-1, 3)
        n = o.shape[0]
        tmin, tmax = f32(np.broadcast_to(tmin, (n,))), f32(np.broadcast_to(tmax, (n,)))
        hit = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        st = np.zeros((n, 3), np.uint32) if stats else None
        lib().orc_trace_closest(C.c_void_p(self.h), _p(o), _p(d), _p(tmin), _p(tmax),
                                C.c_int64(n), C.c_int32(skip), int(brute), threads, _p(hit),
                                _p(t), _p(st))
        return (hit, t, st) if stats else (hit, t)

    def trace_any(self, o, d, tmin, tmax, skip=-1, brute=False, threads=8):
        o, d = f32(o).reshape(-1, 3), f32(d).reshape(-1, 3)
        n = o.shape[0]
        tmin, tmax = f32(np.broadcast_to(tmin, (n,))), f32(np.broadcast_to(tmax, (n,)))
        out = np.empty(n, np.uint8)
        lib().orc_trace_any(C.c_void_p(self.h), _p(o), _p(d), _p(tmin), _p(tmax), C.c_int64(n),
                            C.c_int32(skip), int(brute), threads, _p(out), None)
        return out.astype(bool)

    def test_lines(self, starts, stops, skip=-1, brute=False, threads=8):
        a, b = f32(starts).reshape(-1, 3), f32(stops).reshape(-1, 3)
        out = np.empty(a.shape[0], np.float32)
        lib().orc_test_lines(C.c_void_p(self.h), _p(a), _p(b), C.c_int64(a.shape[0]),
                             C.c_int32(skip), int(brute), threads, _p(out))
        return out

    def trace_coverage(self, cover, o, d, tmin, tmax, skip=-1, threads=8):
        """Transparent-shadow trace (brute force): recorded hit, t, coverage
        per ray; triangles flagged transparent add cover[i]."""
        o, d = f32(o).reshape(-1, 3), f32(d).reshape(-1, 3)
        n = o.shape[0]
        tmin, tmax = f32(np.broadcast_to(tmin, (n,))), f32(np.broadcast_to(tmax, (n,)))
        hit, t, cov = np.empty(n, np.int32), np.empty(n, np.float32), np.empty(n, np.float32)
        lib().orc_trace_coverage(C.c_void_p(self.h), _p(f32(cover)), _p(o), _p(d), _p(tmin),
                                 _p(tmax), C.c_int64(n), C.c_int32(skip), threads, _p(hit), _p(t),
                                 _p(cov))
        return hit, t, cov

    def test_lines_coverage(self, cover, starts, stops, skip=-1, threads=8):
        """TestLineDoesHitSky with texture shadows: fraction visible per line."""
        a, b = f32(starts).reshape(-1, 3), f32(stops).reshape(-1, 3)
        out = np.empty(a.shape[0], np.float32)
        lib().orc_test_lines_coverage(C.c_void_p(self.h), _p(f32(cover)), _p(a), _p(b),
                                      C.c_int64(a.shape[0]), C.c_int32(skip), threads, _p(out))
        return out

    def occlusion_mask(self, starts, stops, skip=-1, threads=8, closest=False, stats=False):
        a, b = f32(starts).reshape(-1, 3), f32(stops).reshape(-1, 3)
        n = a.shape[0]
        mask = np.zeros((n + 31) // 32, np.uint32)
        hit = np.empty(n, np.int32) if closest else None
        t = np.empty(n, np.float32) if closest else None
        st = np.zeros((n, 3), np.uint32) if stats else None
        lib().orc_occlusion_mask(C.c_void_p(self.h), _p(a), _p(b), C.c_int64(n), C.c_int32(skip),
                                 threads, _p(mask), _p(hit), _p(t), _p(st))
        res = [mask]
        if closest:
            res += [hit, t]
        if stats:
            res.append(st)
        return res[0] if len(res) == 1 else tuple(res)


def make_lights(lights) -> "C.Array":
    """Run the reference's light setup (ParseLightSpot / SetLightFalloffParams)
    on scene light descriptions and return the oracle light table."""
    L = lib()
    arr = (OLight * max(len(lights), 1))()
    for i, li in enumerate(lights):
        o = arr[i]
        o.type = li.type
        o.origin[:] = li.origin
        o.intensity[:] = li.intensity
        o.normal[:] = li.normal
        k = OKeys()
        for name, val in li.keys.items():
            setattr(k, name, val)
        if li.type == 2:
            L.orc_parse_light_spot(C.byref(k), C.byref(o))
        elif li.type == 1:
            L.orc_set_light_falloff(C.byref(k), C.byref(o))
        else:
            o.start_fade, o.end_fade, o.cap_distance = 0.0, -1.0, 1.0e22
    return arr


def light_table(arr, n) -> np.ndarray:
    """(n, 20) float32/int view of an oracle light table, for comparisons."""
    return np.frombuffer(bytes(arr), dtype=np.uint32).reshape(-1, 20)[:n].copy()


def gather_points(scene: Scene, lights_arr, nlights, pts, nrm, threads=8):
    pts, nrm = f32(pts).reshape(-1, 3), f32(nrm).reshape(-1, 3)
    out = np.empty_like(pts)
    rays = C.c_uint64(0)
    lib().orc_gather_points(C.c_void_p(scene.h), lights_arr, nlights, _p(pts), _p(nrm),
                            C.c_int64(pts.shape[0]), threads, _p(out), C.byref(rays))
    return out, rays.value


def gather_luxels(scene: Scene, lights_arr, nlights, lit, face_begin, face_end, ss=4, seed=0,
                  threads=8, stats=False):
    """RGB of the luxels of faces [face_begin, face_end) and the shadow-line
    count; with stats=True also (lines, kd nodes, triangle tests, leaves)."""
    off = lit.luxel_offset()
    n = int(off[face_end] - off[face_begin])
    out = np.empty((n, 3), np.float32)
    rays = C.c_uint64(0)
    st = np.zeros(4, np.uint64)
    lib().orc_gather_luxels(C.c_void_p(scene.h), lights_arr, nlights, _p(f32(lit.corner)),
                            _p(f32(lit.u)), _p(f32(lit.v)), _p(f32(lit.normal)),
                            _p(np.ascontiguousarray(lit.nu)), _p(np.ascontiguousarray(lit.nv)),
                            _p(off), face_begin, face_end, ss, C.c_uint64(seed), threads, _p(out),
                            C.byref(rays), _p(st))
    return (out, rays.value, st) if stats else (out, rays.value)


def luxel_samples(lit, face, ss=4, seed=0):
    off = lit.luxel_offset()
    n = int(lit.nu[face]) * int(lit.nv[face]) * ss
    out = np.empty((n, 3), np.float32)
    lib().orc_luxel_samples(_p(f32(lit.corner)), _p(f32(lit.u)), _p(f32(lit.v)),
                            _p(f32(lit.normal)), _p(np.ascontiguousarray(lit.nu)),
                            _p(np.ascontiguousarray(lit.nv)), _p(off), face, ss,
                            C.c_uint64(seed), _p(out))
    return out


def make_patches(lit, max_chop=4.0, min_chop=4.0):
    L = lib()
    args = [_p(f32(lit.corner)), _p(f32(lit.u)), _p(f32(lit.v)), _p(f32(lit.normal)),
            _p(f32(lit.luxscale)), C.c_int32(lit.n_faces), C.c_float(max_chop),
            C.c_float(min_chop)]
    n = L.orc_make_patches(*args, *([None] * 11))
    P = dict(mins=np.zeros((n, 3), np.float32), maxs=np.zeros((n, 3), np.float32),
             center=np.zeros((n, 3), np.float32), area=np.zeros(n, np.float32),
             face=np.zeros(n, np.int32), parent=np.zeros(n, np.int32),
             child1=np.zeros(n, np.int32), child2=np.zeros(n, np.int32),
             split_axis=np.zeros(n, np.int32), split_dist=np.zeros(n, np.float32),
             leaf_index=np.zeros(n, np.int32))
    L.orc_make_patches(*args, *[_p(P[k]) for k in ("mins", "maxs", "center", "area", "face",
                                                     "parent", "child1", "child2", "split_axis",
                                                     "split_dist", "leaf_index")])
    root = np.full(lit.n_faces, -1, np.int32)
    for i in range(n - 1, -1, -1):
        if P["parent"][i] < 0:
            root[P["face"][i]] = i
    P["face_root"] = root
    return P


def make_transfers(scene: Scene, lit, P, dirs, threads=8):
    L = lib()
    nleaf = int((P["leaf_index"] >= 0).sum())
    row_ptr = np.zeros(nleaf + 1, np.int64)
    k = dirs.shape[0]
    cap = nleaf * k
    col = np.zeros(max(cap, 1), np.int32)
    cnt = np.zeros(max(cap, 1), np.int32)
    nnz = L.orc_make_transfers(C.c_void_p(scene.h), _p(np.ascontiguousarray(lit.tri_face)),
                               C.c_int64(len(P["face"])), _p(P["mins"]), _p(P["maxs"]),
                               _p(P["center"]), _p(P["face"]), _p(P["child1"]), _p(P["child2"]),
                               _p(P["split_axis"]), _p(P["split_dist"]), _p(P["leaf_index"]),
                               _p(P["face_root"]), _p(f32(lit.normal)), _p(f32(lit.u)),
                               _p(f32(dirs)), C.c_int32(k), threads, _p(row_ptr), _p(col),
                               _p(cnt), C.c_int64(cap))
    return row_ptr, col[:nnz].copy(), cnt[:nnz].copy()


def make_transfer_rows(scene: Scene, lit, P, dirs, rows, threads=8):
    """Transfer rows of the dense leaf indices `rows` only (in that order):
    (row_ptr[len(rows)+1], col, hit count), each row as make_transfers
    builds it."""
    L = lib()
    L.orc_make_transfer_rows.restype = C.c_int64
    rows = np.ascontiguousarray(rows, np.int64)
    k = dirs.shape[0]
    cap = max(len(rows) * k, 1)
    row_ptr = np.zeros(len(rows) + 1, np.int64)
    col = np.zeros(cap, np.int32)
    cnt = np.zeros(cap, np.int32)
    nnz = L.orc_make_transfer_rows(C.c_void_p(scene.h), _p(np.ascontiguousarray(lit.tri_face)),
                                   C.c_int64(len(P["face"])), _p(P["center"]), _p(P["face"]),
                                   _p(P["child1"]), _p(P["child2"]), _p(P["split_axis"]),
                                   _p(P["split_dist"]), _p(P["leaf_index"]), _p(P["face_root"]),
                                   _p(f32(lit.normal)), _p(f32(lit.u)), _p(f32(dirs)),
                                   C.c_int32(k), threads, _p(rows), C.c_int64(len(rows)),
                                   _p(row_ptr), _p(col), _p(cnt), C.c_int64(cap))
    if nnz < 0:
        raise ValueError("make_transfer_rows: row index out of range")
    return row_ptr, col[:nnz].copy(), cnt[:nnz].copy()


def bounce_f64(row_ptr, col, w, refl, direct, base, max_bounces, tol, threads=1):
    """Float64 Jacobi bounce; the result does not depend on `threads`."""
    n = row_ptr.shape[0] - 1
    total = np.zeros((n, 3), np.float64)
    deltas = np.zeros(max(max_bounces, 1), np.float64)
    L = lib()
    L.orc_bounce_f64_mt.restype = C.c_int
    it = L.orc_bounce_f64_mt(C.c_int64(n), _p(np.ascontiguousarray(row_ptr, np.int64)),
                             _p(np.ascontiguousarray(col, np.int32)), _p(f32(w)),
                             _p(f32(refl)), _p(f32(direct)), _p(f32(base)), max_bounces,
                             C.c_double(tol), _p(total), _p(deltas), int(threads))
    return total, it, deltas[:it]


def encode_sample(r, g, b) -> int:
    """Shared-exponent lightmap sample word of one light."""
    return int(lib().orc_encode_sample(float(r), float(g), float(b)))


def lightmap(lit, P, direct, total):
    """Sample words (uint32 per luxel) of direct luxel light + bounced light of
    the leaf patch at each luxel centre; P as make_patches returns it."""
    off = lit.luxel_offset()
    out = np.zeros(max(int(off[-1]), 1), np.uint32)
    lib().orc_lightmap(_p(f32(lit.corner)), _p(f32(lit.u)), _p(f32(lit.v)), _p(f32(lit.normal)),
                       _p(np.ascontiguousarray(lit.nu, np.int32)),
                       _p(np.ascontiguousarray(lit.nv, np.int32)), _p(off),
                       C.c_int32(lit.n_faces), _p(P["child1"]), _p(P["child2"]),
                       _p(P["split_axis"]), _p(P["split_dist"]), _p(P["leaf_index"]),
                       _p(P["face_root"]), _p(f32(direct)), _p(f32(total)), _p(out))
    return out[: int(off[-1])]


def calc_face_extents(vertices, lightmap_vecs):
    """(mins, size, too_big) of CalcFaceExtents, or None for no vertices or
    values beyond int32."""
    v = f32(vertices).reshape(-1, 3)
    vecs = f32(lightmap_vecs).reshape(2, 4)
    mins, size, big = np.zeros(2, np.int32), np.zeros(2, np.int32), np.zeros(1, np.int32)
    rc = lib().orc_calc_face_extents(_p(v), v.shape[0], _p(vecs), _p(mins), _p(size), _p(big))
    if rc != 0:
        return None
    return (int(mins[0]), int(mins[1])), (int(size[0]), int(size[1])), bool(big[0])


def base_winding(normal, dist):
    out = np.zeros((4, 3), np.float32)
    lib().orc_base_winding(_p(f32(normal)), C.c_float(dist), _p(out))
    return out


def chop_winding(points, normal, dist, eps=0.0):
    """The part of the winding in front of the plane, or None past 64 points."""
    pts = f32(points).reshape(-1, 3)
    w = np.zeros((68, 3), np.float32)
    w[: len(pts)] = pts
    n = lib().orc_chop_winding(_p(w), C.c_int(len(pts)), _p(f32(normal)), C.c_float(dist),
                               C.c_float(eps))
    return None if n < 0 else w[:n].copy()


def bsp_world_triangles(lumps, headnode=0, first_face=0, num_model_faces=None):
    """(xyz (n, 9), ids, brush triangle count) of the world's brushes and sky faces."""
    def arr(name, dt, per):
        return np.ascontiguousarray(lumps.get(name, np.zeros((0, per))), dtype=dt).reshape(-1, per)

    planes = arr("planes", np.float32, 4)
    children = arr("node_children", np.int32, 2)
    ranges = arr("leaf_brush_ranges", np.int32, 2)
    lb = arr("leaf_brushes", np.int32, 1)
    brushes = arr("brushes", np.int32, 3)
    sides = arr("brush_sides", np.int32, 4)
    tflags = arr("texinfo_flags", np.int32, 1)
    verts = arr("vertexes", np.float32, 3)
    edges = arr("edges", np.int32, 2)
    se = arr("surf_edges", np.int32, 1)
    faces = arr("faces", np.int32, 3)
    nmf = len(faces) - first_face if num_model_faces is None else num_model_faces
    cap = 64 * len(sides) + 64 * len(faces) + 1
    xyz = np.zeros((cap, 9), np.float32)
    ids = np.zeros(cap, np.int32)
    nb = C.c_int64()
    L = lib()
    L.orc_bsp_world_triangles.restype = C.c_int64
    n = L.orc_bsp_world_triangles(_p(planes), _p(children), C.c_int32(len(children)), _p(ranges),
                                  C.c_int32(len(ranges)), _p(lb), _p(brushes),
                                  C.c_int32(len(brushes)), _p(sides), _p(tflags), _p(verts),
                                  _p(edges), _p(se), _p(faces), C.c_int32(headnode),
                                  C.c_int32(first_face), C.c_int32(nmf), _p(xyz), _p(ids),
                                  C.c_int64(cap), C.byref(nb))
    if n < 0:
        return None
    return xyz[:n].copy(), ids[:n].copy(), nb.value
