"""Regenerate the golden fixtures in this folder.

    python tests/golden/make_golden.py

``trace_geometry.npz`` -- shadow lines and rays against a box scene, answered
by float64 geometry written here from the definitions alone (segment/plane
crossing, signed distances to the three edges), independent of the oracle's
float32 intersection format and of its kd tree.  Semantics followed
(raytracer/trace/testline.go:22-57,91-93; raytracer/environment.go:140-145):
a line from a to b is traced over [0, |b-a|) along the unit direction,
triangles whose id equals the skip id are ignored, the closest hit wins, and
the line is occluded iff that hit exists and its id lacks TRACE_ID_SKY.
Float32 arithmetic may decide a case differently only when the line passes
within a few float32 rounding errors of an edge, an endpoint lies on a plane,
the line grazes a plane, or two hits lie at nearly the same distance; such
lines get the answer "undecided" (-2 / -1) and the tests skip them.  The
margin is 0.02 world units (about 40 float32 ulps at the 4,096-unit room
scale), widened by 1/cos of the angle to the plane.

``pipeline_small.npz`` -- the oracle's outputs for a small lit scene (60
faces of boxes 512-1,536 units wide, 128-unit luxels, 12 point lights, 4
spots, the sky): luxel RGB, the patch tree digest, the transfer CSR digest
(K = 256), leaf-patch direct light and the float64 bounce.  It pins the
restatement against drift; the product is compared to it within the
tolerances of its tests.
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from vrad_gb300 import scenes  # noqa: E402

EPS = 0.02
UNDECIDED_HIT = -2
UNDECIDED_OCC = -1

PIPE = dict(seed=21, n_faces=60, spacing=128.0, edge=(512.0, 1536.0), n_point=12, n_spot=4, ss=4,
            gather_seed=7, k=256)


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype.str).encode() + str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def geometry_scene(seed: int = 17, n_boxes: int = 96, n_lines: int = 2048):
    """Room (ceiling sky) + boxes with their own ids: every fourth one sky,
    every fourth (offset 1) a static prop (TRACE_ID_STATICPROP | index), the
    rest opaque; half of the lines end inside a box so that most of them hit
    something."""
    soup = scenes.TriangleSoup()
    soup.add_box(scenes.TRACE_ID_OPAQUE, (0.0, 0.0, 0.0), (scenes.ROOM,) * 3,
                 ceiling_id=scenes.TRACE_ID_SKY)
    mins, maxs = scenes._random_boxes(scenes.Stream(seed, scenes.S_BOXES), n_boxes, 64.0, 512.0)
    box_id = []
    for b in range(n_boxes):
        flag = (scenes.TRACE_ID_SKY, scenes.TRACE_ID_STATICPROP)[b % 4] if b % 4 < 2 \
            else scenes.TRACE_ID_OPAQUE
        box_id.append(flag | (b << 1))
        soup.add_box(box_id[-1], mins[b], maxs[b])
    xyz, ids = soup.arrays()
    rr = scenes.Stream(seed, scenes.S_RAYS)
    starts = rr.uniform(3 * n_lines, 1.0, scenes.ROOM - 1.0).reshape(n_lines, 3)
    stops = rr.uniform(3 * n_lines, 1.0, scenes.ROOM - 1.0).reshape(n_lines, 3)
    pick = (rr.uniform(n_lines) * np.float32(n_boxes)).astype(np.int64) % n_boxes
    frac = rr.uniform(3 * n_lines).reshape(n_lines, 3)
    inside = (mins[pick] + (maxs[pick] - mins[pick]) * frac).astype(np.float32)
    stops[1::2] = inside[1::2]
    return xyz, ids, np.ascontiguousarray(starts), np.ascontiguousarray(stops)


def _tri_frames(xyz):
    v = xyz.astype(np.float64).reshape(-1, 3, 3)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    edges = []
    for i in range(3):
        p, q = v[:, (i + 1) % 3], v[:, (i + 2) % 3]  # edge opposite vertex i
        e = q - p
        edges.append((p, e / np.linalg.norm(e, axis=1, keepdims=True)))
    return v, n, edges


def exact_line(frames, ids, a, b, skip):
    """(hit index or -1 / UNDECIDED_HIT, t in float64) for one segment."""
    v, n, edges = frames
    a = a.astype(np.float64)
    d = b.astype(np.float64) - a
    L = float(np.linalg.norm(d))
    dn = d / L
    use = ids != skip
    sa = np.einsum("ij,ij->i", a - v[:, 0], n)
    sb = sa + L * (n @ dn)
    cosang = np.abs(n @ dn)
    eps = EPS * (1.0 + 1.0 / np.maximum(cosang, 1e-12))
    cross = (sa * sb <= 0) | (np.minimum(np.abs(sa), np.abs(sb)) < eps)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(np.abs(sa - sb) > 0, L * sa / (sa - sb), np.nan)
    h = a + t[:, None] * dn
    dist = np.stack([np.einsum("ij,ij->i", np.cross(e, h - p), n) for p, e in edges], axis=1)
    inside_clear = (dist > eps[:, None]).all(axis=1)
    outside_clear = (dist < -eps[:, None]).any(axis=1)
    t_clear = (t > eps) & (t < L - eps)
    t_out = (t < -eps) | (t > L + eps)
    nan = ~np.isfinite(t)
    clear_hit = use & cross & ~nan & inside_clear & t_clear
    clear_miss = ~use | ~cross | outside_clear | t_out
    amb = use & ~clear_hit & ~clear_miss
    hits = np.nonzero(clear_hit)[0]
    best, best_t = -1, np.inf
    if hits.size:
        order = hits[np.argsort(t[hits], kind="stable")]
        best, best_t = int(order[0]), float(t[order[0]])
        if order.size > 1 and t[order[1]] - best_t <= 2 * (eps[order[0]] + eps[order[1]]):
            return UNDECIDED_HIT, np.nan
    ai = np.nonzero(amb)[0]
    if ai.size:
        ta = np.where(np.isfinite(t[ai]), t[ai], -np.inf)
        if (ta <= best_t + 2 * (eps[ai] + (eps[best] if best >= 0 else 0.0))).any():
            return UNDECIDED_HIT, np.nan
    return best, best_t


def _answer(frames, ids, starts, stops, skip):
    hit = np.empty(len(starts), np.int32)
    t = np.empty(len(starts), np.float64)
    for i in range(len(starts)):
        hit[i], t[i] = exact_line(frames, ids, starts[i], stops[i], skip)
    occ = np.where(hit == UNDECIDED_HIT, UNDECIDED_OCC,
                   (hit >= 0) & ((ids[np.maximum(hit, 0)] & scenes.TRACE_ID_SKY) == 0))
    return hit, t, occ.astype(np.int8)


def make_trace_geometry():
    xyz, ids, starts, stops = geometry_scene()
    frames = _tri_frames(xyz)
    hit0, t0, occ0 = _answer(frames, ids, starts, stops, -1)
    # skip the static-prop id that is the closest hit of the most lines (so
    # that TestLineDoesHitSky's staticPropToSkip can name it too)
    hit_ids, counts = np.unique(ids[hit0[hit0 >= 0]], return_counts=True)
    prop = (hit_ids & scenes.TRACE_ID_STATICPROP) != 0
    hit_ids, counts = hit_ids[prop], counts[prop]
    skip = int(hit_ids[np.argmax(counts)])
    hit1, t1, occ1 = _answer(frames, ids, starts, stops, skip)
    out = dict(xyz=xyz, ids=ids, starts=starts, stops=stops,
               skip_ids=np.array([-1, skip], np.int32), hit0=hit0, t0=t0, occ0=occ0,
               hit1=hit1, t1=t1, occ1=occ1)
    np.savez_compressed(HERE / "trace_geometry.npz", **out)
    for k in (0, 1):
        h = out[f"hit{k}"]
        print(f"skip {out['skip_ids'][k]:#x}: {np.mean(h != UNDECIDED_HIT):.3f} decided, "
              f"{np.mean(h >= 0):.3f} hit, {np.mean(out[f'occ{k}'] == 1):.3f} occluded")


def pipeline_scene():
    return scenes.lit_scene(PIPE["seed"], n_faces=PIPE["n_faces"], spacing=PIPE["spacing"],
                            n_point=PIPE["n_point"], n_spot=PIPE["n_spot"], edge=PIPE["edge"])


def pipeline_inputs_digest(lit) -> str:
    return sha(lit.xyz, lit.ids, lit.tri_face, lit.corner, lit.u, lit.v, lit.normal, lit.nu,
               lit.nv, lit.luxscale, lit.refl)


def patch_digest(P) -> str:
    return sha(*[P[k] for k in ("mins", "maxs", "center", "area", "face", "parent", "child1",
                                "child2", "split_axis", "split_dist", "leaf_index")])


def oracle_pipeline(oracle, threads: int = 8):
    """Everything the pipeline fixture holds, computed by the oracle now."""
    lit = pipeline_scene()
    s = oracle.Scene(lit.xyz, lit.ids)
    lights = oracle.make_lights(lit.lights)
    rgb, rays = oracle.gather_luxels(s, lights, len(lit.lights), lit, 0, lit.n_faces,
                                     ss=PIPE["ss"], seed=PIPE["gather_seed"], threads=threads)
    P = oracle.make_patches(lit)
    dirs = scenes.transfer_directions(PIPE["k"])
    row_ptr, col, cnt = oracle.make_transfers(s, lit, P, dirs, threads=threads)
    leaf = np.nonzero(P["leaf_index"] >= 0)[0]
    face = P["face"][leaf]
    pts = (P["center"][leaf] + lit.normal[face] * np.float32(0.125)).astype(np.float32)
    direct, _ = oracle.gather_points(s, lights, len(lit.lights), pts, lit.normal[face],
                                     threads=threads)
    w = (cnt / np.float32(PIPE["k"])).astype(np.float32)
    refl = lit.refl[face]
    total, iters, deltas = oracle.bounce_f64(row_ptr, col, w, refl, direct, np.zeros_like(refl),
                                             100, 1e-3)
    return dict(inputs=pipeline_inputs_digest(lit), luxel_rgb=rgb, rays=np.uint64(rays),
                patches=patch_digest(P), n_leaves=np.int64(leaf.size),
                transfers=sha(row_ptr, col, cnt), nnz=np.int64(col.size), patch_direct=direct,
                bounce_total=total, bounce_iters=np.int64(iters), bounce_deltas=deltas)


def make_pipeline():
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import pyoracle

    pyoracle.build()
    res = oracle_pipeline(pyoracle)
    np.savez_compressed(HERE / "pipeline_small.npz", **{k: np.asarray(v) for k, v in res.items()})
    print(f"pipeline: {res['luxel_rgb'].shape[0]} luxels, {int(res['rays'])} rays, "
          f"{int(res['n_leaves'])} leaves, {int(res['nnz'])} nnz, "
          f"{int(res['bounce_iters'])} bounces")


if __name__ == "__main__":
    make_trace_geometry()
    make_pipeline()
