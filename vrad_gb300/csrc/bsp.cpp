// bsp.cpp -- the world's brushes and sky faces as triangles of the ray-trace
// environment: addBrushesForRayTrace / addBrushToRaytraceEnvironment
// (cmd/tasks/loadbsp/main.go:241-340) over lump arrays the caller has parsed
// (the reference reads them through galaco/bsp, which is not part of it), with
// BaseWindingForPlane and ChopWindingInPlace (vmath/polygon/winding.go:25-170).
//
// Behaviour kept from the reference, with these defects fixed:
//   - brush sides: the reference skips every side WITHOUT SURF_SKY (the test
//     at main.go:255 is inverted, so only sky sides become triangles); here
//     sky sides and displacement sides are skipped and the rest are added;
//   - BaseWindingForPlane reads normal[1] for every axis when it picks the
//     major axis (winding.go:36), its Go switch has no fallthrough so axis 0
//     gets a zero up vector (winding.go:46-52), and it writes Points[0] where
//     Points[3] is meant (winding.go:77-78);
//   - ChopWindingInPlace never sets the wrap-around entry sides[n] = sides[0]
//     (its loop variable shadows the outer i, winding.go:112) and its
//     split-point loop advances i instead of j (winding.go:149);
//   - the vertex index of a sky face is checked against the vertex count, not
//     the edge count (main.go:328-329).
// Arithmetic is float32, one rounding per operation in the order written
// (mgl32's Dot, Cross, Normalize as published: sums left to right,
// 1 / sqrt of the squared length).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <system_error>
#include <thread>
#include <vector>

#include "vrg_internal.h"

namespace {

constexpr float kWindingExtent = 16384.0f * 4.0f;  // MAX_COORD_INTEGER * 4 (common/constants/constants.go:6)
constexpr int kMaxWindingPoints = 64;              // MAX_POINTS_ON_WINDING (constants.go:32)
enum { kFront = 0, kBack = 1, kOn = 2 };            // vmath/polygon/vplane.go:3-5

struct V3 {
    float x, y, z;
};

float dot(const V3 &a, const V3 &b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// A quad of side 2 * 65536 centred on the plane's point nearest the origin.
void base_winding(const float *n, float dist, V3 *out) {
    int x = -1;
    float mx = -1.0f;
    for (int i = 0; i < 3; i++) {
        const float v = std::fabs(n[i]);
        if (v > mx) {
            x = i;
            mx = v;
        }
    }
    V3 up{0.0f, 0.0f, 0.0f};
    if (x == 2) up.x = 1.0f;
    else up.z = 1.0f;
    const V3 N{n[0], n[1], n[2]};
    const float v = dot(up, N);
    up = V3{up.x + -v * N.x, up.y + -v * N.y, up.z + -v * N.z};
    const float il = 1.0f / std::sqrt(dot(up, up));
    up = V3{up.x * il, up.y * il, up.z * il};
    const V3 org{N.x * dist, N.y * dist, N.z * dist};
    V3 right{up.y * N.z - up.z * N.y, up.z * N.x - up.x * N.z, up.x * N.y - up.y * N.x};
    up = V3{up.x * kWindingExtent, up.y * kWindingExtent, up.z * kWindingExtent};
    right = V3{right.x * kWindingExtent, right.y * kWindingExtent, right.z * kWindingExtent};
    out[0] = V3{(org.x - right.x) + up.x, (org.y - right.y) + up.y, (org.z - right.z) + up.z};
    out[1] = V3{(org.x + right.x) + up.x, (org.y + right.y) + up.y, (org.z + right.z) + up.z};
    out[2] = V3{(org.x + right.x) - up.x, (org.y + right.y) - up.y, (org.z + right.z) - up.z};
    out[3] = V3{(org.x - right.x) - up.x, (org.y - right.y) - up.y, (org.z - right.z) - up.z};
}

// A winding with room for the limit plus the points one chop can add.
struct Winding {
    V3 p[kMaxWindingPoints + 4];
    int n = 0;
};

// Keeps the part of w in front of the plane (n . p - dist > -epsilon).
// Returns 0 with w emptied when nothing is in front, -1 when the result would
// pass the winding limit.
int chop_winding(Winding &w, const float *n, float dist, float epsilon) {
    const int np = w.n;
    if (np == 0) return 0;
    const V3 N{n[0], n[1], n[2]};
    float dists[kMaxWindingPoints + 5];
    int sides[kMaxWindingPoints + 5];
    int counts[3] = {0, 0, 0};
    for (int i = 0; i < np; i++) {
        const float d = dot(w.p[i], N) - dist;
        dists[i] = d;
        sides[i] = d > epsilon ? kFront : (d < -epsilon ? kBack : kOn);
        counts[sides[i]]++;
    }
    sides[np] = sides[0];
    dists[np] = dists[0];
    if (counts[kFront] == 0) {
        w.n = 0;
        return 0;
    }
    if (counts[kBack] == 0) return 0;
    Winding f;
    for (int i = 0; i < np; i++) {
        const V3 &p1 = w.p[i];
        if (f.n > kMaxWindingPoints + 2) return -1;  // room for the two pushes below
        if (sides[i] == kOn) {
            f.p[f.n++] = p1;
            continue;
        }
        if (sides[i] == kFront) f.p[f.n++] = p1;
        if (sides[i + 1] == kOn || sides[i + 1] == sides[i]) continue;
        const V3 &p2 = w.p[(i + 1) % np];
        const float t = dists[i] / (dists[i] - dists[i + 1]);
        const float a[3] = {p1.x, p1.y, p1.z}, b[3] = {p2.x, p2.y, p2.z};
        float m[3];
        for (int j = 0; j < 3; j++) {
            if (n[j] == 1.0f) m[j] = dist;
            else if (n[j] == -1.0f) m[j] = -dist;
            else m[j] = a[j] + t * (b[j] - a[j]);
        }
        f.p[f.n++] = V3{m[0], m[1], m[2]};
    }
    if (f.n > kMaxWindingPoints) return -1;
    w = f;
    return 0;
}

bool finite_plane(const float *p) {
    return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]) && std::isfinite(p[3]);
}

// Every index the walk below can follow, checked before anything is added.
int check_world(const vrg_bsp_world &w) {
    auto in = [](int64_t i, int64_t n) { return i >= 0 && i < n; };
    if (w.num_planes < 0 || w.num_nodes < 0 || w.num_leafs < 0 || w.num_leaf_brushes < 0 ||
        w.num_brushes < 0 || w.num_brush_sides < 0 || w.num_texinfo < 0 || w.num_vertexes < 0 ||
        w.num_edges < 0 || w.num_surf_edges < 0 || w.num_faces < 0)
        return VRG_ERR_INVALID;
    if ((w.num_planes && !w.planes) || (w.num_nodes && !w.node_children) ||
        (w.num_leafs && !w.leaf_brush_ranges) || (w.num_leaf_brushes && !w.leaf_brushes) ||
        (w.num_brushes && !w.brushes) || (w.num_brush_sides && !w.brush_sides) ||
        (w.num_texinfo && !w.texinfo_flags) || (w.num_vertexes && !w.vertexes) ||
        (w.num_edges && !w.edges) || (w.num_surf_edges && !w.surf_edges) || (w.num_faces && !w.faces))
        return VRG_ERR_INVALID;
    for (int32_t i = 0; i < w.num_planes; i++)
        if (!finite_plane(w.planes + 4 * i)) return VRG_ERR_INVALID;
    for (int64_t i = 0; i < 2 * (int64_t)w.num_nodes; i++) {
        const int32_t c = w.node_children[i];
        if (c >= 0 ? !in(c, w.num_nodes) : !in(-1 - (int64_t)c, w.num_leafs)) return VRG_ERR_INVALID;
    }
    for (int32_t i = 0; i < w.num_leafs; i++) {
        const int64_t first = w.leaf_brush_ranges[2 * i], n = w.leaf_brush_ranges[2 * i + 1];
        if (first < 0 || n < 0 || first + n > w.num_leaf_brushes) return VRG_ERR_INVALID;
    }
    for (int32_t i = 0; i < w.num_leaf_brushes; i++)
        if (!in(w.leaf_brushes[i], w.num_brushes)) return VRG_ERR_INVALID;
    for (int32_t i = 0; i < w.num_brushes; i++) {
        const int64_t first = w.brushes[3 * i], n = w.brushes[3 * i + 1];
        if (first < 0 || n < 0 || first + n > w.num_brush_sides) return VRG_ERR_INVALID;
    }
    for (int32_t i = 0; i < w.num_brush_sides; i++) {
        const int32_t *s = w.brush_sides + 4 * i;
        // planes come in pairs (p, p ^ 1 facing the other way)
        if (!in(s[0], w.num_planes) || !in(s[0] ^ 1, w.num_planes)) return VRG_ERR_INVALID;
        if (s[1] >= w.num_texinfo) return VRG_ERR_INVALID;  // negative: no texinfo
    }
    if (w.num_nodes > 0 || w.num_leafs > 0) {
        if (w.headnode >= 0 ? !in(w.headnode, w.num_nodes) : !in(-1 - (int64_t)w.headnode, w.num_leafs))
            return VRG_ERR_INVALID;
    }
    if (w.first_face < 0 || w.num_model_faces < 0 || (int64_t)w.first_face + w.num_model_faces > w.num_faces)
        return VRG_ERR_INVALID;
    // the world's faces, and for its sky faces every surfedge, edge and vertex
    // read (edge 0 and other records no face uses are not looked at)
    for (int32_t k = 0; k < w.num_model_faces; k++) {
        const int32_t *f = w.faces + 3 * (int64_t)(w.first_face + k);
        if (f[0] < 0 || f[1] < 0 || (int64_t)f[0] + f[1] > w.num_surf_edges || f[2] >= w.num_texinfo)
            return VRG_ERR_INVALID;
        if (f[1] > kMaxWindingPoints) return VRG_ERR_INVALID;  // main.go:311-313
        if (((f[2] >= 0 ? w.texinfo_flags[f[2]] : 0) & VRG_SURF_SKY) == 0) continue;
        for (int32_t j = 0; j < f[1]; j++) {
            const int64_t e = w.surf_edges[f[0] + j];
            if (!in(e < 0 ? -e : e, w.num_edges)) return VRG_ERR_INVALID;
            const int32_t v = e < 0 ? w.edges[2 * -e + 1] : w.edges[2 * e];
            if (!in(v, w.num_vertexes)) return VRG_ERR_INVALID;
            for (int a = 0; a < 3; a++)
                if (!std::isfinite(w.vertexes[3 * (int64_t)v + a])) return VRG_ERR_INVALID;
        }
    }
    return VRG_OK;
}

// GetBrushRecursive (cmd/tasks/loadbsp/brush/brush.go:7-36): children[0]
// then children[1], each leaf's brushes in order, a brush listed once at its
// first appearance.  Iterative, with a seen-bitmap in place of the list scan.
// Returns VRG_ERR_INVALID when the nodes do not form a tree (an internal
// node reached twice), which would otherwise never end on a cycle.
int brush_list(const vrg_bsp_world &w, std::vector<int32_t> &out) {
    if (w.num_nodes == 0 && w.num_leafs == 0) return VRG_OK;
    std::vector<uint8_t> seen(w.num_brushes, 0);
    std::vector<int32_t> stack{w.headnode};
    int64_t internal = 0;
    while (!stack.empty()) {
        const int32_t node = stack.back();
        stack.pop_back();
        if (node < 0) {
            const int32_t leaf = -1 - node;
            const int32_t first = w.leaf_brush_ranges[2 * leaf], n = w.leaf_brush_ranges[2 * leaf + 1];
            for (int32_t i = 0; i < n; i++) {
                const int32_t b = w.leaf_brushes[first + i];
                if (!seen[b]) {
                    seen[b] = 1;
                    out.push_back(b);
                }
            }
        } else {
            if (++internal > w.num_nodes) return VRG_ERR_INVALID;
            stack.push_back(w.node_children[2 * node + 1]);
            stack.push_back(w.node_children[2 * node]);
        }
    }
    return VRG_OK;
}

}  // namespace

using namespace vrg;

extern "C" {

int vrg_base_winding_for_plane(const float *normal, float dist, float *out12) {
    if (!normal || !out12 || !std::isfinite(normal[0]) || !std::isfinite(normal[1]) ||
        !std::isfinite(normal[2]) || !std::isfinite(dist))
        return VRG_ERR_INVALID;
    V3 p[4];
    base_winding(normal, dist, p);
    memcpy(out12, p, sizeof(p));
    return VRG_OK;
}

int vrg_chop_winding(const float *points, int32_t n, const float *normal, float dist, float epsilon,
                     float *out, int32_t *out_n) {
    if (n < 0 || n > kMaxWindingPoints || (n && !points) || !normal || !out || !out_n) return VRG_ERR_INVALID;
    Winding w;
    w.n = n;
    if (n) memcpy(w.p, points, sizeof(V3) * (size_t)n);
    if (chop_winding(w, normal, dist, epsilon) != 0) return VRG_ERR_UNSUPPORTED;
    if (w.n) memcpy(out, w.p, sizeof(V3) * (size_t)w.n);
    *out_n = w.n;
    return VRG_OK;
}

int vrg_env_add_bsp_world(vrg_env *env, const vrg_bsp_world *world, int64_t *brush_triangles,
                          int64_t *sky_triangles) {
    if (!env || !world) return VRG_ERR_INVALID;
    const vrg_bsp_world &w = *world;
    if (check_world(w) != VRG_OK) return fail(env->ctx, VRG_ERR_INVALID, "BSP lumps hold an index out of range or a non-finite value");
    // build every triangle first, so a failure adds none
    std::vector<float> xyz;
    std::vector<int32_t> ids;
    auto put = [&](const V3 &a, const V3 &b, const V3 &c, int32_t id) {
        const float t[9] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z};
        xyz.insert(xyz.end(), t, t + 9);
        ids.push_back(id);
    };
    std::vector<int32_t> brushes;
    if (brush_list(w, brushes) != VRG_OK) return fail(env->ctx, VRG_ERR_INVALID, "BSP nodes do not form a tree");
    // Brushes are independent: contiguous runs of the list go to threads,
    // each filling its own triangle list, joined in list order afterwards.
    const int64_t nb = (int64_t)brushes.size();
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nth = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)hw, 16, nb / 256}));
    std::vector<std::vector<float>> part_xyz(nth);
    std::vector<int64_t> part_tris(nth, 0);
    std::vector<int> part_rc(nth, 0);
    auto run = [&](int t) {
        const int64_t b0 = nb * t / nth, b1 = nb * (t + 1) / nth;
        std::vector<float> &out = part_xyz[t];
        Winding poly;
        for (int64_t k = b0; k < b1; k++) {
            const int32_t *b = w.brushes + 3 * brushes[k];
            if ((b[2] & VRG_MASK_OPAQUE) == 0) continue;
            for (int32_t i = 0; i < b[1]; i++) {
                const int32_t *side = w.brush_sides + 4 * (b[0] + i);
                const int32_t tflags = side[1] >= 0 ? w.texinfo_flags[side[1]] : 0;
                if ((tflags & VRG_SURF_SKY) != 0 || side[2] != 0) continue;
                const float *pl = w.planes + 4 * side[0];
                poly.n = 4;
                base_winding(pl, pl[3], poly.p);
                for (int32_t j = 0; j < b[1] && poly.n > 0; j++) {
                    if (j == i) continue;
                    const int32_t *other = w.brush_sides + 4 * (b[0] + j);
                    if (other[3] != 0) continue;  // bevel
                    const float *op = w.planes + 4 * (other[0] ^ 1);
                    if (chop_winding(poly, op, op[3], 0.0f) != 0) {
                        part_rc[t] = 1;
                        return;
                    }
                }
                for (int j = 2; j < poly.n; j++) {
                    const V3 *v[3] = {&poly.p[0], &poly.p[j - 1], &poly.p[j]};
                    for (const V3 *q : v) {
                        out.push_back(q->x);
                        out.push_back(q->y);
                        out.push_back(q->z);
                    }
                    part_tris[t]++;
                }
            }
        }
    };
    try {
        std::vector<std::thread> pool;
        for (int t = 1; t < nth; t++) pool.emplace_back(run, t);
        run(0);
        for (auto &th : pool) th.join();
    } catch (const std::bad_alloc &) {
        return fail(env->ctx, VRG_ERR_NOMEM, "out of host memory in the brush ingest");
    } catch (const std::system_error &) {
        return fail(env->ctx, VRG_ERR_NOMEM, "could not start the brush ingest threads");
    }
    for (int t = 0; t < nth; t++) {
        if (part_rc[t]) return fail(env->ctx, VRG_ERR_UNSUPPORTED, "brush side winding passed 64 points");
        xyz.insert(xyz.end(), part_xyz[t].begin(), part_xyz[t].end());
        ids.insert(ids.end(), (size_t)part_tris[t], VRG_TRACE_ID_OPAQUE);
    }
    const int64_t nbrush = (int64_t)ids.size();
    for (int32_t k = 0; k < w.num_model_faces; k++) {
        const int32_t *f = w.faces + 3 * (w.first_face + k);
        const int32_t tflags = f[2] >= 0 ? w.texinfo_flags[f[2]] : 0;
        if ((tflags & VRG_SURF_SKY) == 0) continue;
        std::vector<V3> pts(f[1]);
        for (int32_t j = 0; j < f[1]; j++) {
            const int32_t e = w.surf_edges[f[0] + j];
            const int32_t v = e < 0 ? w.edges[2 * -(int64_t)e + 1] : w.edges[2 * (int64_t)e];
            pts[j] = V3{w.vertexes[3 * v], w.vertexes[3 * v + 1], w.vertexes[3 * v + 2]};
        }
        for (int32_t j = 2; j < f[1]; j++) put(pts[0], pts[j - 1], pts[j], VRG_TRACE_ID_SKY);
    }
    // AddTriangle (environment.go:41-43) for each, in one append: flags 0,
    // material 0, colour fullCoverage = (1, 0, 0) (main.go:275,337)
    {
        std::lock_guard<std::mutex> lk(env->mu);
        if (env->built) return fail(env->ctx, VRG_ERR_STATE, "triangles added after SetupAccelerationStructure");
        const size_t n = ids.size();
        env->cover.resize(env->ids.size(), 0.0f);
        env->cover.insert(env->cover.end(), n, 1.0f);  // fullCoverage's x
        env->xyz.insert(env->xyz.end(), xyz.begin(), xyz.end());
        env->ids.insert(env->ids.end(), ids.begin(), ids.end());
        env->flags.insert(env->flags.end(), n, 0);
        env->materials.insert(env->materials.end(), n, 0);
        env->colours.reserve(env->colours.size() + 3 * n);
        for (size_t t = 0; t < n; t++) {
            env->colours.push_back(1.0f);
            env->colours.push_back(0.0f);
            env->colours.push_back(0.0f);
        }
    }
    if (brush_triangles) *brush_triangles = nbrush;
    if (sky_triangles) *sky_triangles = (int64_t)ids.size() - nbrush;
    return VRG_OK;
}

}  // extern "C"
