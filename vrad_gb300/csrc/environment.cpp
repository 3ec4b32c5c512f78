// environment.cpp -- the ray-trace environment (raytracer/environment.go):
// triangle soup, intersection format, acceleration structure and its
// upload to the device.
#include <algorithm>
#include <limits>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "vrg_internal.h"

namespace vrg {

// GetEdgeEquation (vmath/polygon/edge.go:5-24): the line through p1,p2 in the
// (c1,c2) projection, signed and scaled so it equals 1 at `inside`.
void edge_equation(const float *p1, const float *p2, int c1, int c2, const float *inside,
                   float *out3) {
    float nx = p1[c2] - p2[c2];
    float ny = p2[c1] - p1[c1];
    float d = -(nx * p1[c1] + ny * p1[c2]);
    float trial = (inside[c1] * nx + inside[c2] * ny) + d;
    if (trial < 0) {
        nx = -nx;
        ny = -ny;
        d = -d;
        trial = -trial;
    }
    out3[0] = nx / trial;
    out3[1] = ny / trial;
    out3[2] = d / trial;
}

// ChangeIntoIntersectionFormat (raytracer/cache/optimisedtriangle.go:30-78):
// N = normalize(e1 x e2) as v * (1/sqrt((x*x + y*y) + z*z)), D = N.p1, drop the
// axis of largest |N| (first on ties), edge equations of p1p2 (1 at p3) and
// p2p3 (1 at p1) in the two kept coordinates.
void tri_intersect_format(const float *xyz9, int32_t id, uint8_t flags, TriRecord *out,
                          uint32_t tri_index) {
    (void)flags;
    const float *p1 = xyz9, *p2 = xyz9 + 3, *p3 = xyz9 + 6;
    const float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const float e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                  e1[0] * e2[1] - e1[1] * e2[0]};
    const float len = std::sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
    const float inv = 1.0f / len;
    for (float &c : n) c = c * inv;
    int drop = 0;
    for (int c = 1; c < 3; c++)
        if (std::fabs(n[c]) > std::fabs(n[drop])) drop = c;
    const int cs0 = (drop + 1) % 3, cs1 = (drop + 2) % 3;
    float ea[3], eb[3];
    edge_equation(p1, p2, cs0, cs1, p3, ea);
    edge_equation(p2, p3, cs0, cs1, p1, eb);
    out->nx = n[0];
    out->ny = n[1];
    out->nz = n[2];
    out->d = (n[0] * p1[0] + n[1] * p1[1]) + n[2] * p1[2];
    out->e0 = ea[0];
    out->e1 = ea[1];
    out->e2 = ea[2];
    out->e3 = eb[0];
    out->e4 = eb[1];
    out->e5 = eb[2];
    out->id = id;
    out->idx_drop = (tri_index << 2) | (uint32_t)drop;
}

// Largest number of inner nodes on a root-to-leaf path of a tree in the
// node format (type | left index << 2, children adjacent), iteratively; a
// child index that does not point forward inside the array counts as too
// deep.
int inner_depth(const std::vector<uint32_t> &children) {
    const int64_t n = (int64_t)children.size();
    if (n == 0) return 0;
    std::vector<std::pair<int64_t, int>> todo{{0, 0}};
    int deepest = 0;
    while (!todo.empty()) {
        const std::pair<int64_t, int> top = todo.back();
        todo.pop_back();
        const int64_t node = top.first;
        if ((children[node] & 3u) == kLeaf) continue;
        const int d = top.second + 1;
        deepest = std::max(deepest, d);
        const int64_t left = (int64_t)(children[node] >> 2);
        if (left <= node || left + 1 >= n) return std::numeric_limits<int>::max();
        todo.push_back({left, d});
        todo.push_back({left + 1, d});
    }
    return deepest;
}

}  // namespace vrg

using namespace vrg;

extern "C" {

int vrg_env_setup_acceleration_structure(vrg_env *env) {
    if (!env) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    const int64_t n = (int64_t)env->ids.size();
    if (n >= (int64_t)1 << 30) return fail(ctx, VRG_ERR_UNSUPPORTED, "more than 2^30 triangles");
    // the reference's tree is built when first asked for (vrg_env_tree_info /
    // vrg_env_get_tree): the device walks the walk tree
    scene_bounds(env->xyz, env->min_bound, env->max_bound);
    env->tree = HostTree();
    env->ref_tree_built = false;
    // the GPU build gives trees of the same size and walk speed as the host
    // sweep (within 1 %) in a fraction of the time (7 ms against 25 at 12k
    // triangles, 0.17 s against 4.4 s at 790k), so it is the default
    // whenever there is a device
    const bool on_device = !ctx->host_only && env->walk_builder != 0;

    // the intersection records and the scene constants do not depend on the
    // tree: they are made on a host thread while the tree is built
    env->tri_records.resize(n);
    SceneGeom &g = env->geom;
    memset(&g, 0, sizeof g);
    for (int a = 0; a < 3; a++) {
        g.bmin[a] = env->min_bound[a];
        g.bmax[a] = env->max_bound[a];
        g.smin[a] = INFINITY;
        g.smax[a] = -INFINITY;
    }
    g.ntris = n;
    std::thread records([env, n, &g]() {
        float scale = 0.0f;
        for (int64_t t = 0; t < n; t++) {
            const float *v = &env->xyz[9 * t];
            tri_intersect_format(v, env->ids[t], env->flags[t], &env->tri_records[t], (uint32_t)t);
            for (int k = 0; k < 9; k++) scale = std::max(scale, std::fabs(v[k]));
            if (env->ids[t] & VRG_TRACE_ID_SKY) {
                g.has_sky = 1;
                for (int k = 0; k < 9; k++) {
                    g.smin[k % 3] = std::min(g.smin[k % 3], v[k]);
                    g.smax[k % 3] = std::max(g.smax[k % 3], v[k]);
                }
            }
        }
        g.scale = scale;
    });
    int rc = VRG_OK;
    if (on_device) {
        const cudaError_t e = cudaSetDevice(ctx->device);
        rc = e == cudaSuccess ? build_walk_tree_device(env, env->walk_tree) : cuda_fail(ctx, e, "cudaSetDevice");
    } else {
        build_walk_tree(env->xyz, env->min_bound, env->max_bound, env->walk_costs, env->walk_tree);
    }
    records.join();
    if (rc != VRG_OK) return rc;
    // A walk pushes at most one subtree per inner node on its path, so a tree
    // whose paths hold fewer inner nodes than the device's stack has entries
    // never fills it.  The depth is measured here on the node array that is
    // uploaded, not taken from the builder, so a builder that misreports its
    // tree's height cannot hand the device a tree that would overflow.
    if (env->walk_tree.height >= kStackMax || inner_depth(env->walk_tree.children) >= kStackMax)
        return fail(ctx, VRG_ERR_UNSUPPORTED, "kd tree deeper than the traversal stack");

    // device upload of the walk tree: nodes (8 B), then in leaf order the
    // triangle planes (16 B each) followed by the edge parts (32 B each:
    // (e0, e3, e1, e4), (e2, e5, id, index << 2 | drop)), NTriangleID per
    // triangle
    const HostTree &wt = env->walk_tree;
    const size_t nn = wt.children.size(), nr = wt.refs.size();
    if (nn >= (size_t)kTopRef || nr >= ((size_t)1 << 30))
        return fail(ctx, VRG_ERR_UNSUPPORTED, "kd tree too large for the device node format");
    std::vector<uint2> nodes(nn);
    for (size_t i = 0; i < nn; i++) {
        uint32_t sbits, ch = wt.children[i];
        memcpy(&sbits, &wt.split[i], 4);
        if ((ch & 3u) != kLeaf) {  // flag children that are leaves without triangles
            const uint32_t left = ch >> 2;
            for (uint32_t c = 0; c < 2; c++)
                if ((wt.children[left + c] & 3u) == kLeaf && wt.split[left + c] == 0.0f)
                    ch |= c == 0 ? kLeftEmpty : kRightEmpty;
        }
        nodes[i] = make_uint2(ch, sbits);
    }
    // top table: breadth-first from the root, a pair of children at a
    // time, while it fits; children words of nodes whose children made it
    // into the table point into the table (index | kTopRef)
    std::vector<uint2> top;
    {
        std::vector<int64_t> at(nn, -1);
        std::vector<uint32_t> order;  // node array index of each table entry
        top.push_back(nodes[0]);
        order.push_back(0);
        at[0] = 0;
        for (size_t q = 0; q < order.size(); q++) {
            const uint32_t x = order[q];
            if ((nodes[x].x & 3u) == kLeaf || top.size() + 2 > (size_t)kTopNodes) continue;
            const uint32_t left = (nodes[x].x >> 2) & kChildIndexMask;
            for (uint32_t c = 0; c < 2; c++) {
                at[left + c] = (int64_t)top.size();
                top.push_back(nodes[left + c]);
                order.push_back(left + c);
            }
        }
        for (size_t t = 0; t < top.size(); t++) {
            const uint32_t x = order[t];
            if ((nodes[x].x & 3u) == kLeaf) continue;
            const int64_t l = at[(nodes[x].x >> 2) & kChildIndexMask];
            if (l >= 0)
                top[t].x = (nodes[x].x & (3u | kLeftEmpty | kRightEmpty)) |
                           (((uint32_t)l | kTopRef) << 2);
        }
    }
    env->ntop = (uint32_t)top.size();
    // walls: per face of the scene box, the opaque triangles lying in that
    // face (a closed room's walls and floor, or the brush sides a map's walls
    // are made of), as extra leaf records after the leaf entries: in the
    // face's slots when no face has more than kWallSlots of them, otherwise
    // behind a grid over each face whose cells list the triangles whose
    // extent overlaps them, largest first, at most kWallCellMax.  A shadow
    // line tests the slots or the cell of the face it leaves the box through
    // before walking
    // (wall_occludes).  The first kWallSlots triangles of each face are
    // what vrg_env_wall_slots reports.
    std::vector<int32_t> wall[6];
    std::vector<double> wall_area[6];
    {
        std::vector<std::pair<double, int32_t>> cand[6];
        for (int64_t t = 0; t < (env->use_wall_slots ? n : 0); t++) {
            if (env->ids[t] & VRG_TRACE_ID_SKY) continue;
            const float *v = &env->xyz[9 * t];
            for (int a = 0; a < 3; a++)
                for (int side = 0; side < 2; side++) {
                    const float bound = side ? env->max_bound[a] : env->min_bound[a];
                    if (v[a] != bound || v[3 + a] != bound || v[6 + a] != bound) continue;
                    double e1[3], e2[3];
                    for (int c = 0; c < 3; c++) {
                        e1[c] = (double)v[3 + c] - v[c];
                        e2[c] = (double)v[6 + c] - v[c];
                    }
                    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                                 cz = e1[0] * e2[1] - e1[1] * e2[0];
                    cand[2 * a + side].push_back({-(cx * cx + cy * cy + cz * cz), (int32_t)t});
                }
        }
        for (int f = 0; f < 6; f++) {
            std::stable_sort(cand[f].begin(), cand[f].end());
            for (const auto &c : cand[f]) {
                wall[f].push_back(c.second);
                wall_area[f].push_back(-c.first);
            }
        }
    }
    // one layout per scene, so that the direct-light kernel can be built for
    // it alone: a scene whose faces have at most kWallSlots triangles each (a
    // box room's walls) keeps them in the slots at fixed records
    // nr + kWallSlots * f + i, tested without a table; otherwise every face
    // that has any gets a cell grid over records after the slots
    bool use_cells = false;
    for (int f = 0; f < 6; f++) use_cells = use_cells || wall[f].size() > (size_t)kWallSlots;
    env->wall_layout = use_cells ? 1 : 0;
    size_t nw = 6 * (size_t)kWallSlots;
    for (int f = 0; f < 6; f++)
        if (use_cells) nw += wall[f].size();
    const size_t ne = nr + nw;  // leaf entries + wall slots + wall-cell records
    std::vector<float4> leaf(3 * ne, make_float4(0, 0, 0, 0));
    auto put = [&](size_t r, int32_t tri) {
        const TriRecord &t = env->tri_records[tri];
        float id_bits, idx_bits;
        memcpy(&id_bits, &t.id, 4);
        memcpy(&idx_bits, &t.idx_drop, 4);
        leaf[r] = make_float4(t.nx, t.ny, t.nz, t.d);
        // edge part as pairs (e0, e3) (e1, e4) (e2, e5): b0 and b1 side by side
        leaf[ne + 2 * r] = make_float4(t.e0, t.e3, t.e1, t.e4);
        leaf[ne + 2 * r + 1] = make_float4(t.e2, t.e5, id_bits, idx_bits);
    };
    g.wall_base = (uint32_t)nr;
    g.wall_count = 0;
    g.wall_cell_mask = 0;
    env->n_wall_records = nw;
    // the cell table: 6 face descriptors of kWallFaceWords words (cell origin
    // and inverse size in the face's two in-plane axes as float bits, cells
    // per axis, offset of the face's cell starts), then per face with walls
    // gu * gv + 1 cell starts (indices into this table) and the entries
    // (leaf-record indices)
    std::vector<uint32_t> &cells = env->wall_cells;
    cells.assign(6 * kWallFaceWords, 0u);
    size_t rec = nr + 6 * (size_t)kWallSlots;
    for (int f = 0; f < 6; f++) {
        for (int i = 0; i < kWallSlots; i++)
            env->wall_tris[kWallSlots * f + i] = i < (int)wall[f].size() ? wall[f][i] : -1;
        env->wall_counts[f] = (int32_t)std::min<size_t>(wall[f].size(), kWallSlots);
        const size_t nf = wall[f].size();
        if (nf == 0) continue;
        if (!use_cells) {
            for (size_t i = 0; i < nf; i++) put(nr + (size_t)kWallSlots * f + i, wall[f][i]);
            g.wall_count |= (uint32_t)nf << (3 * f);
            continue;
        }
        const int a = f >> 1, au = (a + 1) % 3, av = (a + 2) % 3;
        const int gs = std::max(1, std::min(kWallGridMax, (int)std::ceil(std::sqrt((double)nf / 2.0))));
        const float u0 = env->min_bound[au], v0 = env->min_bound[av];
        const float du = (env->max_bound[au] - u0) / (float)gs, dv = (env->max_bound[av] - v0) / (float)gs;
        const int gu = du > 0.0f ? gs : 1, gv = dv > 0.0f ? gs : 1;
        const float iu = du > 0.0f ? 1.0f / du : 0.0f, iv = dv > 0.0f ? 1.0f / dv : 0.0f;
        std::vector<std::vector<uint32_t>> cl((size_t)gu * gv);
        for (size_t i = 0; i < nf; i++, rec++) {
            put(rec, wall[f][i]);
            const float *v = &env->xyz[9 * (size_t)wall[f][i]];
            const float umin = std::min(v[au], std::min(v[3 + au], v[6 + au]));
            const float umax = std::max(v[au], std::max(v[3 + au], v[6 + au]));
            const float vmin = std::min(v[av], std::min(v[3 + av], v[6 + av]));
            const float vmax = std::max(v[av], std::max(v[3 + av], v[6 + av]));
            // the cells the triangle's extent overlaps (an extent ending on a
            // cell edge does not reach into the next cell)
            auto span = [](float lo, float hi, float x0, float inv, int g, int &c0, int &c1) {
                const float a = (lo - x0) * inv, b = (hi - x0) * inv;
                c0 = (int)std::min((float)(g - 1), std::max(0.0f, std::floor(a)));
                c1 = (int)std::min((float)(g - 1), std::max((float)c0, std::ceil(b) - 1.0f));
            };
            int c0, c1, r0, r1;
            span(umin, umax, u0, iu, gu, c0, c1);
            span(vmin, vmax, v0, iv, gv, r0, r1);
            for (int cu = c0; cu <= c1; cu++)
                for (int cv = r0; cv <= r1; cv++)
                    if (cl[(size_t)cu * gv + cv].size() < (size_t)kWallCellMax)
                        cl[(size_t)cu * gv + cv].push_back((uint32_t)rec);
        }
        uint32_t *d = &cells[(size_t)f * kWallFaceWords];
        memcpy(&d[0], &u0, 4);
        memcpy(&d[1], &v0, 4);
        memcpy(&d[2], &iu, 4);
        memcpy(&d[3], &iv, 4);
        d[4] = (uint32_t)gu;
        d[5] = (uint32_t)gv;
        d[6] = (uint32_t)cells.size();
        const size_t starts = cells.size();
        cells.resize(starts + (size_t)gu * gv + 1);
        for (size_t c = 0; c < cl.size(); c++) {
            cells[starts + c] = (uint32_t)cells.size();
            cells.insert(cells.end(), cl[c].begin(), cl[c].end());
        }
        cells[starts + cl.size()] = (uint32_t)cells.size();
        g.wall_cell_mask |= 1u << f;
    }
    {  // the cell table after the edge part (wall_table), padded to whole float4s
        cells.resize((cells.size() + 3) & ~(size_t)3, 0u);
        const size_t at = leaf.size();
        leaf.resize(at + cells.size() / 4);
        memcpy(&leaf[at], cells.data(), cells.size() * sizeof(uint32_t));
    }
    {  // the leaf entries, in parallel chunks
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const size_t nt = nr < 65536 ? 1 : hw, chunk = (nr + nt - 1) / nt;
        std::vector<std::thread> pool;
        for (size_t w = 1; w < nt; w++)
            pool.emplace_back([&, w]() {
                for (size_t r = w * chunk; r < std::min(nr, (w + 1) * chunk); r++) put(r, wt.refs[r]);
            });
        for (size_t r = 0; r < std::min(nr, chunk); r++) put(r, wt.refs[r]);
        for (std::thread &t : pool) t.join();
    }
    env->built = true;
    env->cover_ready = false;
    if (ctx->host_only) return VRG_OK;
    VRG_CUDA(ctx, cudaSetDevice(ctx->device));
    VRG_CUDA(ctx, env->d_nodes.reserve(nn * sizeof(uint2)));
    VRG_CUDA(ctx, env->d_leaf_tris.reserve(leaf.size() * sizeof(float4)));
    VRG_CUDA(ctx, env->d_tri_ids.reserve((n ? n : 1) * sizeof(int32_t)));
    VRG_CUDA(ctx, env->d_top.reserve(std::max<size_t>(top.size(), 1) * sizeof(uint2)));
    if (!top.empty())
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_top.ptr, top.data(), top.size() * sizeof(uint2),
                                      cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaMemcpyAsync(env->d_nodes.ptr, nodes.data(), nn * sizeof(uint2),
                                  cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaMemcpyAsync(env->d_leaf_tris.ptr, leaf.data(), leaf.size() * sizeof(float4),
                                  cudaMemcpyHostToDevice, ctx->stream));
    if (n)
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_tri_ids.ptr, env->ids.data(), n * sizeof(int32_t),
                                      cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    env->built = true;
    env->cover_ready = false;
    return VRG_OK;
}

namespace {
// Builds the reference's tree on first use (under the environment's lock).
const HostTree &reference_tree(const vrg_env *cenv) {
    vrg_env *env = const_cast<vrg_env *>(cenv);
    std::lock_guard<std::mutex> lk(env->mu);
    if (!env->ref_tree_built) {
        float mn[3], mx[3];
        build_kd_tree(env->xyz, env->tree, mn, mx);
        env->ref_tree_built = true;
    }
    return env->tree;
}
}  // namespace

int vrg_env_tree_info(const vrg_env *env, int64_t *nodes, int64_t *refs, int32_t *height) {
    if (!env || !env->built) return VRG_ERR_STATE;
    reference_tree(env);
    if (nodes) *nodes = (int64_t)env->tree.children.size();
    if (refs) *refs = (int64_t)env->tree.refs.size();
    if (height) *height = env->tree.height;
    return VRG_OK;
}

int vrg_env_get_tree(const vrg_env *env, uint32_t *children, float *split, int32_t *refs) {
    if (!env || !env->built) return VRG_ERR_STATE;
    reference_tree(env);
    if (children) memcpy(children, env->tree.children.data(), env->tree.children.size() * 4);
    if (split) memcpy(split, env->tree.split.data(), env->tree.split.size() * 4);
    if (refs) memcpy(refs, env->tree.refs.data(), env->tree.refs.size() * 4);
    return VRG_OK;
}

int vrg_env_set_walk_tree_costs(vrg_env *env, float traversal, float intersection,
                                float empty_bonus, int32_t max_depth) {
    if (!env || !(traversal > 0.0f) || !(intersection > 0.0f) || !(empty_bonus > 0.0f) ||
        !(empty_bonus <= 1.0f) || max_depth < 1 || max_depth >= kStackMax)
        return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "walk tree costs set after the build");
    env->walk_costs.traversal = traversal;
    env->walk_costs.intersection = intersection;
    env->walk_costs.empty_bonus = empty_bonus;
    env->walk_costs.max_depth = max_depth;
    return VRG_OK;
}

int vrg_env_wall_slots(const vrg_env *env, int32_t *tris, int32_t *counts) {
    if (!env || !env->built) return VRG_ERR_STATE;
    if (tris) memcpy(tris, env->wall_tris, sizeof env->wall_tris);
    if (counts) memcpy(counts, env->wall_counts, sizeof env->wall_counts);
    return VRG_OK;
}

int vrg_env_set_walk_tree_builder(vrg_env *env, int32_t mode) {
    if (!env || mode < -1 || mode > 1) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "walk tree builder set after the build");
    env->walk_builder = mode;
    return VRG_OK;
}

int vrg_env_set_wall_slots(vrg_env *env, int32_t enable) {
    if (!env || enable < 0 || enable > 1) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "wall slots set after the build");
    env->use_wall_slots = enable != 0;
    return VRG_OK;
}

int vrg_env_walk_tree_info(const vrg_env *env, int64_t *nodes, int64_t *refs, int32_t *height) {
    if (!env || !env->built) return VRG_ERR_STATE;
    if (nodes) *nodes = (int64_t)env->walk_tree.children.size();
    if (refs) *refs = (int64_t)env->walk_tree.refs.size();
    if (height) *height = env->walk_tree.height;
    return VRG_OK;
}

int vrg_env_get_walk_tree(const vrg_env *env, uint32_t *children, float *split, int32_t *refs) {
    if (!env || !env->built) return VRG_ERR_STATE;
    const HostTree &t = env->walk_tree;
    if (children) memcpy(children, t.children.data(), t.children.size() * 4);
    if (split) memcpy(split, t.split.data(), t.split.size() * 4);
    if (refs) memcpy(refs, t.refs.data(), t.refs.size() * 4);
    return VRG_OK;
}

// TriIntersectData layout: Nx,Ny,Nz,D, NTriangleID, edges[6], cs0, cs1,
// flags, unused (raytracer/cache/triangle/triintersectdata.go:3-22)
int vrg_env_get_triangle(const vrg_env *env, int64_t index, void *out48) {
    if (!env || !out48) return VRG_ERR_INVALID;
    if (!env->built) return VRG_ERR_STATE;
    if (index < 0 || index >= (int64_t)env->tri_records.size()) return VRG_ERR_INVALID;
    const TriRecord &t = env->tri_records[index];
    unsigned char *o = static_cast<unsigned char *>(out48);
    const float head[4] = {t.nx, t.ny, t.nz, t.d};
    const float edges[6] = {t.e0, t.e1, t.e2, t.e3, t.e4, t.e5};
    const int drop = (int)(t.idx_drop & 3u);
    const uint8_t tail[4] = {(uint8_t)((drop + 1) % 3), (uint8_t)((drop + 2) % 3),
                             env->flags[index], 0};
    memcpy(o, head, 16);
    memcpy(o + 16, &t.id, 4);
    memcpy(o + 20, edges, 24);
    memcpy(o + 44, tail, 4);
    return VRG_OK;
}

int vrg_env_bounds(const vrg_env *env, float *mins, float *maxs) {
    if (!env || !env->built) return VRG_ERR_STATE;
    if (mins) memcpy(mins, env->min_bound, 12);
    if (maxs) memcpy(maxs, env->max_bound, 12);
    return VRG_OK;
}

}  // extern "C"
