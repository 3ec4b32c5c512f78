// kdbuild.cpp -- SAH kd-tree builder for SetupAccelerationStructure
// (raytracer/environment.go:119-138, RefineNode :238-387,
// CalculateCostsOfSplit :181-236, ClassifyAgainstAxisSplit
// raytracer/cache/optimisedtriangle.go:83-103).
//
// Same candidates, costs, tie-breaking, partition order and node numbering
// as the reference with its evident defects fixed: vertices read x,y,z
// (optimisedtriangle.go:22-28 reads index 3i+1 three times), the root bounds
// are written (raytracer/math/trianglelist.go:9-21 assigns to local copies),
// the midpoint candidate is 0.5*(min+max) (environment.go:274), the split
// counts and the grown split value reach the caller (they are passed by
// value at :181-182), and the left partition index is post-incremented
// (:348-349).
//
// Unlike the reference, each node does not classify every triangle for
// every candidate.  It sorts the per-axis triangle extents once and counts
// each candidate's left/right/straddling sets by binary search, which gives
// the same integers, hence the same float32 costs and the same tree.
#include <algorithm>
#include <cstring>

#include "vrg_internal.h"

namespace vrg {

namespace {

struct Builder {
    const float *xyz;
    HostTree &tree;
    std::vector<float> lo[3], hi[3];  // per triangle extent on each axis

    Builder(const float *x, int64_t n, HostTree &t) : xyz(x), tree(t) {
        for (int a = 0; a < 3; a++) {
            lo[a].resize(n);
            hi[a].resize(n);
        }
        for (int64_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) {
                float v0 = xyz[9 * i + a], v1 = xyz[9 * i + 3 + a], v2 = xyz[9 * i + 6 + a];
                lo[a][i] = std::min(v0, std::min(v1, v2));
                hi[a][i] = std::max(v0, std::max(v1, v2));
            }
    }

    static float box_area(const float *mn, const float *mx) {
        float d0 = mx[0] - mn[0], d1 = mx[1] - mn[1], d2 = mx[2] - mn[2];
        return 2.0f * (((d0 * d2) + (d0 * d1)) + (d1 * d2));
    }

    // PLANECHECK_* of ClassifyAgainstAxisSplit: +1 right, -1 left, 0 both
    int classify(int32_t t, int axis, float s) const {
        float l = lo[axis][t], h = hi[axis][t];
        if (l >= s) return 1;
        if (h <= s) return -1;
        if (l == h) return 1;
        return 0;
    }

    void leaf(int node, const int32_t *list, int n) {
        tree.children[node] = kLeaf + ((uint32_t)tree.refs.size() << 2);
        tree.split[node] = (float)n;
        tree.refs.insert(tree.refs.end(), list, list + n);
    }

    void refine(int node, const int32_t *list, int n, const float *mn, const float *mx, int depth,
                int level) {
        tree.height = std::max(tree.height, level + 1);
        if (n < 3) {
            leaf(node, list, n);
            return;
        }
        float best_cost = 1.0e23f, best_used = 0.0f, best_trial = 0.0f;
        int best_l = 0, best_r = 0, best_b = 0, best_axis = 0;
        const int skip = 1 + n / 10;
        const float isa = 1.0f / box_area(mn, mx);
        std::vector<float> slo(n), shi(n), flat;
        for (int axis = 0; axis < 3; axis++) {
            flat.clear();
            for (int i = 0; i < n; i++) {
                slo[i] = lo[axis][list[i]];
                shi[i] = hi[axis][list[i]];
                if (slo[i] == shi[i]) flat.push_back(slo[i]);
            }
            std::sort(slo.begin(), slo.end());
            std::sort(shi.begin(), shi.end());
            std::sort(flat.begin(), flat.end());
            const float minc = slo.front(), maxc = shi.back();
            auto evaluate = [&](float trial) {
                const int nr = n - (int)(std::lower_bound(slo.begin(), slo.end(), trial) - slo.begin());
                const int nhi = (int)(std::upper_bound(shi.begin(), shi.end(), trial) - shi.begin());
                auto fr = std::equal_range(flat.begin(), flat.end(), trial);
                const int nl = nhi - (int)(fr.second - fr.first);
                const int nb = n - nl - nr;
                float used = trial;
                if (nl != 0 && nb == 0 && nr == 0) used = maxc;
                if (nr != 0 && nb == 0 && nl == 0) used = minc;
                float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
                lmx[axis] = used;
                rmn[axis] = used;
                const float sal = box_area(mn, lmx), sar = box_area(rmn, mx);
                const float inner = ((float)nb + (sal * isa) * (float)nl) + (sar * isa) * (float)nr;
                const float cost = (float)kCostOfTraversal + (float)kCostOfIntersection * inner;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_l = nl;
                    best_r = nr;
                    best_b = nb;
                    best_used = used;
                    best_trial = trial;
                }
            };
            evaluate(0.5f * (mn[axis] + mx[axis]));
            for (int ts = skip - 1; ts < n; ts += skip) {
                for (int tv = 0; tv < 3; tv++) {
                    const float v = xyz[9 * (int64_t)list[ts] + 3 * tv + axis];
                    if (v > mx[axis] || v < mn[axis]) continue;
                    evaluate(v);
                }
            }
        }
        const float no_split = (float)(kCostOfIntersection * n);
        if (no_split <= best_cost || depth > kMaxTreeDepth) {
            leaf(node, list, n);
            return;
        }
        // left block in order, straddling block after it, right block filled
        // from the back (environment.go:343-359)
        std::vector<int32_t> part(n);
        int lo_out = 0, both_out = 0, right_out = 0;
        for (int t = 0; t < n; t++) {
            const int c = classify(list[t], best_axis, best_trial);
            if (c < 0) part[lo_out++] = list[t];
            else if (c > 0) part[n - ++right_out] = list[t];
            else part[best_l + both_out++] = list[t];
        }
        float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
        lmx[best_axis] = best_used;
        rmn[best_axis] = best_used;
        const int left = (int)tree.children.size();
        tree.children[node] = (uint32_t)best_axis + ((uint32_t)left << 2);
        tree.split[node] = best_used;
        tree.children.push_back(0);
        tree.children.push_back(0);
        tree.split.push_back(0.0f);
        tree.split.push_back(0.0f);
        if (n < 20 && (best_l == 0 || best_r == 0)) depth += 100;
        refine(left, part.data(), best_l + best_b, mn, lmx, depth + 1, level + 1);
        refine(left + 1, part.data() + best_l, best_r + best_b, rmn, mx, depth + 1, level + 1);
    }
};

// The tree the device walks.  Any tree whose leaves hold every triangle
// that touches their cell gives the walk the same answers (closest hit =
// brute force, ties to the lower index), so the device is free to use a
// better one than the reference's, whose SAH only tries the vertices of
// every (1 + n/10)-th triangle.  This one evaluates every candidate plane:
// the triangles' extents clamped to the node's box, swept in sorted order on
// each axis (the event sweep of Wald & Havran, "On building fast kd-trees
// for ray tracing, and on doing that in O(N log N)", 2006, here with a sort
// per node).  Cost of a split = traversal + intersection * (P_L * N_L +
// P_R * N_R) (P = surface-area ratio), times empty_bonus when one side is
// empty; triangles lying in the plane go to the cheaper side.  A node
// becomes a leaf when no split is cheaper than intersection * N, when it
// holds one triangle, or at depth max_depth.  The node numbering (children
// in adjacent pairs, left at the odd index) and the leaf format are those of
// the reference's tree.
struct WalkBuilder {
    const float *xyz;
    HostTree &tree;
    WalkTreeCosts cost;
    std::vector<float> lo[3], hi[3];

    struct Event {
        float p;
        int kind;  // 0 ends here, 1 lies in the plane, 2 starts here
    };

    WalkBuilder(const float *x, int64_t n, HostTree &t, const WalkTreeCosts &c)
        : xyz(x), tree(t), cost(c) {
        for (int a = 0; a < 3; a++) {
            lo[a].resize(n);
            hi[a].resize(n);
        }
        for (int64_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) {
                const float v0 = x[9 * i + a], v1 = x[9 * i + 3 + a], v2 = x[9 * i + 6 + a];
                lo[a][i] = std::min(v0, std::min(v1, v2));
                hi[a][i] = std::max(v0, std::max(v1, v2));
            }
    }

    static double area(const float *mn, const float *mx) {
        const double d0 = (double)mx[0] - mn[0], d1 = (double)mx[1] - mn[1],
                     d2 = (double)mx[2] - mn[2];
        return 2.0 * (d0 * d1 + d0 * d2 + d1 * d2);
    }

    void leaf(int node, const std::vector<int32_t> &list) {
        tree.children[node] = kLeaf + ((uint32_t)tree.refs.size() << 2);
        tree.split[node] = (float)list.size();
        tree.refs.insert(tree.refs.end(), list.begin(), list.end());
    }

    void refine(int node, std::vector<int32_t> list, const float *mn, const float *mx, int level) {
        tree.height = std::max(tree.height, level + 1);
        const int n = (int)list.size();
        if (n <= 1 || level + 1 >= cost.max_depth) {
            leaf(node, list);
            return;
        }
        const double sa = area(mn, mx);
        double best = (double)cost.intersection * n;
        int bax = -1;
        float bp = 0.0f;
        bool planar_left = false;
        std::vector<Event> ev;
        ev.reserve(2 * (size_t)n);
        for (int a = 0; a < 3; a++) {
            if (!(mx[a] > mn[a]) || !(sa > 0.0)) continue;
            ev.clear();
            for (int32_t t : list) {
                const float l = std::max(lo[a][t], mn[a]), h = std::min(hi[a][t], mx[a]);
                if (l == h) {
                    ev.push_back({l, 1});
                } else {
                    ev.push_back({l, 2});
                    ev.push_back({h, 0});
                }
            }
            std::sort(ev.begin(), ev.end(), [](const Event &x, const Event &y) {
                return x.p < y.p || (x.p == y.p && x.kind < y.kind);
            });
            // nl: triangles starting below p (or in an earlier plane);
            // nr: triangles ending above p
            int nl = 0, nr = n;
            for (size_t i = 0; i < ev.size();) {
                const float p = ev[i].p;
                int ends = 0, planar = 0, starts = 0;
                for (; i < ev.size() && ev[i].p == p && ev[i].kind == 0; i++) ends++;
                for (; i < ev.size() && ev[i].p == p && ev[i].kind == 1; i++) planar++;
                for (; i < ev.size() && ev[i].p == p && ev[i].kind == 2; i++) starts++;
                nr -= planar + ends;
                if (p > mn[a] && p < mx[a]) {
                    float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
                    lmx[a] = p;
                    rmn[a] = p;
                    const double pl = area(mn, lmx) / sa, pr = area(rmn, mx) / sa;
                    for (int side = 0; side < 2; side++) {
                        const int cl = nl + (side == 0 ? planar : 0);
                        const int cr = nr + (side == 1 ? planar : 0);
                        double c = cost.traversal + cost.intersection * (pl * cl + pr * cr);
                        if (cl == 0 || cr == 0) c *= cost.empty_bonus;
                        if (c < best) {
                            best = c;
                            bax = a;
                            bp = p;
                            planar_left = side == 0;
                        }
                    }
                }
                nl += starts + planar;
            }
        }
        if (bax < 0) {
            leaf(node, list);
            return;
        }
        std::vector<int32_t> L, R;
        for (int32_t t : list) {
            const float l = std::max(lo[bax][t], mn[bax]), h = std::min(hi[bax][t], mx[bax]);
            if (l == h && l == bp) {
                (planar_left ? L : R).push_back(t);
                continue;
            }
            if (l < bp) L.push_back(t);
            if (h > bp) R.push_back(t);
        }
        std::vector<int32_t>().swap(list);
        float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
        lmx[bax] = bp;
        rmn[bax] = bp;
        const int left = (int)tree.children.size();
        tree.children[node] = (uint32_t)bax + ((uint32_t)left << 2);
        tree.split[node] = bp;
        tree.children.push_back(0);
        tree.children.push_back(0);
        tree.split.push_back(0.0f);
        tree.split.push_back(0.0f);
        refine(left, std::move(L), mn, lmx, level + 1);
        refine(left + 1, std::move(R), rmn, mx, level + 1);
    }
};

}  // namespace

void build_walk_tree(const std::vector<float> &xyz, const float *mn, const float *mx,
                     const WalkTreeCosts &cost, HostTree &tree) {
    const int64_t n = (int64_t)(xyz.size() / 9);
    tree.children.assign(1, 0);
    tree.split.assign(1, 0.0f);
    tree.refs.clear();
    tree.height = 0;
    WalkBuilder b(xyz.data(), n, tree, cost);
    std::vector<int32_t> root(n);
    for (int64_t i = 0; i < n; i++) root[i] = (int32_t)i;
    b.refine(0, std::move(root), mn, mx, 0);
}

void scene_bounds(const std::vector<float> &xyz, float *mn, float *mx) {
    const int64_t n = (int64_t)(xyz.size() / 9);
    for (int a = 0; a < 3; a++) {
        mn[a] = 1.0e23f;
        mx[a] = -1.0e23f;
    }
    for (int64_t i = 0; i < 9 * n; i++) {
        mn[i % 3] = std::min(mn[i % 3], xyz[i]);
        mx[i % 3] = std::max(mx[i % 3], xyz[i]);
    }
    if (n == 0)
        for (int a = 0; a < 3; a++) mn[a] = mx[a] = 0.0f;
}

void build_kd_tree(const std::vector<float> &xyz, HostTree &tree, float *mn, float *mx) {
    const int64_t n = (int64_t)(xyz.size() / 9);
    tree.children.assign(1, 0);
    tree.split.assign(1, 0.0f);
    tree.refs.clear();
    tree.height = 0;
    scene_bounds(xyz, mn, mx);
    Builder b(xyz.data(), n, tree);
    std::vector<int32_t> root(n);
    for (int64_t i = 0; i < n; i++) root[i] = (int32_t)i;
    b.refine(0, root.data(), (int)n, mn, mx, 0, 0);
}

}  // namespace vrg
