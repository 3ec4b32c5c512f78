// patches.cpp -- MakePatches / SubdividePatches for axis-aligned rectangular
// faces (rad/patches/build.go:21-68, face.go:30-197, subdivide.go:25-411).
//
// A face becomes one root patch; SubdividePatch splits a patch at the
// midpoint of its widest axis (extent scaled by LuxScale) while some axis
// spans at least `chop` and `min_chop` luxels, with the "make more square"
// rule (subdivide.go:204-212) and the edge rule of CreateChildPatch
// (:398-408).  ClipWindingEpsilon's front half (coordinate > dist) is child1.
// On rectangles the clipped windings are rectangles, so the patch is kept as
// its bounds: area = product of the two in-plane extents, centre = midpoint.
#include <cmath>

#include "vrg_internal.h"

namespace vrg {

namespace {

struct P {
    float mins[3], maxs[3], fmins[3], fmaxs[3];
    float chop, luxscale;
    int32_t face, parent, child1 = -1, child2 = -1, axis = -1;
    float dist = 0.0f;
    int nax;
};

float rect_area(const float *mn, const float *mx, int nax) {
    const int a = (nax + 1) % 3, b = (nax + 2) % 3;
    return (mx[a] - mn[a]) * (mx[b] - mn[b]);
}

struct Subdivider {
    std::vector<P> &ps;
    float min_chop;

    void run(size_t ip) {
        float total[3];
        {
            const P &p = ps[ip];
            for (int i = 0; i < 3; i++) total[i] = (p.maxs[i] - p.mins[i]) * p.luxscale;
        }
        float widest = -1.0f;
        int wa = -1;
        bool should = false;
        for (int i = 0; i < 3; i++) {
            if (total[i] > widest) {
                wa = i;
                widest = total[i];
            }
            if (total[i] >= ps[ip].chop && total[i] >= min_chop) should = true;
        }
        if (!should && wa != -1 && total[wa] > total[(wa + 1) % 3] * 2.0f &&
            total[wa] > total[(wa + 2) % 3] * 2.0f && ps[ip].chop > min_chop) {
            should = true;
            ps[ip].chop = std::fmax(min_chop, ps[ip].chop / 2.0f);
        }
        if (!should) return;
        const P parent = ps[ip];
        const float dist = (parent.mins[wa] + parent.maxs[wa]) * 0.5f;
        P kid[2] = {parent, parent};
        kid[0].mins[wa] = dist;  // front: coordinate >= dist
        kid[1].maxs[wa] = dist;
        if (rect_area(kid[0].mins, kid[0].maxs, parent.nax) == 0.0f ||
            rect_area(kid[1].mins, kid[1].maxs, parent.nax) == 0.0f)
            return;
        for (P &c : kid) {
            c.parent = (int32_t)ip;
            c.child1 = c.child2 = c.axis = -1;
            c.dist = 0.0f;
            float t[3];
            for (int i = 0; i < 3; i++) t[i] = (c.maxs[i] - c.mins[i]) * c.luxscale;
            if (c.chop > min_chop && t[0] < c.chop && t[1] < c.chop && t[2] < c.chop) {
                for (int i = 0; i < 3; i++) {
                    if ((c.fmaxs[i] == c.maxs[i] || c.fmins[i] == c.mins[i]) && t[i] > min_chop) {
                        c.chop = std::fmax(min_chop, c.chop / 2.0f);
                        break;
                    }
                }
            }
        }
        const size_t i1 = ps.size();
        ps.push_back(kid[0]);
        ps.push_back(kid[1]);
        ps[ip].child1 = (int32_t)i1;
        ps[ip].child2 = (int32_t)i1 + 1;
        ps[ip].axis = wa;
        ps[ip].dist = dist;
        run(i1);
        run(i1 + 1);
    }
};

}  // namespace

int make_rect_patches(const vrg_env &env, float max_chop, float min_chop, PatchSet &out) {
    std::vector<P> ps;
    ps.reserve((size_t)env.nfaces * 8);
    for (int32_t f = 0; f < env.nfaces; f++) {
        P p{};
        const float *c = &env.f_corner[3 * f], *U = &env.f_u[3 * f], *V = &env.f_v[3 * f],
                    *N = &env.f_normal[3 * f];
        int nax = 0;
        for (int i = 1; i < 3; i++)
            if (std::fabs(N[i]) > std::fabs(N[nax])) nax = i;
        for (int i = 0; i < 3; i++) {
            const float pts[4] = {c[i], c[i] + U[i], c[i] + V[i], (c[i] + U[i]) + V[i]};
            p.mins[i] = p.maxs[i] = pts[0];
            for (int k = 1; k < 4; k++) {
                p.mins[i] = std::fmin(p.mins[i], pts[k]);
                p.maxs[i] = std::fmax(p.maxs[i], pts[k]);
            }
            p.fmins[i] = p.mins[i];
            p.fmaxs[i] = p.maxs[i];
        }
        p.nax = nax;
        p.chop = max_chop;
        p.luxscale = env.f_luxscale[f];
        p.face = f;
        p.parent = -1;
        if (!(rect_area(p.mins, p.maxs, nax) > 0.0f)) continue;  // degenerate face (face.go:50-55)
        ps.push_back(p);
    }
    Subdivider sub{ps, min_chop};
    const size_t roots = ps.size();
    for (size_t i = 0; i < roots; i++) sub.run(i);

    const size_t n = ps.size();
    out = PatchSet();
    out.mins.resize(3 * n);
    out.maxs.resize(3 * n);
    out.center.resize(3 * n);
    out.area.resize(n);
    out.split_dist.resize(n);
    out.face.resize(n);
    out.parent.resize(n);
    out.child1.resize(n);
    out.child2.resize(n);
    out.split_axis.resize(n);
    out.leaf_index.resize(n);
    out.face_root.assign(env.nfaces, -1);
    int32_t leaf = 0;
    for (size_t i = 0; i < n; i++) {
        const P &p = ps[i];
        for (int a = 0; a < 3; a++) {
            out.mins[3 * i + a] = p.mins[a];
            out.maxs[3 * i + a] = p.maxs[a];
            out.center[3 * i + a] = (p.mins[a] + p.maxs[a]) * 0.5f;
        }
        out.area[i] = rect_area(p.mins, p.maxs, p.nax);
        out.face[i] = p.face;
        out.parent[i] = p.parent;
        out.child1[i] = p.child1;
        out.child2[i] = p.child2;
        out.split_axis[i] = p.axis;
        out.split_dist[i] = p.dist;
        if (p.parent < 0) out.face_root[p.face] = (int32_t)i;
        if (p.child1 < 0) {
            out.leaf_index[i] = leaf++;
            out.leaf_patch.push_back((int32_t)i);
        } else {
            out.leaf_index[i] = -1;
        }
    }
    return VRG_OK;
}

}  // namespace vrg
