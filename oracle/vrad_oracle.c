/*
 * vrad_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see vrad_oracle.h).
 *
 * Compiled with -O2 -ffp-contract=off -fno-fast-math: every float32
 * expression below rounds once per operation, in the order written, so the
 * GPU kernels (built with FMA contraction off and *_rn intrinsics) can be
 * compared bit for bit where the semantics say so.
 *
 * Two modes exist for the pieces the reference actually contains:
 *   ORC_MODE_LITERAL reproduces the Go code as written (defects included);
 *   ORC_MODE_FIXED   is the evident intent, and is what the GPU path matches.
 */
#include "vrad_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../vrad_gb300/csrc/anorms_table.h"

#define COST_OF_TRAVERSAL 75     /* raytracer/kdtree/constants.go:25 */
#define COST_OF_INTERSECTION 167 /* raytracer/kdtree/constants.go:26 */
#define MAX_TREE_DEPTH 21        /* raytracer/kdtree/constants.go:28 */
#define KD_LEAF 3                /* raytracer/cache/optimisedkdnode.go:6 */
#define PLANE_POS 1              /* raytracer/cache/optimisedtriangle.go:10-12 */
#define PLANE_NEG (-1)
#define PLANE_STRADDLE 0
/* common/constants/constants.go:19  MAX_TRACE_LENGTH = sqrt(3) * 2 * 16384 */
#define MAX_TRACE_LENGTH ((float)(1.732050807569 * 32768.0))
/* project constant: sample points sit this far off their surface */
#define SAMPLE_OFFSET 0.125f
#define STACK_MAX 64

static const float k_anorms[VRG_NUM_ANORMS * 3] = VRG_ANORMS_INIT;

struct orc_scene {
    int64_t ntris;
    float *xyz;
    int32_t *ids;
    uint8_t *flags;
    int8_t *tmp0, *tmp1;
    orc_tri *tris;
    uint32_t *children;
    float *split;
    int64_t nnodes, cap_nodes;
    int32_t *refs;
    int64_t nrefs, cap_refs;
    float bmin[3], bmax[3];
    float coord_scale;
    int has_sky;
    float sky_min[3], sky_max[3];
    int mode;
    int depth;
    int skip_empty; /* walk: do not visit leaves without triangles (same answers) */
    int use_walls;  /* shadow lines test the wall triangles of their exit face first */
    int32_t walls[6][4];
    int nwalls[6];
};

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */

static float dot3(const float *a, const float *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* OptimisedTriangle.Vertex (optimisedtriangle.go:22-28).  The Go reads
 * VertexCoordData[3i+1] for all three components (defect D1); the fixed
 * form reads x, y, z. */
static void tri_vertex(const orc_scene *s, int64_t t, int v, float out[3]) {
    const float *p = s->xyz + 9 * t + 3 * v;
    if (s->mode == ORC_MODE_LITERAL) {
        out[0] = p[1];
        out[1] = p[1];
        out[2] = p[1];
    } else {
        out[0] = p[0];
        out[1] = p[1];
        out[2] = p[2];
    }
}

/* BoxSurfaceArea (vmath/polygon/surface.go:5-8) */
static float box_area(const float *mn, const float *mx) {
    float d0 = mx[0] - mn[0], d1 = mx[1] - mn[1], d2 = mx[2] - mn[2];
    return 2.0f * (((d0 * d2) + (d0 * d1)) + (d1 * d2));
}

/* ClassifyAgainstAxisSplit (optimisedtriangle.go:83-103) */
static int classify(const orc_scene *s, int64_t t, int axis, float split) {
    float v[3];
    tri_vertex(s, t, 0, v);
    float minc = v[axis], maxc = minc;
    for (int k = 0; k < 3; k++) {
        tri_vertex(s, t, k, v);
        if (v[axis] < minc) minc = v[axis];
        if (v[axis] > maxc) maxc = v[axis];
    }
    if (minc >= split) return PLANE_POS;
    if (maxc <= split) return PLANE_NEG;
    if (minc == maxc) return PLANE_POS;
    return PLANE_STRADDLE;
}

/* ------------------------------------------------------------------ */
/* intersection format                                                 */
/* ------------------------------------------------------------------ */

/* GetEdgeEquation (vmath/polygon/edge.go:5-24): the edge line through p1,p2
 * in the (c1,c2) projection, signed and scaled to equal 1 at `inside`. */
void orc_edge_equation(const float *p1, const float *p2, int c1, int c2, const float *inside,
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

/* ChangeIntoIntersectionFormat (optimisedtriangle.go:30-78).  Normalize is
 * v * (1/|v|) with |v| = sqrt((x*x + y*y) + z*z) in float32. */
void orc_tri_format(const float *xyz9, int32_t id, uint8_t flags, orc_tri *out) {
    const float *p1 = xyz9, *p2 = xyz9 + 3, *p3 = xyz9 + 6;
    float e1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    float e2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                  e1[0] * e2[1] - e1[1] * e2[0]};
    float len = sqrtf(dot3(n, n));
    float inv = 1.0f / len;
    n[0] = n[0] * inv;
    n[1] = n[1] * inv;
    n[2] = n[2] * inv;
    int drop = 0;
    for (int c = 1; c < 3; c++)
        if (fabsf(n[c]) > fabsf(n[drop])) drop = c;
    memset(out, 0, sizeof(*out));
    out->nx = n[0];
    out->ny = n[1];
    out->nz = n[2];
    out->d = dot3(n, p1);
    out->id = id;
    out->flags = flags;
    out->cs0 = (uint8_t)((drop + 1) % 3);
    out->cs1 = (uint8_t)((drop + 2) % 3);
    orc_edge_equation(p1, p2, out->cs0, out->cs1, p3, out->e);
    orc_edge_equation(p2, p3, out->cs0, out->cs1, p1, out->e + 3);
}

/* ------------------------------------------------------------------ */
/* kd builder (environment.go:119-387)                                 */
/* ------------------------------------------------------------------ */

static int push_node(orc_scene *s) {
    if (s->nnodes == s->cap_nodes) {
        s->cap_nodes = s->cap_nodes ? 2 * s->cap_nodes : 1024;
        s->children = realloc(s->children, s->cap_nodes * sizeof(uint32_t));
        s->split = realloc(s->split, s->cap_nodes * sizeof(float));
    }
    s->children[s->nnodes] = 0;
    s->split[s->nnodes] = 0.0f;
    return (int)s->nnodes++;
}

static void push_ref(orc_scene *s, int32_t r) {
    if (s->nrefs == s->cap_refs) {
        s->cap_refs = s->cap_refs ? 2 * s->cap_refs : 4096;
        s->refs = realloc(s->refs, s->cap_refs * sizeof(int32_t));
    }
    s->refs[s->nrefs++] = r;
}

static void make_leaf(orc_scene *s, int node, const int *list, int n) {
    s->children[node] = KD_LEAF + ((uint32_t)s->nrefs << 2);
    s->split[node] = (float)n;
    for (int t = 0; t < n; t++) push_ref(s, list[t]);
}

/* CalculateCostsOfSplit (environment.go:181-236).  The Go passes the counts
 * and the split value by value (defect D4), so the "grown" split value and
 * the counts never reach the caller; the fixed form returns all of them. */
static float split_cost(orc_scene *s, int axis, const int *list, int n, const float *mn,
                        const float *mx, float *split_io, int *nl, int *nr, int *nb) {
    int l = 0, r = 0, b = 0;
    double minc = 1.0e23, maxc = -1.0e23;
    float split = *split_io;
    float v[3];
    for (int t = 0; t < n; t++) {
        for (int k = 0; k < 3; k++) {
            tri_vertex(s, list[t], k, v);
            if ((double)v[axis] < minc) minc = v[axis];
            if ((double)v[axis] > maxc) maxc = v[axis];
        }
        int c = classify(s, list[t], axis, split);
        if (c == PLANE_NEG) l++;
        else if (c == PLANE_POS) r++;
        else b++;
        s->tmp0[list[t]] = (int8_t)c;
    }
    if (l != 0 && b == 0 && r == 0) split = (float)maxc;
    if (r != 0 && b == 0 && l == 0) split = (float)minc;
    float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
    lmx[axis] = split;
    rmn[axis] = split;
    float sal = box_area(mn, lmx), sar = box_area(rmn, mx);
    float isa = 1.0f / box_area(mn, mx);
    float inner = ((float)b + (sal * isa) * (float)l) + (sar * isa) * (float)r;
    float cost = (float)COST_OF_TRAVERSAL + (float)COST_OF_INTERSECTION * inner;
    if (s->mode == ORC_MODE_FIXED) {
        *split_io = split;
        *nl = l;
        *nr = r;
        *nb = b;
    }
    return cost;
}

/* RefineNode (environment.go:238-387) */
static void refine(orc_scene *s, int node, const int *list, int n, const float *mn,
                   const float *mx, int depth) {
    if (depth > s->depth) s->depth = depth;
    if (n < 3) {
        make_leaf(s, node, list, n);
        return;
    }
    float best_cost = 1.0e23f, best_split = 0.0f;
    int best_l = 0, best_r = 0, best_b = 0, axis_best = 0;
    int skip = 1 + n / 10;
    float v[3];
    for (int axis = 0; axis < 3; axis++) {
        for (int ts = -1; ts < n; ts += skip) {
            for (int tv = 0; tv < 3; tv++) {
                int tl = 0, tr = 0, tb = 0;
                float trial;
                if (ts == -1) {
                    if (s->mode == ORC_MODE_LITERAL)
                        trial = 0.5f * mn[axis] + mx[axis]; /* defect D3 */
                    else
                        trial = 0.5f * (mn[axis] + mx[axis]);
                } else {
                    tri_vertex(s, list[ts], tv, v);
                    trial = v[axis];
                    if (trial > mx[axis] || trial < mn[axis]) continue;
                }
                float used = trial;
                float cost = split_cost(s, axis, list, n, mn, mx, &used, &tl, &tr, &tb);
                if (cost < best_cost) {
                    axis_best = axis;
                    best_cost = cost;
                    best_l = tl;
                    best_r = tr;
                    best_b = tb;
                    best_split = (s->mode == ORC_MODE_FIXED) ? used : trial;
                    for (int t = 0; t < n; t++) s->tmp1[list[t]] = s->tmp0[list[t]];
                }
                if (ts == -1) break;
            }
        }
    }
    float no_split = (float)(COST_OF_INTERSECTION * n);
    if (no_split <= best_cost || depth > MAX_TREE_DEPTH) {
        make_leaf(s, node, list, n);
        return;
    }
    if (s->mode == ORC_MODE_LITERAL) {
        /* With the literal builder the root bounds are never written (D2),
         * every cost is NaN and this point is unreachable; the partition as
         * written (D4 counts of zero, D5 pre-increment) would index past the
         * list.  Fall back to a leaf rather than reproduce an out-of-range
         * write. */
        make_leaf(s, node, list, n);
        return;
    }
    int *nl = malloc(sizeof(int) * (size_t)n);
    int lo = 0, bo = 0, ro = 0;
    for (int t = 0; t < n; t++) {
        int c = s->tmp1[list[t]];
        if (c == PLANE_NEG) nl[lo++] = list[t];
        else if (c == PLANE_POS) nl[n - ++ro] = list[t];
        else nl[best_l + bo++] = list[t];
    }
    float lmx[3] = {mx[0], mx[1], mx[2]}, rmn[3] = {mn[0], mn[1], mn[2]};
    lmx[axis_best] = best_split;
    rmn[axis_best] = best_split;
    int left = (int)s->nnodes;
    s->children[node] = (uint32_t)axis_best + ((uint32_t)left << 2);
    s->split[node] = best_split;
    push_node(s);
    push_node(s);
    if (n < 20 && (best_l == 0 || best_r == 0)) depth += 100;
    refine(s, left, nl, best_l + best_b, mn, lmx, depth + 1);
    refine(s, left + 1, nl + best_l, best_r + best_b, rmn, mx, depth + 1);
    free(nl);
}

orc_scene *orc_scene_new(const float *xyz, const int32_t *ids, const uint8_t *flags,
                         int64_t ntris, int mode) {
    orc_scene *s = calloc(1, sizeof(orc_scene));
    s->ntris = ntris;
    s->mode = mode;
    s->xyz = malloc(sizeof(float) * 9 * (size_t)(ntris ? ntris : 1));
    s->ids = malloc(sizeof(int32_t) * (size_t)(ntris ? ntris : 1));
    s->flags = calloc((size_t)(ntris ? ntris : 1), 1);
    s->tmp0 = calloc((size_t)(ntris ? ntris : 1), 1);
    s->tmp1 = calloc((size_t)(ntris ? ntris : 1), 1);
    s->tris = calloc((size_t)(ntris ? ntris : 1), sizeof(orc_tri));
    memcpy(s->xyz, xyz, sizeof(float) * 9 * (size_t)ntris);
    memcpy(s->ids, ids, sizeof(int32_t) * (size_t)ntris);
    if (flags) memcpy(s->flags, flags, (size_t)ntris);

    /* CalculateTriangleListBounds (raytracer/math/trianglelist.go:9-21).  The
     * Go assigns to local pointer copies (D2) so the bounds stay (0,0,0). */
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    if (mode == ORC_MODE_FIXED) {
        mn[0] = mn[1] = mn[2] = 1.0e23f;
        mx[0] = mx[1] = mx[2] = -1.0e23f;
        for (int64_t t = 0; t < ntris; t++)
            for (int k = 0; k < 9; k++) {
                float c = xyz[9 * t + k];
                if (c < mn[k % 3]) mn[k % 3] = c;
                if (c > mx[k % 3]) mx[k % 3] = c;
            }
        if (ntris == 0) mn[0] = mn[1] = mn[2] = mx[0] = mx[1] = mx[2] = 0.0f;
    }
    memcpy(s->bmin, mn, sizeof mn);
    memcpy(s->bmax, mx, sizeof mx);

    push_node(s);
    int *root = malloc(sizeof(int) * (size_t)(ntris ? ntris : 1));
    for (int64_t t = 0; t < ntris; t++) root[t] = (int)t;
    refine(s, 0, root, (int)ntris, mn, mx, 0);
    free(root);

    float scale = 0.0f;
    s->sky_min[0] = s->sky_min[1] = s->sky_min[2] = INFINITY;
    s->sky_max[0] = s->sky_max[1] = s->sky_max[2] = -INFINITY;
    for (int64_t t = 0; t < ntris; t++) {
        orc_tri_format(xyz + 9 * t, ids[t], s->flags[t], &s->tris[t]);
        for (int k = 0; k < 9; k++) {
            float a = fabsf(xyz[9 * t + k]);
            if (a > scale) scale = a;
        }
        if (ids[t] & ORC_TRACE_ID_SKY) {
            s->has_sky = 1;
            for (int k = 0; k < 9; k++) {
                if (xyz[9 * t + k] < s->sky_min[k % 3]) s->sky_min[k % 3] = xyz[9 * t + k];
                if (xyz[9 * t + k] > s->sky_max[k % 3]) s->sky_max[k % 3] = xyz[9 * t + k];
            }
        }
    }
    s->coord_scale = scale;
    return s;
}

void orc_scene_free(orc_scene *s) {
    if (!s) return;
    free(s->xyz);
    free(s->ids);
    free(s->flags);
    free(s->tmp0);
    free(s->tmp1);
    free(s->tris);
    free(s->children);
    free(s->split);
    free(s->refs);
    free(s);
}

int64_t orc_scene_num_nodes(const orc_scene *s) { return s->nnodes; }
int64_t orc_scene_num_refs(const orc_scene *s) { return s->nrefs; }
int orc_scene_depth(const orc_scene *s) { return s->depth; }
void orc_scene_get_tree(const orc_scene *s, uint32_t *children, float *split, int32_t *refs) {
    if (children) memcpy(children, s->children, sizeof(uint32_t) * (size_t)s->nnodes);
    if (split) memcpy(split, s->split, sizeof(float) * (size_t)s->nnodes);
    if (refs) memcpy(refs, s->refs, sizeof(int32_t) * (size_t)s->nrefs);
}
/* Replaces the scene's tree with another of the same format (children word,
 * split or leaf count, triangle index list), e.g. the library's walk tree,
 * so that its walk can be checked against brute force and counted.  The
 * walk visits at most one stacked subtree per level: depth < STACK_MAX. */
int orc_scene_set_tree(orc_scene *s, const uint32_t *children, const float *split,
                       int64_t nnodes, const int32_t *refs, int64_t nrefs) {
    if (nnodes < 1) return -1;
    uint32_t *c = malloc(sizeof(uint32_t) * (size_t)nnodes);
    float *f = malloc(sizeof(float) * (size_t)nnodes);
    int32_t *r = malloc(sizeof(int32_t) * (size_t)(nrefs > 0 ? nrefs : 1));
    if (!c || !f || !r) {
        free(c);
        free(f);
        free(r);
        return -1;
    }
    memcpy(c, children, sizeof(uint32_t) * (size_t)nnodes);
    memcpy(f, split, sizeof(float) * (size_t)nnodes);
    if (nrefs > 0) memcpy(r, refs, sizeof(int32_t) * (size_t)nrefs);
    free(s->children);
    free(s->split);
    free(s->refs);
    s->children = c;
    s->split = f;
    s->refs = r;
    s->nnodes = s->cap_nodes = nnodes;
    s->nrefs = s->cap_refs = nrefs;
    return 0;
}

void orc_scene_set_skip_empty(orc_scene *s, int on) { s->skip_empty = on != 0; }

void orc_scene_set_walls(orc_scene *s, const int32_t *tris, const int32_t *counts) {
    s->use_walls = 0;
    for (int f = 0; f < 6; f++) {
        s->nwalls[f] = 0;
        if (!tris || !counts) continue;
        for (int i = 0; i < counts[f] && i < 4; i++) {
            const int32_t t = tris[4 * f + i];
            if (t < 0 || t >= s->ntris) continue;
            s->walls[f][s->nwalls[f]++] = t;
            s->use_walls = 1;
        }
    }
}

void orc_scene_get_tris(const orc_scene *s, orc_tri *out) {
    memcpy(out, s->tris, sizeof(orc_tri) * (size_t)s->ntris);
}
void orc_scene_bounds(const orc_scene *s, float *bmin, float *bmax) {
    memcpy(bmin, s->bmin, sizeof(float) * 3);
    memcpy(bmax, s->bmax, sizeof(float) * 3);
}

/* ------------------------------------------------------------------ */
/* ray / triangle test and traversal (Trace4Rays, environment.go:140)  */
/* ------------------------------------------------------------------ */

/* Project-defined ray/triangle test, in this exact operation order:
 *   den = (Nx*dx + Ny*dy) + Nz*dz ;  t = (D - ((Nx*ox + Ny*oy) + Nz*oz)) / den
 *   accept only tmin <= t < tmax
 *   h0 = o[cs0] + t*d[cs0] ; h1 = o[cs1] + t*d[cs1]
 *   b0 = (e0*h0 + e1*h1) + e2 ; b1 = (e3*h0 + e4*h1) + e5 ; b2 = (1 - b0) - b1
 *   hit iff b0 >= 0 && b1 >= 0 && b2 >= 0.
 * Edge equations are positive inside (defect D7: the Go comment says
 * negative; the code in edge.go makes inside positive). */
static int tri_hit(const orc_tri *tr, const float *o, const float *d, float tmin, float tmax,
                   float *t_out) {
    float den = (tr->nx * d[0] + tr->ny * d[1]) + tr->nz * d[2];
    float on = (tr->nx * o[0] + tr->ny * o[1]) + tr->nz * o[2];
    float t = (tr->d - on) / den;
    if (!(t >= tmin && t < tmax)) return 0;
    float h0 = o[tr->cs0] + t * d[tr->cs0];
    float h1 = o[tr->cs1] + t * d[tr->cs1];
    float b0 = (tr->e[0] * h0 + tr->e[1] * h1) + tr->e[2];
    float b1 = (tr->e[3] * h0 + tr->e[4] * h1) + tr->e[5];
    float b2 = (1.0f - b0) - b1;
    if (b0 >= 0.0f && b1 >= 0.0f && b2 >= 0.0f) {
        *t_out = t;
        return 1;
    }
    return 0;
}

typedef struct {
    uint32_t node;
    float t0, t1;
} stk_t;

/* Conservative slack for split planes: a computed hit point lies within a
 * few float32 rounding errors of its triangle; the traversal treats every
 * split plane as a slab this thick so that no leaf holding such a triangle
 * is skipped.  2^-17 * (scene scale + |origin|) is several times the
 * rounding bound of the test above. */
static float ray_slack(const orc_scene *s, const float *o) {
    float om = fmaxf(fabsf(o[0]), fmaxf(fabsf(o[1]), fabsf(o[2])));
    return 7.62939453125e-06f * ((s->coord_scale + om) + 1.0f);
}

static int empty_leaf(const orc_scene *s, uint32_t node) {
    return (int)(s->children[node] & 3u) == KD_LEAF && s->split[node] == 0.0f;
}

/* Walks the tree; closest = 0 stops at the first accepted hit.  Results are
 * identical to testing every triangle (brute force): for closest hits the
 * minimum t wins and equal t goes to the lower triangle index. */
static int trace_kd(const orc_scene *s, const float *o, const float *d, float tmin, float tmax,
                    int32_t skip, int closest, int32_t *hit, float *thit, uint32_t *st) {
    uint32_t nodes = 0, tests = 0, leaves = 0;
    int32_t best = -1;
    float best_t = INFINITY;
    if (s->ntris == 0 || !(tmin <= tmax)) goto done;
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    float slack = ray_slack(s, o);
    float t0 = tmin, t1 = tmax;
    for (int a = 0; a < 3; a++) {
        float lo = (s->bmin[a] - slack) - o[a], hi = (s->bmax[a] + slack) - o[a];
        float ta = lo * inv[a], tb = hi * inv[a];
        float enter = signbit(d[a]) ? tb : ta, leave = signbit(d[a]) ? ta : tb;
        t0 = fmaxf(t0, enter);
        t1 = fminf(t1, leave);
    }
    if (!(t0 <= t1)) goto done;
    stk_t stack[STACK_MAX];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        for (;;) {
            nodes++;
            uint32_t ch = s->children[node];
            int type = (int)(ch & 3u);
            if (type == KD_LEAF) break;
            uint32_t left = ch >> 2;
            float sv = s->split[node];
            int neg = signbit(d[type]) != 0;
            uint32_t near = neg ? left + 1 : left, far = neg ? left : left + 1;
            float sd = neg ? -slack : slack;
            float tne = ((sv + sd) - o[type]) * inv[type];
            float tfe = ((sv - sd) - o[type]) * inv[type];
            int vn = !(tne < t0), vf = !(tfe > t1);
            if (s->skip_empty) { /* the library's kOptSkip walk: never enter an empty leaf */
                vn = vn && !empty_leaf(s, near);
                vf = vf && !empty_leaf(s, far);
            }
            if (vn && vf) {
                stack[sp].node = far;
                stack[sp].t0 = fmaxf(t0, tfe);
                stack[sp].t1 = t1;
                sp++;
                node = near;
                t1 = fminf(t1, tne);
            } else if (vn) {
                node = near;
                t1 = fminf(t1, tne);
            } else if (vf) {
                node = far;
                t0 = fmaxf(t0, tfe);
            } else {
                goto pop;
            }
        }
        leaves++;
        {
            uint32_t start = s->children[node] >> 2;
            int cnt = (int)s->split[node];
            for (int k = 0; k < cnt; k++) {
                int32_t ti = s->refs[start + k];
                const orc_tri *tr = &s->tris[ti];
                if (tr->id == skip) continue;
                tests++;
                float th;
                if (tri_hit(tr, o, d, tmin, tmax, &th)) {
                    if (!closest) {
                        best = ti;
                        best_t = th;
                        goto done;
                    }
                    if (th < best_t || (th == best_t && ti < best)) {
                        best = ti;
                        best_t = th;
                    }
                }
            }
        }
    pop:
        for (;;) {
            if (sp == 0) goto done;
            sp--;
            if (closest && stack[sp].t0 > best_t) continue;
            node = stack[sp].node;
            t0 = stack[sp].t0;
            t1 = stack[sp].t1;
            break;
        }
    }
done:
    *hit = best;
    *thit = best_t;
    if (st) {
        st[0] = nodes;
        st[1] = tests;
        st[2] = leaves;
    }
    return best >= 0;
}

static int trace_brute(const orc_scene *s, const float *o, const float *d, float tmin, float tmax,
                       int32_t skip, int closest, int32_t *hit, float *thit) {
    int32_t best = -1;
    float best_t = INFINITY;
    for (int64_t t = 0; t < s->ntris; t++) {
        if (s->tris[t].id == skip) continue;
        float th;
        if (tri_hit(&s->tris[t], o, d, tmin, tmax, &th)) {
            if (!closest) {
                best = (int32_t)t;
                best_t = th;
                break;
            }
            if (th < best_t) {
                best = (int32_t)t;
                best_t = th;
            }
        }
    }
    *hit = best;
    *thit = best_t;
    return best >= 0;
}

static int trace_one(const orc_scene *s, const float *o, const float *d, float tmin, float tmax,
                     int32_t skip, int closest, int brute, int32_t *hit, float *thit,
                     uint32_t *st) {
    if (brute) {
        if (st) st[0] = st[1] = st[2] = 0;
        return trace_brute(s, o, d, tmin, tmax, skip, closest, hit, thit);
    }
    return trace_kd(s, o, d, tmin, tmax, skip, closest, hit, thit, st);
}

/* TestLineDoesHitSky (raytracer/trace/testline.go:22-57,91-93), fixed:
 *   dir = stop - start ; len = sqrt((x*x + y*y) + z*z) ; dir = dir * (1/len)
 *   trace [0, len) skipping triangles whose id == skip_id
 *   occluded iff the closest hit has t < len and its id lacks TRACE_ID_SKY.
 * Returns 1 when occluded.  A zero-length line is never occluded. */
/* The library's wall test (its shadow lines' shortcut, same verdicts): the
 * face of the slack-padded scene box the line leaves through, and the
 * opaque triangles set for it (orc_scene_set_walls) tested first.  A hit
 * before any_limit -- the entry into the sky triangles' box padded by
 * 2*slack, before which no sky triangle can be hit -- occludes the line
 * whatever lies in front of it.  *tests counts the triangles tested. */
static int wall_occludes(const orc_scene *s, const float *a, const float *dir, float len,
                         int32_t skip, uint32_t *tests) {
    const float slack = ray_slack(s, a);
    int f = 0;
    float tex = INFINITY;
    for (int ax = 0; ax < 3; ax++) {
        const int neg = signbit(dir[ax]) != 0;
        const float bound = neg ? s->bmin[ax] - slack : s->bmax[ax] + slack;
        const float t = (bound - a[ax]) / dir[ax];
        if (t < tex) {
            tex = t;
            f = 2 * ax + (neg ? 0 : 1);
        }
    }
    if (!(tex < 2.0f * len)) return 0;
    float any_limit = INFINITY;
    if (s->has_sky) {
        float ts0 = -INFINITY, ts1 = INFINITY;
        for (int ax = 0; ax < 3; ax++) {
            const float ta = ((s->sky_min[ax] - 2.0f * slack) - a[ax]) / dir[ax];
            const float tb = ((s->sky_max[ax] + 2.0f * slack) - a[ax]) / dir[ax];
            const int neg = signbit(dir[ax]) != 0;
            ts0 = fmaxf(ts0, neg ? tb : ta);
            ts1 = fminf(ts1, neg ? ta : tb);
        }
        if (ts0 <= ts1 && ts0 < len) any_limit = ts0;
    }
    for (int i = 0; i < s->nwalls[f]; i++) {
        const orc_tri *tr = &s->tris[s->walls[f][i]];
        if (tr->id == skip) continue;
        (*tests)++;
        float th;
        if (tri_hit(tr, a, dir, 0.0f, len, &th) && th < any_limit) return 1;
    }
    return 0;
}

static int line_occluded(const orc_scene *s, const float *a, const float *b, int32_t skip,
                         int brute, int32_t *hit_out, float *t_out, uint32_t *st) {
    float dir[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    float len = sqrtf(dot3(dir, dir));
    float r = 1.0f / len;
    dir[0] = dir[0] * r;
    dir[1] = dir[1] * r;
    dir[2] = dir[2] * r;
    int32_t hit = -1;
    float th = INFINITY;
    if (st) st[0] = st[1] = st[2] = 0;
    if (!(len > 0.0f)) {
        if (hit_out) *hit_out = -1;
        if (t_out) *t_out = INFINITY;
        return 0;
    }
    uint32_t wall_tests = 0;
    if (s->use_walls && !hit_out && !t_out && !brute &&
        wall_occludes(s, a, dir, len, skip, &wall_tests)) {
        if (st) st[1] = wall_tests;
        return 1;
    }
    trace_one(s, a, dir, 0.0f, len, skip, 1, brute, &hit, &th, st);
    if (st) st[1] += wall_tests;
    if (hit_out) *hit_out = hit;
    if (t_out) *t_out = th;
    return hit >= 0 && th < len && (s->tris[hit].id & ORC_TRACE_ID_SKY) == 0;
}

/* ------------------------------------------------------------------ */
/* threading                                                           */
/* ------------------------------------------------------------------ */

typedef void (*range_fn)(void *ctx, int64_t begin, int64_t end, int worker);
typedef struct {
    range_fn fn;
    void *ctx;
    int64_t n, chunk;
    int64_t next;
    pthread_mutex_t mu;
    int worker;
} pool_t;

static void *pool_main(void *arg) {
    pool_t *p = (pool_t *)arg;
    pthread_mutex_lock(&p->mu);
    int w = p->worker++;
    pthread_mutex_unlock(&p->mu);
    for (;;) {
        pthread_mutex_lock(&p->mu);
        int64_t b = p->next;
        p->next += p->chunk;
        pthread_mutex_unlock(&p->mu);
        if (b >= p->n) break;
        int64_t e = b + p->chunk < p->n ? b + p->chunk : p->n;
        p->fn(p->ctx, b, e, w);
    }
    return NULL;
}

static void parallel_for(int64_t n, int threads, int64_t chunk, range_fn fn, void *ctx) {
    if (threads <= 1 || n <= chunk) {
        fn(ctx, 0, n, 0);
        return;
    }
    pool_t p;
    p.fn = fn;
    p.ctx = ctx;
    p.n = n;
    p.chunk = chunk;
    p.next = 0;
    p.worker = 0;
    pthread_mutex_init(&p.mu, NULL);
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, pool_main, &p);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&p.mu);
}

/* ------------------------------------------------------------------ */
/* batched trace entry points                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    const orc_scene *s;
    const float *o, *d, *tmin, *tmax, *b;
    int32_t skip;
    int brute, closest;
    int32_t *hit;
    float *t;
    uint8_t *any;
    float *frac;
    uint32_t *mask, *stats;
} trace_job;

static void closest_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    trace_job *j = (trace_job *)ctx;
    for (int64_t i = b; i < e; i++) {
        int32_t h;
        float t;
        trace_one(j->s, j->o + 3 * i, j->d + 3 * i, j->tmin[i], j->tmax[i], j->skip, 1, j->brute,
                  &h, &t, j->stats ? j->stats + 3 * i : NULL);
        j->hit[i] = h;
        j->t[i] = t;
    }
}

void orc_trace_closest(const orc_scene *s, const float *orig, const float *dir, const float *tmin,
                       const float *tmax, int64_t n, int32_t skip_id, int brute, int threads,
                       int32_t *out_hit, float *out_t, uint32_t *stats) {
    trace_job j = {0};
    j.s = s;
    j.o = orig;
    j.d = dir;
    j.tmin = tmin;
    j.tmax = tmax;
    j.skip = skip_id;
    j.brute = brute;
    j.hit = out_hit;
    j.t = out_t;
    j.stats = stats;
    parallel_for(n, threads, 1024, closest_range, &j);
}

static void any_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    trace_job *j = (trace_job *)ctx;
    for (int64_t i = b; i < e; i++) {
        int32_t h;
        float t;
        j->any[i] = (uint8_t)trace_one(j->s, j->o + 3 * i, j->d + 3 * i, j->tmin[i], j->tmax[i],
                                       j->skip, 0, j->brute, &h, &t,
                                       j->stats ? j->stats + 3 * i : NULL);
    }
}

void orc_trace_any(const orc_scene *s, const float *orig, const float *dir, const float *tmin,
                   const float *tmax, int64_t n, int32_t skip_id, int brute, int threads,
                   uint8_t *out_hit, uint32_t *stats) {
    trace_job j = {0};
    j.s = s;
    j.o = orig;
    j.d = dir;
    j.tmin = tmin;
    j.tmax = tmax;
    j.skip = skip_id;
    j.brute = brute;
    j.any = out_hit;
    j.stats = stats;
    parallel_for(n, threads, 1024, any_range, &j);
}

static void lines_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    trace_job *j = (trace_job *)ctx;
    for (int64_t i = b; i < e; i++)
        j->frac[i] = line_occluded(j->s, j->o + 3 * i, j->b + 3 * i, j->skip, j->brute, NULL,
                                   NULL, NULL)
                         ? 0.0f
                         : 1.0f;
}

void orc_test_lines(const orc_scene *s, const float *start, const float *stop, int64_t n,
                    int32_t skip_id, int brute, int threads, float *out_frac) {
    trace_job j = {0};
    j.s = s;
    j.o = start;
    j.b = stop;
    j.skip = skip_id;
    j.brute = brute;
    j.frac = out_frac;
    parallel_for(n, threads, 1024, lines_range, &j);
}

/* ------------------------------------------------------------------ */
/* transparent shadows (project semantics; see the header)             */
/* ------------------------------------------------------------------ */

typedef struct {
    float t;
    int32_t idx;
} tri_hit_t;

static int cmp_hit(const void *a, const void *b) {
    const tri_hit_t *x = (const tri_hit_t *)a, *y = (const tri_hit_t *)b;
    if (x->t < y->t) return -1;
    if (x->t > y->t) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

/* Every accepted hit of the ray (brute force over all triangles, tri_hit on
 * [tmin, tmax), ids equal to skip ignored), sorted by (t, triangle index);
 * then taken in that order: an opaque hit is recorded and ends the walk; a
 * transparent hit adds its coverage, c = min(c + cover, 1), and when c
 * reaches 1 that triangle is recorded and the walk ends. */
static void coverage_trace(const orc_scene *s, const float *cover, const float *o, const float *d,
                           float tmin, float tmax, int32_t skip, tri_hit_t *buf, int32_t *hit,
                           float *thit, float *cov) {
    int64_t nh = 0;
    for (int64_t i = 0; i < s->ntris; i++) {
        const orc_tri *tr = &s->tris[i];
        if (tr->id == skip) continue;
        float t;
        if (tri_hit(tr, o, d, tmin, tmax, &t)) {
            buf[nh].t = t;
            buf[nh].idx = (int32_t)i;
            nh++;
        }
    }
    qsort(buf, (size_t)nh, sizeof(tri_hit_t), cmp_hit);
    float c = 0.0f;
    *hit = -1;
    *thit = INFINITY;
    for (int64_t k = 0; k < nh; k++) {
        const int32_t i = buf[k].idx;
        if (!(s->flags && (s->flags[i] & ORC_TRI_TRANSPARENT))) {
            *hit = i;
            *thit = buf[k].t;
            break;
        }
        c = fminf(c + cover[i], 1.0f);
        if (c >= 1.0f) {
            *hit = i;
            *thit = buf[k].t;
            break;
        }
    }
    *cov = c;
}

typedef struct {
    const orc_scene *s;
    const float *cover, *a, *b, *tmin, *tmax;
    int32_t skip;
    int lines;
    int32_t *hit;
    float *t, *cov, *frac;
} cov_job;

static void cov_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    const cov_job *j = (const cov_job *)ctx;
    tri_hit_t *buf = malloc(sizeof(tri_hit_t) * (size_t)(j->s->ntris ? j->s->ntris : 1));
    for (int64_t i = b; i < e; i++) {
        int32_t h;
        float th, c;
        if (!j->lines) {
            coverage_trace(j->s, j->cover, j->a + 3 * i, j->b + 3 * i, j->tmin[i], j->tmax[i],
                           j->skip, buf, &h, &th, &c);
            j->hit[i] = h;
            j->t[i] = th;
            j->cov[i] = c;
            continue;
        }
        /* TestLineDoesHitSky with texture shadows (testline.go:22-33,42-55,91-93) */
        const float *a = j->a + 3 * i, *bb = j->b + 3 * i;
        float dir[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
        float len = sqrtf(dot3(dir, dir));
        if (!(len > 0.0f)) {
            j->frac[i] = 1.0f;
            continue;
        }
        float r = 1.0f / len;
        dir[0] = dir[0] * r;
        dir[1] = dir[1] * r;
        dir[2] = dir[2] * r;
        coverage_trace(j->s, j->cover, a, dir, 0.0f, len, j->skip, buf, &h, &th, &c);
        float occ = (h >= 0 && th < len && (j->s->tris[h].id & ORC_TRACE_ID_SKY) == 0) ? 1.0f : 0.0f;
        occ = fmaxf(occ, c);
        occ = fminf(fmaxf(occ, 0.0f), 1.0f);
        j->frac[i] = 1.0f - occ;
    }
    free(buf);
}

void orc_trace_coverage(const orc_scene *s, const float *cover, const float *orig, const float *dir,
                        const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                        int threads, int32_t *out_hit, float *out_t, float *out_coverage) {
    cov_job j = {s, cover, orig, dir, tmin, tmax, skip_id, 0, out_hit, out_t, out_coverage, NULL};
    parallel_for(n, threads, 64, cov_range, &j);
}

void orc_test_lines_coverage(const orc_scene *s, const float *cover, const float *start,
                             const float *stop, int64_t n, int32_t skip_id, int threads,
                             float *out_frac) {
    cov_job j = {s, cover, start, stop, NULL, NULL, skip_id, 1, NULL, NULL, NULL, out_frac};
    parallel_for(n, threads, 64, cov_range, &j);
}

static void mask_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    trace_job *j = (trace_job *)ctx;
    /* ranges are multiples of 32 except the last, so words are private */
    for (int64_t i = b; i < e; i++) {
        int32_t h;
        float t;
        int occ = line_occluded(j->s, j->o + 3 * i, j->b + 3 * i, j->skip, 0, &h, &t,
                                j->stats ? j->stats + 3 * i : NULL);
        if (occ) j->mask[i >> 5] |= 1u << (i & 31);
        if (j->hit) {
            j->hit[i] = h;
            j->t[i] = t;
        }
    }
}

void orc_occlusion_mask(const orc_scene *s, const float *start, const float *stop, int64_t n,
                        int32_t skip_id, int threads, uint32_t *out_mask, int32_t *out_hit,
                        float *out_t, uint32_t *stats) {
    trace_job j = {0};
    j.s = s;
    j.o = start;
    j.b = stop;
    j.skip = skip_id;
    j.mask = out_mask;
    j.hit = out_hit;
    j.t = out_t;
    j.stats = stats;
    memset(out_mask, 0, sizeof(uint32_t) * (size_t)((n + 31) / 32));
    parallel_for(n, threads, 1024, mask_range, &j);
}

/* ------------------------------------------------------------------ */
/* lights (rad/lightmap/lights.go, vmath/quadratic/solver.go)          */
/* ------------------------------------------------------------------ */

/* SolveInverseQuadratic (solver.go:48-63), float32, as written. */
int orc_solve_inverse_quadratic(float x1, float y1, float x2, float y2, float x3, float y3,
                                float *a, float *b, float *c) {
    float det = ((x1 - x2) * (x1 - x3)) * (x2 - x3);
    if (det == 0.0f) return 0;
    *a = ((x3 * (-y1 + y2) + x2 * (y1 - y3)) + x1 * (-y2 + y3)) / det;
    *b = (((x3 * x3) * (y1 - y2) + (x1 * x1) * (y2 - y3)) + (x2 * x2) * (-y1 + y3)) / det;
    *c = ((((x1 * x3) * (-x1 + x3)) * y2 + (x2 * x2) * ((x3 * y1) - (x1 * y3))) +
          x2 * (-((x3 * x3) * y1) + (x1 * x1) * y3)) /
         det;
    return 1;
}

/* FLerp (vmath/quadratic/lerp.go:14-16) */
static double flerp(float f1, float f2, float i1, float i2, float x) {
    return (double)(f1 + ((f2 - f1) * (x - i1)) / (i2 - i1));
}

/* SolveInverseQuadraticMonotonic (solver.go:4-45).  vSwap swaps local
 * pointers in the Go (defect D16); the fixed form swaps the values. */
int orc_solve_inverse_quadratic_monotonic(float x1, float y1, float x2, float y2, float x3,
                                          float y3, float *a, float *b, float *c) {
    float t;
#define SWAPF(p, q) (t = (p), (p) = (q), (q) = t)
    if (x1 > x2) {
        SWAPF(x1, x2);
        SWAPF(y1, y2);
    }
    if (x2 > x3) {
        SWAPF(x2, x3);
        SWAPF(y2, y3);
    }
    if (x1 > x2) {
        SWAPF(x1, x2);
        SWAPF(y1, y2);
    }
#undef SWAPF
    for (double blend = 0.0; blend <= 1.0; blend += 0.05) {
        double ty2 = (double)(1.0 - blend) * (double)y2 + blend * flerp(y1, y3, x1, x3, x2);
        if (!orc_solve_inverse_quadratic(x1, y1, x2, (float)ty2, x3, y3, a, b, c)) return 0;
        float deriv = 2.0f * (*a) + (*b);
        if (y1 < y2 && y2 < y3) {
            if (deriv >= 0.0f) return 1;
        } else if (y1 > y2 && y2 > y3) {
            if (deriv <= 0.0f) return 1;
        } else {
            return 1;
        }
    }
    return 1;
}

/* SetLightFalloffParams (lights.go:259-341) */
void orc_set_light_falloff(const orc_light_keys *k, orc_light *l) {
    const float eq_eps = 0.001f; /* vmath/constants.go:9 EQUAL_EPSILON */
    float d50 = k->fifty_percent_distance;
    l->start_fade = 0.0f;
    l->end_fade = -1.0f;
    l->cap_distance = 1.0e22f;
    if (d50 != 0.0f) {
        float d0 = k->zero_percent_distance;
        if (d0 < d50) d0 = 2.0f * d50;
        float a = 0.0f, b = 1.0f, c = 0.0f;
        orc_solve_inverse_quadratic_monotonic(0.0f, 1.0f, d50, 2.0f, d0, 256.0f, &a, &b, &c);
        float v50 = c + d50 * (b + d50 * a);
        float scale = 2.0f / v50;
        a *= scale;
        b *= scale;
        c *= scale;
        l->quadratic_attn = a;
        l->linear_attn = b;
        l->constant_attn = c;
        if (k->hard_falloff != 0) {
            l->end_fade = d0;
            l->start_fade = 0.75f * d0 + 0.25f * d50;
        } else if (fabs((double)a) > 0.0) {
            float fmax = b / (-2.0f * a);
            if (fmax > 0.0f) {
                l->cap_distance = fmax;
                l->start_fade = fmax;
                l->end_fade = 10.0f * fmax;
            }
        }
    } else {
        l->constant_attn = k->constant_attn;
        l->linear_attn = k->linear_attn;
        l->quadratic_attn = k->quadratic_attn;
        l->radius = k->distance;
        if (l->constant_attn < eq_eps) l->constant_attn = 0.0f;
        if (l->linear_attn < eq_eps) l->linear_attn = 0.0f;
        if (l->quadratic_attn < eq_eps) l->quadratic_attn = 0.0f;
        if (l->constant_attn < eq_eps && l->linear_attn < eq_eps && l->quadratic_attn < eq_eps)
            l->constant_attn = 1.0f;
        float ratio = (l->constant_attn + 100.0f * l->linear_attn) + 10000.0f * l->quadratic_attn;
        if (ratio > 0.0f)
            for (int i = 0; i < 3; i++) l->intensity[i] = l->intensity[i] * ratio;
    }
}

/* ParseLightSpot (lights.go:210-257) from the cone keys; origin, intensity
 * and normal are set by the caller beforehand. */
void orc_parse_light_spot(const orc_light_keys *k, orc_light *l) {
    const float pi = (float)3.14159265358979323846;
    l->type = 2;
    l->stopdot = k->inner_cone;
    if (l->stopdot == 0.0f) l->stopdot = 10.0f;
    l->stopdot2 = k->cone;
    if (l->stopdot2 == 0.0f) l->stopdot2 = l->stopdot;
    if (l->stopdot2 < l->stopdot) l->stopdot2 = l->stopdot;
    if (l->stopdot == 180.0f && l->stopdot2 == 180.0f) {
        l->stopdot = l->stopdot2 = 0.0f;
        l->type = 1;
        l->exponent = 0.0f;
    } else {
        if (l->stopdot > 90.0f) l->stopdot = 90.0f;
        if (l->stopdot2 > 90.0f) l->stopdot2 = 90.0f;
        l->stopdot2 = (float)cos((double)((l->stopdot2 / 180.0f) * pi));
        l->stopdot = (float)cos((double)((l->stopdot / 180.0f) * pi));
        l->exponent = k->exponent;
    }
    orc_set_light_falloff(k, l);
}

/* ------------------------------------------------------------------ */
/* direct light gather (absent in the reference; project semantics)    */
/* ------------------------------------------------------------------ */

/* Visibility as TestLineDoesHitSky with staticPropToSkip = -1, i.e. the skip
 * id TRACE_ID_STATICPROP | -1 == -1, which no triangle carries. */
static int visible(const orc_scene *s, const float *p, const float *q, uint64_t *acc) {
    uint32_t st[3];
    int occ = line_occluded(s, p, q, -1, 0, NULL, NULL, st);
    acc[0]++;
    acc[1] += st[0];
    acc[2] += st[1];
    acc[3] += st[2];
    return !occ;
}

/* Irradiance at p (normal n), summed over the lights in table order:
 *  point/spot: delta = origin - p ; dist2 = (dx*dx + dy*dy) + dz*dz
 *    skip if radius > 0 and dist2 > radius*radius, or dist2 == 0
 *    dist = sqrt(dist2) ; L = delta * (1/dist) ; cosr = (n.L)
 *    skip unless cosr > 0
 *    dc, dc2 = dist, dist2 (or cap, cap*cap beyond cap_distance)
 *    denom = (c + b*dc) + a*dc2 ; skip unless denom > 0 ; f = 1/denom
 *    if end_fade > start_fade and dist > start_fade:
 *        skip if dist >= end_fade, else s = (dist-start)/(end-start),
 *        f = f * (((1-s)*(1-s)) * (1 + 2*s))
 *    spot: dot2 = -(L.normal) ; skip unless dot2 > stopdot2
 *        if dot2 < stopdot: f = f * ((dot2 - stopdot2) / (stopdot - stopdot2))
 *        exponent 1: f = f * dot2 ; other nonzero exponent: f = f * powf(dot2, e)
 *    visible(p, origin) ? rgb += I * (f * cosr)
 *  skylight: dir = -normal ; cosr = n.dir ; skip unless > 0 ;
 *    visible(p, p + dir*MAX_TRACE_LENGTH) ? rgb += I * cosr
 *  skyambient: over the 162 directions a_j with w = n.a_j > 0:
 *    sw += w ; visible(p, p + a_j*MAX_TRACE_LENGTH) ? sv += w
 *    rgb += I * (sv / sw) when sw > 0 */
static void gather_point(const orc_scene *s, const orc_light *lights, int nl, const float *p,
                         const float *n, float *rgb, uint64_t *rays) {
    /* rays[0..3]: shadow lines, kd nodes visited, triangles tested, leaves */
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (int li = 0; li < nl; li++) {
        const orc_light *l = &lights[li];
        if (l->type == 1 || l->type == 2) {
            float dl[3] = {l->origin[0] - p[0], l->origin[1] - p[1], l->origin[2] - p[2]};
            float dist2 = dot3(dl, dl);
            if (l->radius > 0.0f && dist2 > l->radius * l->radius) continue;
            if (dist2 == 0.0f) continue;
            float dist = sqrtf(dist2);
            float inv = 1.0f / dist;
            float L[3] = {dl[0] * inv, dl[1] * inv, dl[2] * inv};
            float cosr = dot3(n, L);
            if (!(cosr > 0.0f)) continue;
            float dc = dist, dc2 = dist2;
            if (dist > l->cap_distance) {
                dc = l->cap_distance;
                dc2 = l->cap_distance * l->cap_distance;
            }
            float denom = (l->constant_attn + l->linear_attn * dc) + l->quadratic_attn * dc2;
            if (!(denom > 0.0f)) continue;
            float f = 1.0f / denom;
            if (l->end_fade > l->start_fade && dist > l->start_fade) {
                if (dist >= l->end_fade) continue;
                float sfr = (dist - l->start_fade) / (l->end_fade - l->start_fade);
                f = f * (((1.0f - sfr) * (1.0f - sfr)) * (1.0f + 2.0f * sfr));
            }
            if (l->type == 2) {
                float dot2 = -dot3(L, l->normal);
                if (!(dot2 > l->stopdot2)) continue;
                if (dot2 < l->stopdot) f = f * ((dot2 - l->stopdot2) / (l->stopdot - l->stopdot2));
                if (l->exponent == 1.0f) f = f * dot2;
                else if (l->exponent != 0.0f) f = f * powf(dot2, l->exponent);
            }
            if (!visible(s, p, l->origin, rays)) continue;
            float sc = f * cosr;
            acc[0] = acc[0] + l->intensity[0] * sc;
            acc[1] = acc[1] + l->intensity[1] * sc;
            acc[2] = acc[2] + l->intensity[2] * sc;
        } else if (l->type == 3) {
            float dir[3] = {-l->normal[0], -l->normal[1], -l->normal[2]};
            float cosr = dot3(n, dir);
            if (!(cosr > 0.0f)) continue;
            float q[3] = {p[0] + dir[0] * MAX_TRACE_LENGTH, p[1] + dir[1] * MAX_TRACE_LENGTH,
                          p[2] + dir[2] * MAX_TRACE_LENGTH};
            if (!visible(s, p, q, rays)) continue;
            acc[0] = acc[0] + l->intensity[0] * cosr;
            acc[1] = acc[1] + l->intensity[1] * cosr;
            acc[2] = acc[2] + l->intensity[2] * cosr;
        } else if (l->type == 5) {
            float sw = 0.0f, sv = 0.0f;
            for (int j = 0; j < VRG_NUM_ANORMS; j++) {
                const float *a = k_anorms + 3 * j;
                float w = dot3(n, a);
                if (!(w > 0.0f)) continue;
                sw = sw + w;
                float q[3] = {p[0] + a[0] * MAX_TRACE_LENGTH, p[1] + a[1] * MAX_TRACE_LENGTH,
                              p[2] + a[2] * MAX_TRACE_LENGTH};
                if (visible(s, p, q, rays)) sv = sv + w;
            }
            if (sw > 0.0f) {
                float fr = sv / sw;
                acc[0] = acc[0] + l->intensity[0] * fr;
                acc[1] = acc[1] + l->intensity[1] * fr;
                acc[2] = acc[2] + l->intensity[2] * fr;
            }
        }
    }
    rgb[0] = acc[0];
    rgb[1] = acc[1];
    rgb[2] = acc[2];
}

typedef struct {
    const orc_scene *s;
    const orc_light *lights;
    int nl;
    const float *pts, *nrm;
    float *rgb;
    uint64_t *rays; /* per worker, 4 counters each */
    /* luxel mode */
    const float *corner, *u, *v;
    const int32_t *nu, *nv;
    const int64_t *off;
    int32_t fbegin;
    int ss;
    uint64_t seed;
} gather_job;

static void gather_pts_range(void *ctx, int64_t b, int64_t e, int w) {
    gather_job *j = (gather_job *)ctx;
    uint64_t r[4] = {0, 0, 0, 0};
    for (int64_t i = b; i < e; i++)
        gather_point(j->s, j->lights, j->nl, j->pts + 3 * i, j->nrm + 3 * i, j->rgb + 3 * i, r);
    for (int k = 0; k < 4; k++) j->rays[4 * w + k] += r[k];
}

void orc_gather_points(const orc_scene *s, const orc_light *lights, int nlights, const float *pts,
                       const float *nrm, int64_t n, int threads, float *out_rgb,
                       uint64_t *rays_out) {
    gather_job j = {0};
    uint64_t rays[4 * 256] = {0};
    if (threads > 256) threads = 256;
    j.s = s;
    j.lights = lights;
    j.nl = nlights;
    j.pts = pts;
    j.nrm = nrm;
    j.rgb = out_rgb;
    j.rays = rays;
    parallel_for(n, threads, 64, gather_pts_range, &j);
    uint64_t tot = 0;
    for (int i = 0; i < 256; i++) tot += rays[4 * i];
    if (rays_out) *rays_out = tot;
}

/* SplitMix64 (Steele, Lea & Flood 2014): output for state seed + (i+1)*gamma */
static uint64_t splitmix(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Luxel supersample position (project semantics).  Face f has nu x nv luxels
 * spanning corner + U*su + V*sv, su,sv in [0,1].  Sample k of luxel
 * (iu,iv), global sample index g = (luxel_offset[f] + iv*nu + iu)*S + k:
 *   h = splitmix(seed, g) ; r1 = (h >> 40) * 2^-24 ; r2 = ((h >> 16) & 0xffffff) * 2^-24
 *   S == 4: su = (iu + ((k & 1) + r1) * 0.5) * (1/nu) ; sv = (iv + ((k >> 1) + r2) * 0.5) * (1/nv)
 *   S == 1: su = (iu + 0.5) * (1/nu) ; sv = (iv + 0.5) * (1/nv)
 *   p = ((corner + U*su) + V*sv) + N*0.125 per component. */
static void luxel_sample(const float *c, const float *U, const float *V, const float *N, int nu,
                         int nv, int64_t lux_global, int iu, int iv, int k, int ss, uint64_t seed,
                         float *p) {
    float su, sv;
    float inu = 1.0f / (float)nu, inv = 1.0f / (float)nv;
    if (ss == 4) {
        uint64_t h = splitmix(seed, (uint64_t)(lux_global * 4 + k));
        float r1 = (float)(h >> 40) * 5.9604644775390625e-08f;
        float r2 = (float)((h >> 16) & 0xffffffu) * 5.9604644775390625e-08f;
        su = ((float)iu + ((float)(k & 1) + r1) * 0.5f) * inu;
        sv = ((float)iv + ((float)(k >> 1) + r2) * 0.5f) * inv;
    } else {
        su = ((float)iu + 0.5f) * inu;
        sv = ((float)iv + 0.5f) * inv;
    }
    for (int a = 0; a < 3; a++) p[a] = ((c[a] + U[a] * su) + V[a] * sv) + N[a] * SAMPLE_OFFSET;
}

void orc_luxel_samples(const float *corner, const float *u, const float *v, const float *nrm,
                       const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                       int32_t f, int ss, uint64_t seed, float *out_pts) {
    int64_t idx = 0;
    for (int iv = 0; iv < nv[f]; iv++)
        for (int iu = 0; iu < nu[f]; iu++)
            for (int k = 0; k < ss; k++) {
                luxel_sample(corner + 3 * f, u + 3 * f, v + 3 * f, nrm + 3 * f, nu[f], nv[f],
                             luxel_offset[f] + (int64_t)iv * nu[f] + iu, iu, iv, k, ss, seed,
                             out_pts + 3 * idx);
                idx++;
            }
}

static void gather_lux_range(void *ctx, int64_t b, int64_t e, int w) {
    gather_job *j = (gather_job *)ctx;
    uint64_t r[4] = {0, 0, 0, 0};
    for (int64_t fi = b; fi < e; fi++) {
        int32_t f = j->fbegin + (int32_t)fi;
        const float *c = j->corner + 3 * f, *U = j->u + 3 * f, *V = j->v + 3 * f,
                    *N = j->nrm + 3 * f;
        for (int iv = 0; iv < j->nv[f]; iv++)
            for (int iu = 0; iu < j->nu[f]; iu++) {
                int64_t lux = j->off[f] + (int64_t)iv * j->nu[f] + iu;
                float sum[3] = {0.0f, 0.0f, 0.0f};
                for (int k = 0; k < j->ss; k++) {
                    float p[3], rgb[3];
                    luxel_sample(c, U, V, N, j->nu[f], j->nv[f], lux, iu, iv, k, j->ss, j->seed,
                                 p);
                    gather_point(j->s, j->lights, j->nl, p, N, rgb, r);
                    sum[0] = sum[0] + rgb[0];
                    sum[1] = sum[1] + rgb[1];
                    sum[2] = sum[2] + rgb[2];
                }
                float sc = 1.0f / (float)j->ss;
                float *out = j->rgb + 3 * (lux - j->off[j->fbegin]);
                out[0] = sum[0] * sc;
                out[1] = sum[1] * sc;
                out[2] = sum[2] * sc;
            }
    }
    for (int k = 0; k < 4; k++) j->rays[4 * w + k] += r[k];
}

/* Writes RGB for the luxels of faces [face_begin, face_end), indexed from
 * the first luxel of face_begin. */
void orc_gather_luxels(const orc_scene *s, const orc_light *lights, int nlights,
                       const float *corner, const float *u, const float *v, const float *nrm,
                       const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                       int32_t face_begin, int32_t face_end, int supersamples, uint64_t seed,
                       int threads, float *out_rgb, uint64_t *rays_out, uint64_t *stats_out) {
    gather_job j = {0};
    uint64_t rays[4 * 256] = {0};
    if (threads > 256) threads = 256;
    j.s = s;
    j.lights = lights;
    j.nl = nlights;
    j.corner = corner;
    j.u = u;
    j.v = v;
    j.nrm = nrm;
    j.nu = nu;
    j.nv = nv;
    j.off = luxel_offset;
    j.fbegin = face_begin;
    j.ss = supersamples;
    j.seed = seed;
    j.rgb = out_rgb;
    j.rays = rays;
    parallel_for(face_end - face_begin, threads, 1, gather_lux_range, &j);
    /* stats_out (optional, 4 counters): shadow lines, kd nodes visited,
     * triangles tested, leaves visited */
    uint64_t tot[4] = {0, 0, 0, 0};
    for (int i = 0; i < 256; i++)
        for (int k = 0; k < 4; k++) tot[k] += rays[4 * i + k];
    if (rays_out) {
        rays_out[0] = tot[0];
        if (stats_out) memcpy(stats_out, tot, sizeof tot);
    }
}

/* ------------------------------------------------------------------ */
/* patches (rad/patches/subdivide.go:166-411, face.go:30-197)          */
/* ------------------------------------------------------------------ */

typedef struct {
    float mins[3], maxs[3], fmins[3], fmaxs[3], center[3];
    float area, chop, luxscale;
    int32_t face, parent, child1, child2, axis;
    float dist;
    int nax; /* normal axis of the face */
} opatch;

typedef struct {
    opatch *p;
    int64_t n, cap;
    float min_chop;
} plist;

static int64_t padd(plist *L, const opatch *src) {
    if (L->n == L->cap) {
        L->cap = L->cap ? 2 * L->cap : 1024;
        L->p = realloc(L->p, sizeof(opatch) * (size_t)L->cap);
    }
    L->p[L->n] = *src;
    return L->n++;
}

/* Area of an axis-aligned rectangle: product of the two extents off the
 * face's normal axis. */
static float rect_area(const float *mn, const float *mx, int nax) {
    int a = (nax + 1) % 3, b = (nax + 2) % 3;
    return (mx[a] - mn[a]) * (mx[b] - mn[b]);
}

/* SubdividePatch for rectangles: split the widest axis (scaled by LuxScale)
 * at its midpoint while any axis spans >= chop and >= minChop luxels; the
 * "make more square" and edge-chop rules of subdivide.go:204-212,398-408
 * apply.  ClipWindingEpsilon's front side (coordinate > dist) becomes child1. */
static void subdivide(plist *L, int64_t ip) {
    opatch *p = &L->p[ip];
    float total[3];
    for (int i = 0; i < 3; i++) total[i] = (p->maxs[i] - p->mins[i]) * p->luxscale;
    float widest = -1.0f;
    int wa = -1, should = 0;
    for (int i = 0; i < 3; i++) {
        if (total[i] > widest) {
            wa = i;
            widest = total[i];
        }
        if (total[i] >= p->chop && total[i] >= L->min_chop) should = 1;
    }
    if (!should && wa != -1) {
        if (total[wa] > total[(wa + 1) % 3] * 2.0f && total[wa] > total[(wa + 2) % 3] * 2.0f) {
            if (p->chop > L->min_chop) {
                should = 1;
                p->chop = fmaxf(L->min_chop, p->chop / 2.0f);
            }
        }
    }
    if (!should) return;
    float dist = (p->mins[wa] + p->maxs[wa]) * 0.5f;
    opatch c1 = *p, c2 = *p;
    c1.mins[wa] = dist;
    c2.maxs[wa] = dist;
    c1.area = rect_area(c1.mins, c1.maxs, p->nax);
    c2.area = rect_area(c2.mins, c2.maxs, p->nax);
    if (c1.area == 0.0f || c2.area == 0.0f) return;
    opatch *kids[2] = {&c1, &c2};
    for (int k = 0; k < 2; k++) {
        opatch *c = kids[k];
        c->parent = (int32_t)ip;
        c->child1 = c->child2 = -1;
        c->axis = -1;
        c->dist = 0.0f;
        for (int i = 0; i < 3; i++) c->center[i] = (c->mins[i] + c->maxs[i]) * 0.5f;
        float t[3];
        for (int i = 0; i < 3; i++) t[i] = (c->maxs[i] - c->mins[i]) * c->luxscale;
        if (c->chop > L->min_chop && t[0] < c->chop && t[1] < c->chop && t[2] < c->chop) {
            for (int i = 0; i < 3; i++) {
                if ((c->fmaxs[i] == c->maxs[i] || c->fmins[i] == c->mins[i]) && t[i] > L->min_chop) {
                    c->chop = fmaxf(L->min_chop, c->chop / 2.0f);
                    break;
                }
            }
        }
    }
    int64_t i1 = padd(L, &c1);
    int64_t i2 = padd(L, &c2);
    p = &L->p[ip];
    p->child1 = (int32_t)i1;
    p->child2 = (int32_t)i2;
    p->axis = wa;
    p->dist = dist;
    subdivide(L, i1);
    subdivide(L, i2);
}

int64_t orc_make_patches(const float *corner, const float *u, const float *v, const float *nrm,
                         const float *luxscale, int32_t nfaces, float max_chop, float min_chop,
                         float *mins, float *maxs, float *center, float *area, int32_t *face,
                         int32_t *parent, int32_t *child1, int32_t *child2, int32_t *split_axis,
                         float *split_dist, int32_t *leaf_index) {
    plist L = {0};
    L.min_chop = min_chop;
    for (int32_t f = 0; f < nfaces; f++) {
        opatch p;
        memset(&p, 0, sizeof p);
        const float *c = corner + 3 * f, *U = u + 3 * f, *V = v + 3 * f, *N = nrm + 3 * f;
        int nax = 0;
        for (int i = 1; i < 3; i++)
            if (fabsf(N[i]) > fabsf(N[nax])) nax = i;
        for (int i = 0; i < 3; i++) {
            float pts[4] = {c[i], c[i] + U[i], c[i] + V[i], (c[i] + U[i]) + V[i]};
            p.mins[i] = p.maxs[i] = pts[0];
            for (int k = 1; k < 4; k++) {
                if (pts[k] < p.mins[i]) p.mins[i] = pts[k];
                if (pts[k] > p.maxs[i]) p.maxs[i] = pts[k];
            }
            p.fmins[i] = p.mins[i];
            p.fmaxs[i] = p.maxs[i];
            p.center[i] = (p.mins[i] + p.maxs[i]) * 0.5f;
        }
        p.nax = nax;
        p.area = rect_area(p.mins, p.maxs, nax);
        p.chop = max_chop;
        p.luxscale = luxscale[f];
        p.face = f;
        p.parent = p.child1 = p.child2 = -1;
        p.axis = -1;
        if (p.area <= 0.0f) continue;
        padd(&L, &p);
    }
    int64_t roots = L.n;
    for (int64_t i = 0; i < roots; i++) subdivide(&L, i);
    int32_t leaf = 0;
    for (int64_t i = 0; i < L.n; i++) {
        opatch *p = &L.p[i];
        if (mins) memcpy(mins + 3 * i, p->mins, 12);
        if (maxs) memcpy(maxs + 3 * i, p->maxs, 12);
        if (center) memcpy(center + 3 * i, p->center, 12);
        if (area) area[i] = p->area;
        if (face) face[i] = p->face;
        if (parent) parent[i] = p->parent;
        if (child1) child1[i] = p->child1;
        if (child2) child2[i] = p->child2;
        if (split_axis) split_axis[i] = p->axis;
        if (split_dist) split_dist[i] = p->dist;
        if (leaf_index) leaf_index[i] = p->child1 < 0 ? leaf++ : -1;
    }
    int64_t n = L.n;
    free(L.p);
    return n;
}

/* ------------------------------------------------------------------ */
/* transfers (absent in the reference; project semantics)             */
/* ------------------------------------------------------------------ */

/* Row i (leaf patch with center c, face normal N, face edge U):
 *   q = c + N*0.125 ; T1 = U * (1/sqrt(U.U)) ; T2 = N x T1
 *   ray k: d = ((lx*T1 + ly*T2) + lz*N) per component, closest hit on
 *   [0, MAX_TRACE_LENGTH) skipping nothing.
 *   A hit triangle h with tri_face[h] = g >= 0 lands on face g; the hit
 *   point x = q + t*d descends g's patch tree (coordinate >= dist goes to
 *   child1) to a leaf patch j.  Row i lists each j with its hit count,
 *   sorted by j; the transfer weight is count / K. */
typedef struct {
    const orc_scene *s;
    const int32_t *tri_face, *child1, *child2, *split_axis, *leaf_index, *face_root, *pface;
    const float *center, *split_dist, *fnormal, *fu, *dirs;
    int32_t k;
    const int64_t *leaf_patch; /* dense leaf -> patch index */
    const int64_t *row_list;   /* rows to build (NULL: 0, 1, 2, ...) */
    int32_t *cnt_rows;         /* per built row: list of targets (k entries) */
    int32_t *nnz;
} xfer_job;

static int cmp_i32(const void *a, const void *b) {
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static void xfer_range(void *ctx, int64_t b, int64_t e, int w) {
    (void)w;
    xfer_job *j = (xfer_job *)ctx;
    for (int64_t slot = b; slot < e; slot++) {
        const int64_t row = j->row_list ? j->row_list[slot] : slot;
        int64_t pi = j->leaf_patch[row];
        int32_t f = j->pface[pi];
        const float *N = j->fnormal + 3 * f, *U = j->fu + 3 * f, *c = j->center + 3 * pi;
        float q[3] = {c[0] + N[0] * SAMPLE_OFFSET, c[1] + N[1] * SAMPLE_OFFSET,
                      c[2] + N[2] * SAMPLE_OFFSET};
        float il = 1.0f / sqrtf(dot3(U, U));
        float T1[3] = {U[0] * il, U[1] * il, U[2] * il};
        float T2[3] = {N[1] * T1[2] - N[2] * T1[1], N[2] * T1[0] - N[0] * T1[2],
                       N[0] * T1[1] - N[1] * T1[0]};
        int32_t *tg = j->cnt_rows + slot * (int64_t)j->k;
        for (int32_t r = 0; r < j->k; r++) {
            const float *L = j->dirs + 3 * r;
            float d[3];
            for (int a = 0; a < 3; a++) d[a] = (L[0] * T1[a] + L[1] * T2[a]) + L[2] * N[a];
            int32_t h;
            float t;
            int32_t target = -1;
            if (trace_kd(j->s, q, d, 0.0f, MAX_TRACE_LENGTH, -1, 1, &h, &t, NULL)) {
                int32_t g = j->tri_face[h];
                if (g >= 0 && j->face_root[g] >= 0) {
                    float x[3] = {q[0] + t * d[0], q[1] + t * d[1], q[2] + t * d[2]};
                    int32_t node = j->face_root[g];
                    while (j->child1[node] >= 0) {
                        int ax = j->split_axis[node];
                        node = (x[ax] >= j->split_dist[node]) ? j->child1[node] : j->child2[node];
                    }
                    target = j->leaf_index[node];
                }
            }
            tg[r] = target;
        }
        qsort(tg, (size_t)j->k, sizeof(int32_t), cmp_i32);
        int32_t distinct = 0;
        for (int32_t r = 0; r < j->k; r++)
            if (tg[r] >= 0 && (r == 0 || tg[r] != tg[r - 1])) distinct++;
        j->nnz[slot] = distinct;
    }
}

static int64_t make_transfer_rows(const orc_scene *s, const int32_t *tri_face, int64_t npatches_all,
                                  const float *center, const int32_t *face, const int32_t *child1,
                                  const int32_t *child2, const int32_t *split_axis,
                                  const float *split_dist, const int32_t *leaf_index,
                                  const int32_t *face_root, const float *fnormal, const float *fu,
                                  const float *dirs_local, int32_t k, int threads,
                                  const int64_t *row_list, int64_t nrows, int64_t *row_ptr,
                                  int32_t *col, int32_t *cnt, int64_t cap) {
    int64_t nleaf = 0;
    for (int64_t i = 0; i < npatches_all; i++)
        if (leaf_index[i] >= 0) nleaf++;
    if (!row_list) nrows = nleaf;
    for (int64_t r = 0; row_list && r < nrows; r++)
        if (row_list[r] < 0 || row_list[r] >= nleaf) return -2;
    int64_t *leaf_patch = malloc(sizeof(int64_t) * (size_t)(nleaf ? nleaf : 1));
    for (int64_t i = 0; i < npatches_all; i++)
        if (leaf_index[i] >= 0) leaf_patch[leaf_index[i]] = i;
    int32_t *rows = malloc(sizeof(int32_t) * (size_t)(nrows ? nrows : 1) * (size_t)k);
    int32_t *nnz = calloc((size_t)(nrows ? nrows : 1), sizeof(int32_t));
    xfer_job j = {0};
    j.s = s;
    j.tri_face = tri_face;
    j.child1 = child1;
    j.child2 = child2;
    j.split_axis = split_axis;
    j.leaf_index = leaf_index;
    j.face_root = face_root;
    j.pface = face;
    j.center = center;
    j.split_dist = split_dist;
    j.fnormal = fnormal;
    j.fu = fu;
    j.dirs = dirs_local;
    j.k = k;
    j.leaf_patch = leaf_patch;
    j.row_list = row_list;
    j.cnt_rows = rows;
    j.nnz = nnz;
    parallel_for(nrows, threads, 4, xfer_range, &j);
    int64_t total = 0;
    row_ptr[0] = 0;
    for (int64_t r = 0; r < nrows; r++) {
        total += nnz[r];
        row_ptr[r + 1] = total;
    }
    if (total <= cap) {
        for (int64_t r = 0; r < nrows; r++) {
            const int32_t *tg = rows + r * (int64_t)k;
            int64_t o = row_ptr[r];
            for (int32_t i = 0; i < k; i++) {
                if (tg[i] < 0) continue;
                if (i > 0 && tg[i] == tg[i - 1]) {
                    cnt[o - 1]++;
                } else {
                    col[o] = tg[i];
                    cnt[o] = 1;
                    o++;
                }
            }
        }
    }
    free(leaf_patch);
    free(rows);
    free(nnz);
    return total <= cap ? total : -1;
}

int64_t orc_make_transfers(const orc_scene *s, const int32_t *tri_face, int64_t npatches_all,
                           const float *mins, const float *maxs, const float *center,
                           const int32_t *face, const int32_t *child1, const int32_t *child2,
                           const int32_t *split_axis, const float *split_dist,
                           const int32_t *leaf_index, const int32_t *face_root,
                           const float *fnormal, const float *fu, const float *dirs_local,
                           int32_t k, int threads, int64_t *row_ptr, int32_t *col, int32_t *cnt,
                           int64_t cap) {
    (void)mins;
    (void)maxs;
    return make_transfer_rows(s, tri_face, npatches_all, center, face, child1, child2, split_axis,
                              split_dist, leaf_index, face_root, fnormal, fu, dirs_local, k,
                              threads, NULL, 0, row_ptr, col, cnt, cap);
}

int64_t orc_make_transfer_rows(const orc_scene *s, const int32_t *tri_face, int64_t npatches_all,
                               const float *center, const int32_t *face, const int32_t *child1,
                               const int32_t *child2, const int32_t *split_axis,
                               const float *split_dist, const int32_t *leaf_index,
                               const int32_t *face_root, const float *fnormal, const float *fu,
                               const float *dirs_local, int32_t k, int threads,
                               const int64_t *rows, int64_t nrows, int64_t *row_ptr, int32_t *col,
                               int32_t *cnt, int64_t cap) {
    if (!rows) return -2;
    return make_transfer_rows(s, tri_face, npatches_all, center, face, child1, child2, split_axis,
                              split_dist, leaf_index, face_root, fnormal, fu, dirs_local, k,
                              threads, rows, nrows, row_ptr, col, cnt, cap);
}

/* ------------------------------------------------------------------ */
/* bounce (absent in the reference; project semantics), float64        */
/* ------------------------------------------------------------------ */

/* Jacobi gather over the transfer rows:
 *   emit_i = refl_i * direct_i + base_i ; total_i = 0
 *   per bounce: add_i = sum_j w_ij emit_j ; total_i += add_i ; emit_i = refl_i * add_i
 *   delta = sum_i |add_i|_1 / sum_i |total_i|_1 ; stop after the bounce
 *   whose delta < tol, or after max_bounces.  Returns bounces run. */
typedef struct {
    const int64_t *row_ptr;
    const int32_t *col;
    const float *w;
    const double *emit;
    double *add;
} spmv_job;

/* add_i = sum_j w_ij emit_j for rows [b, e), each row summed in entry order */
static void spmv_range(void *ctx, int64_t b, int64_t e, int wk) {
    (void)wk;
    const spmv_job *j = (const spmv_job *)ctx;
    for (int64_t i = b; i < e; i++) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int64_t k = j->row_ptr[i]; k < j->row_ptr[i + 1]; k++) {
            const double wv = (double)j->w[k];
            const double *em = j->emit + 3 * (int64_t)j->col[k];
            acc[0] += wv * em[0];
            acc[1] += wv * em[1];
            acc[2] += wv * em[2];
        }
        for (int c = 0; c < 3; c++) j->add[3 * i + c] = acc[c];
    }
}

int orc_bounce_f64(int64_t nrows, const int64_t *row_ptr, const int32_t *col, const float *w,
                   const float *refl, const float *direct, const float *base, int max_bounces,
                   double tol, double *out_total, double *out_deltas) {
    return orc_bounce_f64_mt(nrows, row_ptr, col, w, refl, direct, base, max_bounces, tol,
                             out_total, out_deltas, 1);
}

/* The same, rows spread over `threads` (each row's sum and the energy sums
 * keep their order, so the result does not depend on the thread count). */
int orc_bounce_f64_mt(int64_t nrows, const int64_t *row_ptr, const int32_t *col, const float *w,
                      const float *refl, const float *direct, const float *base, int max_bounces,
                      double tol, double *out_total, double *out_deltas, int threads) {
    double *emit = malloc(sizeof(double) * 3 * (size_t)(nrows ? nrows : 1));
    double *add = malloc(sizeof(double) * 3 * (size_t)(nrows ? nrows : 1));
    for (int64_t i = 0; i < 3 * nrows; i++) {
        emit[i] = (double)refl[i] * (double)direct[i] + (double)base[i];
        out_total[i] = 0.0;
    }
    spmv_job j = {row_ptr, col, w, emit, add};
    int b;
    for (b = 0; b < max_bounces; b++) {
        double sa = 0.0, st = 0.0;
        parallel_for(nrows, threads, 256, spmv_range, &j);
        for (int64_t i = 0; i < 3 * nrows; i++) {
            out_total[i] += add[i];
            emit[i] = (double)refl[i] * add[i];
            sa += fabs(add[i]);
            st += fabs(out_total[i]);
        }
        double delta = st > 0.0 ? sa / st : 0.0;
        if (out_deltas) out_deltas[b] = delta;
        if (delta < tol) {
            b++;
            break;
        }
    }
    free(emit);
    free(add);
    return b;
}

/* ---- lightmap samples (project semantics) ----
 * The reference computes face extents and drops them (CalcFaceExtents takes
 * its output arrays by value, rad/world/face.go:14, rad/start.go:110), its
 * write-out is a stub (cmd/tasks/finish/main.go:8-40) and the sample encoder
 * it names (compute/leafambient/lighting.go:67) is not in the project.
 *
 * Sample of one light: Ward's RGBE ("Real Pixels", Graphics Gems II) with a
 * signed exponent byte.  A channel that is not > 0 counts as 0, +inf as
 * FLT_MAX; m = the largest channel, 0 -> the all-zero sample; frexp gives
 * m = f * 2^e with 0.5 <= f < 1; x = max(e - 8, -128);
 * byte = floor(ldexp(c, -x)); the word is r | g << 8 | b << 16 | (x & 255) << 24. */
static float sample_channel(float c) {
    if (!(c > 0.0f)) return 0.0f;
    return c > 3.4028234663852886e38f ? 3.4028234663852886e38f : c;
}

uint32_t orc_encode_sample(float r, float g, float b) {
    float c[3] = {sample_channel(r), sample_channel(g), sample_channel(b)};
    float m = c[0];
    if (c[1] > m) m = c[1];
    if (c[2] > m) m = c[2];
    if (m == 0.0f) return 0u;
    int e = 0;
    (void)frexpf(m, &e);
    int x = e - 8 < -128 ? -128 : e - 8;
    uint32_t w = (uint32_t)(x & 255) << 24;
    for (int a = 0; a < 3; a++) {
        float s = floorf(ldexpf(c[a], -x));
        w |= (uint32_t)(s > 255.0f ? 255.0f : s) << (8 * a);
    }
    return w;
}

/* Per luxel (face order, row-major nu x nv): light = direct[lux] +
 * total[leaf], leaf = the face's patch tree descended at the luxel centre
 * (the S == 1 sample point, centre + 0.125 N; coordinate >= dist ->
 * child1), no bounced term when the face has no patches; then the sample. */
void orc_lightmap(const float *corner, const float *u, const float *v, const float *nrm,
                  const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                  int32_t nfaces, const int32_t *child1, const int32_t *child2,
                  const int32_t *split_axis, const float *split_dist, const int32_t *leaf_index,
                  const int32_t *face_root, const float *direct, const float *total,
                  uint32_t *out) {
    for (int32_t f = 0; f < nfaces; f++)
        for (int iv = 0; iv < nv[f]; iv++)
            for (int iu = 0; iu < nu[f]; iu++) {
                int64_t lux = luxel_offset[f] + (int64_t)iv * nu[f] + iu;
                float light[3] = {direct[3 * lux], direct[3 * lux + 1], direct[3 * lux + 2]};
                if (face_root[f] >= 0) {
                    float p[3];
                    luxel_sample(corner + 3 * f, u + 3 * f, v + 3 * f, nrm + 3 * f, nu[f], nv[f],
                                 lux, iu, iv, 0, 1, 0, p);
                    int32_t node = face_root[f];
                    while (child1[node] >= 0)
                        node = p[split_axis[node]] >= split_dist[node] ? child1[node] : child2[node];
                    const float *t = total + 3 * (int64_t)leaf_index[node];
                    for (int a = 0; a < 3; a++) light[a] = light[a] + t[a];
                }
                out[lux] = orc_encode_sample(light[0], light[1], light[2]);
            }
}

/* CalcFaceExtents (rad/world/face.go:14-90) with its results returned: for
 * each lightmap axis j, val = ((x*L[j][0] + y*L[j][1]) + z*L[j][2]) + L[j][3]
 * over the face's vertices (float32, one rounding per operation), min/max
 * seeded with +-1e24; mins = floor(min), size = ceil(max) - floor(min) (the
 * subtraction in float32, then truncated to int32).  *too_big = 1 when a
 * size exceeds 125 + 1 (MAX_LIGHTMAP_DIM_WITHOUT_BORDER, the same for
 * displacements; common/constants/constants.go:22,27), which the reference
 * logs and carries on from.  Returns 0, or -1 for no vertices or values that
 * do not fit an int32. */
int orc_calc_face_extents(const float *verts, int32_t nverts, const float *vecs,
                          int32_t *mins_out, int32_t *size_out, int32_t *too_big) {
    if (nverts < 1) return -1;
    float mins[2] = {1e24f, 1e24f}, maxs[2] = {-1e24f, -1e24f};
    for (int32_t i = 0; i < nverts; i++) {
        const float *p = verts + 3 * i;
        for (int j = 0; j < 2; j++) {
            const float *L = vecs + 4 * j;
            float val = ((p[0] * L[0] + p[1] * L[1]) + p[2] * L[2]) + L[3];
            if (val < mins[j]) mins[j] = val;
            if (val > maxs[j]) maxs[j] = val;
        }
    }
    *too_big = 0;
    for (int j = 0; j < 2; j++) {
        float lo = (float)floor((double)mins[j]), hi = (float)ceil((double)maxs[j]);
        float sz = hi - lo;
        if (!(lo >= -2147483648.0f && lo < 2147483648.0f && sz >= -2147483648.0f && sz < 2147483648.0f))
            return -1;
        mins_out[j] = (int32_t)lo;
        size_out[j] = (int32_t)sz;
        if (size_out[j] > 125 + 1) *too_big = 1;
    }
    return 0;
}

/* ---- brush ingest (fixed mode) ----
 * addBrushesForRayTrace / addBrushToRaytraceEnvironment
 * (cmd/tasks/loadbsp/main.go:241-340), BaseWindingForPlane and
 * ChopWindingInPlace (vmath/polygon/winding.go:25-170), with the defects the
 * fixed mode repairs: sky sides are skipped (the reference keeps only them,
 * main.go:255); the major axis reads normal[i] and axes 0 and 1 share the
 * up vector (0,0,1) (winding.go:36,45-51); the fourth point is written
 * (winding.go:77-78); the wrap-around side/distance entry is set and the
 * split loop advances j (winding.go:112,149).  No literal mode: the Go
 * as written never leaves the split loop. */
#define ORC_WPTS 68

static float dot3f(const float *a, const float *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

void orc_base_winding(const float *n, float dist, float *out12) {
    int x = -1;
    float mx = -1.0f;
    for (int i = 0; i < 3; i++) {
        float v = fabsf(n[i]);
        if (v > mx) { x = i; mx = v; }
    }
    float up[3] = {0.0f, 0.0f, 0.0f};
    if (x == 0 || x == 1) up[2] = 1.0f;
    else up[0] = 1.0f;
    float v = dot3f(up, n);
    for (int a = 0; a < 3; a++) up[a] = up[a] + (-v) * n[a];
    float il = 1.0f / sqrtf(dot3f(up, up));
    for (int a = 0; a < 3; a++) up[a] = up[a] * il;
    float org[3], right[3];
    for (int a = 0; a < 3; a++) org[a] = n[a] * dist;
    right[0] = up[1] * n[2] - up[2] * n[1];
    right[1] = up[2] * n[0] - up[0] * n[2];
    right[2] = up[0] * n[1] - up[1] * n[0];
    for (int a = 0; a < 3; a++) {
        up[a] = up[a] * 65536.0f;
        right[a] = right[a] * 65536.0f;
    }
    for (int a = 0; a < 3; a++) {
        out12[0 + a] = (org[a] - right[a]) + up[a];
        out12[3 + a] = (org[a] + right[a]) + up[a];
        out12[6 + a] = (org[a] + right[a]) - up[a];
        out12[9 + a] = (org[a] - right[a]) - up[a];
    }
}

/* In-place chop of w (n points, room for ORC_WPTS); returns the new count
 * (0: nothing in front) or -1 past 64 points. */
int orc_chop_winding(float *w, int n, const float *nrm, float dist, float eps) {
    float dists[ORC_WPTS + 1], tmp[3 * ORC_WPTS];
    int sides[ORC_WPTS + 1], counts[3] = {0, 0, 0};
    if (n <= 0) return 0;
    for (int i = 0; i < n; i++) {
        dists[i] = dot3f(w + 3 * i, nrm) - dist;
        sides[i] = dists[i] > eps ? 0 : (dists[i] < -eps ? 1 : 2);
        counts[sides[i]]++;
    }
    sides[n] = sides[0];
    dists[n] = dists[0];
    if (counts[0] == 0) return 0;
    if (counts[1] == 0) return n;
    int m = 0;
    for (int i = 0; i < n; i++) {
        const float *p1 = w + 3 * i;
        if (sides[i] == 2) {
            if (m >= ORC_WPTS) return -1;
            memcpy(tmp + 3 * m++, p1, 12);
            continue;
        }
        if (sides[i] == 0) {
            if (m >= ORC_WPTS) return -1;
            memcpy(tmp + 3 * m++, p1, 12);
        }
        if (sides[i + 1] == 2 || sides[i + 1] == sides[i]) continue;
        const float *p2 = w + 3 * ((i + 1) % n);
        float t = dists[i] / (dists[i] - dists[i + 1]);
        if (m >= ORC_WPTS) return -1;
        for (int j = 0; j < 3; j++) {
            if (nrm[j] == 1.0f) tmp[3 * m + j] = dist;
            else if (nrm[j] == -1.0f) tmp[3 * m + j] = -dist;
            else tmp[3 * m + j] = p1[j] + t * (p2[j] - p1[j]);
        }
        m++;
    }
    if (m > 64) return -1;
    memcpy(w, tmp, 12 * (size_t)m);
    return m;
}

static void brushes_recursive(int32_t node, const int32_t *children, const int32_t *leaf_ranges,
                              const int32_t *leaf_brushes, int32_t *list, int32_t *count) {
    if (node < 0) {
        int32_t leaf = -1 - node;
        for (int32_t i = 0; i < leaf_ranges[2 * leaf + 1]; i++) {
            int32_t b = leaf_brushes[leaf_ranges[2 * leaf] + i], found = 0;
            for (int32_t k = 0; k < *count; k++)
                if (list[k] == b) { found = 1; break; }
            if (!found) list[(*count)++] = b;
        }
        return;
    }
    brushes_recursive(children[2 * node], children, leaf_ranges, leaf_brushes, list, count);
    brushes_recursive(children[2 * node + 1], children, leaf_ranges, leaf_brushes, list, count);
}

/* Triangles of the world (model 0): opaque brushes then sky faces, in the
 * reference's order; ids ORC_TRACE_ID_OPAQUE / ORC_TRACE_ID_SKY.  Inputs are
 * assumed valid (the tests build them).  Returns the triangle count, or -1
 * when cap is too small or a winding passes 64 points; *n_brush = brush
 * triangles. */
int64_t orc_bsp_world_triangles(const float *planes, const int32_t *node_children, int32_t num_nodes,
                                const int32_t *leaf_ranges, int32_t num_leafs,
                                const int32_t *leaf_brushes, const int32_t *brushes,
                                int32_t num_brushes, const int32_t *brush_sides,
                                const int32_t *texinfo_flags, const float *vertexes,
                                const int32_t *edges, const int32_t *surf_edges,
                                const int32_t *faces, int32_t headnode, int32_t first_face,
                                int32_t num_model_faces, float *xyz, int32_t *ids, int64_t cap,
                                int64_t *n_brush) {
    int32_t *list = (int32_t *)malloc(sizeof(int32_t) * (size_t)(num_brushes > 0 ? num_brushes : 1));
    int32_t count = 0;
    int64_t nt = 0;
    if (num_nodes > 0 || num_leafs > 0)
        brushes_recursive(headnode, node_children, leaf_ranges, leaf_brushes, list, &count);
    float w[3 * ORC_WPTS];
    for (int32_t k = 0; k < count; k++) {
        const int32_t *b = brushes + 3 * list[k];
        if ((b[2] & (0x1 | 0x4000 | 0x80)) == 0) continue;
        for (int32_t i = 0; i < b[1]; i++) {
            const int32_t *side = brush_sides + 4 * (b[0] + i);
            int32_t tf = side[1] >= 0 ? texinfo_flags[side[1]] : 0;
            if ((tf & 0x4) != 0 || side[2] != 0) continue;
            orc_base_winding(planes + 4 * side[0], planes[4 * side[0] + 3], w);
            int n = 4;
            for (int32_t j = 0; j < b[1] && n > 0; j++) {
                if (j == i) continue;
                const int32_t *o = brush_sides + 4 * (b[0] + j);
                if (o[3] != 0) continue;
                const float *op = planes + 4 * (o[0] ^ 1);
                n = orc_chop_winding(w, n, op, op[3], 0.0f);
                if (n < 0) { free(list); return -1; }
            }
            for (int j = 2; j < n; j++) {
                if (nt >= cap) { free(list); return -1; }
                memcpy(xyz + 9 * nt, w, 12);
                memcpy(xyz + 9 * nt + 3, w + 3 * (j - 1), 12);
                memcpy(xyz + 9 * nt + 6, w + 3 * j, 12);
                ids[nt++] = ORC_TRACE_ID_OPAQUE;
            }
        }
    }
    free(list);
    *n_brush = nt;
    for (int32_t k = 0; k < num_model_faces; k++) {
        const int32_t *f = faces + 3 * (first_face + k);
        int32_t tf = f[2] >= 0 ? texinfo_flags[f[2]] : 0;
        if ((tf & 0x4) == 0) continue;
        for (int32_t j = 2; j < f[1]; j++) {
            int32_t vv[3] = {0, j - 1, j};
            if (nt >= cap) return -1;
            for (int c = 0; c < 3; c++) {
                int32_t e = surf_edges[f[0] + vv[c]];
                int32_t v = e < 0 ? edges[2 * (-e) + 1] : edges[2 * e];
                memcpy(xyz + 9 * nt + 3 * c, vertexes + 3 * v, 12);
            }
            ids[nt++] = ORC_TRACE_ID_SKY;
        }
    }
    return nt;
}
