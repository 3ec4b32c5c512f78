/*
 * vrad_oracle.h -- CPU oracle for the VRAD radiosity hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithm, which tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg compare the library against.  The product library never
 * links, loads or calls it.  Parity with the reference itself is unpinned:
 * the reference's path cannot be built or run, and its tests hold no golden
 * vectors for it; known-answer tests pin this restatement instead.
 *
 * Reference files restated (paths inside the reference project):
 *   raytracer/environment.go:41-138,181-403   triangle soup, SAH kd builder
 *   raytracer/cache/optimisedtriangle.go:14-103  intersection format, classify
 *   raytracer/cache/optimisedkdnode.go:8-54    packed node
 *   raytracer/kdtree/constants.go:25-28        SAH constants
 *   vmath/polygon/edge.go:5-24, surface.go:5-8 edge equations, box area
 *   raytracer/trace/testline.go:18-94          shadow-line semantics
 *   rad/lightmap/lights.go:23,210-341          light falloff parameters
 *   vmath/quadratic/solver.go:4-63             inverse quadratic solve
 *   rad/patches/subdivide.go:166-411           patch subdivision
 *   common/types/patch.go, transfer.go         patch / transfer layout
 *   rad/world/face.go:14-90                    face lightmap extents
 *   cmd/tasks/loadbsp/main.go:241-340          brushes and sky faces -> triangles
 *   vmath/polygon/winding.go:25-170            base winding, winding chop
 * Gather, transfer building and the bounce loop are absent from the
 * reference; their semantics are the project's own and are written out in
 * the comments of vrad_oracle.c beside each function.
 *
 * Parity status: unpinned against the reference itself (it has no Go
 * toolchain here and no golden vectors for this path); pinned by the
 * known-answer tests in tests/test_oracle_kat.py and, for the trace
 * semantics, by float64 geometry in tests/golden/trace_geometry.npz.
 */
#ifndef VRAD_ORACLE_H
#define VRAD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_TRACE_ID_SKY        0x01000000
#define ORC_TRACE_ID_OPAQUE     0x02000000
#define ORC_TRACE_ID_STATICPROP 0x04000000
/* Triangle flag of a transparent triangle (the NFlags byte of
 * raytracer/cache/triangle/trigeometrydata.go:8; the reference defines no
 * bit, the project uses bit 0). */
#define ORC_TRI_TRANSPARENT 0x01

#define ORC_MODE_FIXED   0
#define ORC_MODE_LITERAL 1

/* TriIntersectData (raytracer/cache/triangle/triintersectdata.go:3-22), 48 B. */
typedef struct {
    float nx, ny, nz, d;
    int32_t id;
    float e[6];
    uint8_t cs0, cs1, flags, unused;
} orc_tri;

/* The parts of DirectLight / WorldLight (common/types/light.go:10-44) that
 * the gather reads.  type uses Source's emittype order:
 * 0 surface, 1 point, 2 spotlight, 3 skylight, 4 quakelight, 5 skyambient. */
typedef struct {
    int32_t type;
    float origin[3];
    float intensity[3];
    float normal[3];
    float stopdot, stopdot2, exponent;
    float constant_attn, linear_attn, quadratic_attn;
    float radius;
    float start_fade, end_fade, cap_distance;
} orc_light;

/* Entity key/values that SetLightFalloffParams / ParseLightSpot read. */
typedef struct {
    float fifty_percent_distance, zero_percent_distance;
    int32_t hard_falloff;
    float constant_attn, linear_attn, quadratic_attn, distance;
    float inner_cone, cone, exponent;
} orc_light_keys;

typedef struct orc_scene orc_scene;

/* ---- scene / kd tree ---- */
orc_scene *orc_scene_new(const float *xyz, const int32_t *ids, const uint8_t *flags,
                         int64_t ntris, int mode);
void orc_scene_free(orc_scene *s);
int64_t orc_scene_num_nodes(const orc_scene *s);
int64_t orc_scene_num_refs(const orc_scene *s);
void orc_scene_get_tree(const orc_scene *s, uint32_t *children, float *split, int32_t *refs);
void orc_scene_get_tris(const orc_scene *s, orc_tri *out);
/* walk without visiting leaves that hold no triangle (answers unchanged;
 * only the node counts of the stats differ) */
void orc_scene_set_skip_empty(orc_scene *s, int on);
/* shadow lines (no hit output) first test the opaque triangles lying in
 * the scene-box face they leave through, as the library does: tris[4*f+i]
 * for i < counts[f] (face f = 2*axis + 1 for a max side); NULL: off.
 * Verdicts are unchanged; node and triangle counts follow the library. */
void orc_scene_set_walls(orc_scene *s, const int32_t *tris, const int32_t *counts);
/* replace the tree (same format as orc_scene_get_tree); 0 on success */
int orc_scene_set_tree(orc_scene *s, const uint32_t *children, const float *split,
                       int64_t nnodes, const int32_t *refs, int64_t nrefs);
void orc_scene_bounds(const orc_scene *s, float *bmin, float *bmax);
int orc_scene_depth(const orc_scene *s);

/* intersection format of one triangle (fixed semantics) */
void orc_tri_format(const float *xyz9, int32_t id, uint8_t flags, orc_tri *out);
/* GetEdgeEquation (vmath/polygon/edge.go:5-24); p1,p2,inside are xyz */
void orc_edge_equation(const float *p1, const float *p2, int c1, int c2, const float *inside,
                       float *out3);

/* ---- trace ---- */
/* closest hit: out_hit = triangle index (insertion order) or -1; out_t = t.
 * brute != 0 tests every triangle instead of walking the tree.
 * stats (optional, 3 x n): nodes visited, triangles tested, leaves visited. */
void orc_trace_closest(const orc_scene *s, const float *orig, const float *dir,
                       const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                       int brute, int threads, int32_t *out_hit, float *out_t, uint32_t *stats);
void orc_trace_any(const orc_scene *s, const float *orig, const float *dir,
                   const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                   int brute, int threads, uint8_t *out_hit, uint32_t *stats);
/* TestLineDoesHitSky semantics per line; frac = fractionVisible (0 or 1). */
void orc_test_lines(const orc_scene *s, const float *start, const float *stop, int64_t n,
                    int32_t skip_id, int brute, int threads, float *out_frac);
/* 1-bit occlusion mask (bit i of word i/32 set = occluded) and, if out_hit is
 * non-null, the closest-hit triangle index and t of the normalised segment. */
void orc_occlusion_mask(const orc_scene *s, const float *start, const float *stop, int64_t n,
                        int32_t skip_id, int threads, uint32_t *out_mask,
                        int32_t *out_hit, float *out_t, uint32_t *stats);

/* ---- lights ---- */
int orc_solve_inverse_quadratic(float x1, float y1, float x2, float y2, float x3, float y3,
                                float *a, float *b, float *c);
int orc_solve_inverse_quadratic_monotonic(float x1, float y1, float x2, float y2, float x3,
                                          float y3, float *a, float *b, float *c);
void orc_set_light_falloff(const orc_light_keys *k, orc_light *l);
void orc_parse_light_spot(const orc_light_keys *k, orc_light *l);

/* ---- direct light ---- */
/* Gather at explicit points (one sample each). rays_out counts shadow rays. */
void orc_gather_points(const orc_scene *s, const orc_light *lights, int nlights,
                       const float *pts, const float *nrm, int64_t n, int threads,
                       float *out_rgb, uint64_t *rays_out);
/* Luxel supersample gather.  faces: corner,u,v,normal (3 floats each), nu,nv.
 * luxel_offset[f] = first luxel of face f.  Writes RGB per luxel. */
void orc_gather_luxels(const orc_scene *s, const orc_light *lights, int nlights,
                       const float *corner, const float *u, const float *v, const float *nrm,
                       const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                       int32_t face_begin, int32_t face_end, int supersamples, uint64_t seed,
                       int threads, float *out_rgb, uint64_t *rays_out, uint64_t *stats_out);
/* the sample points the luxel gather uses (for cross-checks) */
void orc_luxel_samples(const float *corner, const float *u, const float *v, const float *nrm,
                       const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                       int32_t face, int supersamples, uint64_t seed, float *out_pts);

/* ---- patches ---- */
/* Subdivide axis-aligned rectangular faces.  Returns the number of patches
 * (parents included) and fills the arrays when they are non-null (call once
 * with nulls to size).  leaf_index[p] = dense leaf number or -1. */
int64_t orc_make_patches(const float *corner, const float *u, const float *v, const float *nrm,
                         const float *luxscale, int32_t nfaces, float max_chop, float min_chop,
                         float *mins, float *maxs, float *center, float *area, int32_t *face,
                         int32_t *parent, int32_t *child1, int32_t *child2, int32_t *split_axis,
                         float *split_dist, int32_t *leaf_index);

/* ---- transparent shadows (project semantics) ----
 * The reference's Trace4Rays takes a transparent-triangle callback
 * (raytracer/environment.go:140-142) whose one counting implementation adds
 * each hit triangle's colour x as coverage and clamps at 1
 * (raytracer/types/coverageCount.go:27-41); texture coverage is a stub
 * (rad/staticprops/compute.go:4-12).  The reference never fixes the order in
 * which hits reach the callback.  Here: a triangle with ORC_TRI_TRANSPARENT
 * in its flags is transparent with coverage cover[i] (the caller passes the
 * colours' x); a ray's accepted hits are taken in ascending (t, triangle
 * index): an opaque hit is recorded and ends the walk, a transparent one
 * adds c = min(c + cover, 1) and, when c reaches 1, is recorded and ends it.
 * orc_trace_coverage returns the recorded hit, its t and c;
 * orc_test_lines_coverage is TestLineDoesHitSky with texture shadows
 * (raytracer/trace/testline.go:29-33,53-55): occlusion = max(opaque, c),
 * clamped, fraction visible = 1 - occlusion.  Brute force over all
 * triangles (small scenes only). */
void orc_trace_coverage(const orc_scene *s, const float *cover, const float *orig, const float *dir,
                        const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                        int threads, int32_t *out_hit, float *out_t, float *out_coverage);
void orc_test_lines_coverage(const orc_scene *s, const float *cover, const float *start,
                             const float *stop, int64_t n, int32_t skip_id, int threads,
                             float *out_frac);

/* ---- transfers ---- */
/* Per leaf patch, K rays along dirs_local (lx,ly,lz) in the frame (T1,T2,N);
 * counts closest hits per target leaf patch.  Rows are written into the
 * caller's buffers: row_ptr[P+1] (int64), col/cnt arrays of capacity cap.
 * Returns total nnz (or -1 if cap is too small; row_ptr is still filled). */
int64_t orc_make_transfers(const orc_scene *s, const int32_t *tri_face, int64_t npatches_all,
                           const float *mins, const float *maxs, const float *center,
                           const int32_t *face, const int32_t *child1, const int32_t *child2,
                           const int32_t *split_axis, const float *split_dist,
                           const int32_t *leaf_index, const int32_t *face_root,
                           const float *fnormal, const float *fu,
                           const float *dirs_local, int32_t k, int threads,
                           int64_t *row_ptr, int32_t *col, int32_t *cnt, int64_t cap);
/* The same rows for a subset of leaf rows (dense indices `rows[0..nrows)`, in
 * that order): row_ptr[nrows+1] and col/cnt as above.  -1: cap too small;
 * -2: a row index out of range. */
int64_t orc_make_transfer_rows(const orc_scene *s, const int32_t *tri_face, int64_t npatches_all,
                               const float *center, const int32_t *face, const int32_t *child1,
                               const int32_t *child2, const int32_t *split_axis,
                               const float *split_dist, const int32_t *leaf_index,
                               const int32_t *face_root, const float *fnormal, const float *fu,
                               const float *dirs_local, int32_t k, int threads,
                               const int64_t *rows, int64_t nrows, int64_t *row_ptr, int32_t *col,
                               int32_t *cnt, int64_t cap);

/* ---- bounce (float64) ---- */
int orc_bounce_f64(int64_t nrows, const int64_t *row_ptr, const int32_t *col, const float *w,
                   const float *refl, const float *direct, const float *base, int max_bounces,
                   double tol, double *out_total, double *out_deltas);
int orc_bounce_f64_mt(int64_t nrows, const int64_t *row_ptr, const int32_t *col, const float *w,
                      const float *refl, const float *direct, const float *base, int max_bounces,
                      double tol, double *out_total, double *out_deltas, int threads);

/* ---- lightmap samples ---- */
/* Shared-exponent sample (r | g << 8 | b << 16 | exponent << 24) of one light. */
uint32_t orc_encode_sample(float r, float g, float b);
/* Samples of every luxel: direct light + bounced light of the leaf patch at
 * the luxel centre.  direct: 3 floats per luxel; total: 3 floats per leaf. */
void orc_lightmap(const float *corner, const float *u, const float *v, const float *nrm,
                  const int32_t *nu, const int32_t *nv, const int64_t *luxel_offset,
                  int32_t nfaces, const int32_t *child1, const int32_t *child2,
                  const int32_t *split_axis, const float *split_dist, const int32_t *leaf_index,
                  const int32_t *face_root, const float *direct, const float *total,
                  uint32_t *out);
/* CalcFaceExtents: vecs = LightmapVecsLuxelsPerWorldUnits (2 x 4 floats). */
int orc_calc_face_extents(const float *verts, int32_t nverts, const float *vecs,
                          int32_t *mins_out, int32_t *size_out, int32_t *too_big);

/* ---- brush ingest (fixed mode) ---- */
void orc_base_winding(const float *n, float dist, float *out12);
/* w has room for 68 points; returns the new point count, 0 = nothing in
 * front, -1 = past 64 points. */
int orc_chop_winding(float *w, int n, const float *nrm, float dist, float eps);
int64_t orc_bsp_world_triangles(const float *planes, const int32_t *node_children, int32_t num_nodes,
                                const int32_t *leaf_ranges, int32_t num_leafs,
                                const int32_t *leaf_brushes, const int32_t *brushes,
                                int32_t num_brushes, const int32_t *brush_sides,
                                const int32_t *texinfo_flags, const float *vertexes,
                                const int32_t *edges, const int32_t *surf_edges,
                                const int32_t *faces, int32_t headnode, int32_t first_face,
                                int32_t num_model_faces, float *xyz, int32_t *ids, int64_t cap,
                                int64_t *n_brush);

#ifdef __cplusplus
}
#endif
#endif
