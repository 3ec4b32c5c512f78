/*
 * vradgpu.h -- C ABI of the GB300 (sm_103a) radiosity hot path.
 *
 * One shared library (libvradgpu.so) stands behind the reference's Go entry
 * points for the ray tracer, direct-light gathering, transfer building and
 * the bounce loop, and for the stages on either side: reading a compiled
 * map's brushes into the ray tracer, and face extents and lightmap samples
 * after the bake.  Plain pointers and sizes only; every call returns an int
 * status (VRG_OK = 0, negative on error) and the message of the most recent
 * failure on a context is available from vrg_last_error().
 *
 * Ownership: host buffers belong to the caller and are only borrowed for the
 * duration of the call.  Device memory is owned by the handle that created
 * it.  Functions ending in _d take device pointers; all others take host
 * pointers.  The trace entry points (vrg_env_occlusion_mask,
 * vrg_env_trace_closest, vrg_env_test_line_does_hit_sky) read page-locked
 * host inputs (cudaHostAlloc / cudaHostRegister) in place over the CPU-GPU
 * link; other host buffers are copied in and out inside the call.
 *
 * Threading: a context may be shared by several host threads; each
 * environment serialises its own calls with a mutex.
 *
 * Reference citations are paths inside the reference project.
 */
#ifndef VRADGPU_H
#define VRADGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VRG_OK 0
#define VRG_ERR_INVALID (-1)     /* bad argument */
#define VRG_ERR_NOMEM (-2)       /* host or device allocation failed */
#define VRG_ERR_CUDA (-3)        /* CUDA runtime error */
#define VRG_ERR_TIMEOUT (-4)     /* a bounded device wait ran out */
#define VRG_ERR_STATE (-5)       /* call out of order (e.g. trace before build) */
#define VRG_ERR_UNSUPPORTED (-6) /* feature or size outside the build's limits */

/* raytracer/constants.go:9-11 */
#define VRG_TRACE_ID_SKY 0x01000000
#define VRG_TRACE_ID_OPAQUE 0x02000000
#define VRG_TRACE_ID_STATICPROP 0x04000000
/* raytracer/constants.go:5-7 */
#define VRG_RTE_FLAGS_FAST_TREE_GENERATION 1
#define VRG_RTE_FLAGS_DONT_STORE_TRIANGLE_COLORS 2
#define VRG_RTE_FLAGS_DONT_STORE_TRIANGLE_MATERIALS 4
/* Triangle flag (the NFlags byte, raytracer/cache/triangle/trigeometrydata.go:8,
 * set from AddTriangleWithMaterial's flags, environment.go:58) that marks a
 * transparent triangle for the coverage traces below.  The reference defines
 * no bit for it; bit 0 is the project's. */
#define VRG_TRIFLAG_TRANSPARENT 1

/* BSP contents and surface flags the brush ingest reads (Source's bspflags
 * values, which galaco/bsp's flags package carries):
 * MASK_OPAQUE = CONTENTS_SOLID | CONTENTS_MOVEABLE | CONTENTS_OPAQUE. */
#define VRG_CONTENTS_SOLID 0x1
#define VRG_CONTENTS_OPAQUE 0x80
#define VRG_CONTENTS_MOVEABLE 0x4000
#define VRG_MASK_OPAQUE (VRG_CONTENTS_SOLID | VRG_CONTENTS_MOVEABLE | VRG_CONTENTS_OPAQUE)
#define VRG_SURF_SKY 0x4

/* Source's emittype order, as galaco/bsp worldlight EMIT_* uses it. */
#define VRG_EMIT_SURFACE 0
#define VRG_EMIT_POINT 1
#define VRG_EMIT_SPOTLIGHT 2
#define VRG_EMIT_SKYLIGHT 3
#define VRG_EMIT_QUAKELIGHT 4
#define VRG_EMIT_SKYAMBIENT 5

typedef struct vrg_ctx vrg_ctx;
typedef struct vrg_env vrg_env;

/* The light fields the gather reads: DirectLight + WorldLight
 * (common/types/light.go:10-44).  20 x 4 bytes. */
typedef struct vrg_light {
    int32_t type;
    float origin[3];
    float intensity[3];
    float normal[3];
    float stopdot, stopdot2, exponent;
    float constant_attn, linear_attn, quadratic_attn;
    float radius;
    float start_fade, end_fade, cap_distance;
} vrg_light;

/* Entity keys that rad/lightmap/lights.go:210-341 reads. */
typedef struct vrg_light_keys {
    float fifty_percent_distance, zero_percent_distance;
    int32_t hard_falloff;
    float constant_attn, linear_attn, quadratic_attn, distance;
    float inner_cone, cone, exponent;
} vrg_light_keys;

/* ------------------------------------------------------------------ */
/* context                                                              */
/* ------------------------------------------------------------------ */

/* Creates a context on CUDA device `device` with its own non-blocking stream.
 * device < 0 creates a host-only context: the host algorithms (kd-tree build,
 * intersection records, light parameters, patch subdivision) work, every
 * device call returns VRG_ERR_STATE.
 * (no reference counterpart: the reference is one process with globals) */
int vrg_ctx_create(int device, vrg_ctx **out);
void vrg_ctx_destroy(vrg_ctx *ctx);
/* Message of the last failure on this context ("" if none). */
const char *vrg_last_error(const vrg_ctx *ctx);
/* Launch on `stream` (a cudaStream_t) instead of the context's own stream;
 * NULL restores the context stream. */
int vrg_ctx_set_stream(vrg_ctx *ctx, void *stream);
int vrg_ctx_synchronize(vrg_ctx *ctx);
/* Per-kernel CUDA-event timing of every launch (off by default). */
int vrg_ctx_set_timing(vrg_ctx *ctx, int enable);
/* Accumulated device time and launch count of kernel `name` since the last
 * reset; names: "trace_mask", "trace_closest", "trace_lines",
 * "direct_luxels", "direct_points", "transfer_rows", "transfer_rows_sorted",
 * "transfer_gather",
 * "bounce_init", "bounce_spmv", "bounce_reduce", "batch_gather",
 * "batch_bounce_init", "batch_spmv", "batch_reduce", "relight_gather",
 * "lightmap". */
int vrg_ctx_kernel_stats(vrg_ctx *ctx, const char *name, double *total_ms, int64_t *launches);
int vrg_ctx_reset_stats(vrg_ctx *ctx);
/* Kernels launched by this context since creation (all names). */
int64_t vrg_ctx_launch_count(const vrg_ctx *ctx);

/* Per-scene-size autotuning (no reference counterpart).  Tuned launch
 * sites ("trace_mask", "trace_mask_hit", "direct_luxels", "transfer_rows",
 * "bounce_spmv", "batch_gather") offer variants that give identical results (the bounce
 * variants: the same sums); the first launch in a bucket
 * "<site>/t<log2 triangles>/n<log2 work items>" times each twice on the real
 * input and keeps the fastest.  On by default; off, or inside a stream
 * capture, an untuned bucket runs variant 0. */
int vrg_ctx_set_autotune(vrg_ctx *ctx, int enable);
/* The variant chosen for `key` (-1 if untuned) and, when `ms` is not NULL,
 * up to `cap` per-variant times of the tuning run. */
int vrg_ctx_autotune_choice(vrg_ctx *ctx, const char *key, int32_t *variant, double *ms, int32_t cap);
/* Save / load the tuned choices as text lines "key variant" (a launch site
 * has at most 32 variants; a line naming another number is ignored). */
int vrg_ctx_autotune_save(vrg_ctx *ctx, const char *path);
int vrg_ctx_autotune_load(vrg_ctx *ctx, const char *path);

/* ------------------------------------------------------------------ */
/* Environment: raytracer/environment.go                                */
/* ------------------------------------------------------------------ */

/* NewEnvironment (environment.go:434-442) */
int vrg_env_create(vrg_ctx *ctx, vrg_env **out);
void vrg_env_destroy(vrg_env *env);
/* AddTriangleWithMaterial (environment.go:45-69); colour may be NULL. */
int vrg_env_add_triangle(vrg_env *env, int32_t id, const float *v1, const float *v2,
                         const float *v3, const float *colour, uint16_t flags, int32_t material);
/* AddQuad (environment.go:71-75): (v1,v2,v3) id, (v1,v3,v4) id+1 */
int vrg_env_add_quad(vrg_env *env, int32_t id, const float *v1, const float *v2, const float *v3,
                     const float *v4, const float *colour);
/* AddAxisAlignedRectangularSolid (environment.go:77-117) */
int vrg_env_add_axis_aligned_rectangular_solid(vrg_env *env, int32_t id, const float *mins,
                                               const float *maxs, const float *colour);
/* Bulk AddTriangle for n triangles (xyz: 9 floats each), the loop of
 * cmd/tasks/loadbsp/main.go:276,338. */
int vrg_env_add_triangles(vrg_env *env, const float *xyz, const int32_t *ids, int64_t n);

/* The lumps of a compiled map that addBrushesForRayTrace reads
 * (cmd/tasks/loadbsp/main.go:283-340), as arrays the caller has parsed
 * (lump records reduced to the fields used; counts are record counts).
 * planes: num_planes x {normal xyz, dist}, in the BSP's pairs (p ^ 1 is p
 * facing the other way); node_children: num_nodes x {child0, child1}
 * (negative = -1 - leaf); leaf_brush_ranges: num_leafs x {firstleafbrush,
 * numleafbrushes}; leaf_brushes: brush indices; brushes: num_brushes x
 * {firstside, numsides, contents}; brush_sides: num_brush_sides x {planenum,
 * texinfo (-1: none), dispinfo, bevel}; texinfo_flags: num_texinfo surface
 * flags; vertexes: num_vertexes x xyz; edges: num_edges x {v0, v1};
 * surf_edges: signed edge indices; faces: num_faces x {firstedge, numedges,
 * texinfo}.  headnode, first_face and num_model_faces describe model 0 (the
 * world). */
typedef struct vrg_bsp_world {
    const float *planes;
    int32_t num_planes;
    const int32_t *node_children;
    int32_t num_nodes;
    const int32_t *leaf_brush_ranges;
    int32_t num_leafs;
    const int32_t *leaf_brushes;
    int32_t num_leaf_brushes;
    const int32_t *brushes;
    int32_t num_brushes;
    const int32_t *brush_sides;
    int32_t num_brush_sides;
    const int32_t *texinfo_flags;
    int32_t num_texinfo;
    const float *vertexes;
    int32_t num_vertexes;
    const int32_t *edges;
    int32_t num_edges;
    const int32_t *surf_edges;
    int32_t num_surf_edges;
    const int32_t *faces;
    int32_t num_faces;
    int32_t headnode;
    int32_t first_face;
    int32_t num_model_faces;
} vrg_bsp_world;
/* addBrushesForRayTrace (cmd/tasks/loadbsp/main.go:283-340) and
 * addBrushToRaytraceEnvironment (:241-282): every opaque brush (contents &
 * VRG_MASK_OPAQUE) of the world, in GetBrushRecursive order (brush.go:7-36),
 * adds each side that is neither sky nor a displacement as the fan of its
 * winding -- BaseWindingForPlane chopped by every other non-bevel side's
 * flipped plane (planenum ^ 1) -- with id VRG_TRACE_ID_OPAQUE; then every
 * sky face of the world adds the fan of its vertices with id
 * VRG_TRACE_ID_SKY.  Colour (1, 0, 0) as the reference's fullCoverage.  The
 * reference adds only the sky sides of brushes (an inverted test at
 * main.go:255); sky sides are skipped here.  Every index is checked before a
 * triangle is added (VRG_ERR_INVALID); the counts of brush and sky
 * triangles added may be returned (NULL to skip). */
int vrg_env_add_bsp_world(vrg_env *env, const vrg_bsp_world *world, int64_t *brush_triangles,
                          int64_t *sky_triangles);
/* A compiled map's bytes decoded into the lumps vrg_bsp_world names (the
 * reference reads them through galaco/bsp, cmd/tasks/loadbsp/main.go:31-40).
 * Source BSP versions 19-21, little-endian; leaf lump version 0 (56-byte
 * leaves) or 1 (32-byte); compressed lumps give VRG_ERR_UNSUPPORTED, a bad
 * magic, a lump outside the data or a lump that is not whole records
 * VRG_ERR_INVALID.  The handle owns the decoded arrays; `data` is not
 * kept. */
typedef struct vrg_bsp vrg_bsp;
int vrg_bsp_open(const uint8_t *data, size_t size, vrg_bsp **out);
void vrg_bsp_close(vrg_bsp *bsp);
/* Fills `world` with pointers into the handle's arrays (valid until
 * vrg_bsp_close) and model 0's headnode and face range. */
int vrg_bsp_get_world(const vrg_bsp *bsp, vrg_bsp_world *world);
/* The world's faces from the HDR face lump (58) instead of lump 7, as
 * loadbsp picks its target faces with -hdr (cmd/tasks/loadbsp/main.go:80-88).
 * A face lump shorter than model 0's face range makes vrg_env_add_bsp_world
 * refuse the world (the reference would index past it). */
int vrg_bsp_use_hdr_faces(vrg_bsp *bsp, int32_t hdr);
/* BSP version, texinfo count and the texinfos' LightmapVecsLuxelsPerWorldUnits
 * (8 floats each, for vrg_calc_face_extents); any pointer may be NULL. */
int vrg_bsp_info(const vrg_bsp *bsp, int32_t *version, int32_t *num_texinfo,
                 const float **lightmap_vecs);
/* BaseWindingForPlane (vmath/polygon/winding.go:25-83): the quad
 * (4 x xyz) of half-side 65536 on the plane, around normal * dist. */
int vrg_base_winding_for_plane(const float *normal, float dist, float *out12);
/* ChopWindingInPlace (winding.go:85-170): the part of the n-point winding
 * in front of the plane (points with normal . p - dist >= -epsilon kept,
 * crossing edges split); *out_n = 0 when nothing is in front.  out holds up
 * to n + 4 points; more than 64 points give VRG_ERR_UNSUPPORTED. */
int vrg_chop_winding(const float *points, int32_t n, const float *normal, float dist, float epsilon,
                     float *out, int32_t *out_n);
/* The vertices (9 floats) and ids of triangles [first, first + n) in the
 * order they were added (OptimisedTriangle.Vertex, raytracer/cache/
 * optimisedtriangle.go:22-28, reading x, y, z). */
int vrg_env_get_triangle_vertices(const vrg_env *env, int64_t first, int64_t n, float *xyz,
                                  int32_t *ids);
/* SetupAccelerationStructure (environment.go:119-138): builds on the host
 * and uploads the tree the device walks (the walk tree: the reference's node
 * format, SAH over every candidate plane) with the intersection records;
 * they stay resident.  The reference's own tree (its candidates, costs and
 * partition order) is built when vrg_env_tree_info or vrg_env_get_tree first
 * asks for it.  Both trees give the same answers: every query returns what
 * testing every triangle would. */
int vrg_env_setup_acceleration_structure(vrg_env *env);
int64_t vrg_env_num_triangles(const vrg_env *env);
/* Size of the reference's tree: nodes, triangle-index-list length, height. */
int vrg_env_tree_info(const vrg_env *env, int64_t *nodes, int64_t *refs, int32_t *height);
/* OptimizedKDTree (children word, split float) and TriangleIndexList. */
int vrg_env_get_tree(const vrg_env *env, uint32_t *children, float *split, int32_t *refs);
/* SAH costs of the walk tree (defaults 1, 1.2, 0.9, 28): a split costs
 * traversal + intersection * (P_left * N_left + P_right * N_right), times
 * empty_bonus when a side is empty; depth at most max_depth (< 32).  Only
 * before vrg_env_setup_acceleration_structure. */
int vrg_env_set_walk_tree_costs(vrg_env *env, float traversal, float intersection,
                                float empty_bonus, int32_t max_depth);
/* Wall cells: per face of the scene box (face 2*axis + 1 for a max side),
 * the opaque triangles lying in that face (a room's walls and floor, or the
 * brush sides a map's walls are made of): up to 4 per face in fixed slots
 * when no face has more, otherwise a grid over each face whose cells list
 * the triangles overlapping them.  A shadow line of the gathers first tests
 * the slots or the cell of the face through which it leaves the box: a hit
 * before the sky region occludes it whatever lies in between, so the walk
 * is skipped.
 * This call reports, per face, the number of such triangles (at most 4
 * counted) and the first 4, largest first (tris[4*face+i], -1 unused).
 * (no reference counterpart) */
int vrg_env_wall_slots(const vrg_env *env, int32_t *tris, int32_t *counts);
/* Wall cells on (1, the default) or off (0: every line is walked; the
 * answers are the same).  Only before vrg_env_setup_acceleration_structure.
 * (no reference counterpart) */
int vrg_env_set_wall_slots(vrg_env *env, int32_t enable);
/* Where the walk tree is built: 0 on the host (every extent boundary a
 * candidate plane), 1 or -1 (default) on the context's GPU (nodes of up to
 * 512 triangles weigh every extent boundary, larger ones the first start
 * and last end in each of 256 bins per axis).  A host-only context always
 * builds on the host.  Only before vrg_env_setup_acceleration_structure. */
int vrg_env_set_walk_tree_builder(vrg_env *env, int32_t mode);
/* The walk tree, in the format of vrg_env_tree_info / vrg_env_get_tree. */
int vrg_env_walk_tree_info(const vrg_env *env, int64_t *nodes, int64_t *refs, int32_t *height);
int vrg_env_get_walk_tree(const vrg_env *env, uint32_t *children, float *split, int32_t *refs);
/* GetTriangle (environment.go:422-424): the 48-byte TriIntersectData
 * (raytracer/cache/triangle/triintersectdata.go:3-22) of triangle `index`. */
int vrg_env_get_triangle(const vrg_env *env, int64_t index, void *out48);
int vrg_env_bounds(const vrg_env *env, float *mins, float *maxs);

/* Trace4Rays (environment.go:140-145; FourRays raytracer/types/fourrays.go:8-11,
 * RayTracingResult raytracer/types/result.go:8-12).  origin/direction are
 * FourVectors in x x x x y y y y z z z z order; hit_ids[i] = triangle index or
 * -1; surface_normal (may be NULL) in the same SoA order. */
int vrg_env_trace4_rays(vrg_env *env, const float *origin, const float *direction,
                        const float *tmin, const float *tmax, int32_t skip_id, int32_t *hit_ids,
                        float *hit_distance, float *surface_normal);
/* Closest hit of n rays (origin/direction 3 floats each, AoS); the batched
 * form of Trace4Rays. */
int vrg_env_trace_closest(vrg_env *env, const float *origin, const float *direction,
                          const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                          int32_t *out_hit, float *out_t);
int vrg_env_trace_closest_d(vrg_env *env, const float *origin, const float *direction,
                            const float *tmin, const float *tmax, int64_t n, int32_t skip_id,
                            int32_t *out_hit, float *out_t);
/* TestLineDoesHitSky (raytracer/trace/testline.go:18-94) for n lines:
 * fraction_visible[i] is 1 or 0; the skip id is TRACE_ID_STATICPROP |
 * static_prop_to_skip as at testline.go:36. */
int vrg_env_test_line_does_hit_sky(vrg_env *env, const float *start, const float *stop,
                                   int64_t n, int32_t static_prop_to_skip,
                                   float *fraction_visible);

/* Transparent shadows.  Trace4Rays with a transparent-triangle callback
 * (environment.go:140-142) that counts coverage as types.CoverageCount does
 * (raytracer/types/coverageCount.go:27-41: each transparent hit adds its
 * triangle's colour x, clamped at 1).  The reference never fixes the order
 * in which hits reach the callback; here a ray's accepted hits are taken in
 * ascending (t, triangle index): an opaque hit is recorded and ends the walk,
 * a transparent one (VRG_TRIFLAG_TRANSPARENT) adds coverage and, when the sum
 * reaches 1, is recorded and ends it.  Per ray: the recorded hit (-1 none),
 * its t (+inf none) and the coverage.  Host buffers; origins and unit
 * directions as in vrg_env_trace_closest. */
int vrg_env_trace_coverage(vrg_env *env, const float *origin, const float *direction, const float *tmin,
                           const float *tmax, int64_t n, int32_t skip_id, int32_t *out_hit, float *out_t,
                           float *out_coverage);
/* TestLineDoesHitSky with texture shadows on (raytracer/trace/testline.go:29-33,
 * 53-55): occlusion = max(1 if the recorded hit lies before the stop point
 * and is not TRACE_ID_SKY, coverage), clamped; fraction_visible = 1 -
 * occlusion.  Texture coverage is a stub in the reference
 * (rad/staticprops/compute.go:4-12); the triangle's colour x stands for it,
 * as in CoverageCount. */
int vrg_env_test_line_coverage(vrg_env *env, const float *start, const float *stop, int64_t n,
                               int32_t static_prop_to_skip, float *fraction_visible);
/* Flags and colours of triangles [first, first + n) added earlier (the bulk
 * form of AddTriangleWithMaterial's flags and colour, environment.go:45-66;
 * no counterpart in the reference); colours (3 per triangle) may be NULL.
 * Only before SetupAccelerationStructure. */
int vrg_env_set_triangle_flags(vrg_env *env, int64_t first, int64_t n, const uint8_t *flags,
                               const float *colours);
/* Shadow lines as a 1-bit mask (bit i%32 of word i/32 set = occluded), with
 * the same semantics; out_hit/out_t (may be NULL) add the closest hit of the
 * normalised segment. */
int vrg_env_occlusion_mask(vrg_env *env, const float *start, const float *stop, int64_t n,
                           int32_t skip_id, uint32_t *out_mask, int32_t *out_hit, float *out_t);
int vrg_env_occlusion_mask_d(vrg_env *env, const float *start, const float *stop, int64_t n,
                             int32_t skip_id, uint32_t *out_mask, int32_t *out_hit, float *out_t);
/* CanLeafTraceToSky (rad/lightmap/lightmap.go:425-451) for n leaves given
 * by their integer bounds (leaf_mins / leaf_maxs: n x 3, the BSP leaf's
 * mins and maxs): from the centre (float)(mins + maxs) * 0.5, one shadow
 * line per Anorms direction a_j (162) to a_j * -MAX_TRACE_LENGTH + centre
 * (per component, float32), with TestLineDoesHitSky's semantics and no
 * static prop skipped; out[i] = 1 when any line's fraction visible is above
 * 0.  The reference traces from the origin (its centre vector is never
 * loaded, lightmap.go:432) and its direction loader keeps only x
 * (vmath/ssemath/fourvectors.go:15-28); here the lines leave the centre. */
int vrg_env_can_leaf_trace_to_sky(vrg_env *env, const int32_t *leaf_mins, const int32_t *leaf_maxs,
                                  int64_t n, uint8_t *out);
/* The lines vrg_env_can_leaf_trace_to_sky traces (n x 162 starts and stops,
 * 3 floats each, leaf-major).  Host only; needs no context. */
int vrg_leaf_sky_lines(const int32_t *leaf_mins, const int32_t *leaf_maxs, int64_t n, float *starts,
                       float *stops);
/* Ray stream (AddToRayStream / FlushStreamEntry / FinishRayStream,
 * environment.go:162-175): lines are queued on the host, traced in large
 * batches, and their fraction_visible values are returned in queue order. */
int vrg_env_add_to_ray_stream(vrg_env *env, const float *start, const float *stop,
                              int32_t skip_id);
int vrg_env_flush_stream_entry(vrg_env *env);
int vrg_env_finish_ray_stream(vrg_env *env, float *fraction_visible, int64_t capacity,
                              int64_t *count);

/* ------------------------------------------------------------------ */
/* Lights: rad/lightmap/lights.go                                       */
/* ------------------------------------------------------------------ */

/* SetLightFalloffParams (lights.go:259-341) */
int vrg_light_set_falloff_params(const vrg_light_keys *keys, vrg_light *light);
/* ParseLightSpot (lights.go:210-257) without the entity parse: origin,
 * intensity and normal are set by the caller. */
int vrg_light_parse_spot(const vrg_light_keys *keys, vrg_light *light);
/* ParseLightPoint (lights.go:417-426) */
int vrg_light_parse_point(const vrg_light_keys *keys, vrg_light *light);
/* The active light list CreateDirectLights (lights.go:38-116) produces,
 * copied to the device. */
int vrg_env_set_lights(vrg_env *env, const vrg_light *lights, int32_t n);

/* ------------------------------------------------------------------ */
/* Faces, luxels and the direct-light gather                            */
/* ------------------------------------------------------------------ */

/* Lightmapped faces: axis-aligned rectangles corner + s*u + t*v with unit
 * normal, nu x nv luxels (the extents CalcFaceExtents computes,
 * rad/world/face.go:14-90), luxscale = luxels per world unit,
 * reflectivity/baselight RGB (BaseLightForFace, rad/patches/face.go:210-231;
 * reflectivity is clamped to 0.99).  tri_face (ntris entries) maps each
 * triangle to its face or -1.  NULL reflectivity/baselight mean 0. */
int vrg_env_set_faces(vrg_env *env, int32_t nfaces, const float *corner, const float *u,
                      const float *v, const float *normal, const int32_t *nu, const int32_t *nv,
                      const float *luxscale, const float *reflectivity, const float *baselight,
                      const int32_t *tri_face);
int64_t vrg_env_num_luxels(const vrg_env *env);
/* Direct light of every luxel (RGB, luxel order = face order, row-major
 * nu x nv), averaged over `supersamples` (1 or 4) seeded samples. */
int vrg_env_gather_direct_light(vrg_env *env, int32_t supersamples, uint64_t seed,
                                float *out_rgb, uint64_t *out_shadow_rays);
int vrg_env_gather_direct_light_d(vrg_env *env, int32_t supersamples, uint64_t seed,
                                  float *out_rgb, uint64_t *out_shadow_rays);
/* Direct light at n explicit points with normals. */
int vrg_env_gather_points(vrg_env *env, const float *points, const float *normals, int64_t n,
                          float *out_rgb, uint64_t *out_shadow_rays);

/* ------------------------------------------------------------------ */
/* Patches, transfers, bounce: rad/patches, common/types/patch.go       */
/* ------------------------------------------------------------------ */

/* MakePatches + SubdividePatches (rad/patches/build.go:21-68,
 * subdivide.go:25-251) for the faces set above. */
int vrg_env_make_patches(vrg_env *env, float max_chop, float min_chop, int64_t *num_patches,
                         int64_t *num_leaves);
/* All patches (parents included); any pointer may be NULL. */
int vrg_env_get_patches(const vrg_env *env, float *mins, float *maxs, float *center, float *area,
                        int32_t *face, int32_t *parent, int32_t *child1, int32_t *child2,
                        int32_t *split_axis, float *split_dist, int32_t *leaf_index);
/* Transfer lists (Patch.NumTransfers/Transfers, common/types/patch.go:60-61,
 * Transfer common/types/transfer.go:3-6) of every leaf patch, from k
 * closest-hit rays along dirs_local (k x 3, local frame: tangent, bitangent,
 * normal; k a power of two in [32, 65536]).  Built on the device into CSR
 * and kept resident. */
int vrg_env_make_transfers(vrg_env *env, const float *dirs_local, int32_t k, int64_t *out_nnz);
/* CSR copy-out: row_ptr[leaves+1], col[nnz], weight[nnz] (= hits / k). */
int vrg_env_get_transfers(const vrg_env *env, int64_t *row_ptr, int32_t *col, float *weight);
/* The last build's ray count k, entry count, and how many of its rows had
 * more distinct targets than the shared-memory row table holds (those rows
 * are rebuilt by a global-memory sort; the CSR is the same either way).
 * (no reference counterpart: transfer building is absent there) */
int vrg_env_transfer_info(const vrg_env *env, int32_t *k, int64_t *nnz, int64_t *overflow_rows);
/* Distinct targets a transfer row may collect in its shared-memory table
 * before the row is rebuilt by the global-memory sort (default and maximum
 * 7168; a lower limit sends more rows down that path, which tests use).
 * (no reference counterpart) */
int vrg_ctx_set_transfer_table_limit(vrg_ctx *ctx, int32_t limit);
/* Direct light at every leaf patch (one sample at centre + 0.125 * normal). */
int vrg_env_gather_patch_direct(vrg_env *env, float *out_rgb);
/* Bounce loop: emit = refl * direct + baselight; per bounce add = T emit,
 * total += add, emit = refl * add; stop after the bounce whose energy delta
 * sum|add| / sum|total| < rel_tol, or after max_bounces.  out_total (leaves x
 * 3, may be NULL) is the bounced light (TotalLight, patch.go:33). */
int vrg_env_bounce_light(vrg_env *env, int32_t max_bounces, float rel_tol, float *out_total,
                         int32_t *out_bounces, float *out_delta);
/* The same bounce loop for callers that may not allocate device memory while
 * they run (a serving loop that reserved its memory up front, a process whose
 * device memory is carved out in advance by a framework pool, code that must
 * not trigger the device-wide synchronisation of cudaMalloc/cudaFree).  This
 * call allocates nothing: its working state lives in one fixed device array
 * of 8 MiB + 16 KiB that every GPU loading the library holds until exit, so a
 * scene may have at most 262144 leaf patches (larger scenes get
 * VRG_ERR_UNSUPPORTED).  total_out is a DEVICE buffer of this context's
 * GPU, 16-byte aligned, of 4 floats per leaf (RGB + padding); a host pointer,
 * another GPU's memory or a misaligned pointer is refused with
 * VRG_ERR_INVALID before anything is launched.  The result lives only in
 * total_out: vrg_env_get_bake and vrg_env_get_lightmap keep returning the
 * scene's last allocating bake.  vrg_env_make_transfers and
 * vrg_env_gather_patch_direct must have run.  vrg_ctx_create already looks
 * up the array's device address and loads this call's kernels, so every
 * call, the first included, allocates nothing (if that set-up failed, the
 * first call retries it).  All calls on a device share the one array, so
 * calls that overlap on the GPU (two streams, two threads) race: serialise
 * them.  No counterpart in the reference. */
int vrg_env_bounce_light_noalloc(vrg_env *env, int32_t max_bounces, float rel_tol,
                                 float *total_out, int32_t *out_bounces, float *out_delta);

/* ------------------------------------------------------------------ */
/* Whole bakes: one scene, or many resident scenes batched              */
/* (RadWorld_Go's direct pass and bounce, cmd/tasks/computerad/main.go:7) */
/* ------------------------------------------------------------------ */

typedef struct vrg_batch vrg_batch;

/* One scene: direct light of every luxel and leaf patch, then the bounce
 * loop; results stay on the device (read them with vrg_env_get_bake).  The
 * scene needs lights, faces, patches and transfers. */
int vrg_env_bake(vrg_env *env, int32_t supersamples, uint64_t seed, int32_t max_bounces,
                 float rel_tol, uint64_t *out_shadow_rays);
/* Results of the last bake of this scene (any pointer may be NULL):
 * luxel RGB, leaf-patch direct light and bounced light (3 floats each),
 * bounces run and the final energy delta. */
int vrg_env_get_bake(vrg_env *env, float *luxel_rgb, float *patch_direct, float *patch_total,
                     int32_t *bounces, float *delta);

/* ------------------------------------------------------------------ */
/* Lightmap output: face extents and lightmap samples                  */
/* (rad/world/face.go:14-90; cmd/tasks/finish/main.go:8-40 is a stub)  */
/* ------------------------------------------------------------------ */

/* CalcFaceExtents (rad/world/face.go:14-90) for one face: vertices (nverts
 * x 3, winding order -- the surfedge walk of face.go:29-36 resolved by the
 * caller: edge e >= 0 gives vertex edges[e][0], e < 0 gives edges[-e][1]),
 * lightmap_vecs = the texinfo's LightmapVecsLuxelsPerWorldUnits (2 x 4).
 * Writes LightmapTextureMinsInLuxels and LightmapTextureSizeInLuxels (the
 * reference passes them by value and loses them, rad/start.go:110).
 * *too_big (may be NULL) = 1 when a size exceeds 125 + 1, which the
 * reference logs and carries on from.  Host only; needs no context. */
int vrg_calc_face_extents(const float *vertices, int32_t nverts, const float *lightmap_vecs,
                          int32_t *mins, int32_t *size, int32_t *too_big);
/* Lightmap samples of the last bake (or relight) of this scene: per luxel,
 * in the luxel order of vrg_env_gather_direct_light, the direct light plus
 * the bounced light (TotalLight, common/types/patch.go:33) of the leaf patch
 * holding the luxel centre, as one 4-byte shared-exponent sample
 * {r, g, b, signed exponent x}, channel = byte * 2^x, x = max(e - 8, -128)
 * for the largest channel m = f * 2^e (0.5 <= f < 1), byte = floor(channel
 * * 2^-x); channels that are not > 0 store 0.  samples: 4 x num_luxels
 * bytes; face_offset: nfaces + 1 byte offsets of each face's first sample
 * (its lightofs in a lighting lump of one style).  Either may be NULL.
 * Needs a bake of the current faces and patches (VRG_ERR_STATE otherwise). */
int vrg_env_get_lightmap(vrg_env *env, uint8_t *samples, int64_t *face_offset);
/* A batch of resident scenes baked together: the direct pass of every
 * scene in one persistent launch over a device work queue, then one
 * block-diagonal bounce loop (CUDA graph) with a per-scene stop. */
int vrg_batch_create(vrg_ctx *ctx, vrg_batch **out);
void vrg_batch_destroy(vrg_batch *batch);
int vrg_batch_add(vrg_batch *batch, vrg_env *env);
int32_t vrg_batch_size(const vrg_batch *batch);
int vrg_batch_bake(vrg_batch *batch, int32_t supersamples, uint64_t seed, int32_t max_bounces,
                   float rel_tol, uint64_t *out_shadow_rays);

/* ------------------------------------------------------------------ */
/* Relighting resident scenes, and a server for relight requests        */
/* ------------------------------------------------------------------ */

/* Replace light `index` of a scene's light table with `light`. */
typedef struct vrg_light_edit {
    int32_t index;
    vrg_light light;
} vrg_light_edit;

typedef struct vrg_server vrg_server;

/* Bake a scene (as vrg_env_bake) and keep, per luxel sample and leaf point,
 * the multiplier of each sky-type light and one visibility bit per light, so
 * that later light edits re-trace only the edited lights.  Admission: checks
 * free device memory first (VRG_ERR_NOMEM when the scene's relight state does
 * not fit with the context's HBM reserve to spare). */
int vrg_env_relight_prepare(vrg_env *env, int32_t supersamples, uint64_t seed,
                            int32_t max_bounces, float rel_tol);
/* Device memory that admission keeps free for other work (default 1 GiB). */
int vrg_ctx_set_hbm_reserve(vrg_ctx *ctx, uint64_t bytes);
/* Apply light edits and update the scene: luxels and leaf points of the faces
 * within the old or new radius of an edited light are re-gathered (the same
 * values a full gather would give), then the bounce restarts from the
 * resident solution until the relative change falls below rel_tol or
 * max_iters iterations.  Sky-type lights may change intensity only. */
int vrg_env_relight(vrg_env *env, const vrg_light_edit *edits, int32_t n, int32_t max_iters,
                    float rel_tol, int32_t *out_bounces, float *out_delta);
/* A relight server with `slots` concurrent requests (one CUDA stream each).
 * A worker thread admits pending requests into free slots as soon as they
 * free up; requests on different scenes overlap on the GPU, requests on the
 * same scene run in submission order.  A scene added to a server must only
 * be changed through it while the server lives: in particular it must not be
 * relit with vrg_env_relight meanwhile, since both use the scene's one bounce
 * control block and loop graph. */
int vrg_server_create(vrg_ctx *ctx, int32_t slots, int32_t max_iters, float rel_tol,
                      vrg_server **out);
void vrg_server_destroy(vrg_server *server);
int vrg_server_add_scene(vrg_server *server, vrg_env *env, int32_t *scene_id);
int vrg_server_submit(vrg_server *server, int32_t scene_id, const vrg_light_edit *edits,
                      int32_t n, int64_t *ticket);
/* Waits for one request (returns its status: 0 done, negative error) or for
 * every submitted request; VRG_ERR_TIMEOUT after timeout_s seconds. */
int vrg_server_wait(vrg_server *server, int64_t ticket, double timeout_s);
int vrg_server_drain(vrg_server *server, double timeout_s);
/* times = {submitted, started, finished} (seconds, steady clock);
 * digest = {sum of the scene's luxel RGB, sum of its bounced light} after
 * the request. */
int vrg_server_result(vrg_server *server, int64_t ticket, int32_t *status, int32_t *bounces,
                      float *delta, double *times, double *digest);

#ifdef __cplusplus
}
#endif
#endif
