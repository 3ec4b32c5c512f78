// vrg_internal.h -- host-side state behind the C ABI in include/vradgpu.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vradgpu.h"
#include "vrg_device.h"

namespace vrg {

// kd-tree SAH constants (raytracer/kdtree/constants.go:25-28)
constexpr int kCostOfTraversal = 75;
constexpr int kCostOfIntersection = 167;
constexpr int kMaxTreeDepth = 21;
constexpr uint32_t kLeaf = 3;  // KDNODE_STATE_LEAF (raytracer/cache/optimisedkdnode.go:6)
// MAX_LIGHTMAP_DIM_WITHOUT_BORDER = MAX_DISP_LIGHTMAP_DIM_WITHOUT_BORDER
// (common/constants/constants.go:22,27)
constexpr int32_t kMaxLightmapDim = 125;

struct Error {
    int code;
    std::string msg;
};

// Owns a device allocation.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    // (re)allocates when the capacity is too small; contents are not kept
    cudaError_t reserve(size_t n) {
        if (n <= bytes && ptr) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess) bytes = n;
        else ptr = nullptr;
        return e;
    }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

struct RelightState;  // relight.cu: serial scratch and loop graphs of a scene
struct BounceGraph;   // bounce.cu: the scene's bounce loop as a graph

struct KernelStat {
    double ms = 0.0;
    int64_t launches = 0;
};

struct PendingTiming {
    std::string name;
    cudaEvent_t start, stop;
};

}  // namespace vrg

struct vrg_ctx {
    int device = 0;
    bool host_only = false;  // created with device < 0: host algorithms only
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    mutable std::mutex mu;
    std::string last_error;
    bool timing = false;
    std::map<std::string, vrg::KernelStat> stats;
    std::vector<vrg::PendingTiming> pending;
    std::vector<cudaEvent_t> event_pool;
    int64_t launches = 0;
    bool autotune = true;
    uint64_t hbm_reserve = (uint64_t)1 << 30;  // kept free when admitting a relight scene
    int32_t xfer_table_limit = 7168;            // distinct targets per transfer row held in shared memory
    std::map<std::string, int> tuned;                   // bucket key -> variant
    std::map<std::string, std::vector<double>> tune_ms;  // bucket key -> variant times
};

// Built kd tree + intersection records (host copy).
struct HostTree {
    std::vector<uint32_t> children;
    std::vector<float> split;
    std::vector<int32_t> refs;
    int height = 0;
};

// SAH costs of the tree the device walks (build_walk_tree).  Measured on
// the 12,300-triangle any-hit room and the 8,208-triangle direct-light room:
// intersection costs from 0.8 to 10 and empty-space bonuses from 0.7 to 1
// give walks within 5 % of each other; 1.2 and 0.9 make the smallest trees
// that keep the direct-light gather fastest (16.0 ms against 16.6 at 1.5 /
// 0.8), at 1-2 % of the any-hit walk.
struct WalkTreeCosts {
    float traversal = 1.0f;
    float intersection = 1.2f;
    float empty_bonus = 0.9f;
    int max_depth = 28;  // below the traversal stack (kStackMax)
};

struct PatchSet {
    // all patches, parents included, in creation order
    std::vector<float> mins, maxs, center, area, split_dist;
    std::vector<int32_t> face, parent, child1, child2, split_axis, leaf_index;
    std::vector<int32_t> face_root;  // face -> root patch (or -1)
    std::vector<int32_t> leaf_patch; // dense leaf -> patch index
};

struct vrg_env {
    vrg_ctx *ctx = nullptr;
    mutable std::mutex mu;  // const readers (tree and triangle getters) lock it too

    // Environment fields (raytracer/environment.go:28-39)
    std::vector<float> xyz;  // 9 per triangle (TriGeometryData.VertexCoordData)
    std::vector<int32_t> ids;
    std::vector<uint8_t> flags;
    std::vector<float> colours;
    std::vector<float> cover;  // per triangle: colour x, the coverage of a transparent triangle
    std::vector<int32_t> materials;
    float min_bound[3] = {0, 0, 0}, max_bound[3] = {0, 0, 0};

    bool built = false;
    HostTree tree;        // the reference's tree, built on first request
    bool ref_tree_built = false;
    HostTree walk_tree;   // the tree the device walks (build_walk_tree)
    int32_t wall_tris[6 * vrg::kWallSlots];  // wall slots per scene-box face (-1: unused)
    int32_t wall_counts[6] = {0, 0, 0, 0, 0, 0};
    std::vector<uint32_t> wall_cells;  // the wall-cell table (see vrg_device.h)
    size_t n_wall_records = 0;          // wall triangles' leaf records after the leaf entries
    int wall_layout = 0;                // 0: wall slots, 1: wall cells (see vrg_device.h)
    WalkTreeCosts walk_costs;
    int walk_builder = -1;  // walk tree: 0 host (full sweep), 1 GPU (binned), -1 by size
    bool use_wall_slots = true;  // shadow lines test their exit face's walls before walking
    std::vector<vrg::TriRecord> tri_records;  // per triangle, insertion order
    vrg::SceneGeom geom{};                     // bounds, sky box, scale

    // device scene
    vrg::DevBuf d_nodes, d_leaf_tris, d_tri_ids, d_tri_normals;
    vrg::DevBuf d_top;       // top levels of the tree (kTopNodes entries at most)
    uint32_t ntop = 0;

    // transparent shadows (coverage.cu): per-triangle flags and coverage
    vrg::DevBuf d_tri_flags, d_tri_cover;
    bool cover_ready = false;
    int32_t n_transparent = 0;

    // lights
    std::vector<vrg_light> lights;
    vrg::DevBuf d_lights;

    // faces
    int32_t nfaces = 0;
    std::vector<float> f_corner, f_u, f_v, f_normal, f_luxscale, f_refl, f_base;
    std::vector<int32_t> f_nu, f_nv, tri_face;
    std::vector<int64_t> luxel_offset;
    vrg::DevBuf d_faces, d_luxel_offset, d_tri_face;

    // patches / transfers / bounce
    bool have_patches = false;
    PatchSet patches;
    vrg::DevBuf d_patch_nodes, d_leaf_info, d_face_root;
    vrg::DevBuf d_face_tree;  // int4 per face: see face_tree_ranges (capi.cpp)
    bool have_transfers = false;
    int64_t nnz = 0;
    int32_t transfer_k = 0;
    int64_t transfer_overflow_rows = 0;  // rows of the last build past the shared-memory row table
    vrg::DevBuf d_row_ptr, d_col, d_weight;
    vrg::DevBuf d_leaf_direct;
    bool have_patch_direct = false;
    vrg::DevBuf d_emit, d_total, d_partials, d_control;
    vrg::DevBuf d_patch_pts, d_patch_nrm;  // leaf sample points (centre + 0.125 N), resident
    vrg::DevBuf d_bake_rgb;                 // luxel RGB of the last bake
    bool have_bake = false;
    int32_t bake_bounces = 0;
    float bake_delta = 0.0f;

    // relighting: sky multipliers cached per sample, warm-start bounce state
    bool relight_ready = false;
    int32_t relight_ss = 4;
    uint64_t relight_seed = 0;
    int32_t sky_slots = 0;
    int32_t vis_words = 0;                  // visibility-cache words per sample / point
    vrg::DevBuf d_sky_lux, d_sky_pts, d_emit0, d_x;
    vrg::DevBuf d_vis_lux, d_vis_pts;       // point/spot shadow-line bits per sample / point
    vrg::RelightState *relight = nullptr;   // owned; freed by relight_release
    vrg::BounceGraph *bounce_graph = nullptr;  // owned; freed by bounce_release
    std::vector<float> face_mid, face_ext;      // face centres / padded half extents, axis-major ([a * nfaces + f])
    std::vector<int32_t> face_leaf_begin;     // leaves of face f: [begin[f], begin[f+1])

    // scratch for host-buffer entry points
    vrg::DevBuf d_in0, d_in1, d_out0, d_out1, d_out2, d_counter;
    vrg::DevBuf d_work;  // work-queue counters of the persistent kernels

    // ray stream queue
    std::vector<float> rs_start, rs_stop;
    std::vector<int32_t> rs_skip;
};

namespace vrg {

// error plumbing
int fail(vrg_ctx *ctx, int code, const std::string &msg);
int cuda_fail(vrg_ctx *ctx, cudaError_t e, const char *what);
#define VRG_CUDA(ctx, call)                                  \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return vrg::cuda_fail((ctx), _e, #call); \
    } while (0)

// per-scene-size autotuning (tune.cpp).  tune_pick returns the bucket's
// variant, first timing every variant through `launch` when the bucket is
// new; tune_run then launches the chosen one unless tuning just did.
std::string tune_key(const char *kernel, int64_t scene_size, int64_t work);
constexpr int kTuneMaxVariants = 32;  // variants of one launch site, at most
int tune_pick(vrg_ctx *ctx, const std::string &key, int nvar,
              const std::function<cudaError_t(int)> &launch, int *variant);
int tune_run(vrg_ctx *ctx, const std::string &key, int nvar,
             const std::function<cudaError_t(int)> &launch);

// timing around kernel launches
void timing_begin(vrg_ctx *ctx, const char *name, cudaEvent_t *start);
void timing_end(vrg_ctx *ctx, const char *name, cudaEvent_t start);
void collect_timings(vrg_ctx *ctx);

// host algorithms (C++)
void tri_intersect_format(const float *xyz9, int32_t id, uint8_t flags, TriRecord *out,
                          uint32_t tri_index);
void edge_equation(const float *p1, const float *p2, int c1, int c2, const float *inside,
                   float *out3);
void scene_bounds(const std::vector<float> &xyz, float *mn, float *mx);
void build_kd_tree(const std::vector<float> &xyz, HostTree &tree, float *mn, float *mx);
void build_walk_tree(const std::vector<float> &xyz, const float *mn, const float *mx,
                     const WalkTreeCosts &cost, HostTree &tree);
int build_walk_tree_device(vrg_env *env, HostTree &tree);  // kdbuild_gpu.cu
void light_set_falloff(const vrg_light_keys &k, vrg_light &l);
void light_parse_spot(const vrg_light_keys &k, vrg_light &l);
int make_rect_patches(const vrg_env &env, float max_chop, float min_chop, PatchSet &out);

// device launchers (trace.cu, direct.cu, transfer.cu, bounce.cu)
DevScene scene_view(const vrg_env *env);
int launch_occlusion_mask(vrg_env *env, const float *start, const float *stop, int64_t n,
                          int32_t skip_id, uint32_t *mask, int32_t *hit, float *t);
int launch_trace_closest(vrg_env *env, const float *orig, const float *dir, const float *tmin,
                         const float *tmax, int64_t n, int32_t skip_id, int32_t *hit, float *t);
int launch_test_lines(vrg_env *env, const float *start, const float *stop, int64_t n,
                      int32_t skip_id, float *frac);
// Luxel samples of every face, then (optionally) npts extra sample points
// in the same persistent launch.
int launch_gather_luxels(vrg_env *env, int ss, uint64_t seed, float *out_rgb,
                         unsigned long long *d_rays, const float *pts = nullptr,
                         const float *nrm = nullptr, int64_t npts = 0, float *pts_out = nullptr);
int launch_gather_points(vrg_env *env, const float *pts, const float *nrm, int64_t n,
                         float *out_rgb, unsigned long long *d_rays);
void pack_lights(const std::vector<vrg_light> &src, std::vector<float4> &dst);
int run_make_transfers(vrg_env *env, const float *dirs_local, int32_t k);
int run_bounce(vrg_env *env, int32_t max_bounces, float rel_tol, int32_t *bounces,
               float *delta);
void relight_release(vrg_env *env);
void bounce_release(vrg_env *env);
int noalloc_prepare(vrg_ctx *ctx);  // bounce.cu: the no-alloc bounce's array and kernels
// Inner nodes on the longest root-to-leaf path (environment.cpp).
int inner_depth(const std::vector<uint32_t> &children);

}  // namespace vrg
