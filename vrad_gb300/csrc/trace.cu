// trace.cu -- batched ray queries against a resident scene (Trace4Rays,
// raytracer/environment.go:140-145, and TestLineDoesHitSky,
// raytracer/trace/testline.go:18-94).
#include "vrg_internal.h"
#include "vrg_trace.cuh"

namespace vrg {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ void load3(const float *p, int64_t i, float &x, float &y, float &z) {
    x = __ldg(p + 3 * i);
    y = __ldg(p + 3 * i + 1);
    z = __ldg(p + 3 * i + 2);
}

// The refill loops read each line's end points when a lane takes the line,
// one lane at a time and out of step with its neighbours, so a line that is
// not yet in L2 costs the lane a full HBM round trip.  At launch every
// thread asks L2 for its share of the two end-point arrays (128-byte lines,
// addresses inside the arrays only), so they stream in at full bandwidth
// instead.
__device__ __forceinline__ void prefetch_lines(const float *start, const float *stop, int64_t n) {
    const int64_t bytes = 12 * n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x * 128;
    const char *a = reinterpret_cast<const char *>(start), *b = reinterpret_cast<const char *>(stop);
    for (int64_t off = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 128; off < bytes; off += stride) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a + off));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(b + off));
    }
}

// Shadow lines with per-lane refill.  Independent lines diverge: some stop
// at their first leaf, some cross the whole scene.  Each lane therefore
// walks its own line one leaf at a time, and as soon as a lane's line is
// done the warp hands it the next unclaimed line (one atomic per refill on
// a device counter zeroed before the launch).  The occlusion bit goes into
// the 1-bit mask with an atomic OR (the mask is zeroed before the launch).
// WANT_HIT also writes the closest hit of the normalised segment.
template <bool WANT_HIT, int LB, int OPT = 0>
__global__ void __launch_bounds__(kThreads) k_trace_mask(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, uint32_t *__restrict__ mask,
                                                          int32_t *__restrict__ hit,
                                                          float *__restrict__ thit,
                                                          unsigned long long *__restrict__ work) {
    if (OPT & kOptTop) stage_top(s);
    prefetch_lines(start, stop, n);
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int64_t ri = 0;
    LinePlan p;
    TraceState st;
    for (;;) {
        const unsigned idle = __ballot_sync(full, !active && !exhausted);
        if (idle == 0 && !__any_sync(full, active)) break;
        if (idle) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (!active && !exhausted) {
                const int64_t i = (int64_t)base + __popc(idle & below);
                if (i >= n) {
                    exhausted = true;
                } else {
                    ri = i;
                    float sx, sy, sz, ex, ey, ez;
                    load3(start, i, sx, sy, sz);
                    load3(stop, i, ex, ey, ez);
                    p = plan_line(s, make_line(sx, sy, sz, ex, ey, ez));
                    active = !p.trivial && trace_init(s, p.ray, p.rp, p.slack, 0.0f, p.len, st, root_ref<OPT>(s));
                    if (!active && WANT_HIT) {
                        hit[ri] = -1;
                        thit[ri] = kInf;
                    }
                }
            }
        }
        if (active) {
            const bool done =
                WANT_HIT ? trace_step<kClosest, LB, OPT>(s, p.ray, p.rp, 0.0f, p.len, skip, 0.0f, st)
                         : trace_step<kSkyOcc, LB, OPT>(s, p.ray, p.rp, 0.0f, p.len, skip, p.any_limit, st);
            if (done) {
                active = false;
                bool occ;
                if (WANT_HIT) {
                    hit[ri] = st.best;
                    thit[ri] = st.best_t;
                    occ = st.best >= 0 && st.best_t < p.len &&
                          (__ldg(&s.tri_ids[st.best]) & kTraceIdSky) == 0;
                } else {
                    occ = line_verdict(s, p, st.best, st.best_t);
                }
                if (occ) atomicOr(mask + (ri >> 5), 1u << (ri & 31));
            }
        }
    }
}

// Shadow lines walked one unit of work per lane per round: each round every
// busy lane either steps through one inner node or tests one triangle (a
// lane that arrives at a leaf takes its triangle range and tests the first
// one in the same round), so lanes at different depths and in leaves of
// different sizes advance together instead of waiting for the slowest lane
// of a descent or of a leaf (the "if-if" loop of Aila & Laine, HPG 2009).
// Finished lanes take new lines when at least THRESH lanes are idle (or
// none is busy), so the line setup runs for several lanes at once.  With
// VOTE a round runs only the kind of unit (node step or triangle test) that
// most lanes want, so the warp does not pay for both branches every round.
// MINB is the resident-block hint of __launch_bounds__ (register cap).
// Leaf order, pruning and tie rule are those of trace_step: same verdicts
// and closest hits.
template <bool WANT_HIT, int THRESH, bool VOTE, int MINB, int OPT = 0>
__global__ void __launch_bounds__(kThreads, MINB) k_trace_unit(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, uint32_t *__restrict__ mask,
                                                          int32_t *__restrict__ hit,
                                                          float *__restrict__ thit,
                                                          unsigned long long *__restrict__ work) {
    if (OPT & kOptTop) stage_top(s);
    prefetch_lines(start, stop, n);
    constexpr int MODE = WANT_HIT ? kClosest : kSkyOcc;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int64_t ri = 0;
    Ray ray{};
    RayPre rp{};
    float len = 0.0f, any_limit = 0.0f;
    uint32_t node = 0;
    uint2 nd = make_uint2(0u, 0u);
    float t0 = 0.0f, t1 = 0.0f;
    int sp = 0;
    uint32_t lpos = 0, lend = 0;  // triangles of the current leaf still to test
    float4 next_plane = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // kOptPipe: plane of lpos, loaded ahead
    bool have_next = false;
    int32_t best = -1;
    float best_t = kInf;
    uint4 stk[kStackMax];
    unsigned out_of_work = 0u;  // kOptOneVote: the lanes with `exhausted` set (warp-uniform)
    for (;;) {
        const unsigned busy = __ballot_sync(full, active);
        const unsigned idle = (OPT & kOptOneVote) ? ~busy & ~out_of_work
                                                  : __ballot_sync(full, !active && !exhausted);
        if (idle == 0 && busy == 0) break;
        if (idle != 0 && (__popc(idle) >= THRESH || busy == 0)) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (!active && !exhausted) {
                const int64_t i = (int64_t)base + __popc(idle & below);
                if (i >= n) {
                    exhausted = true;
                } else {
                    ri = i;
                    float sx, sy, sz, ex, ey, ez;
                    load3(start, i, sx, sy, sz);
                    load3(stop, i, ex, ey, ez);
                    const LinePlan p = plan_line(s, make_line(sx, sy, sz, ex, ey, ez));
                    ray = p.ray;
                    rp = p.rp;
                    if (OPT & kOptShRay) {
#pragma unroll
                        for (int a = 0; a < 3; a++)
                            g_ray_axes[a * kShRayLanes + threadIdx.x] = make_float4(
                                rp.inv[a], rp.A[a], rp.B[a], __uint_as_float((rp.neg >> a) & 1u));
                    }
                    len = p.len;
                    any_limit = p.any_limit;
                    best = -1;
                    best_t = kInf;
                    sp = 0;
                    lpos = lend = 0;
                    t0 = 0.0f;
                    t1 = p.len;
                    bool go = !p.trivial && s.g.ntris > 0;
                    if (go) {
                        clip_box(s.g.bmin, s.g.bmax, p.slack, ray, rp, t0, t1);
                        go = t0 <= t1;
                    }
                    if (go) {
                        node = root_ref<OPT>(s);
                        nd = fetch_node<OPT>(s, node);
                        active = true;
                    } else if (WANT_HIT) {
                        hit[ri] = -1;
                        thit[ri] = kInf;
                    }
                }
            }
            if (OPT & kOptOneVote) out_of_work = __ballot_sync(full, exhausted);
        }
        bool done = false;
        if (active && lpos == lend && (nd.x & 3u) == 3u) {
            lpos = nd.x >> 2;
            lend = lpos + (uint32_t)__uint_as_float(nd.y);
            have_next = false;
            if (lpos == lend) {  // empty leaf
                if (pop_next<MODE>(stk, sp, best_t, node, t0, t1))
                    nd = fetch_node<OPT>(s, node);
                else
                    done = true;
            }
        }
        // (a leaf popped after an empty one waits a round)
        bool run_tri = active && !done && lpos < lend;
        bool run_node = active && !done && lpos == lend && (nd.x & 3u) != 3u;
        if (VOTE) {
            const int ct = __popc(__ballot_sync(full, run_tri));
            const int cn = __popc(__ballot_sync(full, run_node));
            run_tri = run_tri && ct >= cn;
            run_node = run_node && cn > ct;
        }
        if (run_tri) {
            float4 w0;
            if (OPT & kOptPipe) {
                w0 = have_next ? next_plane : leaf_load<OPT>(s.leaf_planes + lpos);
                have_next = lpos + 1 < lend;
                if (have_next) next_plane = leaf_load<OPT>(s.leaf_planes + lpos + 1);
            } else {
                w0 = leaf_load<OPT>(s.leaf_planes + lpos);
            }
            if (tri_test<MODE, OPT>(s, ray, 0.0f, len, skip, any_limit, w0, lpos, best, best_t)) {
                done = true;
            } else if (++lpos == lend) {
                if (pop_next<MODE>(stk, sp, best_t, node, t0, t1))
                    nd = fetch_node<OPT>(s, node);
                else
                    done = true;
            }
        } else if (run_node) {
            if (inner_step<OPT>(rp, nd, t0, t1, stk, sp, node) ||
                pop_next<MODE>(stk, sp, best_t, node, t0, t1))
                nd = fetch_node<OPT>(s, node);
            else
                done = true;
        }
        if (done) {
            active = false;
            bool occ;
            if (WANT_HIT) {
                hit[ri] = best;
                thit[ri] = best_t;
                occ = best >= 0 && best_t < len && (__ldg(&s.tri_ids[best]) & kTraceIdSky) == 0;
            } else {
                occ = best >= 0 &&
                      (best_t < any_limit || (__ldg(&s.tri_ids[best]) & kTraceIdSky) == 0);
            }
            if (occ) atomicOr(mask + (ri >> 5), 1u << (ri & 31));
        }
    }
}

// Closest hits of independent rays, with the same per-lane refill.
__global__ void __launch_bounds__(kThreads) k_trace_closest(DevScene s, const float *__restrict__ orig,
                                                             const float *__restrict__ dir,
                                                             const float *__restrict__ tmin,
                                                             const float *__restrict__ tmax, int64_t n,
                                                             int32_t skip, int32_t *__restrict__ hit,
                                                             float *__restrict__ thit,
                                                             unsigned long long *__restrict__ work) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    bool active = false, exhausted = false;
    int64_t ri = 0;
    Ray ray;
    RayPre rp;
    float r0 = 0.0f, r1 = 0.0f;
    TraceState st;
    for (;;) {
        const unsigned idle = __ballot_sync(full, !active && !exhausted);
        if (idle == 0 && !__any_sync(full, active)) break;
        if (idle) {
            const int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (!active && !exhausted) {
                const int64_t i = (int64_t)base + __popc(idle & below);
                if (i >= n) {
                    exhausted = true;
                } else {
                    ri = i;
                    load3(orig, i, ray.ox, ray.oy, ray.oz);
                    load3(dir, i, ray.dx, ray.dy, ray.dz);
                    r0 = __ldg(tmin + i);
                    r1 = __ldg(tmax + i);
                    const float slack = ray_slack(s.g, ray.ox, ray.oy, ray.oz);
                    rp = ray_pre(ray, slack);
                    active = trace_init(s, ray, rp, slack, r0, r1, st);
                    if (!active) {
                        hit[i] = -1;
                        thit[i] = kInf;
                    }
                }
            }
        }
        if (active && trace_step<kClosest, 1>(s, ray, rp, r0, r1, skip, 0.0f, st)) {
            active = false;
            hit[ri] = st.best;
            thit[ri] = st.best_t;
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_test_lines(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, float *__restrict__ frac) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float sx, sy, sz, ex, ey, ez;
        load3(start, i, sx, sy, sz);
        load3(stop, i, ex, ey, ez);
        frac[i] = line_occluded(s, make_line(sx, sy, sz, ex, ey, ez), skip) ? 0.0f : 1.0f;
    }
}

int grid_for(const vrg_ctx *ctx, int64_t n) {
    int64_t blocks = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

// Persistent grid: resident blocks per SM times SMs, but no more blocks
// than the rays can keep busy.
template <class K>
int persistent_grid(const vrg_ctx *ctx, K kernel, int64_t n) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 4;
    int64_t blocks = (int64_t)ctx->num_sms * per_sm;
    const int64_t need = (n + kThreads - 1) / kThreads;
    if (blocks > need) blocks = need;
    return (int)(blocks < 1 ? 1 : blocks);
}

using MaskKernel = void (*)(DevScene, const float *, const float *, int64_t, int32_t, uint32_t *,
                            int32_t *, float *, unsigned long long *);

// Variants of the shadow-line walk, picked per scene-size bucket: per-lane
// refill with whole-leaf steps; unit rounds (new lines at 4 or 8 idle
// lanes, with or without the vote, at the default or a 40-register cap,
// leaf records kept out of L1 or not, top of the tree in shared memory or
// not, next plane loaded ahead, children without triangles skipped or not,
// the walk constants in shared memory or not, one ballot per round or two).
const MaskKernel kMaskOcc[] = {
    k_trace_mask<false, 1>,          k_trace_unit<false, 4, false, 1>,
    k_trace_unit<false, 4, true, 1>, k_trace_unit<false, 8, true, 1>,
    k_trace_unit<false, 4, false, 12>, k_trace_unit<false, 4, true, 12>,
    k_trace_unit<false, 4, false, 1, kOptStream>, k_trace_unit<false, 8, false, 1, kOptStream>,
    k_trace_mask<false, 1, kOptStream>,
    k_trace_unit<false, 4, false, 1, kOptStream | kOptTop>, k_trace_unit<false, 8, false, 1, kOptStream | kOptTop>,
    k_trace_unit<false, 4, false, 1, kOptStream | kOptPipe>,
    k_trace_mask<false, 1, kOptSkip>, k_trace_unit<false, 4, false, 1, kOptSkip>,
    k_trace_unit<false, 8, true, 1, kOptSkip>, k_trace_unit<false, 4, false, 1, kOptStream | kOptSkip>,
    k_trace_unit<false, 4, false, 1, kOptSkip | kOptShRay>, k_trace_unit<false, 8, true, 1, kOptSkip | kOptShRay>,
    k_trace_unit<false, 8, true, 12, kOptSkip | kOptShRay>, k_trace_unit<false, 8, true, 1, kOptSkip | kOptOneVote>,
};
const MaskKernel kMaskHit[] = {
    k_trace_mask<true, 1>,          k_trace_unit<true, 4, false, 1>,
    k_trace_unit<true, 4, true, 1>, k_trace_unit<true, 8, true, 1>,
    k_trace_unit<true, 4, false, 12>, k_trace_unit<true, 4, true, 12>,
    k_trace_unit<true, 4, false, 1, kOptStream>, k_trace_unit<true, 8, false, 1, kOptStream>,
    k_trace_mask<true, 1, kOptStream>,
    k_trace_unit<true, 4, false, 1, kOptStream | kOptTop>, k_trace_unit<true, 8, false, 1, kOptStream | kOptTop>,
    k_trace_unit<true, 4, false, 1, kOptStream | kOptPipe>,
    k_trace_mask<true, 1, kOptSkip>, k_trace_unit<true, 4, false, 1, kOptSkip>,
    k_trace_unit<true, 8, true, 1, kOptSkip>, k_trace_unit<true, 4, false, 1, kOptStream | kOptSkip>,
    k_trace_unit<true, 4, false, 1, kOptSkip | kOptShRay>, k_trace_unit<true, 8, true, 1, kOptSkip | kOptShRay>,
    k_trace_unit<true, 8, true, 12, kOptSkip | kOptShRay>, k_trace_unit<true, 8, true, 1, kOptSkip | kOptOneVote>,
};
constexpr int kMaskVariants = 20;
static_assert(kThreads <= kShRayLanes, "kOptShRay keeps one slot per thread of a block");

}  // namespace

DevScene scene_view(const vrg_env *env) {
    DevScene s;
    s.nodes = env->d_nodes.as<uint2>();
    s.leaf_planes = env->d_leaf_tris.as<float4>();
    s.leaf_edges = s.leaf_planes + env->walk_tree.refs.size() + env->n_wall_records;
    s.tri_ids = env->d_tri_ids.as<int32_t>();
    s.top = env->d_top.as<uint2>();
    s.ntop = env->ntop;
    s.g = env->geom;
    return s;
}

int launch_occlusion_mask(vrg_env *env, const float *start, const float *stop, int64_t n,
                          int32_t skip_id, uint32_t *mask, int32_t *hit, float *t) {
    vrg_ctx *ctx = env->ctx;
    if (n <= 0) return VRG_OK;
    DevScene s = scene_view(env);
    VRG_CUDA(ctx, env->d_work.reserve(256));
    unsigned long long *work = env->d_work.as<unsigned long long>();
    const bool want = hit && t;
    if (!want) {
        hit = nullptr;
        t = nullptr;
    }
    auto launch = [&](int v) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(work, 0, 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(mask, 0, 4 * (size_t)((n + 31) / 32), ctx->stream);
        if (e != cudaSuccess) return e;
        const MaskKernel k = want ? kMaskHit[v] : kMaskOcc[v];
        cudaEvent_t ev = nullptr;
        timing_begin(ctx, "trace_mask", &ev);
        k<<<persistent_grid(ctx, k, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask,
                                                                     hit, t, work);
        e = cudaGetLastError();
        timing_end(ctx, "trace_mask", ev);
        return e;
    };
    const std::string key = tune_key(want ? "trace_mask_hit" : "trace_mask", env->geom.ntris, n);
    return tune_run(ctx, key, kMaskVariants, launch);
}

int launch_trace_closest(vrg_env *env, const float *orig, const float *dir, const float *tmin,
                         const float *tmax, int64_t n, int32_t skip_id, int32_t *hit, float *t) {
    vrg_ctx *ctx = env->ctx;
    if (n <= 0) return VRG_OK;
    VRG_CUDA(ctx, env->d_work.reserve(256));
    unsigned long long *work = env->d_work.as<unsigned long long>() + 2;
    VRG_CUDA(ctx, cudaMemsetAsync(work, 0, 8, ctx->stream));
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "trace_closest", &ev);
    k_trace_closest<<<persistent_grid(ctx, k_trace_closest, n), kThreads, 0, ctx->stream>>>(
        scene_view(env), orig, dir, tmin, tmax, n, skip_id, hit, t, work);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "trace_closest", ev);
    return VRG_OK;
}

int launch_test_lines(vrg_env *env, const float *start, const float *stop, int64_t n,
                      int32_t skip_id, float *frac) {
    vrg_ctx *ctx = env->ctx;
    if (n <= 0) return VRG_OK;
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "trace_lines", &ev);
    k_test_lines<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(scene_view(env), start, stop, n, skip_id, frac);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "trace_lines", ev);
    return VRG_OK;
}

}  // namespace vrg
