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

// Shadow lines with per-lane refill.  Independent lines diverge: some stop
// at their first leaf, some cross the whole scene.  Each lane therefore
// walks its own line one leaf at a time, and as soon as a lane's line is
// done the warp hands it the next unclaimed line (one atomic per refill on
// a device counter zeroed before the launch).  The occlusion bit goes into
// the 1-bit mask with an atomic OR (the mask is zeroed before the launch).
// WANT_HIT also writes the closest hit of the normalised segment.
template <bool WANT_HIT, int LB>
__global__ void __launch_bounds__(kThreads) k_trace_mask(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, uint32_t *__restrict__ mask,
                                                          int32_t *__restrict__ hit,
                                                          float *__restrict__ thit,
                                                          unsigned long long *__restrict__ work) {
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
                    active = !p.trivial && trace_init(s, p.ray, p.rp, p.slack, 0.0f, p.len, st);
                    if (!active && WANT_HIT) {
                        hit[i] = -1;
                        thit[i] = kInf;
                    }
                }
            }
        }
        if (active) {
            const bool done =
                WANT_HIT ? trace_step<kClosest, LB>(s, p.ray, p.rp, 0.0f, p.len, skip, 0.0f, st)
                         : trace_step<kSkyOcc, LB>(s, p.ray, p.rp, 0.0f, p.len, skip, p.any_limit, st);
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

}  // namespace

DevScene scene_view(const vrg_env *env) {
    DevScene s;
    s.nodes = env->d_nodes.as<uint2>();
    s.leaf_planes = env->d_leaf_tris.as<float4>();
    s.leaf_edges = s.leaf_planes + std::max<size_t>(env->tree.refs.size(), 1);
    s.tri_ids = env->d_tri_ids.as<int32_t>();
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
    // variants: triangle planes fetched 1, 2 or 4 at a time (more overlap of
    // loads against fewer resident warps); picked per scene-size bucket
    auto launch = [&](int v) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(work, 0, 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(mask, 0, 4 * (size_t)((n + 31) / 32), ctx->stream);
        if (e != cudaSuccess) return e;
        cudaEvent_t ev = nullptr;
        timing_begin(ctx, "trace_mask", &ev);
        if (want) {
            if (v == 0) k_trace_mask<true, 1><<<persistent_grid(ctx, k_trace_mask<true, 1>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, hit, t, work);
            else if (v == 1) k_trace_mask<true, 2><<<persistent_grid(ctx, k_trace_mask<true, 2>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, hit, t, work);
            else k_trace_mask<true, 4><<<persistent_grid(ctx, k_trace_mask<true, 4>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, hit, t, work);
        } else {
            if (v == 0) k_trace_mask<false, 1><<<persistent_grid(ctx, k_trace_mask<false, 1>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, nullptr, nullptr, work);
            else if (v == 1) k_trace_mask<false, 2><<<persistent_grid(ctx, k_trace_mask<false, 2>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, nullptr, nullptr, work);
            else k_trace_mask<false, 4><<<persistent_grid(ctx, k_trace_mask<false, 4>, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, nullptr, nullptr, work);
        }
        e = cudaGetLastError();
        timing_end(ctx, "trace_mask", ev);
        return e;
    };
    const std::string key = tune_key(want ? "trace_mask_hit" : "trace_mask", env->geom.ntris, n);
    return tune_run(ctx, key, 3, launch);
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
