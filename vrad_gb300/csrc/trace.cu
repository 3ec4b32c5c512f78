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

// Persistent warps: each warp takes the next 32 lines from a device counter
// (zeroed before the launch), so uneven lines balance across the GPU; the
// 1-bit mask word of the 32 lines is written with one ballot.  WANT_HIT adds
// the closest hit of the normalised segment (hit index and t).
template <bool WANT_HIT>
__global__ void __launch_bounds__(kThreads) k_trace_mask(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, uint32_t *__restrict__ mask,
                                                          int32_t *__restrict__ hit,
                                                          float *__restrict__ thit,
                                                          unsigned long long *__restrict__ work) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(work, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned long long)n) break;
        const int64_t i = (int64_t)base + lane;
        bool occ = false;
        if (i < n) {
            float sx, sy, sz, ex, ey, ez;
            load3(start, i, sx, sy, sz);
            load3(stop, i, ex, ey, ez);
            const Line L = make_line(sx, sy, sz, ex, ey, ez);
            if (WANT_HIT) {
                int32_t h = -1;
                float t = __int_as_float(0x7f800000);
                if (L.len > 0.0f) h = trace_ray<kClosest>(s, Ray{L.ox, L.oy, L.oz, L.dx, L.dy, L.dz}, 0.0f, L.len, skip, &t);
                occ = h >= 0 && t < L.len && (__ldg(&s.tri_ids[h]) & kTraceIdSky) == 0;
                hit[i] = h;
                thit[i] = t;
            } else {
                occ = line_occluded(s, L, skip);
            }
        }
        const unsigned bits = __ballot_sync(0xffffffffu, occ);
        if (lane == 0) mask[base >> 5] = bits;
    }
}

__global__ void __launch_bounds__(kThreads) k_trace_closest(DevScene s, const float *__restrict__ orig,
                                                             const float *__restrict__ dir,
                                                             const float *__restrict__ tmin,
                                                             const float *__restrict__ tmax, int64_t n,
                                                             int32_t skip, int32_t *__restrict__ hit,
                                                             float *__restrict__ thit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float ox, oy, oz, dx, dy, dz;
        load3(orig, i, ox, oy, oz);
        load3(dir, i, dx, dy, dz);
        float t;
        hit[i] = trace_ray<kClosest>(s, Ray{ox, oy, oz, dx, dy, dz}, __ldg(tmin + i), __ldg(tmax + i), skip, &t);
        thit[i] = t;
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
// than 32-line chunks.
template <class K>
int persistent_grid(const vrg_ctx *ctx, K kernel, int64_t n) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 4;
    int64_t blocks = (int64_t)ctx->num_sms * per_sm;
    const int64_t chunks = (n + 31) / 32;
    const int64_t need = (chunks + kThreads / 32 - 1) / (kThreads / 32);
    if (blocks > need) blocks = need;
    return (int)(blocks < 1 ? 1 : blocks);
}

}  // namespace

DevScene scene_view(const vrg_env *env) {
    DevScene s;
    s.nodes = env->d_nodes.as<uint2>();
    s.leaf_tris = env->d_leaf_tris.as<float4>();
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
    VRG_CUDA(ctx, cudaMemsetAsync(work, 0, 8, ctx->stream));
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "trace_mask", &ev);
    if (hit && t)
        k_trace_mask<true><<<persistent_grid(ctx, k_trace_mask<true>, n), kThreads, 0, ctx->stream>>>(
            s, start, stop, n, skip_id, mask, hit, t, work);
    else
        k_trace_mask<false><<<persistent_grid(ctx, k_trace_mask<false>, n), kThreads, 0, ctx->stream>>>(
            s, start, stop, n, skip_id, mask, nullptr, nullptr, work);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "trace_mask", ev);
    return VRG_OK;
}

int launch_trace_closest(vrg_env *env, const float *orig, const float *dir, const float *tmin,
                         const float *tmax, int64_t n, int32_t skip_id, int32_t *hit, float *t) {
    vrg_ctx *ctx = env->ctx;
    if (n <= 0) return VRG_OK;
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "trace_closest", &ev);
    k_trace_closest<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(scene_view(env), orig, dir, tmin, tmax, n, skip_id, hit, t);
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
