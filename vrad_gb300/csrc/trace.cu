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

// One line per thread; a warp covers 32 consecutive lines so the 1-bit mask
// word is written with one ballot.  WANT_HIT adds the closest hit of the
// normalised segment (hit index and t).
template <bool WANT_HIT>
__global__ void __launch_bounds__(kThreads) k_trace_mask(DevScene s, const float *__restrict__ start,
                                                          const float *__restrict__ stop, int64_t n,
                                                          int32_t skip, uint32_t *__restrict__ mask,
                                                          int32_t *__restrict__ hit,
                                                          float *__restrict__ thit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool occ = false;
        if (i < n) {
            float sx, sy, sz, ex, ey, ez;
            load3(start, i, sx, sy, sz);
            load3(stop, i, ex, ey, ez);
            const Line L = make_line(sx, sy, sz, ex, ey, ez);
            if (WANT_HIT) {
                int32_t h = -1;
                float t = __int_as_float(0x7f800000);
                if (L.len > 0.0f) h = kd_trace<true>(s, L.ox, L.oy, L.oz, L.dx, L.dy, L.dz, 0.0f, L.len, skip, &t);
                occ = h >= 0 && t < L.len && (__ldg(&s.tri_ids[h]) & kTraceIdSky) == 0;
                hit[i] = h;
                thit[i] = t;
            } else {
                occ = line_occluded(s, L, skip);
            }
        }
        const unsigned bits = __ballot_sync(0xffffffffu, occ);
        if ((threadIdx.x & 31) == 0 && i < n) mask[i >> 5] = bits;
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
        hit[i] = kd_trace<true>(s, ox, oy, oz, dx, dy, dz, __ldg(tmin + i), __ldg(tmax + i), skip, &t);
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
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "trace_mask", &ev);
    if (hit && t)
        k_trace_mask<true><<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, hit, t);
    else
        k_trace_mask<false><<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(s, start, stop, n, skip_id, mask, nullptr, nullptr);
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
