// capi.cpp -- context, errors, timing and the host-facing entry points of
// include/vradgpu.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "anorms_table.h"
#include "vrg_internal.h"

namespace vrg {

int fail(vrg_ctx *ctx, int code, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->last_error = msg;
    }
    return code;
}

int cuda_fail(vrg_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(ctx, e == cudaErrorMemoryAllocation ? VRG_ERR_NOMEM : VRG_ERR_CUDA, m);
}

void timing_begin(vrg_ctx *ctx, const char *name, cudaEvent_t *start) {
    (void)name;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->launches++;
    *start = nullptr;
    if (!ctx->timing) return;
    cudaEvent_t e;
    if (!ctx->event_pool.empty()) {
        e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        return;
    }
    cudaEventRecord(e, ctx->stream);
    *start = e;
}

void timing_end(vrg_ctx *ctx, const char *name, cudaEvent_t start) {
    if (!start) return;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaEvent_t e;
    if (!ctx->event_pool.empty()) {
        e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        ctx->event_pool.push_back(start);
        return;
    }
    cudaEventRecord(e, ctx->stream);
    ctx->pending.push_back({name, start, e});
}

void collect_timings(vrg_ctx *ctx) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::vector<PendingTiming> keep;
    for (auto &p : ctx->pending) {
        if (cudaEventQuery(p.stop) != cudaSuccess) {
            keep.push_back(p);
            continue;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, p.start, p.stop);
        KernelStat &s = ctx->stats[p.name];
        s.ms += ms;
        s.launches++;
        ctx->event_pool.push_back(p.start);
        ctx->event_pool.push_back(p.stop);
    }
    ctx->pending.swap(keep);
}

}  // namespace vrg

using namespace vrg;

namespace {

bool finite3(const float *v) {
    return v && std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

int sync(vrg_ctx *ctx) {
    if (ctx->host_only) return VRG_OK;
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VRG_OK;
}

int upload(vrg_ctx *ctx, DevBuf &buf, const void *src, size_t bytes) {
    if (ctx->host_only) return VRG_OK;
    VRG_CUDA(ctx, buf.reserve(bytes));
    if (bytes) VRG_CUDA(ctx, cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return VRG_OK;
}

// The device's address of a host buffer that is page-locked (cudaHostAlloc,
// cudaHostRegister, a pinned torch tensor): kernels read it in place, over
// the CPU-GPU link, instead of waiting for a copy.  NULL for any other
// memory (pageable buffers are copied).
const void *pinned_view(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int download(vrg_ctx *ctx, void *dst, const DevBuf &buf, size_t bytes) {
    if (bytes) VRG_CUDA(ctx, cudaMemcpyAsync(dst, buf.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return VRG_OK;
}

#define TRY(x)                  \
    do {                        \
        int _r = (x);           \
        if (_r != VRG_OK) return _r; \
    } while (0)

int need_built(vrg_env *env) {
    if (!env) return VRG_ERR_INVALID;
    if (env->ctx->host_only) return fail(env->ctx, VRG_ERR_STATE, "host-only context has no device");
    if (!env->built) return fail(env->ctx, VRG_ERR_STATE, "SetupAccelerationStructure has not run");
    return VRG_OK;
}

}  // namespace

namespace vrg {
void pack_lights(const std::vector<vrg_light> &src, std::vector<float4> &dst);
}

extern "C" {

/* ---------------- context ---------------- */

int vrg_ctx_create(int device, vrg_ctx **out) {
    if (!out) return VRG_ERR_INVALID;
    *out = nullptr;
    vrg_ctx *ctx = new (std::nothrow) vrg_ctx();
    if (!ctx) return VRG_ERR_NOMEM;
    ctx->device = device;
    if (device < 0) {
        ctx->host_only = true;
        *out = ctx;
        return VRG_OK;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete ctx;
        return e == cudaErrorMemoryAllocation ? VRG_ERR_NOMEM : VRG_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    // the no-alloc bounce's device array and kernels are set up now, so that
    // its calls allocate nothing; a failure here is reported by that call
    if (vrg::noalloc_prepare(ctx) != VRG_OK) ctx->last_error.clear();
    *out = ctx;
    return VRG_OK;
}

void vrg_ctx_destroy(vrg_ctx *ctx) {
    if (!ctx) return;
    if (ctx->host_only) {
        delete ctx;
        return;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &p : ctx->pending) {
        cudaEventDestroy(p.start);
        cudaEventDestroy(p.stop);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char *vrg_last_error(const vrg_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int vrg_ctx_set_stream(vrg_ctx *ctx, void *stream) {
    if (!ctx) return VRG_ERR_INVALID;
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return VRG_OK;
}

int vrg_ctx_synchronize(vrg_ctx *ctx) {
    if (!ctx) return VRG_ERR_INVALID;
    if (ctx->host_only) return VRG_OK;
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    collect_timings(ctx);
    return VRG_OK;
}

int vrg_ctx_set_timing(vrg_ctx *ctx, int enable) {
    if (!ctx) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->timing = enable != 0;
    return VRG_OK;
}

int vrg_ctx_kernel_stats(vrg_ctx *ctx, const char *name, double *total_ms, int64_t *launches) {
    if (!ctx || !name) return VRG_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
    collect_timings(ctx);
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->stats.find(name);
    if (total_ms) *total_ms = it == ctx->stats.end() ? 0.0 : it->second.ms;
    if (launches) *launches = it == ctx->stats.end() ? 0 : it->second.launches;
    return VRG_OK;
}

int vrg_ctx_reset_stats(vrg_ctx *ctx) {
    if (!ctx) return VRG_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
    collect_timings(ctx);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->stats.clear();
    return VRG_OK;
}

int64_t vrg_ctx_launch_count(const vrg_ctx *ctx) {
    if (!ctx) return 0;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return ctx->launches;
}

/* ---------------- environment: triangle soup ---------------- */

int vrg_env_create(vrg_ctx *ctx, vrg_env **out) {
    if (!ctx || !out) return VRG_ERR_INVALID;
    vrg_env *env = new (std::nothrow) vrg_env();
    if (!env) return VRG_ERR_NOMEM;
    env->ctx = ctx;
    *out = env;
    return VRG_OK;
}

void vrg_env_destroy(vrg_env *env) {
    if (!env) return;
    if (env->ctx->host_only) {
        delete env;
        return;
    }
    cudaSetDevice(env->ctx->device);
    cudaStreamSynchronize(env->ctx->stream);
    relight_release(env);
    bounce_release(env);
    delete env;
}

int vrg_env_add_triangle(vrg_env *env, int32_t id, const float *v1, const float *v2,
                         const float *v3, const float *colour, uint16_t flags, int32_t material) {
    if (!env || !v1 || !v2 || !v3) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "triangles added after SetupAccelerationStructure");
    env->xyz.insert(env->xyz.end(), v1, v1 + 3);
    env->xyz.insert(env->xyz.end(), v2, v2 + 3);
    env->xyz.insert(env->xyz.end(), v3, v3 + 3);
    env->ids.push_back(id);
    env->flags.resize(env->ids.size() - 1, 0);
    env->flags.push_back((uint8_t)flags);
    // coverage of the triangle when it is transparent: its colour's x, as
    // types.CoverageCount adds it (raytracer/types/coverageCount.go:27-41)
    env->cover.resize(env->ids.size() - 1, 0.0f);
    env->cover.push_back(colour ? colour[0] : 0.0f);
    // environment.go:61-66: colours and materials unless the flags say not to
    if (!(flags & VRG_RTE_FLAGS_DONT_STORE_TRIANGLE_COLORS)) {
        const float zero[3] = {0, 0, 0};
        const float *c = colour ? colour : zero;
        env->colours.insert(env->colours.end(), c, c + 3);
    }
    if (!(flags & VRG_RTE_FLAGS_DONT_STORE_TRIANGLE_MATERIALS)) env->materials.push_back(material);
    return VRG_OK;
}

int vrg_env_add_quad(vrg_env *env, int32_t id, const float *v1, const float *v2, const float *v3,
                     const float *v4, const float *colour) {
    TRY(vrg_env_add_triangle(env, id, v1, v2, v3, colour, 0, 0));
    return vrg_env_add_triangle(env, id + 1, v1, v3, v4, colour, 0, 0);
}

int vrg_env_add_axis_aligned_rectangular_solid(vrg_env *env, int32_t id, const float *mn,
                                               const float *mx, const float *colour) {
    if (!env || !mn || !mx) return VRG_ERR_INVALID;
    // six quads: far, near, left, right, top, bottom (environment.go:79-116)
    const float q[6][4][3] = {
        {{mn[0], mx[1], mx[2]}, {mx[0], mx[1], mx[2]}, {mx[0], mn[1], mx[2]}, {mn[0], mn[1], mx[2]}},
        {{mn[0], mx[1], mn[2]}, {mx[0], mx[1], mn[2]}, {mx[0], mn[1], mn[2]}, {mn[0], mn[1], mn[2]}},
        {{mn[0], mx[1], mx[2]}, {mn[0], mx[1], mn[2]}, {mn[0], mn[1], mn[2]}, {mn[0], mn[1], mx[2]}},
        {{mx[0], mx[1], mx[2]}, {mx[0], mx[1], mn[2]}, {mx[0], mn[1], mn[2]}, {mx[0], mn[1], mx[2]}},
        {{mn[0], mx[1], mx[2]}, {mx[0], mx[1], mx[2]}, {mx[0], mx[1], mn[2]}, {mn[0], mx[1], mn[2]}},
        {{mn[0], mn[1], mx[2]}, {mx[0], mn[1], mx[2]}, {mx[0], mn[1], mn[2]}, {mn[0], mn[1], mn[2]}},
    };
    for (int f = 0; f < 6; f++) TRY(vrg_env_add_quad(env, id, q[f][0], q[f][1], q[f][2], q[f][3], colour));
    return VRG_OK;
}

int vrg_env_add_triangles(vrg_env *env, const float *xyz, const int32_t *ids, int64_t n) {
    if (!env || n < 0 || (n > 0 && (!xyz || !ids))) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "triangles added after SetupAccelerationStructure");
    env->xyz.insert(env->xyz.end(), xyz, xyz + 9 * n);
    env->ids.insert(env->ids.end(), ids, ids + n);
    env->flags.insert(env->flags.end(), (size_t)n, 0);
    env->colours.insert(env->colours.end(), (size_t)(3 * n), 0.0f);
    env->materials.insert(env->materials.end(), (size_t)n, 0);
    return VRG_OK;
}

int64_t vrg_env_num_triangles(const vrg_env *env) { return env ? (int64_t)env->ids.size() : 0; }

int vrg_env_get_triangle_vertices(const vrg_env *env, int64_t first, int64_t n, float *xyz, int32_t *ids) {
    if (!env || first < 0 || n < 0 || (n && !xyz && !ids)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (first + n > (int64_t)env->ids.size()) return VRG_ERR_INVALID;
    if (xyz && n) memcpy(xyz, env->xyz.data() + 9 * first, sizeof(float) * 9 * (size_t)n);
    if (ids && n) memcpy(ids, env->ids.data() + first, sizeof(int32_t) * (size_t)n);
    return VRG_OK;
}

/* ---------------- trace ---------------- */

int vrg_env_trace_closest_d(vrg_env *env, const float *orig, const float *dir, const float *tmin,
                            const float *tmax, int64_t n, int32_t skip_id, int32_t *out_hit,
                            float *out_t) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!orig || !dir || !tmin || !tmax || !out_hit || !out_t))) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    return launch_trace_closest(env, orig, dir, tmin, tmax, n, skip_id, out_hit, out_t);
}

int vrg_env_trace_closest(vrg_env *env, const float *orig, const float *dir, const float *tmin,
                          const float *tmax, int64_t n, int32_t skip_id, int32_t *out_hit,
                          float *out_t) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!orig || !dir || !tmin || !tmax || !out_hit || !out_t))) return VRG_ERR_INVALID;
    if (n == 0) return VRG_OK;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    // page-locked inputs are read in place, others copied first
    const float *d_orig = static_cast<const float *>(pinned_view(orig));
    const float *d_dir = static_cast<const float *>(pinned_view(dir));
    const float *d_tmin = static_cast<const float *>(pinned_view(tmin));
    const float *d_tmax = static_cast<const float *>(pinned_view(tmax));
    if (!d_orig || !d_dir || !d_tmin || !d_tmax) {
        TRY(upload(ctx, env->d_in0, orig, 12 * n));
        TRY(upload(ctx, env->d_in1, dir, 12 * n));
        VRG_CUDA(ctx, env->d_out2.reserve(8 * n));
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_out2.as<float>(), tmin, 4 * n, cudaMemcpyHostToDevice, ctx->stream));
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_out2.as<float>() + n, tmax, 4 * n, cudaMemcpyHostToDevice, ctx->stream));
        d_orig = env->d_in0.as<float>();
        d_dir = env->d_in1.as<float>();
        d_tmin = env->d_out2.as<float>();
        d_tmax = env->d_out2.as<float>() + n;
    }
    VRG_CUDA(ctx, env->d_out0.reserve(4 * n));
    VRG_CUDA(ctx, env->d_out1.reserve(4 * n));
    TRY(launch_trace_closest(env, d_orig, d_dir, d_tmin, d_tmax, n, skip_id, env->d_out0.as<int32_t>(),
                             env->d_out1.as<float>()));
    TRY(download(ctx, out_hit, env->d_out0, 4 * n));
    TRY(download(ctx, out_t, env->d_out1, 4 * n));
    return sync(ctx);
}

int vrg_env_trace4_rays(vrg_env *env, const float *origin, const float *direction, const float *tmin,
                        const float *tmax, int32_t skip_id, int32_t *hit_ids, float *hit_distance,
                        float *surface_normal) {
    if (!origin || !direction || !tmin || !tmax || !hit_ids || !hit_distance) return VRG_ERR_INVALID;
    float o[12], d[12];
    for (int i = 0; i < 4; i++)
        for (int a = 0; a < 3; a++) {
            o[3 * i + a] = origin[4 * a + i];
            d[3 * i + a] = direction[4 * a + i];
        }
    TRY(vrg_env_trace_closest(env, o, d, tmin, tmax, 4, skip_id, hit_ids, hit_distance));
    if (surface_normal) {
        for (int i = 0; i < 4; i++) {
            const int h = hit_ids[i];
            const TriRecord *t = h >= 0 ? &env->tri_records[h] : nullptr;
            surface_normal[i] = t ? t->nx : 0.0f;
            surface_normal[4 + i] = t ? t->ny : 0.0f;
            surface_normal[8 + i] = t ? t->nz : 0.0f;
        }
    }
    return VRG_OK;
}

int vrg_env_occlusion_mask_d(vrg_env *env, const float *start, const float *stop, int64_t n,
                             int32_t skip_id, uint32_t *out_mask, int32_t *out_hit, float *out_t) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!start || !stop || !out_mask))) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    return launch_occlusion_mask(env, start, stop, n, skip_id, out_mask, out_hit, out_t);
}

int vrg_env_occlusion_mask(vrg_env *env, const float *start, const float *stop, int64_t n,
                           int32_t skip_id, uint32_t *out_mask, int32_t *out_hit, float *out_t) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!start || !stop || !out_mask))) return VRG_ERR_INVALID;
    if (n == 0) return VRG_OK;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    const bool want = out_hit && out_t;
    const int64_t words = (n + 31) / 32;
    // page-locked end points are read where they are (the walk reads each
    // line's 24 bytes once, as it takes the line); others are copied first
    const float *d_start = static_cast<const float *>(pinned_view(start));
    const float *d_stop = static_cast<const float *>(pinned_view(stop));
    if (!d_start || !d_stop) {
        TRY(upload(ctx, env->d_in0, start, 12 * n));
        TRY(upload(ctx, env->d_in1, stop, 12 * n));
        d_start = env->d_in0.as<float>();
        d_stop = env->d_in1.as<float>();
    }
    VRG_CUDA(ctx, env->d_out2.reserve(4 * words));
    if (want) {
        VRG_CUDA(ctx, env->d_out0.reserve(4 * n));
        VRG_CUDA(ctx, env->d_out1.reserve(4 * n));
    }
    TRY(launch_occlusion_mask(env, d_start, d_stop, n, skip_id,
                              env->d_out2.as<uint32_t>(), want ? env->d_out0.as<int32_t>() : nullptr,
                              want ? env->d_out1.as<float>() : nullptr));
    TRY(download(ctx, out_mask, env->d_out2, 4 * words));
    if (want) {
        TRY(download(ctx, out_hit, env->d_out0, 4 * n));
        TRY(download(ctx, out_t, env->d_out1, 4 * n));
    }
    return sync(ctx);
}

int vrg_env_test_line_does_hit_sky(vrg_env *env, const float *start, const float *stop, int64_t n,
                                   int32_t static_prop_to_skip, float *fraction_visible) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!start || !stop || !fraction_visible))) return VRG_ERR_INVALID;
    if (n == 0) return VRG_OK;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    // testline.go:36: skip id = TRACE_ID_STATICPROP | staticPropToSkip
    const int32_t skip = VRG_TRACE_ID_STATICPROP | static_prop_to_skip;
    const float *d_start = static_cast<const float *>(pinned_view(start));
    const float *d_stop = static_cast<const float *>(pinned_view(stop));
    if (!d_start || !d_stop) {
        TRY(upload(ctx, env->d_in0, start, 12 * n));
        TRY(upload(ctx, env->d_in1, stop, 12 * n));
        d_start = env->d_in0.as<float>();
        d_stop = env->d_in1.as<float>();
    }
    VRG_CUDA(ctx, env->d_out0.reserve(4 * n));
    TRY(launch_test_lines(env, d_start, d_stop, n, skip, env->d_out0.as<float>()));
    TRY(download(ctx, fraction_visible, env->d_out0, 4 * n));
    return sync(ctx);
}

/* CanLeafTraceToSky (rad/lightmap/lightmap.go:425-451) */

int vrg_leaf_sky_lines(const int32_t *leaf_mins, const int32_t *leaf_maxs, int64_t n, float *starts,
                       float *stops) {
    if (n < 0 || (n > 0 && (!leaf_mins || !leaf_maxs || !starts || !stops))) return VRG_ERR_INVALID;
    static const float anorms[kNumAnorms * 3] = VRG_ANORMS_INIT;
    const float scale = -kMaxTraceLength;
    for (int64_t i = 0; i < n; i++) {
        float c[3];
        for (int a = 0; a < 3; a++) c[a] = (float)(leaf_mins[3 * i + a] + leaf_maxs[3 * i + a]) * 0.5f;
        for (int j = 0; j < kNumAnorms; j++) {
            float *st = starts + 3 * (i * kNumAnorms + j), *sp = stops + 3 * (i * kNumAnorms + j);
            for (int a = 0; a < 3; a++) {
                st[a] = c[a];
                sp[a] = anorms[3 * j + a] * scale + c[a];
            }
        }
    }
    return VRG_OK;
}

int vrg_env_can_leaf_trace_to_sky(vrg_env *env, const int32_t *leaf_mins, const int32_t *leaf_maxs, int64_t n,
                                  uint8_t *out) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!leaf_mins || !leaf_maxs || !out))) return VRG_ERR_INVALID;
    constexpr int64_t kChunk = 4096;  // leaves per trace call: 663,552 lines, 16 MB of end points
    std::vector<float> a, b, frac;
    for (int64_t i0 = 0; i0 < n; i0 += kChunk) {
        const int64_t m = std::min(kChunk, n - i0);
        const int64_t lines = m * kNumAnorms;
        a.resize(3 * lines);
        b.resize(3 * lines);
        frac.resize(lines);
        TRY(vrg_leaf_sky_lines(leaf_mins + 3 * i0, leaf_maxs + 3 * i0, m, a.data(), b.data()));
        TRY(vrg_env_test_line_does_hit_sky(env, a.data(), b.data(), lines, -1, frac.data()));
        for (int64_t i = 0; i < m; i++) {
            uint8_t sky = 0;
            for (int j = 0; j < kNumAnorms && !sky; j++) sky = frac[i * kNumAnorms + j] > 0.0f ? 1 : 0;
            out[i0 + i] = sky;
        }
    }
    return VRG_OK;
}

/* ray stream: queue on the host, trace on finish in one batch */

int vrg_env_add_to_ray_stream(vrg_env *env, const float *start, const float *stop, int32_t skip_id) {
    if (!env || !start || !stop) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    env->rs_start.insert(env->rs_start.end(), start, start + 3);
    env->rs_stop.insert(env->rs_stop.end(), stop, stop + 3);
    env->rs_skip.push_back(skip_id);
    return VRG_OK;
}

int vrg_env_flush_stream_entry(vrg_env *env) {
    // Queued lines are traced together at FinishRayStream; a flush only
    // validates the state so callers written against the reference's
    // 4-ray flush keep working.
    return need_built(env);
}

int vrg_env_finish_ray_stream(vrg_env *env, float *fraction_visible, int64_t capacity, int64_t *count) {
    TRY(need_built(env));
    std::vector<float> a, b;
    std::vector<int32_t> sk;
    {
        std::lock_guard<std::mutex> lk(env->mu);
        a.swap(env->rs_start);
        b.swap(env->rs_stop);
        sk.swap(env->rs_skip);
    }
    const int64_t n = (int64_t)sk.size();
    if (count) *count = n;
    if (n > capacity || (n > 0 && !fraction_visible)) return fail(env->ctx, VRG_ERR_INVALID, "ray stream result buffer too small");
    // lines sharing a skip id go in one launch
    int64_t i = 0;
    while (i < n) {
        int64_t j = i;
        while (j < n && sk[j] == sk[i]) j++;
        uint32_t dummy;
        (void)dummy;
        std::vector<float> frac(j - i);
        // skip ids in the stream are used as given
        std::vector<uint32_t> mask((j - i + 31) / 32);
        TRY(vrg_env_occlusion_mask(env, &a[3 * i], &b[3 * i], j - i, sk[i], mask.data(), nullptr, nullptr));
        for (int64_t k = i; k < j; k++) fraction_visible[k] = (mask[(k - i) >> 5] >> ((k - i) & 31)) & 1u ? 0.0f : 1.0f;
        i = j;
    }
    return VRG_OK;
}

/* ---------------- lights ---------------- */

int vrg_light_set_falloff_params(const vrg_light_keys *keys, vrg_light *light) {
    if (!keys || !light) return VRG_ERR_INVALID;
    light_set_falloff(*keys, *light);
    return VRG_OK;
}

int vrg_light_parse_spot(const vrg_light_keys *keys, vrg_light *light) {
    if (!keys || !light) return VRG_ERR_INVALID;
    light_parse_spot(*keys, *light);
    return VRG_OK;
}

int vrg_light_parse_point(const vrg_light_keys *keys, vrg_light *light) {
    if (!keys || !light) return VRG_ERR_INVALID;
    light->type = VRG_EMIT_POINT;
    light_set_falloff(*keys, *light);
    return VRG_OK;
}

int vrg_env_set_lights(vrg_env *env, const vrg_light *lights, int32_t n) {
    if (!env || n < 0 || (n > 0 && !lights)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    env->relight_ready = false;  // the relight caches belong to the old table
    for (int32_t i = 0; i < n; i++) {
        const vrg_light &l = lights[i];
        if (l.type < 0 || l.type > 5 || !finite3(l.origin) || !finite3(l.intensity))
            return fail(env->ctx, VRG_ERR_INVALID, "light " + std::to_string(i) + " has a bad type or non-finite fields");
    }
    env->lights.assign(lights, lights + n);
    std::vector<float4> packed;
    pack_lights(env->lights, packed);
    TRY(upload(env->ctx, env->d_lights, packed.data(), packed.size() * sizeof(float4)));
    env->have_patch_direct = false;
    return sync(env->ctx);
}

/* ---------------- face lightmap extents ---------------- */

// CalcFaceExtents (rad/world/face.go:14-90), with the two results written
// out (the reference takes them by value and loses them, rad/start.go:110).
// Each vertex is projected onto both lightmap axes in float32, one rounding
// per operation: ((x*L0 + y*L1) + z*L2) + L3; the running bounds start at
// +-1e24; mins = floor(min) and size = ceil(max) - floor(min), the
// subtraction in float32.  A size above the lightmap limit + 1 (125,
// common/constants/constants.go:22,27, for brush and displacement faces
// alike) is reported in *too_big, the case the reference logs and goes on.
int vrg_calc_face_extents(const float *vertices, int32_t nverts, const float *lightmap_vecs,
                          int32_t *mins, int32_t *size, int32_t *too_big) {
    if (!vertices || nverts < 1 || !lightmap_vecs || !mins || !size) return VRG_ERR_INVALID;
    float lo[2] = {1e24f, 1e24f}, hi[2] = {-1e24f, -1e24f};
    for (int32_t i = 0; i < nverts; i++) {
        const float *p = vertices + 3 * i;
        for (int j = 0; j < 2; j++) {
            const float *L = lightmap_vecs + 4 * j;
            const float val = ((p[0] * L[0] + p[1] * L[1]) + p[2] * L[2]) + L[3];
            lo[j] = val < lo[j] ? val : lo[j];
            hi[j] = val > hi[j] ? val : hi[j];
        }
    }
    int32_t m[2], s[2], big = 0;
    for (int j = 0; j < 2; j++) {
        const float fl = (float)std::floor((double)lo[j]), ce = (float)std::ceil((double)hi[j]);
        const float extent = ce - fl;
        if (!(fl >= -2147483648.0f && fl < 2147483648.0f && extent >= -2147483648.0f && extent < 2147483648.0f))
            return VRG_ERR_INVALID;  // non-finite or beyond int32
        m[j] = (int32_t)fl;
        s[j] = (int32_t)extent;
        big |= s[j] > kMaxLightmapDim + 1 ? 1 : 0;
    }
    mins[0] = m[0];
    mins[1] = m[1];
    size[0] = s[0];
    size[1] = s[1];
    if (too_big) *too_big = big;
    return VRG_OK;
}

/* ---------------- faces and the direct-light gather ---------------- */

int vrg_env_set_faces(vrg_env *env, int32_t nfaces, const float *corner, const float *u, const float *v,
                      const float *normal, const int32_t *nu, const int32_t *nv, const float *luxscale,
                      const float *reflectivity, const float *baselight, const int32_t *tri_face) {
    if (!env || nfaces < 0) return VRG_ERR_INVALID;
    if (nfaces > 0 && (!corner || !u || !v || !normal || !nu || !nv || !luxscale)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    env->relight_ready = false;
    vrg_ctx *ctx = env->ctx;
    if (!env->built) return fail(ctx, VRG_ERR_STATE, "set faces after SetupAccelerationStructure");
    for (int32_t f = 0; f < nfaces; f++)
        if (nu[f] < 1 || nv[f] < 1 || !finite3(corner + 3 * f) || !finite3(u + 3 * f) || !finite3(v + 3 * f) ||
            !finite3(normal + 3 * f))
            return fail(ctx, VRG_ERR_INVALID, "face " + std::to_string(f) + " has an empty luxel grid or non-finite geometry");
    const int64_t nt = (int64_t)env->ids.size();
    if (tri_face)
        for (int64_t t = 0; t < nt; t++)
            if (tri_face[t] < -1 || tri_face[t] >= nfaces)
                return fail(ctx, VRG_ERR_INVALID, "tri_face entry out of range");
    env->nfaces = nfaces;
    env->f_corner.assign(corner, corner + 3 * nfaces);
    env->f_u.assign(u, u + 3 * nfaces);
    env->f_v.assign(v, v + 3 * nfaces);
    env->f_normal.assign(normal, normal + 3 * nfaces);
    env->f_nu.assign(nu, nu + nfaces);
    env->f_nv.assign(nv, nv + nfaces);
    env->f_luxscale.assign(luxscale, luxscale + nfaces);
    env->f_refl.assign(3 * (size_t)nfaces, 0.0f);
    env->f_base.assign(3 * (size_t)nfaces, 0.0f);
    if (reflectivity)
        for (int64_t i = 0; i < 3 * (int64_t)nfaces; i++)
            env->f_refl[i] = std::min(reflectivity[i], 0.99f);  // rad/patches/face.go:225-230
    if (baselight) env->f_base.assign(baselight, baselight + 3 * nfaces);
    env->tri_face.assign(nt, -1);
    if (tri_face) env->tri_face.assign(tri_face, tri_face + nt);
    env->luxel_offset.assign(nfaces + 1, 0);
    for (int32_t f = 0; f < nfaces; f++) env->luxel_offset[f + 1] = env->luxel_offset[f] + (int64_t)nu[f] * nv[f];
    std::vector<FaceRec> recs(nfaces ? nfaces : 1);
    for (int32_t f = 0; f < nfaces; f++) {
        FaceRec &r = recs[f];
        r.corner = make_float4(corner[3 * f], corner[3 * f + 1], corner[3 * f + 2], luxscale[f]);
        r.u = make_float4(u[3 * f], u[3 * f + 1], u[3 * f + 2], 0.0f);
        r.v = make_float4(v[3 * f], v[3 * f + 1], v[3 * f + 2], 0.0f);
        r.normal = make_float4(normal[3 * f], normal[3 * f + 1], normal[3 * f + 2], 0.0f);
        r.nu = nu[f];
        r.nv = nv[f];
        r.pad0 = r.pad1 = 0;
    }
    TRY(upload(ctx, env->d_faces, recs.data(), recs.size() * sizeof(FaceRec)));
    TRY(upload(ctx, env->d_luxel_offset, env->luxel_offset.data(), env->luxel_offset.size() * 8));
    TRY(upload(ctx, env->d_tri_face, env->tri_face.data(), std::max<size_t>(1, env->tri_face.size()) * 4));
    env->have_patches = env->have_transfers = env->have_patch_direct = false;
    env->have_bake = false;  // the last bake's buffers were sized for the old faces
    return sync(ctx);
}

int64_t vrg_env_num_luxels(const vrg_env *env) {
    return (env && !env->luxel_offset.empty()) ? env->luxel_offset.back() : 0;
}

int vrg_env_gather_direct_light_d(vrg_env *env, int32_t supersamples, uint64_t seed, float *out_rgb,
                                  uint64_t *out_shadow_rays) {
    TRY(need_built(env));
    if (supersamples != 1 && supersamples != 4) return fail(env->ctx, VRG_ERR_UNSUPPORTED, "supersamples must be 1 or 4");
    if (!out_rgb && vrg_env_num_luxels(env) > 0) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    unsigned long long *cnt = nullptr;
    if (out_shadow_rays) {
        VRG_CUDA(ctx, env->d_counter.reserve(64));
        cnt = env->d_counter.as<unsigned long long>();
        VRG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, ctx->stream));
    }
    TRY(launch_gather_luxels(env, supersamples, seed, out_rgb, cnt));
    if (out_shadow_rays) {
        unsigned long long h = 0;
        VRG_CUDA(ctx, cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
        TRY(sync(ctx));
        *out_shadow_rays = h;
    }
    return VRG_OK;
}

int vrg_env_gather_direct_light(vrg_env *env, int32_t supersamples, uint64_t seed, float *out_rgb,
                                uint64_t *out_shadow_rays) {
    TRY(need_built(env));
    const int64_t nlux = vrg_env_num_luxels(env);
    if (nlux > 0 && !out_rgb) return VRG_ERR_INVALID;
    vrg_ctx *ctx = env->ctx;
    {
        std::lock_guard<std::mutex> lk(env->mu);
        VRG_CUDA(ctx, env->d_out0.reserve(12 * std::max<int64_t>(nlux, 1)));
    }
    TRY(vrg_env_gather_direct_light_d(env, supersamples, seed, env->d_out0.as<float>(), out_shadow_rays));
    std::lock_guard<std::mutex> lk(env->mu);
    TRY(download(ctx, out_rgb, env->d_out0, 12 * nlux));
    return sync(ctx);
}

int vrg_env_gather_points(vrg_env *env, const float *points, const float *normals, int64_t n, float *out_rgb,
                          uint64_t *out_shadow_rays) {
    TRY(need_built(env));
    if (n < 0 || (n > 0 && (!points || !normals || !out_rgb))) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    if (n > 0) {
        TRY(upload(ctx, env->d_in0, points, 12 * n));
        TRY(upload(ctx, env->d_in1, normals, 12 * n));
        VRG_CUDA(ctx, env->d_out0.reserve(12 * n));
    }
    VRG_CUDA(ctx, env->d_counter.reserve(64));
    unsigned long long *cnt = env->d_counter.as<unsigned long long>();
    VRG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, ctx->stream));
    TRY(launch_gather_points(env, env->d_in0.as<float>(), env->d_in1.as<float>(), n, env->d_out0.as<float>(), cnt));
    unsigned long long h = 0;
    VRG_CUDA(ctx, cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (n > 0) TRY(download(ctx, out_rgb, env->d_out0, 12 * n));
    TRY(sync(ctx));
    if (out_shadow_rays) *out_shadow_rays = h;
    return VRG_OK;
}

/* ---------------- patches, transfers, bounce ---------------- */

int vrg_env_make_patches(vrg_env *env, float max_chop, float min_chop, int64_t *num_patches, int64_t *num_leaves) {
    if (!env) return VRG_ERR_INVALID;
    if (!env->built) return fail(env->ctx, VRG_ERR_STATE, "SetupAccelerationStructure has not run");
    if (!(max_chop > 0.0f) || !(min_chop > 0.0f)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    env->relight_ready = false;
    TRY(make_rect_patches(*env, max_chop, min_chop, env->patches));
    const PatchSet &P = env->patches;
    const size_t n = P.face.size(), nl = P.leaf_patch.size();
    std::vector<PatchNode> nodes(n ? n : 1);
    for (size_t i = 0; i < n; i++) {
        PatchNode &d = nodes[i];
        d.child1 = P.child1[i];
        d.child2 = P.child2[i];
        d.axis = P.child1[i] >= 0 ? P.split_axis[i] : -1;
        if (d.axis >= 0) d.dist = P.split_dist[i];
        else d.leaf = P.leaf_index[i];
    }
    std::vector<LeafInfo> info(nl ? nl : 1);
    for (size_t l = 0; l < nl; l++) {
        const int32_t p = P.leaf_patch[l], f = P.face[p];
        float fbits;
        memcpy(&fbits, &f, 4);
        info[l].center = make_float4(P.center[3 * p], P.center[3 * p + 1], P.center[3 * p + 2], P.area[p]);
        info[l].refl = make_float4(env->f_refl[3 * f], env->f_refl[3 * f + 1], env->f_refl[3 * f + 2], fbits);
        info[l].base = make_float4(env->f_base[3 * f], env->f_base[3 * f + 1], env->f_base[3 * f + 2], 0.0f);
    }
    // per face, for the lightmap kernel's shared-memory copy of the face's
    // tree: (first node below the root, nodes below the root, first leaf,
    // leaves).  The subdivision appends a face's nodes in one run and numbers
    // leaves in node order, so both ranges are contiguous; a face where the
    // check below fails gets (-1, 0, -1, 0) and is walked in global memory.
    std::vector<int4> face_tree(std::max<int32_t>(env->nfaces, 1), make_int4(-1, 0, -1, 0));
    {
        const int32_t nf = env->nfaces;
        std::vector<int64_t> n0(nf, INT64_MAX), n1(nf, -1), nc(nf, 0), l0(nf, INT64_MAX), l1(nf, -1), lc(nf, 0);
        std::vector<char> mixed(nf, 0);  // a child of another face: walk in global memory
        for (size_t i = 0; i < n; i++) {
            const int32_t f = P.face[i];
            if (f < 0 || f >= nf) continue;
            for (const int32_t c : {P.child1[i], P.child2[i]})
                if (c >= 0 && ((size_t)c >= n || P.face[c] != f)) mixed[f] = 1;
            if (P.parent[i] >= 0) {
                n0[f] = std::min<int64_t>(n0[f], (int64_t)i);
                n1[f] = std::max<int64_t>(n1[f], (int64_t)i);
                nc[f]++;
            }
            if (P.child1[i] < 0) {
                l0[f] = std::min<int64_t>(l0[f], P.leaf_index[i]);
                l1[f] = std::max<int64_t>(l1[f], P.leaf_index[i]);
                lc[f]++;
            }
        }
        for (int32_t f = 0; f < nf; f++) {
            if (P.face_root[f] < 0 || lc[f] == 0 || mixed[f]) continue;
            const bool nodes_run = nc[f] == 0 || n1[f] - n0[f] + 1 == nc[f];
            const bool leaves_run = l1[f] - l0[f] + 1 == lc[f];
            if (nodes_run && leaves_run && nc[f] < INT32_MAX && lc[f] < INT32_MAX)
                face_tree[f] = make_int4(nc[f] ? (int32_t)n0[f] : 0, (int32_t)nc[f], (int32_t)l0[f], (int32_t)lc[f]);
        }
    }
    TRY(upload(ctx, env->d_face_tree, face_tree.data(), face_tree.size() * sizeof(int4)));
    TRY(upload(ctx, env->d_patch_nodes, nodes.data(), nodes.size() * sizeof(PatchNode)));
    TRY(upload(ctx, env->d_leaf_info, info.data(), info.size() * sizeof(LeafInfo)));
    TRY(upload(ctx, env->d_face_root, P.face_root.data(), std::max<size_t>(1, P.face_root.size()) * 4));
    // leaf sample points for the patch direct light: centre + 0.125 * normal
    {
        std::vector<float> pts(3 * std::max<size_t>(nl, 1)), nrm(3 * std::max<size_t>(nl, 1));
        for (size_t l = 0; l < nl; l++) {
            const int32_t p = P.leaf_patch[l], f = P.face[p];
            for (int a = 0; a < 3; a++) {
                nrm[3 * l + a] = env->f_normal[3 * f + a];
                pts[3 * l + a] = P.center[3 * p + a] + env->f_normal[3 * f + a] * kSampleOffset;
            }
        }
        TRY(upload(ctx, env->d_patch_pts, pts.data(), pts.size() * 4));
        TRY(upload(ctx, env->d_patch_nrm, nrm.data(), nrm.size() * 4));
    }
    env->have_patches = true;
    env->have_transfers = env->have_patch_direct = false;
    env->have_bake = false;  // the last bake's bounced light belongs to the old leaves
    if (num_patches) *num_patches = (int64_t)n;
    if (num_leaves) *num_leaves = (int64_t)nl;
    return sync(ctx);
}

int vrg_env_get_patches(const vrg_env *env, float *mins, float *maxs, float *center, float *area, int32_t *face,
                        int32_t *parent, int32_t *child1, int32_t *child2, int32_t *split_axis, float *split_dist,
                        int32_t *leaf_index) {
    if (!env || !env->have_patches) return VRG_ERR_STATE;
    const PatchSet &P = env->patches;
    const size_t n = P.face.size();
    if (mins) memcpy(mins, P.mins.data(), 12 * n);
    if (maxs) memcpy(maxs, P.maxs.data(), 12 * n);
    if (center) memcpy(center, P.center.data(), 12 * n);
    if (area) memcpy(area, P.area.data(), 4 * n);
    if (face) memcpy(face, P.face.data(), 4 * n);
    if (parent) memcpy(parent, P.parent.data(), 4 * n);
    if (child1) memcpy(child1, P.child1.data(), 4 * n);
    if (child2) memcpy(child2, P.child2.data(), 4 * n);
    if (split_axis) memcpy(split_axis, P.split_axis.data(), 4 * n);
    if (split_dist) memcpy(split_dist, P.split_dist.data(), 4 * n);
    if (leaf_index) memcpy(leaf_index, P.leaf_index.data(), 4 * n);
    return VRG_OK;
}

int vrg_env_make_transfers(vrg_env *env, const float *dirs_local, int32_t k, int64_t *out_nnz) {
    TRY(need_built(env));
    if (!env->have_patches) return fail(env->ctx, VRG_ERR_STATE, "MakePatches has not run");
    if (!dirs_local || k < 32 || k > 65536 || (k & (k - 1)) != 0)
        return fail(env->ctx, VRG_ERR_UNSUPPORTED, "transfer ray count must be a power of two in [32, 65536]");
    std::lock_guard<std::mutex> lk(env->mu);
    env->relight_ready = false;
    TRY(run_make_transfers(env, dirs_local, k));
    if (out_nnz) *out_nnz = env->nnz;
    return VRG_OK;
}

int vrg_env_transfer_info(const vrg_env *env, int32_t *k, int64_t *nnz, int64_t *overflow_rows) {
    if (!env || !env->have_transfers) return VRG_ERR_STATE;
    std::lock_guard<std::mutex> lk(env->mu);
    if (k) *k = env->transfer_k;
    if (nnz) *nnz = env->nnz;
    if (overflow_rows) *overflow_rows = env->transfer_overflow_rows;
    return VRG_OK;
}

int vrg_ctx_set_transfer_table_limit(vrg_ctx *ctx, int32_t limit) {
    if (!ctx || limit < 1) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->xfer_table_limit = std::min<int32_t>(limit, 7168);
    return VRG_OK;
}

int vrg_env_get_transfers(const vrg_env *env, int64_t *row_ptr, int32_t *col, float *weight) {
    if (!env || !env->have_transfers) return VRG_ERR_STATE;
    vrg_ctx *ctx = env->ctx;
    const size_t rows = env->patches.leaf_patch.size();
    if (row_ptr) VRG_CUDA(ctx, cudaMemcpyAsync(row_ptr, env->d_row_ptr.ptr, 8 * (rows + 1), cudaMemcpyDeviceToHost, ctx->stream));
    if (col && env->nnz) VRG_CUDA(ctx, cudaMemcpyAsync(col, env->d_col.ptr, 4 * env->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    if (weight && env->nnz) VRG_CUDA(ctx, cudaMemcpyAsync(weight, env->d_weight.ptr, 4 * env->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VRG_OK;
}

int vrg_env_gather_patch_direct(vrg_env *env, float *out_rgb) {
    TRY(need_built(env));
    if (!env->have_patches) return fail(env->ctx, VRG_ERR_STATE, "MakePatches has not run");
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    VRG_CUDA(ctx, env->d_leaf_direct.reserve(12 * std::max<int64_t>(nl, 1)));
    TRY(launch_gather_points(env, env->d_patch_pts.as<float>(), env->d_patch_nrm.as<float>(), nl,
                             env->d_leaf_direct.as<float>(), nullptr));
    if (out_rgb) TRY(download(ctx, out_rgb, env->d_leaf_direct, 12 * nl));
    TRY(sync(ctx));
    env->have_patch_direct = true;
    return VRG_OK;
}

int vrg_env_bounce_light(vrg_env *env, int32_t max_bounces, float rel_tol, float *out_total, int32_t *out_bounces,
                         float *out_delta) {
    TRY(need_built(env));
    if (!env->have_transfers) return fail(env->ctx, VRG_ERR_STATE, "MakeTransfers has not run");
    if (max_bounces < 0 || !(rel_tol >= 0.0f)) return VRG_ERR_INVALID;
    if (!env->have_patch_direct) TRY(vrg_env_gather_patch_direct(env, nullptr));
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    int32_t b = 0;
    float d = 0.0f;
    TRY(run_bounce(env, max_bounces, rel_tol, &b, &d));
    if (out_bounces) *out_bounces = b;
    if (out_delta) *out_delta = d;
    if (out_total) {
        const int64_t nl = (int64_t)env->patches.leaf_patch.size();
        std::vector<float4> tot(nl);
        if (nl) VRG_CUDA(ctx, cudaMemcpyAsync(tot.data(), env->d_total.ptr, 16 * nl, cudaMemcpyDeviceToHost, ctx->stream));
        TRY(sync(ctx));
        for (int64_t i = 0; i < nl; i++) {
            out_total[3 * i] = tot[i].x;
            out_total[3 * i + 1] = tot[i].y;
            out_total[3 * i + 2] = tot[i].z;
        }
    }
    return VRG_OK;
}

}  // extern "C"
