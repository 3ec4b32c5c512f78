// coverage.cu -- transparent shadows: Trace4Rays with a transparent-triangle
// callback (raytracer/environment.go:140-142) that counts coverage the way
// types.CoverageCount does (raytracer/types/coverageCount.go:27-41: each hit
// triangle adds its colour's x, clamped at 1), and TestLineDoesHitSky with
// texture shadows on (raytracer/trace/testline.go:29-33,53-55).
//
// The reference never fixes the order in which hits reach the callback (its
// Trace4Rays is a stub), and a float sum depends on that order.  The project
// defines it: a ray's accepted hits (tmin <= t < tmax, ids equal to the skip
// id ignored) are taken in ascending (t, triangle index).  An opaque hit is
// recorded and ends the walk; a transparent hit (triangle flag
// VRG_TRIFLAG_TRANSPARENT) adds c = min(c + coverage, 1), and when c reaches
// 1 that triangle is recorded and ends the walk.  For a shadow line,
// occlusion = max(1 if the recorded hit is before the end and not sky,
// c), clamped to [0, 1]; fraction visible = 1 - occlusion.
//
// On the device: one closest-hit walk over the opaque triangles only, then
// one closest-hit walk per transparent hit, each over the transparent
// triangles after the previous one in (t, index) order and before the opaque
// hit.  Every walk is the exact test of the other kernels, so the sum runs
// over the same floats in the same order as the oracle's sorted list.
#include <algorithm>

#include "vrg_internal.h"
#include "vrg_trace.cuh"

namespace vrg {

namespace {

constexpr int kCoverThreads = 128;

// Which triangles a walk accepts: mode 1 the opaque ones; mode 2 the
// transparent ones strictly after (lo_t, lo_i) and, when hi_i >= 0, strictly
// before (hi_t, hi_i), in (t, index) order.
struct CoverFilter {
    const uint8_t *flags;
    int mode;
    float lo_t;
    int32_t lo_i;
    float hi_t;
    int32_t hi_i;
};

// The exact test of tri_test (same operations, same order) with the filter;
// keeps the closest accepted hit (ties to the lower index).
__device__ __forceinline__ void filtered_tri(const DevScene &s, const Ray &ray, float tmin, float tmax,
                                             int32_t skip, const float4 w0, size_t k, const CoverFilter &f,
                                             int32_t &best, float &best_t) {
    const float den = dot3r(w0.x, w0.y, w0.z, ray.dx, ray.dy, ray.dz);
    const float on = dot3r(w0.x, w0.y, w0.z, ray.ox, ray.oy, ray.oz);
    const float t = rdiv(rsub(w0.w, on), den);
    if (!(t >= tmin && t < tmax)) return;
    if (!(t <= best_t)) return;
    const float4 *ed = s.leaf_edges + 2 * k;
    const float4 w2 = __ldg(ed + 1);
    if (__float_as_int(w2.z) == skip) return;
    const float4 w1 = __ldg(ed);
    const uint32_t idx_drop = __float_as_uint(w2.w);
    const int drop = (int)(idx_drop & 3u);
    const float o0 = drop == 0 ? ray.oy : (drop == 1 ? ray.oz : ray.ox);
    const float o1 = drop == 0 ? ray.oz : (drop == 1 ? ray.ox : ray.oy);
    const float d0 = drop == 0 ? ray.dy : (drop == 1 ? ray.dz : ray.dx);
    const float d1 = drop == 0 ? ray.dz : (drop == 1 ? ray.dx : ray.dy);
    const float h0 = radd(o0, rmul(t, d0));
    const float h1 = radd(o1, rmul(t, d1));
    const float b0 = radd(radd(rmul(w1.x, h0), rmul(w1.z, h1)), w2.x);
    const float b1 = radd(radd(rmul(w1.y, h0), rmul(w1.w, h1)), w2.y);
    const float b2 = rsub(rsub(1.0f, b0), b1);
    if (!(b0 >= 0.0f && b1 >= 0.0f && b2 >= 0.0f)) return;
    const int32_t ti = (int32_t)(idx_drop >> 2);
    const bool transparent = (__ldg(f.flags + ti) & VRG_TRIFLAG_TRANSPARENT) != 0;
    if (f.mode == 1 && transparent) return;
    if (f.mode == 2) {
        if (!transparent) return;
        if (!(t > f.lo_t || ti > f.lo_i)) return;
        if (f.hi_i >= 0 && !(t < f.hi_t || (t == f.hi_t && ti < f.hi_i))) return;
    }
    if (t < best_t || ti < best) {
        best = ti;
        best_t = t;
    }
}

// A closest-hit walk (the slab walk of vrg_trace.cuh) whose leaves are
// tested through filtered_tri.
__device__ int32_t filtered_trace(const DevScene &s, const Ray &ray, const RayPre &rp, float slack, float tmin,
                                  float tmax, int32_t skip, const CoverFilter &f, float *t_out) {
    TraceState st;
    if (trace_init(s, ray, rp, slack, tmin, tmax, st, 0u)) {
        for (;;) {
            uint32_t node = st.node;
            float t0 = st.t0, t1 = st.t1;
            int sp = st.sp;
            uint2 nd = fetch_node<0>(s, node);
            bool reached = true;
            while ((nd.x & 3u) != 3u) {
                if (!inner_step<0>(rp, nd, t0, t1, st.stk, sp, node)) {
                    reached = false;
                    break;
                }
                nd = fetch_node<0>(s, node);
            }
            if (reached) {
                const uint32_t start = nd.x >> 2;
                const int cnt = (int)__uint_as_float(nd.y);
                for (int j = 0; j < cnt; j++)
                    filtered_tri(s, ray, tmin, tmax, skip, __ldg(s.leaf_planes + start + j), (size_t)start + j, f,
                                 st.best, st.best_t);
            }
            if (!pop_next<kClosest>(st.stk, sp, st.best_t, st.node, st.t0, st.t1)) break;
            st.sp = sp;
        }
    }
    *t_out = st.best_t;
    return st.best;
}

// One lane per ray (lines = 0: origin a, unit direction b, [tmin, tmax)) or
// per shadow line (lines = 1: start a, stop b, TestLineDoesHitSky setup).
__global__ void __launch_bounds__(kCoverThreads) k_coverage(
    DevScene s, const uint8_t *__restrict__ flags, const float *__restrict__ cover, int32_t ntransparent,
    const float *__restrict__ a, const float *__restrict__ b, const float *__restrict__ tmin_in,
    const float *__restrict__ tmax_in, int64_t n, int32_t skip, int lines, int32_t *__restrict__ out_hit,
    float *__restrict__ out_t, float *__restrict__ out_cov, float *__restrict__ out_frac) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        Ray ray;
        float tmin, tmax;
        if (lines) {
            const Line L = make_line(a[3 * i], a[3 * i + 1], a[3 * i + 2], b[3 * i], b[3 * i + 1], b[3 * i + 2]);
            if (!(L.len > 0.0f)) {
                out_frac[i] = 1.0f;
                continue;
            }
            ray = Ray{L.ox, L.oy, L.oz, L.dx, L.dy, L.dz};
            tmin = 0.0f;
            tmax = L.len;
        } else {
            ray = Ray{a[3 * i], a[3 * i + 1], a[3 * i + 2], b[3 * i], b[3 * i + 1], b[3 * i + 2]};
            tmin = tmin_in[i];
            tmax = tmax_in[i];
        }
        const float slack = ray_slack(s.g, ray.ox, ray.oy, ray.oz);
        const RayPre rp = ray_pre(ray, slack);
        CoverFilter f{flags, 1, 0.0f, -1, 0.0f, -1};
        float t_rec;
        int32_t rec = filtered_trace(s, ray, rp, slack, tmin, tmax, skip, f, &t_rec);
        float c = 0.0f;
        f.mode = 2;
        f.lo_t = tmin;
        f.lo_i = -1;
        f.hi_t = t_rec;
        f.hi_i = rec;
        // each walk returns a different transparent triangle (the next in
        // (t, index) order), so ntransparent walks at most
        for (int32_t it = 0; it < ntransparent; it++) {
            float tt;
            const int32_t ht = filtered_trace(s, ray, rp, slack, f.lo_t, tmax, skip, f, &tt);
            if (ht < 0) break;
            c = fminf(radd(c, __ldg(cover + ht)), 1.0f);
            if (c >= 1.0f) {
                rec = ht;
                t_rec = tt;
                break;
            }
            f.lo_t = tt;
            f.lo_i = ht;
        }
        if (lines) {
            float occ = (rec >= 0 && t_rec < tmax && (__ldg(&s.tri_ids[rec]) & kTraceIdSky) == 0) ? 1.0f : 0.0f;
            occ = fmaxf(occ, c);
            occ = fminf(fmaxf(occ, 0.0f), 1.0f);
            out_frac[i] = rsub(1.0f, occ);
        } else {
            out_hit[i] = rec;
            out_t[i] = t_rec;
            out_cov[i] = c;
        }
    }
}

int cover_fail(vrg_ctx *ctx, int code, const char *msg) { return fail(ctx, code, msg); }

// Per-triangle flags and coverage on the device (built on first use after
// SetupAccelerationStructure).
int cover_upload(vrg_env *env) {
    vrg_ctx *ctx = env->ctx;
    const size_t n = env->ids.size();
    if (env->cover_ready) return VRG_OK;
    std::vector<float> cov(n, 0.0f);
    std::vector<uint8_t> fl(n, 0);
    int32_t nt = 0;
    for (size_t i = 0; i < n; i++) {
        cov[i] = i < env->cover.size() ? env->cover[i] : 0.0f;
        fl[i] = i < env->flags.size() ? env->flags[i] : 0;
        nt += (fl[i] & VRG_TRIFLAG_TRANSPARENT) ? 1 : 0;
    }
    VRG_CUDA(ctx, env->d_tri_cover.reserve(4 * std::max<size_t>(n, 1)));
    VRG_CUDA(ctx, env->d_tri_flags.reserve(std::max<size_t>(n, 16)));
    if (n) {
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_tri_cover.ptr, cov.data(), 4 * n, cudaMemcpyHostToDevice, ctx->stream));
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_tri_flags.ptr, fl.data(), n, cudaMemcpyHostToDevice, ctx->stream));
    }
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope
    env->n_transparent = nt;
    env->cover_ready = true;
    return VRG_OK;
}

int run_coverage(vrg_env *env, const float *a, const float *b, const float *tmin, const float *tmax, int64_t n,
                 int32_t skip, int lines, int32_t *hit, float *t, float *cov, float *frac) {
    vrg_ctx *ctx = env->ctx;
    if (!env->built) return cover_fail(ctx, VRG_ERR_STATE, "SetupAccelerationStructure has not run");
    if (n == 0) return VRG_OK;
    {
        const int rc = cover_upload(env);
        if (rc != VRG_OK) return rc;
    }
    DevBuf da, db, dt0, dt1, dh, dtt, dc, df;
    VRG_CUDA(ctx, da.reserve(12 * (size_t)n));
    VRG_CUDA(ctx, db.reserve(12 * (size_t)n));
    VRG_CUDA(ctx, cudaMemcpyAsync(da.ptr, a, 12 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaMemcpyAsync(db.ptr, b, 12 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    if (!lines) {
        VRG_CUDA(ctx, dt0.reserve(4 * (size_t)n));
        VRG_CUDA(ctx, dt1.reserve(4 * (size_t)n));
        VRG_CUDA(ctx, dh.reserve(4 * (size_t)n));
        VRG_CUDA(ctx, dtt.reserve(4 * (size_t)n));
        VRG_CUDA(ctx, dc.reserve(4 * (size_t)n));
        VRG_CUDA(ctx, cudaMemcpyAsync(dt0.ptr, tmin, 4 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
        VRG_CUDA(ctx, cudaMemcpyAsync(dt1.ptr, tmax, 4 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        VRG_CUDA(ctx, df.reserve(4 * (size_t)n));
    }
    const int grid = (int)std::min<int64_t>((n + kCoverThreads - 1) / kCoverThreads, (int64_t)ctx->num_sms * 16);
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "coverage", &ev);
    k_coverage<<<grid, kCoverThreads, 0, ctx->stream>>>(
        scene_view(env), env->d_tri_flags.as<uint8_t>(), env->d_tri_cover.as<float>(), env->n_transparent,
        da.as<float>(), db.as<float>(), dt0.as<float>(), dt1.as<float>(), n, skip, lines, dh.as<int32_t>(),
        dtt.as<float>(), dc.as<float>(), df.as<float>());
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "coverage", ev);
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->launches++;
    }
    if (lines) {
        VRG_CUDA(ctx, cudaMemcpyAsync(frac, df.ptr, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        VRG_CUDA(ctx, cudaMemcpyAsync(hit, dh.ptr, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        VRG_CUDA(ctx, cudaMemcpyAsync(t, dtt.ptr, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        VRG_CUDA(ctx, cudaMemcpyAsync(cov, dc.ptr, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    collect_timings(ctx);
    return VRG_OK;
}

}  // namespace

}  // namespace vrg

extern "C" {

int vrg_env_set_triangle_flags(vrg_env *env, int64_t first, int64_t n, const uint8_t *flags,
                               const float *colours) {
    using namespace vrg;
    if (!env || first < 0 || n < 0 || (n > 0 && !flags)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    const int64_t ntris = (int64_t)env->ids.size();
    if (first + n > ntris) return fail(env->ctx, VRG_ERR_INVALID, "triangle range out of bounds");
    if (env->built) return fail(env->ctx, VRG_ERR_STATE, "triangle flags set after SetupAccelerationStructure");
    env->flags.resize((size_t)ntris, 0);
    env->cover.resize((size_t)ntris, 0.0f);
    for (int64_t i = 0; i < n; i++) {
        env->flags[first + i] = flags[i];
        if (colours) env->cover[first + i] = colours[3 * i];
    }
    return VRG_OK;
}

int vrg_env_trace_coverage(vrg_env *env, const float *origin, const float *direction, const float *tmin,
                           const float *tmax, int64_t n, int32_t skip_id, int32_t *out_hit, float *out_t,
                           float *out_coverage) {
    using namespace vrg;
    if (!env || n < 0 ||
        (n > 0 && (!origin || !direction || !tmin || !tmax || !out_hit || !out_t || !out_coverage)))
        return VRG_ERR_INVALID;
    if (env->ctx->host_only) return fail(env->ctx, VRG_ERR_STATE, "host-only context has no device");
    std::lock_guard<std::mutex> lk(env->mu);
    return run_coverage(env, origin, direction, tmin, tmax, n, skip_id, 0, out_hit, out_t, out_coverage, nullptr);
}

int vrg_env_test_line_coverage(vrg_env *env, const float *start, const float *stop, int64_t n,
                               int32_t static_prop_to_skip, float *fraction_visible) {
    using namespace vrg;
    if (!env || n < 0 || (n > 0 && (!start || !stop || !fraction_visible))) return VRG_ERR_INVALID;
    if (env->ctx->host_only) return fail(env->ctx, VRG_ERR_STATE, "host-only context has no device");
    std::lock_guard<std::mutex> lk(env->mu);
    // testline.go:36: skip id = TRACE_ID_STATICPROP | staticPropToSkip
    const int32_t skip = VRG_TRACE_ID_STATICPROP | static_prop_to_skip;
    return run_coverage(env, start, stop, nullptr, nullptr, n, skip, 1, nullptr, nullptr, nullptr,
                        fraction_visible);
}

}  // extern "C"
