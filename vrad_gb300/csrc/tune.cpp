// tune.cpp -- per-scene-size autotuning of kernel variants.
//
// A tuned launch site offers a few variants of one kernel that compute the
// same result with different trade-offs (how many triangle planes a walk
// fetches at once, how much work a warp claims at a time).  The first launch
// in a scene-size bucket (log2 of the triangle count and of the work size)
// runs every variant twice on the real input, timed with CUDA events, and
// keeps the fastest; later launches in that bucket use it directly.  Inside
// a stream capture, or with tuning switched off, an untuned bucket runs
// variant 0.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>

#include "vrg_internal.h"

namespace vrg {

std::string tune_key(const char *kernel, int64_t scene_size, int64_t work) {
    auto lg = [](int64_t v) {
        int r = 0;
        while (v > 1) {
            v >>= 1;
            r++;
        }
        return r;
    };
    std::ostringstream k;
    k << kernel << "/t" << lg(scene_size) << "/n" << lg(work);
    return k.str();
}

int tune_pick(vrg_ctx *ctx, const std::string &key, int nvar,
              const std::function<cudaError_t(int)> &launch, int *variant) {
    *variant = 0;
    bool tune = false;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        auto it = ctx->tuned.find(key);
        if (it != ctx->tuned.end()) *variant = it->second < nvar ? it->second : 0;
        else tune = ctx->autotune;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        tune = false;
    if (nvar > kTuneMaxVariants) return fail(ctx, VRG_ERR_INVALID, "too many variants at a tuned launch site");
    if (!tune || nvar < 2) return VRG_OK;
    cudaEvent_t a = nullptr, b = nullptr;
    VRG_CUDA(ctx, cudaEventCreate(&a));
    VRG_CUDA(ctx, cudaEventCreate(&b));
    std::vector<double> ms(nvar, 0.0);
    cudaError_t err = launch(0);  // warm-up: first touch of code and data
    // two passes, the second in reverse order, keeping each variant's
    // faster run: a one-off slow launch or a drift of the clock over the
    // passes does not decide the choice
    for (int pass = 0; pass < 2; pass++)
        for (int j = 0; j < nvar && err == cudaSuccess; j++) {
            const int i = pass == 0 ? j : nvar - 1 - j;
            err = cudaEventRecord(a, ctx->stream);
            if (err == cudaSuccess) err = launch(i);
            if (err == cudaSuccess) err = cudaEventRecord(b, ctx->stream);
            if (err == cudaSuccess) err = cudaEventSynchronize(b);
            float t = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&t, a, b);
            ms[i] = pass == 0 ? t : std::min<double>(ms[i], t);
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (err != cudaSuccess) return cuda_fail(ctx, err, "autotune");
    int best = 0;
    for (int i = 1; i < nvar; i++)
        if (ms[i] < ms[best]) best = i;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuned[key] = best;
    ctx->tune_ms[key] = ms;
    *variant = best;
    return VRG_OK;
}

int tune_run(vrg_ctx *ctx, const std::string &key, int nvar,
             const std::function<cudaError_t(int)> &launch) {
    bool ran = false;
    int v = 0;
    const int rc = tune_pick(ctx, key, nvar, [&](int i) { ran = true; return launch(i); }, &v);
    if (rc != VRG_OK || ran) return rc;  // a tuning run already produced the result
    VRG_CUDA(ctx, launch(v));
    return VRG_OK;
}

}  // namespace vrg

using namespace vrg;

extern "C" {

int vrg_ctx_set_autotune(vrg_ctx *ctx, int enable) {
    if (!ctx) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->autotune = enable != 0;
    return VRG_OK;
}

int vrg_ctx_autotune_choice(vrg_ctx *ctx, const char *key, int32_t *variant, double *ms, int32_t cap) {
    if (!ctx || !key || !variant) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->tuned.find(key);
    if (it == ctx->tuned.end()) {
        *variant = -1;
        return VRG_OK;
    }
    *variant = it->second;
    auto jt = ctx->tune_ms.find(key);
    if (ms && jt != ctx->tune_ms.end())
        for (int32_t i = 0; i < cap && i < (int32_t)jt->second.size(); i++) ms[i] = jt->second[i];
    return VRG_OK;
}

// Tuned choices as text, one "key variant" per line.
int vrg_ctx_autotune_save(vrg_ctx *ctx, const char *path) {
    if (!ctx || !path) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::ofstream f(path);
    if (!f) return fail(nullptr, VRG_ERR_INVALID, "cannot write autotune file");
    for (auto &kv : ctx->tuned) f << kv.first << " " << kv.second << "\n";
    return f.good() ? VRG_OK : VRG_ERR_INVALID;
}

int vrg_ctx_autotune_load(vrg_ctx *ctx, const char *path) {
    if (!ctx || !path) return VRG_ERR_INVALID;
    std::ifstream f(path);
    if (!f) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::string key;
    int v;
    while (f >> key >> v)
        if (v >= 0 && v < kTuneMaxVariants) ctx->tuned[key] = v;
    return VRG_OK;
}

}  // extern "C"
