// bounce.cu -- the radiosity bounce loop over the CSR transfer lists.  The
// reference keeps only the state (Patch.TotalLight, DirectLight,
// Reflectivity, BaseLight: common/types/patch.go:33-42) and the bounce count
// (numBounce, rad/patches/subdivide.go:19); the loop is the project's own
// Jacobi gather:
//   emit = refl * direct + base ; total = 0
//   per bounce: add_i = sum_j w_ij emit_j ; total += add ; emit = refl * add
//   delta = sum |add|_1 / sum |total|_1 ; stop after the bounce whose delta
//   is below the tolerance, or after max_bounces.
// Each bounce is one SpMV kernel plus one single-block reduction; the loop
// is a CUDA graph whose conditional while node repeats a body of two bounces
// until the reduce kernel, reading the device-side control block, clears
// the condition.
#include <algorithm>
#include <memory>

#include "vrg_internal.h"
#include "vrg_spmv.cuh"

namespace vrg {

namespace {

constexpr int kSpmvThreads = 256;
constexpr int kGraphBounces = 8;

struct BounceControl {
    int32_t done;
    int32_t iters;
    int32_t max_iters;
    float tol;
    float last_delta;
    float pad[3];
};

__global__ void k_bounce_init(const LeafInfo *__restrict__ info, const float *__restrict__ direct,
                              float4 *__restrict__ emit, float4 *__restrict__ total, int64_t n,
                              BounceControl *ctl, int32_t max_iters, float tol) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 r = info[i].refl, b = info[i].base;
        emit[i] = make_float4(__fadd_rn(__fmul_rn(r.x, direct[3 * i]), b.x),
                              __fadd_rn(__fmul_rn(r.y, direct[3 * i + 1]), b.y),
                              __fadd_rn(__fmul_rn(r.z, direct[3 * i + 2]), b.z), 0.0f);
        total[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->done = max_iters <= 0;
        ctl->iters = 0;
        ctl->max_iters = max_iters;
        ctl->tol = tol;
        ctl->last_delta = 0.0f;
    }
}

// One warp per row (row_gather with U entries per lane per round), rows
// strided over the grid's warps, so the NT / 32 warps of a block work on
// neighbouring rows (neighbouring patches, which see much the same patches:
// their emission gathers share L1 lines).  Per-block sums of |add| and
// |total| go to partials[2*block].
template <int U, int NT = kSpmvThreads, int MINB = 1, bool NA = false>
__global__ void __launch_bounds__(NT, MINB) k_bounce_spmv(
    const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
    const float *__restrict__ w, const float4 *__restrict__ emit_in, float4 *__restrict__ emit_out,
    float4 *__restrict__ total, const LeafInfo *__restrict__ info, int64_t n,
    const BounceControl *__restrict__ ctl, double *__restrict__ partials) {
    if (*(volatile const int32_t *)&ctl->done) return;
    __shared__ double red[2][NT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double sa = 0.0, st = 0.0;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nwarps) {
        const float3 a = warp_sum3(row_gather<U, NA>(col, w, emit_in, row_ptr[row], row_ptr[row + 1], lane));
        if (lane == 0) {
            float4 t = total[row];
            t.x += a.x;
            t.y += a.y;
            t.z += a.z;
            total[row] = t;
            const float4 r = info[row].refl;
            emit_out[row] = make_float4(r.x * a.x, r.y * a.y, r.z * a.z, 0.0f);
            sa += (double)fabsf(a.x) + (double)fabsf(a.y) + (double)fabsf(a.z);
            st += (double)fabsf(t.x) + (double)fabsf(t.y) + (double)fabsf(t.z);
        }
    }
    if (lane == 0) {
        red[0][wid] = sa;
        red[1][wid] = st;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, t = 0.0;
        for (int k = 0; k < NT / 32; k++) {
            a += red[0][k];
            t += red[1][k];
        }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = t;
    }
}

// Sums the block partials in a fixed order and advances the control block.
// Inside the loop graph (in_loop) thread 0 also sets the loop's condition:
// the while node runs its body again only while the loop is not done.
__global__ void k_bounce_reduce(BounceControl *ctl, const double *__restrict__ partials, int nblocks,
                                int in_loop, cudaGraphConditionalHandle loop) {
    if (*(volatile int32_t *)&ctl->done) {
        if (in_loop && threadIdx.x == 0) cudaGraphSetConditional(loop, 0u);
        return;
    }
    __shared__ double sa[256], st[256];
    double a = 0.0, t = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        a += partials[2 * i];
        t += partials[2 * i + 1];
    }
    sa[threadIdx.x] = a;
    st[threadIdx.x] = t;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sa[threadIdx.x] += sa[threadIdx.x + o];
            st[threadIdx.x] += st[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const float delta = st[0] > 0.0 ? (float)(sa[0] / st[0]) : 0.0f;
        ctl->last_delta = delta;
        ctl->iters += 1;
        const int done = delta < ctl->tol || ctl->iters >= ctl->max_iters;
        if (done) ctl->done = 1;
        if (in_loop) cudaGraphSetConditional(loop, done ? 0u : 1u);
    }
}

}  // namespace

// The bounce loop of a scene as an executable graph (see run_bounce).
struct BounceGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<const void *> key;  // the buffers, sizes and variant it was built on
    ~BounceGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

void bounce_release(vrg_env *env) {
    delete env->bounce_graph;
    env->bounce_graph = nullptr;
}

int run_bounce(vrg_env *env, int32_t max_bounces, float rel_tol, int32_t *bounces, float *delta) {
    vrg_ctx *ctx = env->ctx;
    const int64_t n = (int64_t)env->patches.leaf_patch.size();
    VRG_CUDA(ctx, env->d_emit.reserve(2 * 16 * (size_t)std::max<int64_t>(n, 1)));
    VRG_CUDA(ctx, env->d_total.reserve(16 * (size_t)std::max<int64_t>(n, 1)));
    VRG_CUDA(ctx, env->d_partials.reserve(16 * (size_t)ctx->num_sms * 8));
    VRG_CUDA(ctx, env->d_control.reserve(sizeof(BounceControl)));
    float4 *e0 = env->d_emit.as<float4>(), *e1 = e0 + std::max<int64_t>(n, 1);
    BounceControl *ctl = env->d_control.as<BounceControl>();
    const int ib = (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), (int64_t)ctx->num_sms * 8);
    auto init = [&]() -> cudaError_t {
        cudaEvent_t ev = nullptr;
        timing_begin(ctx, "bounce_init", &ev);
        k_bounce_init<<<ib, 256, 0, ctx->stream>>>(env->d_leaf_info.as<LeafInfo>(), env->d_leaf_direct.as<float>(),
                                                   e0, env->d_total.as<float4>(), n, ctl, max_bounces, rel_tol);
        cudaError_t e = cudaGetLastError();
        timing_end(ctx, "bounce_init", ev);
        return e;
    };
    VRG_CUDA(ctx, init());

    // SpMV variants, picked per (nnz, rows) bucket: 4, 8 or 2 entries per
    // lane per round, 256, 512 or 1024 threads per block (more neighbouring
    // rows per block at a time), and 4 per round at a 5-block register cap
    // with the column / weight stream kept out of L1; the same sums.  Each
    // runs one wave: resident blocks per SM times SMs.
    using SpmvKernel = void (*)(const int64_t *, const int32_t *, const float *, const float4 *,
                                float4 *, float4 *, const LeafInfo *, int64_t,
                                const BounceControl *, double *);
    constexpr int kSpmvVariants = 7;
    const SpmvKernel kvar[kSpmvVariants] = {k_bounce_spmv<4>,       k_bounce_spmv<8>,       k_bounce_spmv<2>,
                                            k_bounce_spmv<4, 512>,  k_bounce_spmv<4, 1024>, k_bounce_spmv<2, 1024>,
                                            k_bounce_spmv<4, 256, 5, true>};
    const int vthreads[kSpmvVariants] = {256, 256, 256, 512, 1024, 1024, 256};
    auto spmv_blocks = [&](int v) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kvar[v], vthreads[v], 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        return ctx->num_sms * std::min(per_sm, 8);
    };
    auto spmv = [&](int v, float4 *in, float4 *out) -> cudaError_t {
        cudaEvent_t ev2 = nullptr;
        timing_begin(ctx, "bounce_spmv", &ev2);
        const SpmvKernel k = kvar[v];
        k<<<spmv_blocks(v), vthreads[v], 0, ctx->stream>>>(
            env->d_row_ptr.as<int64_t>(), env->d_col.as<int32_t>(), env->d_weight.as<float>(), in, out,
            env->d_total.as<float4>(), env->d_leaf_info.as<LeafInfo>(), n, ctl, env->d_partials.as<double>());
        cudaError_t e = cudaGetLastError();
        timing_end(ctx, "bounce_spmv", ev2);
        return e;
    };
    int var = 0;
    if (n > 0 && max_bounces > 0) {
        bool ran = false;
        const int rc = tune_pick(ctx, tune_key("bounce_spmv", env->nnz, n), kSpmvVariants,
                                 [&](int v) { ran = true; return spmv(v, e0, e1); }, &var);
        if (rc != VRG_OK) return rc;
        if (ran) VRG_CUDA(ctx, init());  // tuning ran bounces: start over
    }
    const int nblocks = spmv_blocks(var);

    auto one_bounce = [&](float4 *in, float4 *out) -> cudaError_t {
        cudaError_t e = spmv(var, in, out);
        if (e != cudaSuccess) return e;
        cudaEvent_t ev2 = nullptr;
        timing_begin(ctx, "bounce_reduce", &ev2);
        k_bounce_reduce<<<1, 256, 0, ctx->stream>>>(ctl, env->d_partials.as<double>(), nblocks, 0, 0);
        e = cudaGetLastError();
        timing_end(ctx, "bounce_reduce", ev2);
        return e;
    };

    BounceControl h{};
    int32_t launched = 0;
    // With timing on, bounces launch one by one so each kernel gets events
    // (and the host checks the control block every kGraphBounces); otherwise
    // the whole loop is one launch of the scene's loop graph.
    if (ctx->timing) {
        while (launched < max_bounces) {
            VRG_CUDA(ctx, one_bounce((launched & 1) ? e1 : e0, (launched & 1) ? e0 : e1));
            launched++;
            if ((launched % kGraphBounces) == 0 || launched == max_bounces) {
                VRG_CUDA(ctx, cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
                VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                if (h.done) break;
            }
        }
    } else if (max_bounces > 0) {
        // the loop as a graph with a conditional while node (body: two
        // bounces), kept on the scene and rebuilt only when a buffer it
        // points into, the size or the SpMV variant changes
        const std::vector<const void *> key = {e0, env->d_total.ptr, env->d_row_ptr.ptr, env->d_col.ptr,
                                               env->d_weight.ptr, env->d_leaf_info.ptr, ctl,
                                               env->d_partials.ptr, reinterpret_cast<const void *>((intptr_t)n),
                                               reinterpret_cast<const void *>((intptr_t)nblocks),
                                               reinterpret_cast<const void *>((intptr_t)var)};
        if (!env->bounce_graph || env->bounce_graph->key != key) {
            bounce_release(env);
            std::unique_ptr<BounceGraph> bg(new BounceGraph);
            cudaGraph_t g = nullptr;
            VRG_CUDA(ctx, cudaGraphCreate(&g, 0));
            cudaGraphConditionalHandle hc = 0;
            cudaError_t e = cudaGraphConditionalHandleCreate(&hc, g, 1u, cudaGraphCondAssignDefault);
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hc;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t wn = nullptr;
            if (e == cudaSuccess) e = cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &cp);
            if (e == cudaSuccess)
                e = cudaStreamBeginCaptureToGraph(ctx->stream, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaError_t le = spmv(var, e0, e1);
                k_bounce_reduce<<<1, 256, 0, ctx->stream>>>(ctl, env->d_partials.as<double>(), nblocks, 1, hc);
                if (le == cudaSuccess) le = cudaGetLastError();
                if (le == cudaSuccess) le = spmv(var, e1, e0);
                k_bounce_reduce<<<1, 256, 0, ctx->stream>>>(ctl, env->d_partials.as<double>(), nblocks, 1, hc);
                if (le == cudaSuccess) le = cudaGetLastError();
                cudaGraph_t captured = nullptr;
                e = cudaStreamEndCapture(ctx->stream, &captured);
                if (e == cudaSuccess) e = le;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&bg->exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "bounce loop graph");
            bg->key = key;
            env->bounce_graph = bg.release();
        }
        VRG_CUDA(ctx, cudaGraphLaunch(env->bounce_graph->exec, ctx->stream));
    }
    VRG_CUDA(ctx, cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *bounces = h.iters;
    *delta = h.last_delta;
    return VRG_OK;
}

}  // namespace vrg

// ---------------------------------------------------------------------------
// Bounce loop without allocation.
//
// For callers that must not allocate device memory while they run: a
// serving loop that has reserved its memory up front and may not grow it
// mid-request, a process whose memory is carved out in advance by a
// framework pool (where a stray cudaMalloc can fail or fragment the pool),
// or code queued between other work where an implicit device-wide
// synchronisation by cudaMalloc/cudaFree would stall unrelated streams.
// This entry point reads only what is already resident (the transfer lists
// from vrg_env_make_transfers and the patch direct light from
// vrg_env_gather_patch_direct) and keeps its working state (two emission
// buffers, per-block partial sums, the loop control block) in one
// file-scope device array, held by every GPU that loads the library until
// the process exits.  With lazy module loading the array comes into being
// when bounce.cu's module is first loaded on a device; vrg_ctx_create does
// that (noalloc_prepare below), so the entry point itself allocates
// nothing, its first call included.
namespace vrg {
namespace {

constexpr int64_t kNoAllocMaxRows = 262144;  // leaf patches
constexpr int kNoAllocBlocks = 1024;         // SpMV blocks (partials slots)
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    float4 emit[2][kNoAllocMaxRows];
    double partials[2 * kNoAllocBlocks];
    BounceControl ctl;
};

// 8 MiB + 16 KiB on every GPU that loads the library.
static __device__ __align__(256) NoAllocScratch g_bounce_scratch;

std::mutex g_scratch_mu;
NoAllocScratch *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
// Looked up once per device; host code never passes the symbol itself to a
// kernel, because on the host that name is only a stand-in.
int noalloc_scratch(vrg_ctx *ctx, NoAllocScratch **out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return fail(ctx, VRG_ERR_UNSUPPORTED, "device index out of range for the no-alloc bounce");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_bounce_scratch);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_bounce_scratch)");
        g_scratch_ptr[ctx->device] = static_cast<NoAllocScratch *>(p);
    }
    *out = g_scratch_ptr[ctx->device];
    return VRG_OK;
}

void count_launch(vrg_ctx *ctx) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->launches++;
}

}  // namespace

// Context set-up (device current): resolves the scratch array's address and
// loads the no-alloc path's kernels, so neither happens inside a later call.
int noalloc_prepare(vrg_ctx *ctx) {
    NoAllocScratch *sc = nullptr;
    const int rc = noalloc_scratch(ctx, &sc);
    if (rc != VRG_OK) return rc;
    cudaFuncAttributes fa;
    VRG_CUDA(ctx, cudaFuncGetAttributes(&fa, k_bounce_init));
    VRG_CUDA(ctx, cudaFuncGetAttributes(&fa, k_bounce_spmv<4>));
    VRG_CUDA(ctx, cudaFuncGetAttributes(&fa, k_bounce_reduce));
    return VRG_OK;
}

}  // namespace vrg

extern "C" int vrg_env_bounce_light_noalloc(vrg_env *env, int32_t max_bounces, float rel_tol,
                                            float *total_out, int32_t *out_bounces,
                                            float *out_delta) {
    using namespace vrg;
    if (!env) return VRG_ERR_INVALID;
    vrg_ctx *ctx = env->ctx;
    std::lock_guard<std::mutex> lk(env->mu);
    if (ctx->host_only) return fail(ctx, VRG_ERR_STATE, "host-only context has no device");
    if (!env->built || !env->have_transfers)
        return fail(ctx, VRG_ERR_STATE, "vrg_env_make_transfers has not run");
    if (!env->have_patch_direct)
        return fail(ctx, VRG_ERR_STATE, "vrg_env_gather_patch_direct has not run");
    if (max_bounces < 0 || !(rel_tol >= 0.0f) || !total_out)
        return fail(ctx, VRG_ERR_INVALID, "no-alloc bounce: bad bounce count, tolerance or output");
    const int64_t n = (int64_t)env->patches.leaf_patch.size();
    if (n > kNoAllocMaxRows)
        return fail(ctx, VRG_ERR_UNSUPPORTED,
                    "no-alloc bounce holds at most 262144 leaf patches; this scene has " +
                        std::to_string(n));
    VRG_CUDA(ctx, cudaSetDevice(ctx->device));
    // The output is written as float4: it must be device (or managed) memory
    // of this context's device, 16-byte aligned.  Anything else would fault
    // on the GPU, so it is refused here, before any launch.
    {
        cudaPointerAttributes pa{};
        const cudaError_t e = cudaPointerGetAttributes(&pa, total_out);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, VRG_ERR_INVALID, "no-alloc bounce: total_out is not a device pointer");
        }
        if ((pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) || pa.device != ctx->device)
            return fail(ctx, VRG_ERR_INVALID, "no-alloc bounce: total_out is not device memory of this context's GPU");
        if ((reinterpret_cast<uintptr_t>(total_out) & 15u) != 0)
            return fail(ctx, VRG_ERR_INVALID, "no-alloc bounce: total_out is not 16-byte aligned");
    }
    NoAllocScratch *sc = nullptr;
    {
        const int rc = noalloc_scratch(ctx, &sc);
        if (rc != VRG_OK) return rc;
    }
    float4 *e0 = sc->emit[0], *e1 = sc->emit[1];
    float4 *total = reinterpret_cast<float4 *>(total_out);
    BounceControl *ctl = &sc->ctl;
    double *partials = sc->partials;
    const int nblocks = std::min(kNoAllocBlocks, ctx->num_sms * 4);
    const int ib = (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), (int64_t)ctx->num_sms * 8);
    // k_bounce_init zeroes the totals and resets the control block, so no
    // state of an earlier call leaks into this one.
    k_bounce_init<<<ib, 256, 0, ctx->stream>>>(env->d_leaf_info.as<LeafInfo>(), env->d_leaf_direct.as<float>(),
                                               e0, total, n, ctl, max_bounces, rel_tol);
    VRG_CUDA(ctx, cudaGetLastError());
    count_launch(ctx);
    BounceControl h{};
    int32_t launched = 0;
    while (launched < max_bounces) {
        float4 *in = (launched & 1) ? e1 : e0, *out = (launched & 1) ? e0 : e1;
        k_bounce_spmv<4><<<nblocks, kSpmvThreads, 0, ctx->stream>>>(
            env->d_row_ptr.as<int64_t>(), env->d_col.as<int32_t>(), env->d_weight.as<float>(), in, out, total,
            env->d_leaf_info.as<LeafInfo>(), n, ctl, partials);
        VRG_CUDA(ctx, cudaGetLastError());
        k_bounce_reduce<<<1, 256, 0, ctx->stream>>>(ctl, partials, nblocks, 0, 0);
        VRG_CUDA(ctx, cudaGetLastError());
        count_launch(ctx);
        count_launch(ctx);
        launched++;
        if ((launched % kGraphBounces) == 0 || launched == max_bounces) {
            VRG_CUDA(ctx, cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
            VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (h.done) break;
        }
    }
    VRG_CUDA(ctx, cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (out_bounces) *out_bounces = h.iters;
    if (out_delta) *out_delta = h.last_delta;
    return VRG_OK;
}
