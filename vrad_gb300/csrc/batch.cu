// batch.cu -- whole bakes (direct light at every luxel and leaf patch, then
// the bounce loop) for one scene or for many resident scenes at once.
//
// A batched bake runs the direct pass of every scene in ONE persistent
// launch: warps take 32 work items at a time from a device counter, where
// the work list is every scene's luxel supersamples followed by every
// scene's leaf-patch sample points, so small and large scenes share the GPU
// without per-scene launch tails.  The bounce loop then runs block-diagonal
// over all scenes' transfer rows (one SpMV kernel per bounce for all
// scenes), with a per-scene energy delta, stop flag and bounce count; a CUDA
// graph holds several bounces and is replayed until every scene has
// stopped.  Per scene the arithmetic is the same as the one-scene path, so a
// batched bake with a fixed bounce count gives identical results.
#include <algorithm>
#include <cstring>
#include <new>

#include "vrg_gather.cuh"
#include "vrg_internal.h"
#include "vrg_spmv.cuh"

namespace vrg {

namespace {

constexpr int kThreads = 128;
static_assert(kThreads <= kShRayLanes, "kOptShRay keeps one slot per thread of a block");
constexpr int kSpmvThreads = 256;
constexpr int kGraphBounces = 8;

// What the batched kernels read of one scene.
struct BatchDesc {
    DevScene scene;
    const DevLight *lights;
    const FaceRec *faces;
    const int64_t *luxel_off;
    float *out_rgb;
    const float *ppts, *pnrm;
    float *pout;
    const int64_t *row_ptr;
    const int32_t *col;
    const float *w;
    const LeafInfo *leaf;
    float4 *emit0, *emit1, *total;
    int64_t nlux, npts, rows;
    int32_t nl, nfaces;
};

struct SceneCtl {
    int32_t done, iters, max_iters;
    float tol, last_delta;
    int32_t pad[3];
};

__device__ __forceinline__ int upper_segment(const int64_t *__restrict__ start, int n, int64_t i) {
    // largest s with start[s] <= i, for start[0] = 0 <= i < start[n]
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(start + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Work items: segments [0, E) are scene e's luxel supersamples (ss per
// luxel, in luxel order), segments [E, 2E) scene e's leaf-patch points.
// OPT: walk options (kOptShRay or none); MINB: resident blocks per SM.
template <int OPT, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_batch_gather(
    const BatchDesc *__restrict__ descs, const int64_t *__restrict__ seg, int nscenes, int ss,
    uint64_t seed, unsigned long long *__restrict__ work, unsigned long long *__restrict__ ray_count) {
    const int64_t total = __ldg(seg + 2 * nscenes);
    const int lane = threadIdx.x & 31;
    uint32_t rays = 0;
    for (;;) {
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(work, 32ull);
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (wb >= (unsigned long long)total) break;
        const int64_t gi = (int64_t)wb + lane;
        float r = 0.0f, g = 0.0f, b = 0.0f;
        bool luxel_item = false;
        int64_t lux = 0;
        float *lux_out = nullptr;
        if (gi < total) {
            const int sg = upper_segment(seg, 2 * nscenes, gi);
            const int64_t local = gi - __ldg(seg + sg);
            const BatchDesc *d = descs + (sg < nscenes ? sg : sg - nscenes);
            // the item's point and normal, then one gather_point call site
            // (a second inlined copy of the gather costs through code size)
            float px, py, pz, nx, ny, nz;
            if (sg < nscenes) {
                luxel_item = true;
                lux = local / ss;
                const int k = (int)(local - lux * ss);
                const int f = find_face(d->luxel_off, d->nfaces, lux);
                const FaceRec fr = d->faces[f];
                int iu, iv;  // the face's luxels in 4 x 2 tiles
                tile_luxel(lux - __ldg(d->luxel_off + f), fr.nu, fr.nv, iu, iv);
                lux = __ldg(d->luxel_off + f) + (int64_t)iv * fr.nu + iu;
                luxel_sample(fr, lux, iu, iv, k, ss, seed, px, py, pz);
                nx = fr.normal.x;
                ny = fr.normal.y;
                nz = fr.normal.z;
                lux_out = d->out_rgb;
            } else {
                const float *p = d->ppts + 3 * local, *n = d->pnrm + 3 * local;
                px = __ldg(p);
                py = __ldg(p + 1);
                pz = __ldg(p + 2);
                nx = __ldg(n);
                ny = __ldg(n + 1);
                nz = __ldg(n + 2);
            }
            gather_point<kSkyTrace, OPT>(d->scene, d->lights, d->nl, px, py, pz, nx, ny, nz, r, g, b, rays);
            if (!luxel_item) {
                float *o = d->pout + 3 * local;
                o[0] = r;
                o[1] = g;
                o[2] = b;
            }
        }
        if (ss == 4) {
            // luxel segments start at multiples of 4, so a luxel's samples
            // are the four lanes of one aligned quad
            const float r1 = __shfl_down_sync(0xffffffffu, r, 1), r2 = __shfl_down_sync(0xffffffffu, r, 2),
                        r3 = __shfl_down_sync(0xffffffffu, r, 3);
            const float g1 = __shfl_down_sync(0xffffffffu, g, 1), g2 = __shfl_down_sync(0xffffffffu, g, 2),
                        g3 = __shfl_down_sync(0xffffffffu, g, 3);
            const float b1 = __shfl_down_sync(0xffffffffu, b, 1), b2 = __shfl_down_sync(0xffffffffu, b, 2),
                        b3 = __shfl_down_sync(0xffffffffu, b, 3);
            if (luxel_item && (lane & 3) == 0) {
                lux_out[3 * lux + 0] = rmul(radd(radd(radd(r, r1), r2), r3), 0.25f);
                lux_out[3 * lux + 1] = rmul(radd(radd(radd(g, g1), g2), g3), 0.25f);
                lux_out[3 * lux + 2] = rmul(radd(radd(radd(b, b1), b2), b3), 0.25f);
            }
        } else if (luxel_item) {
            lux_out[3 * lux + 0] = r;
            lux_out[3 * lux + 1] = g;
            lux_out[3 * lux + 2] = b;
        }
    }
    unsigned long long wr = rays;
    for (int o = 16; o > 0; o >>= 1) wr += __shfl_down_sync(0xffffffffu, wr, o);
    if (lane == 0 && ray_count) atomicAdd(ray_count, wr);
}

__global__ void k_batch_bounce_init(const BatchDesc *__restrict__ descs, const int64_t *__restrict__ rstart,
                                    int nscenes, SceneCtl *__restrict__ ctl, int32_t max_iters, float tol,
                                    int32_t *__restrict__ done_count) {
    const int64_t rows = __ldg(rstart + nscenes);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += stride) {
        const int e = upper_segment(rstart, nscenes, r);
        const BatchDesc *d = descs + e;
        const int64_t i = r - __ldg(rstart + e);
        const float4 rf = d->leaf[i].refl, bs = d->leaf[i].base;
        const float *dir = d->pout + 3 * i;
        d->emit0[i] = make_float4(__fadd_rn(__fmul_rn(rf.x, dir[0]), bs.x), __fadd_rn(__fmul_rn(rf.y, dir[1]), bs.y),
                                  __fadd_rn(__fmul_rn(rf.z, dir[2]), bs.z), 0.0f);
        d->total[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nscenes; e += (int)stride) {
        ctl[e].done = max_iters <= 0 || descs[e].rows == 0;
        ctl[e].iters = 0;
        ctl[e].max_iters = max_iters;
        ctl[e].tol = tol;
        ctl[e].last_delta = 0.0f;
        if (ctl[e].done) atomicAdd(done_count, 1);
    }
}

// One warp per row of the stacked (block-diagonal) transfer matrix.  The
// per-row sums in a warp are reduced in the same fixed order as the
// one-scene kernel; |add| and |total| of the row go to rowabs.
__global__ void __launch_bounds__(kSpmvThreads) k_batch_spmv(const BatchDesc *__restrict__ descs,
                                                              const int64_t *__restrict__ rstart, int nscenes,
                                                              int parity, const SceneCtl *__restrict__ ctl,
                                                              float2 *__restrict__ rowabs) {
    const int lane = threadIdx.x & 31;
    const int64_t rows = __ldg(rstart + nscenes);
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nwarps) {
        const int e = upper_segment(rstart, nscenes, r);
        if (*(volatile const int32_t *)&ctl[e].done) continue;
        const BatchDesc *d = descs + e;
        const int64_t row = r - __ldg(rstart + e);
        const float4 *emit_in = parity ? d->emit1 : d->emit0;
        float4 *emit_out = parity ? d->emit0 : d->emit1;
        const int64_t b = d->row_ptr[row], en = d->row_ptr[row + 1];
        const float3 a = warp_sum3(row_gather<4>(d->col, d->w, emit_in, b, en, lane));
        const float ar = a.x, ag = a.y, ab = a.z;
        if (lane == 0) {
            float4 t = d->total[row];
            t.x += ar;
            t.y += ag;
            t.z += ab;
            d->total[row] = t;
            const float4 rf = d->leaf[row].refl;
            emit_out[row] = make_float4(rf.x * ar, rf.y * ag, rf.z * ab, 0.0f);
            rowabs[r] = make_float2((fabsf(ar) + fabsf(ag)) + fabsf(ab), (fabsf(t.x) + fabsf(t.y)) + fabsf(t.z));
        }
    }
}

// One block per scene: fixed-order sum of its rows' |add| and |total|, then
// the stop test.
__global__ void k_batch_reduce(const int64_t *__restrict__ rstart, int nscenes, SceneCtl *__restrict__ ctl,
                               const float2 *__restrict__ rowabs, int32_t *__restrict__ done_count) {
    const int e = blockIdx.x;
    if (e >= nscenes || *(volatile int32_t *)&ctl[e].done) return;
    __shared__ double sa[256], st[256];
    const int64_t r0 = rstart[e], r1 = rstart[e + 1];
    double a = 0.0, t = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const float2 v = rowabs[r];
        a += v.x;
        t += v.y;
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
        ctl[e].last_delta = delta;
        ctl[e].iters += 1;
        if (delta < ctl[e].tol || ctl[e].iters >= ctl[e].max_iters) {
            ctl[e].done = 1;
            atomicAdd(done_count, 1);
        }
    }
}

}  // namespace

}  // namespace vrg

using namespace vrg;

struct vrg_batch {
    vrg_ctx *ctx = nullptr;
    std::vector<vrg_env *> envs;
    DevBuf d_desc, d_seg, d_rstart, d_ctl, d_rowabs, d_count;
};

namespace {

int batch_fail(vrg_ctx *ctx, int code, const std::string &m) { return fail(ctx, code, m); }

// Everything a bake needs must be resident: faces, lights, patches and
// transfers.  Reserves the bake outputs of the scene.
int prepare_env(vrg_env *env) {
    vrg_ctx *ctx = env->ctx;
    if (ctx->host_only) return batch_fail(ctx, VRG_ERR_STATE, "host-only context has no device");
    if (!env->built || !env->have_transfers || env->lights.empty())
        return batch_fail(ctx, VRG_ERR_STATE, "a bake needs lights, faces, patches and transfers");
    const int64_t nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    VRG_CUDA(ctx, env->d_bake_rgb.reserve(12 * (size_t)std::max<int64_t>(nlux, 1)));
    VRG_CUDA(ctx, env->d_leaf_direct.reserve(12 * (size_t)std::max<int64_t>(nl, 1)));
    VRG_CUDA(ctx, env->d_emit.reserve(2 * 16 * (size_t)std::max<int64_t>(nl, 1)));
    VRG_CUDA(ctx, env->d_total.reserve(16 * (size_t)std::max<int64_t>(nl, 1)));
    return VRG_OK;
}

BatchDesc make_desc(vrg_env *env) {
    BatchDesc d;
    memset(&d, 0, sizeof d);
    d.scene = scene_view(env);
    d.lights = env->d_lights.as<DevLight>();
    d.faces = env->d_faces.as<FaceRec>();
    d.luxel_off = env->d_luxel_offset.as<int64_t>();
    d.out_rgb = env->d_bake_rgb.as<float>();
    d.ppts = env->d_patch_pts.as<float>();
    d.pnrm = env->d_patch_nrm.as<float>();
    d.pout = env->d_leaf_direct.as<float>();
    d.row_ptr = env->d_row_ptr.as<int64_t>();
    d.col = env->d_col.as<int32_t>();
    d.w = env->d_weight.as<float>();
    d.leaf = env->d_leaf_info.as<LeafInfo>();
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    d.emit0 = env->d_emit.as<float4>();
    d.emit1 = d.emit0 + std::max<int64_t>(nl, 1);
    d.total = env->d_total.as<float4>();
    d.nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    d.npts = nl;
    d.rows = nl;
    d.nl = (int32_t)env->lights.size();
    d.nfaces = env->nfaces;
    return d;
}

}  // namespace

extern "C" {

int vrg_batch_create(vrg_ctx *ctx, vrg_batch **out) {
    if (!ctx || !out) return VRG_ERR_INVALID;
    if (ctx->host_only) return fail(ctx, VRG_ERR_STATE, "host-only context has no device");
    vrg_batch *b = new (std::nothrow) vrg_batch();
    if (!b) return VRG_ERR_NOMEM;
    b->ctx = ctx;
    *out = b;
    return VRG_OK;
}

void vrg_batch_destroy(vrg_batch *b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
}

int vrg_batch_add(vrg_batch *b, vrg_env *env) {
    if (!b || !env) return VRG_ERR_INVALID;
    if (env->ctx != b->ctx) return fail(b->ctx, VRG_ERR_INVALID, "scene belongs to another context");
    b->envs.push_back(env);
    return VRG_OK;
}

int32_t vrg_batch_size(const vrg_batch *b) { return b ? (int32_t)b->envs.size() : 0; }

int vrg_batch_bake(vrg_batch *b, int32_t supersamples, uint64_t seed, int32_t max_bounces, float rel_tol,
                   uint64_t *out_shadow_rays) {
    if (!b) return VRG_ERR_INVALID;
    vrg_ctx *ctx = b->ctx;
    if (supersamples != 1 && supersamples != 4) return fail(ctx, VRG_ERR_UNSUPPORTED, "supersamples must be 1 or 4");
    if (max_bounces < 0 || !(rel_tol >= 0.0f)) return VRG_ERR_INVALID;
    const int E = (int)b->envs.size();
    if (E == 0) return VRG_OK;
    std::vector<std::unique_lock<std::mutex>> locks;
    for (vrg_env *env : b->envs) {
        bool seen = false;
        for (auto &l : locks)
            if (l.mutex() == &env->mu) seen = true;
        if (seen) return fail(ctx, VRG_ERR_INVALID, "a scene appears twice in the batch");
        locks.emplace_back(env->mu);
        const int rc = prepare_env(env);
        if (rc != VRG_OK) return rc;
    }
    std::vector<BatchDesc> descs(E);
    std::vector<int64_t> seg(2 * E + 1, 0), rstart(E + 1, 0);
    for (int e = 0; e < E; e++) {
        descs[e] = make_desc(b->envs[e]);
        seg[e + 1] = seg[e] + descs[e].nlux * supersamples;
        rstart[e + 1] = rstart[e] + descs[e].rows;
    }
    for (int e = 0; e < E; e++) seg[E + e + 1] = seg[E + e] + descs[e].npts;
    const int64_t rows = rstart[E];
    VRG_CUDA(ctx, b->d_desc.reserve(sizeof(BatchDesc) * E));
    VRG_CUDA(ctx, b->d_seg.reserve(8 * seg.size()));
    VRG_CUDA(ctx, b->d_rstart.reserve(8 * rstart.size()));
    VRG_CUDA(ctx, b->d_ctl.reserve(sizeof(SceneCtl) * E));
    VRG_CUDA(ctx, b->d_rowabs.reserve(8 * (size_t)std::max<int64_t>(rows, 1)));
    VRG_CUDA(ctx, b->d_count.reserve(256));
    cudaStream_t st = ctx->stream;
    VRG_CUDA(ctx, cudaMemcpyAsync(b->d_desc.ptr, descs.data(), sizeof(BatchDesc) * E, cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(b->d_seg.ptr, seg.data(), 8 * seg.size(), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(b->d_rstart.ptr, rstart.data(), 8 * rstart.size(), cudaMemcpyHostToDevice, st));
    // counters: [0] work queue, [1] shadow rays, [2] scenes done (int32)
    unsigned long long *cnt = b->d_count.as<unsigned long long>();
    int32_t *done_count = reinterpret_cast<int32_t *>(cnt + 2);
    VRG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 24, st));
    const BatchDesc *dd = b->d_desc.as<BatchDesc>();
    const int64_t *dseg = b->d_seg.as<int64_t>(), *drs = b->d_rstart.as<int64_t>();
    SceneCtl *ctl = b->d_ctl.as<SceneCtl>();
    float2 *rowabs = b->d_rowabs.as<float2>();

    // direct pass: one persistent launch over every scene, in the variant
    // tuned for the batch's size (the register walk at 8 blocks per SM, or
    // the walk constants in shared memory at 9 or 8; the same results)
    using GatherKernel = void (*)(const BatchDesc *, const int64_t *, int, int, uint64_t, unsigned long long *,
                                  unsigned long long *);
    const GatherKernel gvar[3] = {k_batch_gather<0, 8>, k_batch_gather<kOptShRay, 9>,
                                  k_batch_gather<kOptShRay, 8>};
    const int64_t items = seg[2 * E];
    int64_t tris = 0;
    for (vrg_env *env : b->envs) tris += env->geom.ntris;
    cudaEvent_t ev = nullptr;
    auto gather = [&](int v) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(cnt, 0, 16, st);  // work queue and shadow rays
        if (e != cudaSuccess) return e;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gvar[v], kThreads, 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 4;
        const int ggrid = (int)std::max<int64_t>(1, std::min<int64_t>((items + kThreads - 1) / kThreads,
                                                                      (int64_t)ctx->num_sms * per_sm));
        timing_begin(ctx, "batch_gather", &ev);
        gvar[v]<<<ggrid, kThreads, 0, st>>>(dd, dseg, E, supersamples, seed, cnt, out_shadow_rays ? cnt + 1 : nullptr);
        e = cudaGetLastError();
        timing_end(ctx, "batch_gather", ev);
        return e;
    };
    {
        const int rc = tune_run(ctx, tune_key("batch_gather", tris, items), 3, gather);
        if (rc != VRG_OK) return rc;
    }

    // bounce: block-diagonal over every scene, per-scene stop
    const int ib = (int)std::min<int64_t>(std::max<int64_t>((rows + 255) / 256, 1), (int64_t)ctx->num_sms * 8);
    timing_begin(ctx, "batch_bounce_init", &ev);
    k_batch_bounce_init<<<ib, 256, 0, st>>>(dd, drs, E, ctl, max_bounces, rel_tol, done_count);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "batch_bounce_init", ev);
    const int sgrid = ctx->num_sms * 4;
    auto one = [&](int parity) -> cudaError_t {
        cudaEvent_t e2 = nullptr;
        timing_begin(ctx, "batch_spmv", &e2);
        k_batch_spmv<<<sgrid, kSpmvThreads, 0, st>>>(dd, drs, E, parity, ctl, rowabs);
        cudaError_t e = cudaGetLastError();
        timing_end(ctx, "batch_spmv", e2);
        if (e != cudaSuccess) return e;
        timing_begin(ctx, "batch_reduce", &e2);
        k_batch_reduce<<<E, 256, 0, st>>>(drs, E, ctl, rowabs, done_count);
        e = cudaGetLastError();
        timing_end(ctx, "batch_reduce", e2);
        return e;
    };
    int32_t done_h = 0;
    int32_t launched = 0;
    if (ctx->timing) {
        while (launched < max_bounces) {
            VRG_CUDA(ctx, one(launched & 1));
            launched++;
            if ((launched % kGraphBounces) == 0 || launched == max_bounces) {
                VRG_CUDA(ctx, cudaMemcpyAsync(&done_h, done_count, 4, cudaMemcpyDeviceToHost, st));
                VRG_CUDA(ctx, cudaStreamSynchronize(st));
                if (done_h >= E) break;
            }
        }
    } else if (max_bounces > 0) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        VRG_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaSuccess;
        for (int k = 0; k < kGraphBounces && ce == cudaSuccess; k++) ce = one(k & 1);
        cudaError_t ee = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "batch bounce capture");
        if (ee != cudaSuccess) return cuda_fail(ctx, ee, "cudaStreamEndCapture");
        VRG_CUDA(ctx, cudaGraphInstantiate(&exec, graph, 0));
        cudaGraphDestroy(graph);
        while (launched < max_bounces) {
            cudaError_t le = cudaGraphLaunch(exec, st);
            if (le == cudaSuccess) le = cudaMemcpyAsync(&done_h, done_count, 4, cudaMemcpyDeviceToHost, st);
            if (le == cudaSuccess) le = cudaStreamSynchronize(st);
            if (le != cudaSuccess) {
                cudaGraphExecDestroy(exec);
                return cuda_fail(ctx, le, "batch bounce graph");
            }
            launched += kGraphBounces;
            if (done_h >= E) break;
        }
        cudaGraphExecDestroy(exec);
    }
    std::vector<SceneCtl> hc(E);
    VRG_CUDA(ctx, cudaMemcpyAsync(hc.data(), ctl, sizeof(SceneCtl) * E, cudaMemcpyDeviceToHost, st));
    unsigned long long rays = 0;
    VRG_CUDA(ctx, cudaMemcpyAsync(&rays, cnt + 1, 8, cudaMemcpyDeviceToHost, st));
    VRG_CUDA(ctx, cudaStreamSynchronize(st));
    for (int e = 0; e < E; e++) {
        vrg_env *env = b->envs[e];
        env->have_bake = true;
        env->have_patch_direct = true;
        env->bake_bounces = hc[e].iters;
        env->bake_delta = hc[e].last_delta;
    }
    if (out_shadow_rays) *out_shadow_rays = rays;
    return VRG_OK;
}

// One scene, the way a caller without batching bakes: direct pass (one
// launch), patch direct light (one launch), bounce loop (graph).
int vrg_env_bake(vrg_env *env, int32_t supersamples, uint64_t seed, int32_t max_bounces, float rel_tol,
                 uint64_t *out_shadow_rays) {
    if (!env) return VRG_ERR_INVALID;
    vrg_ctx *ctx = env->ctx;
    if (supersamples != 1 && supersamples != 4) return fail(ctx, VRG_ERR_UNSUPPORTED, "supersamples must be 1 or 4");
    if (max_bounces < 0 || !(rel_tol >= 0.0f)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    int rc = prepare_env(env);
    if (rc != VRG_OK) return rc;
    unsigned long long *cnt = nullptr;
    if (out_shadow_rays) {
        VRG_CUDA(ctx, env->d_counter.reserve(64));
        cnt = env->d_counter.as<unsigned long long>();
        VRG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, ctx->stream));
    }
    // luxel samples and leaf-patch points in one persistent launch
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    rc = launch_gather_luxels(env, supersamples, seed, env->d_bake_rgb.as<float>(), cnt,
                              env->d_patch_pts.as<float>(), env->d_patch_nrm.as<float>(), nl,
                              env->d_leaf_direct.as<float>());
    if (rc != VRG_OK) return rc;
    env->have_patch_direct = true;
    int32_t bounces = 0;
    float delta = 0.0f;
    rc = run_bounce(env, max_bounces, rel_tol, &bounces, &delta);
    if (rc != VRG_OK) return rc;
    env->have_bake = true;
    env->bake_bounces = bounces;
    env->bake_delta = delta;
    if (out_shadow_rays) {
        unsigned long long h = 0;
        VRG_CUDA(ctx, cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, ctx->stream));
        VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        *out_shadow_rays = h;
    }
    return VRG_OK;
}

int vrg_env_get_bake(vrg_env *env, float *luxel_rgb, float *patch_direct, float *patch_total, int32_t *bounces,
                     float *delta) {
    if (!env) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    if (!env->have_bake) return fail(env->ctx, VRG_ERR_STATE, "no bake of the current faces and patches has run on this scene");
    vrg_ctx *ctx = env->ctx;
    const int64_t nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    cudaStream_t st = ctx->stream;
    if (luxel_rgb && nlux) VRG_CUDA(ctx, cudaMemcpyAsync(luxel_rgb, env->d_bake_rgb.ptr, 12 * nlux, cudaMemcpyDeviceToHost, st));
    if (patch_direct && nl) VRG_CUDA(ctx, cudaMemcpyAsync(patch_direct, env->d_leaf_direct.ptr, 12 * nl, cudaMemcpyDeviceToHost, st));
    std::vector<float4> tot;
    if (patch_total && nl) {
        tot.resize(nl);
        VRG_CUDA(ctx, cudaMemcpyAsync(tot.data(), env->d_total.ptr, 16 * nl, cudaMemcpyDeviceToHost, st));
    }
    VRG_CUDA(ctx, cudaStreamSynchronize(st));
    for (int64_t i = 0; i < (int64_t)tot.size(); i++) {
        patch_total[3 * i] = tot[i].x;
        patch_total[3 * i + 1] = tot[i].y;
        patch_total[3 * i + 2] = tot[i].z;
    }
    if (bounces) *bounces = env->bake_bounces;
    if (delta) *delta = env->bake_delta;
    return VRG_OK;
}

}  // extern "C"
