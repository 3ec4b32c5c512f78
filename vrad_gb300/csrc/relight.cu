// relight.cu -- serving light edits on resident scenes.
//
// A relight-ready scene keeps, besides its lightmap and bounce state, the
// multiplier of every sky-type light at every luxel sample and leaf-patch
// point (the sky light's cosine or the sky ambient's visible fraction).
// Those do not depend on any light position, so a request that edits point
// and spot lights re-gathers only the faces within the old or new radius of
// an edited light, re-tracing only the point and spot shadow lines; the
// result is bit-identical to a full gather with the edited table.  The bounce
// then restarts from the resident solution B of B = T (emit + refl * B):
//   x = emit + refl * B ; per iteration y = T x, delta = sum|y - B| / sum|y|,
//   B = y, x = emit + refl * y ; stop when delta < tol or at the cap.
// Iterations are queued all at once and turn into no-ops after the stop, so
// a request never waits on the host between kernels.
//
// The server admits requests into slots (one CUDA stream each) as slots and
// scenes free up: requests on different scenes overlap on the GPU, requests
// on one scene run in submission order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <thread>

#include "vrg_gather.cuh"
#include "vrg_internal.h"
#include "vrg_spmv.cuh"

namespace vrg {

namespace {

constexpr int kThreads = 128;
constexpr int kSpmvThreads = 256;
constexpr int kRelightMaxBlocks = 2048;  // SpMV grid cap of a relight (partials slots)

struct RelightCtl {
    int32_t done, iters, max_iters;
    float tol, last_delta;
    int32_t pad[3];
};

// Work list of one relight: samples of the affected faces (segment 0) and
// leaf points of the affected faces (segment 1).
struct RelightList {
    const int32_t *faces;     // affected face ids
    const int64_t *samp_off;  // prefix of affected faces' sample counts (n+1)
    const int64_t *leaf_off;  // prefix of affected faces' leaf counts (n+1)
    const int32_t *leaf_beg;  // first leaf of each affected face
    int32_t nfaces;
};

__device__ __forceinline__ int seg_of(const int64_t *__restrict__ off, int n, int64_t i) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Gather over a work list: the luxels of listed faces (all faces when
// list.faces is null), then their leaf points.  SKY = kSkyWrite stores the
// sky multipliers and the point/spot visibility bits (vis_words words per
// sample or point), kSkyRead reuses them and traces only the lights flagged
// in `edited`.
template <int SKY>
__global__ void __launch_bounds__(kThreads, 8) k_relight_gather(
    DevScene s, const DevLight *__restrict__ lights, int nl, const FaceRec *__restrict__ faces,
    const int64_t *__restrict__ luxel_off, int nfaces, RelightList list, int ss, uint64_t seed,
    float *__restrict__ lux_out, const float *__restrict__ ppts, const float *__restrict__ pnrm,
    float *__restrict__ pout, float *__restrict__ sky_lux, float *__restrict__ sky_pts, int sky_slots,
    uint32_t *__restrict__ vis_lux, uint32_t *__restrict__ vis_pts, int vis_words,
    const uint32_t *__restrict__ edited, unsigned long long *__restrict__ work,
    unsigned long long *__restrict__ ray_count) {
    const bool all = list.faces == nullptr;
    const int nf = list.nfaces;
    // totals of the two segments (in "all" mode the leaf list is {0, leaves})
    const int64_t nsamp = all ? __ldg(luxel_off + nfaces) * ss : __ldg(list.samp_off + nf);
    const int64_t nleaf = __ldg(list.leaf_off + nf);
    const int64_t total = nsamp + nleaf;
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
        if (gi < nsamp) {
            luxel_item = true;
            int f;
            int64_t local;
            if (all) {
                lux = gi / ss;
                f = find_face(luxel_off, nfaces, lux);
                local = gi - __ldg(luxel_off + f) * ss;
            } else {
                const int k = seg_of(list.samp_off, nf, gi);
                f = __ldg(list.faces + k);
                local = gi - __ldg(list.samp_off + k);
                lux = __ldg(luxel_off + f) + local / ss;
            }
            const int kk = (int)(local % ss);
            const FaceRec fr = faces[f];
            int iu, iv;  // the face's luxels in 4 x 2 tiles
            tile_luxel(lux - __ldg(luxel_off + f), fr.nu, fr.nv, iu, iv);
            lux = __ldg(luxel_off + f) + (int64_t)iv * fr.nu + iu;
            const int64_t gsamp = lux * ss + kk;
            float px, py, pz;
            luxel_sample(fr, lux, iu, iv, kk, ss, seed, px, py, pz);
            gather_point<SKY>(s, lights, nl, px, py, pz, fr.normal.x, fr.normal.y, fr.normal.z, r, g,
                              b, rays, sky_lux + gsamp * sky_slots, vis_lux + gsamp * vis_words, edited);
        } else if (gi < total) {
            const int64_t li = gi - nsamp;
            int64_t leaf;
            if (all) {
                leaf = li;
            } else {
                const int k = seg_of(list.leaf_off, nf, li);
                leaf = __ldg(list.leaf_beg + k) + (li - __ldg(list.leaf_off + k));
            }
            const float *p = ppts + 3 * leaf, *n = pnrm + 3 * leaf;
            gather_point<SKY>(s, lights, nl, __ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(n), __ldg(n + 1),
                              __ldg(n + 2), r, g, b, rays, sky_pts + leaf * sky_slots,
                              vis_pts + leaf * vis_words, edited);
            pout[3 * leaf] = r;
            pout[3 * leaf + 1] = g;
            pout[3 * leaf + 2] = b;
        }
        if (ss == 4) {
            // sample segments hold whole luxels (4 samples, 4-aligned)
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

// emit = refl * direct + base ; x = emit + refl * B ; control reset.
__global__ void k_relight_start(const LeafInfo *__restrict__ info, const float *__restrict__ direct,
                                const float4 *__restrict__ B, float4 *__restrict__ emit, float4 *__restrict__ x,
                                int64_t n, RelightCtl *ctl, int32_t max_iters, float tol) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 rf = info[i].refl, bs = info[i].base, bb = B[i];
        const float4 e = make_float4(__fadd_rn(__fmul_rn(rf.x, direct[3 * i]), bs.x),
                                     __fadd_rn(__fmul_rn(rf.y, direct[3 * i + 1]), bs.y),
                                     __fadd_rn(__fmul_rn(rf.z, direct[3 * i + 2]), bs.z), 0.0f);
        emit[i] = e;
        x[i] = make_float4(__fadd_rn(e.x, __fmul_rn(rf.x, bb.x)), __fadd_rn(e.y, __fmul_rn(rf.y, bb.y)),
                           __fadd_rn(e.z, __fmul_rn(rf.z, bb.z)), 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->done = max_iters <= 0;
        ctl->iters = 0;
        ctl->max_iters = max_iters;
        ctl->tol = tol;
        ctl->last_delta = 0.0f;
    }
}

// y = T x per row (one warp per row), B = y, x' = emit + refl * y; per-block
// sums of |y - B_old| and |y| into partials.
__global__ void __launch_bounds__(kSpmvThreads) k_relight_spmv(
    const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ col, const float *__restrict__ w,
    const float4 *__restrict__ x_in, float4 *__restrict__ x_out, float4 *__restrict__ B,
    const float4 *__restrict__ emit, const LeafInfo *__restrict__ info, int64_t n,
    const RelightCtl *__restrict__ ctl, double *__restrict__ partials) {
    if (*(volatile const int32_t *)&ctl->done) return;
    __shared__ double red[2][kSpmvThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double sd = 0.0, sy = 0.0;
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nwarps) {
        const float3 a = warp_sum3(row_gather<4>(col, w, x_in, row_ptr[row], row_ptr[row + 1], lane));
        const float ar = a.x, ag = a.y, ab = a.z;
        if (lane == 0) {
            const float4 old = B[row];
            B[row] = make_float4(ar, ag, ab, 0.0f);
            const float4 rf = info[row].refl, em = emit[row];
            x_out[row] = make_float4(em.x + rf.x * ar, em.y + rf.y * ag, em.z + rf.z * ab, 0.0f);
            sd += (double)fabsf(ar - old.x) + (double)fabsf(ag - old.y) + (double)fabsf(ab - old.z);
            sy += (double)fabsf(ar) + (double)fabsf(ag) + (double)fabsf(ab);
        }
    }
    if (lane == 0) {
        red[0][wid] = sd;
        red[1][wid] = sy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, t = 0.0;
        for (int k = 0; k < kSpmvThreads / 32; k++) {
            a += red[0][k];
            t += red[1][k];
        }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = t;
    }
}

// Inside the loop graph (in_loop) thread 0 also sets the loop's condition:
// the while node runs its body again only while the loop is not done.
__global__ void k_relight_reduce(RelightCtl *ctl, const double *__restrict__ partials, int nblocks,
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

// Fixed-order checksums of a scene's lightmap and bounce state: per-block
// partial sums over a fixed grid, then one block adds them in order.
constexpr int kDigestBlocks = 64;

__global__ void k_digest_partial(const float *__restrict__ lux, int64_t nlux3, const float4 *__restrict__ B,
                                 int64_t n, double *__restrict__ partials) {
    __shared__ double s0[256], s1[256];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, c = 0.0;
    for (int64_t i = t0; i < nlux3; i += stride) a += (double)lux[i];
    for (int64_t i = t0; i < n; i += stride) c += ((double)B[i].x + (double)B[i].y) + (double)B[i].z;
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s0[0];
        partials[2 * blockIdx.x + 1] = s1[0];
    }
}

__global__ void k_digest_final(const double *__restrict__ partials, int nblocks, double *__restrict__ out) {
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int i = 0; i < nblocks; i++) {
            a += partials[2 * i];
            c += partials[2 * i + 1];
        }
        out[0] = a;
        out[1] = c;
    }
}

// Words of the per-item visibility cache: one bit per light.
int vis_words(size_t nlights) { return (int)((nlights + 31) / 32); }

int count_sky(const std::vector<vrg_light> &lights) {
    int n = 0;
    for (const vrg_light &l : lights)
        if (l.type == VRG_EMIT_SKYLIGHT || l.type == VRG_EMIT_SKYAMBIENT) n++;
    return n;
}

int persistent_blocks(vrg_ctx *ctx, const void *kernel, int64_t items) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 4;
    return (int)std::max<int64_t>(1, std::min<int64_t>((items + kThreads - 1) / kThreads,
                                                       (int64_t)ctx->num_sms * per_sm));
}

int spmv_blocks(const vrg_ctx *ctx) {
    static const int per_sm = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_relight_spmv, kSpmvThreads, 0) != cudaSuccess || v < 1)
            v = 2;
        return v;
    }();
    return std::min(kRelightMaxBlocks, ctx->num_sms * per_sm);
}

}  // namespace

// Per-slot device scratch of a relight request.
struct RelightScratch {
    DevBuf buf;  // [unused | counters | digest | digest partials | offsets | face list | edited mask]
    size_t cap_faces = 0, cap_words = 0;
    unsigned long long *work = nullptr, *rays = nullptr;
    double *digest = nullptr, *partials = nullptr;
    int32_t *faces = nullptr, *leaf_beg = nullptr;
    int64_t *samp_off = nullptr, *leaf_off = nullptr;
    uint32_t *edited = nullptr;

    int reserve(vrg_ctx *ctx, size_t nfaces, size_t nwords) {
        if (nfaces <= cap_faces && nwords <= cap_words && buf.ptr) return VRG_OK;
        nfaces = std::max(nfaces, cap_faces);
        nwords = std::max(nwords, cap_words);
        const size_t head = 256 + 2 * 8 * kRelightMaxBlocks;
        const size_t bytes = head + (nfaces + 1) * (4 + 4 + 8 + 8) + 4 * nwords + 256;
        VRG_CUDA(ctx, buf.reserve(bytes));
        char *p = buf.as<char>();
        work = reinterpret_cast<unsigned long long *>(p + 64);
        rays = work + 1;
        digest = reinterpret_cast<double *>(p + 128);
        partials = reinterpret_cast<double *>(p + 256);
        char *q = p + head;
        samp_off = reinterpret_cast<int64_t *>(q);
        leaf_off = samp_off + (nfaces + 1);
        faces = reinterpret_cast<int32_t *>(leaf_off + (nfaces + 1));
        leaf_beg = faces + (nfaces + 1);
        edited = reinterpret_cast<uint32_t *>(leaf_beg + (nfaces + 1));
        cap_faces = nfaces;
        cap_words = nwords;
        return VRG_OK;
    }
};

struct HostStage {
    void *ptr = nullptr;
    size_t bytes = 0;
    ~HostStage() {
        if (ptr) cudaFreeHost(ptr);
    }
    int reserve(vrg_ctx *ctx, size_t n) {
        if (n <= bytes && ptr) return VRG_OK;
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        bytes = 0;
        VRG_CUDA(ctx, cudaMallocHost(&ptr, n));
        bytes = n;
        return VRG_OK;
    }
};

// The warm-start bounce loop of one (scene, scratch) pair as an executable
// graph: a while node whose body is SpMV x0 -> x1, reduce, SpMV x1 -> x0,
// reduce.  The reduce kernels clear the loop condition once the control
// block is done, so the loop stops on the device after the last useful
// iteration instead of running no-op launches up to the cap.
struct LoopGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<const void *> key;  // the buffers and sizes it was built on
    LoopGraph() = default;
    LoopGraph(const LoopGraph &) = delete;
    LoopGraph &operator=(const LoopGraph &) = delete;
    ~LoopGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// Relight state a scene keeps between requests: the serial entry point's
// scratch and staging buffer, the bounce loop's control block and partial
// sums, and the loop graph built on them.  Requests on one scene never run
// at the same time (the server keeps them in order), so one control block
// and one graph serve every slot.
struct RelightState {
    RelightScratch sc;
    HostStage stage;
    DevBuf loop_buf;  // [RelightCtl | 2 doubles per SpMV block]
    RelightCtl *ctl = nullptr;
    double *partials = nullptr;
    std::unique_ptr<LoopGraph> loop;

    int reserve_loop(vrg_ctx *ctx) {
        if (ctl) return VRG_OK;
        VRG_CUDA(ctx, loop_buf.reserve(256 + 2 * 8 * (size_t)kRelightMaxBlocks));
        ctl = loop_buf.as<RelightCtl>();
        partials = reinterpret_cast<double *>(loop_buf.as<char>() + 256);
        return VRG_OK;
    }
};

void relight_release(vrg_env *env) {
    delete env->relight;
    env->relight = nullptr;
}
}  // namespace vrg

using namespace vrg;

namespace {

// Bake with the sky multipliers stored, then the cold bounce; afterwards the
// scene can take relight requests.
int relight_prepare(vrg_env *env, int32_t ss, uint64_t seed, int32_t max_bounces, float tol) {
    vrg_ctx *ctx = env->ctx;
    if (ctx->host_only) return fail(ctx, VRG_ERR_STATE, "host-only context has no device");
    if (!env->built || !env->have_transfers || env->lights.empty())
        return fail(ctx, VRG_ERR_STATE, "relighting needs lights, faces, patches and transfers");
    if (ss != 1 && ss != 4) return fail(ctx, VRG_ERR_UNSUPPORTED, "supersamples must be 1 or 4");
    const int64_t nlux = env->luxel_offset.back();
    const int64_t nl = (int64_t)env->patches.leaf_patch.size();
    const int sky = count_sky(env->lights);
    const int vw = vis_words(env->lights.size());
    const size_t need = 12 * (size_t)nlux + 4 * (size_t)(nlux * ss + nl) * (std::max(sky, 1) + vw) +
                        16 * 4 * (size_t)nl + 12 * (size_t)nl;
    size_t free_b = 0, total_b = 0;
    VRG_CUDA(ctx, cudaMemGetInfo(&free_b, &total_b));
    uint64_t reserve;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        reserve = ctx->hbm_reserve;
    }
    if ((uint64_t)need > (uint64_t)free_b || (uint64_t)free_b - (uint64_t)need < reserve)
        return fail(ctx, VRG_ERR_NOMEM, "not enough free device memory to admit this scene for relighting");
    relight_release(env);  // loop graphs point into buffers that may move below
    VRG_CUDA(ctx, env->d_bake_rgb.reserve(12 * (size_t)std::max<int64_t>(nlux, 1)));
    VRG_CUDA(ctx, env->d_leaf_direct.reserve(12 * (size_t)std::max<int64_t>(nl, 1)));
    VRG_CUDA(ctx, env->d_sky_lux.reserve(4 * (size_t)std::max<int64_t>(nlux * ss * sky, 1)));
    VRG_CUDA(ctx, env->d_sky_pts.reserve(4 * (size_t)std::max<int64_t>(nl * sky, 1)));
    VRG_CUDA(ctx, env->d_vis_lux.reserve(4 * (size_t)std::max<int64_t>(nlux * ss * vw, 1)));
    VRG_CUDA(ctx, env->d_vis_pts.reserve(4 * (size_t)std::max<int64_t>(nl * vw, 1)));
    VRG_CUDA(ctx, env->d_emit0.reserve(16 * (size_t)std::max<int64_t>(nl, 1)));
    VRG_CUDA(ctx, env->d_x.reserve(2 * 16 * (size_t)std::max<int64_t>(nl, 1)));
    VRG_CUDA(ctx, env->d_work.reserve(256));
    // per-face bounds and leaf ranges for request culling
    const int32_t F = env->nfaces;
    env->face_mid.assign(3 * (size_t)F, 0.0f);  // centres, per axis a: [a * F + f]
    env->face_ext.assign(3 * (size_t)F, 0.0f);  // half extents, same order
    for (int32_t f = 0; f < F; f++)
        for (int a = 0; a < 3; a++) {
            const float c = env->f_corner[3 * f + a], u = env->f_u[3 * f + a], v = env->f_v[3 * f + a];
            const float pts[4] = {c, c + u, c + v, (c + u) + v};
            float lo = pts[0], hi = pts[0];
            for (float p : pts) {
                lo = std::min(lo, p);
                hi = std::max(hi, p);
            }
            // centre and half extent, padded by a quarter unit
            env->face_mid[(size_t)a * F + f] = 0.5f * (lo + hi);
            env->face_ext[(size_t)a * F + f] = 0.5f * (hi - lo) + 0.25f;
        }
    env->face_leaf_begin.assign(2 * (size_t)F, 0);
    for (int32_t f = 0; f < F; f++) env->face_leaf_begin[2 * f] = INT32_MAX;
    for (int64_t l = 0; l < nl; l++) {
        const int32_t f = env->patches.face[env->patches.leaf_patch[l]];
        env->face_leaf_begin[2 * f] = std::min<int32_t>(env->face_leaf_begin[2 * f], (int32_t)l);
        env->face_leaf_begin[2 * f + 1] = std::max<int32_t>(env->face_leaf_begin[2 * f + 1], (int32_t)l + 1);
    }
    for (int32_t f = 0; f < F; f++)
        if (env->face_leaf_begin[2 * f] == INT32_MAX) env->face_leaf_begin[2 * f] = env->face_leaf_begin[2 * f + 1] = 0;

    cudaStream_t st = ctx->stream;
    unsigned long long *work = env->d_work.as<unsigned long long>() + 4;
    VRG_CUDA(ctx, cudaMemsetAsync(work, 0, 8, st));
    VRG_CUDA(ctx, cudaMemsetAsync(env->d_vis_lux.ptr, 0, 4 * (size_t)(nlux * ss * vw), st));
    VRG_CUDA(ctx, cudaMemsetAsync(env->d_vis_pts.ptr, 0, 4 * (size_t)(nl * vw), st));
    RelightList all{};
    // leaf_off of the "all" list: {0, nl} from a tiny device array
    int64_t off2[2] = {0, nl};
    DevBuf d_off;
    VRG_CUDA(ctx, d_off.reserve(16));
    VRG_CUDA(ctx, cudaMemcpyAsync(d_off.ptr, off2, 16, cudaMemcpyHostToDevice, st));
    all.faces = nullptr;
    all.nfaces = 1;
    all.leaf_off = d_off.as<int64_t>();
    const int64_t items = nlux * ss + nl;
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "relight_gather", &ev);
    k_relight_gather<kSkyWrite><<<persistent_blocks(ctx, (const void *)k_relight_gather<kSkyWrite>, items), kThreads, 0, st>>>(
        scene_view(env), env->d_lights.as<DevLight>(), (int)env->lights.size(), env->d_faces.as<FaceRec>(),
        env->d_luxel_offset.as<int64_t>(), env->nfaces, all, ss, seed, env->d_bake_rgb.as<float>(),
        env->d_patch_pts.as<float>(), env->d_patch_nrm.as<float>(), env->d_leaf_direct.as<float>(),
        env->d_sky_lux.as<float>(), env->d_sky_pts.as<float>(), sky, env->d_vis_lux.as<uint32_t>(),
        env->d_vis_pts.as<uint32_t>(), vw, nullptr, work, nullptr);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "relight_gather", ev);
    env->have_patch_direct = true;
    int32_t bounces = 0;
    float delta = 0.0f;
    const int rc = run_bounce(env, max_bounces, tol, &bounces, &delta);
    if (rc != VRG_OK) return rc;
    VRG_CUDA(ctx, cudaStreamSynchronize(st));
    env->sky_slots = sky;
    env->vis_words = vw;
    env->relight_ss = ss;
    env->relight_seed = seed;
    env->relight_ready = true;
    env->have_bake = true;
    env->bake_bounces = bounces;
    env->bake_delta = delta;
    return VRG_OK;
}

bool light_equal(const vrg_light &a, const vrg_light &b) { return memcmp(&a, &b, sizeof a) == 0; }

// Marks (hit[f] |= 1) the faces whose padded bounds come within `radius` of
// centre c.  Branch-free float arithmetic over axis-major centres and half
// extents; without FP-trap semantics the host compiler turns the selects
// into vector blends (about 7x faster than the scalar test at 4,096 faces
// and 32 spheres).  The radius is padded by 1e-4 relative + 1e-2 absolute,
// far beyond the float rounding of the distance and of the stored bounds, so
// a face in reach is never missed (a face marked in excess is only
// re-gathered to the values it already has).
__attribute__((optimize("O3", "no-trapping-math")))
void mark_faces_in_reach(const vrg_env *env, const float *c, float radius, int32_t *hit) {
    const int32_t F = env->nfaces;
    const float *mx = env->face_mid.data(), *my = mx + F, *mz = my + F;
    const float *ex = env->face_ext.data(), *ey = ex + F, *ez = ey + F;
    const float cx = c[0], cy = c[1], cz = c[2];
    const float r = radius * (1.0f + 1e-4f) + 1e-2f, r2 = r * r;
    for (int32_t f = 0; f < F; f++) {
        float dx = std::fabs(cx - mx[f]) - ex[f];
        float dy = std::fabs(cy - my[f]) - ey[f];
        float dz = std::fabs(cz - mz[f]) - ez[f];
        dx = dx > 0.0f ? dx : 0.0f;
        dy = dy > 0.0f ? dy : 0.0f;
        dz = dz > 0.0f ? dz : 0.0f;
        hit[f] |= (int32_t)((dx * dx + dy * dy + dz * dz) <= r2);
    }
}

struct RelightPlan {
    std::vector<vrg_light> table;  // new light table
    std::vector<uint32_t> edited;  // bit k: light k changed (its shadow lines are re-traced)
    std::vector<int32_t> faces;    // affected faces (empty + all=true: every face)
    bool all = false;
    bool any = false;
};

// Applies edits to a copy of the scene's light table and finds the faces a
// full gather would change.
int plan_relight(vrg_env *env, const vrg_light_edit *edits, int32_t n, RelightPlan &p) {
    vrg_ctx *ctx = env->ctx;
    p.table = env->lights;
    p.edited.assign((size_t)vis_words(p.table.size()), 0u);
    std::vector<std::pair<vrg_light, vrg_light>> changed;
    for (int32_t i = 0; i < n; i++) {
        const int32_t k = edits[i].index;
        if (k < 0 || k >= (int32_t)p.table.size()) return fail(ctx, VRG_ERR_INVALID, "light edit index out of range");
        const vrg_light &old = p.table[k], &nw = edits[i].light;
        const bool old_sky = old.type == VRG_EMIT_SKYLIGHT || old.type == VRG_EMIT_SKYAMBIENT;
        const bool new_sky = nw.type == VRG_EMIT_SKYLIGHT || nw.type == VRG_EMIT_SKYAMBIENT;
        if (old_sky || new_sky) {
            // sky multipliers are cached: only the intensity may change
            vrg_light a = old, b = nw;
            memcpy(b.intensity, a.intensity, sizeof a.intensity);
            if (old.type != nw.type || !light_equal(a, b))
                return fail(ctx, VRG_ERR_UNSUPPORTED, "relight can change a sky light's intensity only");
        }
        if (nw.type < 0 || nw.type > 5) return fail(ctx, VRG_ERR_INVALID, "bad light type in edit");
        if (!light_equal(old, nw)) {
            changed.emplace_back(old, nw);
            p.edited[k >> 5] |= 1u << (k & 31);
        }
        p.table[k] = nw;
    }
    p.any = !changed.empty();
    const int32_t F = env->nfaces;
    for (auto &c : changed) {
        for (const vrg_light *l : {&c.first, &c.second}) {
            const bool ranged = (l->type == VRG_EMIT_POINT || l->type == VRG_EMIT_SPOTLIGHT) && l->radius > 0.0f;
            if (!ranged) p.all = true;
        }
    }
    if (p.all || !p.any) return VRG_OK;
    std::vector<int32_t> hit(F, 0);
    for (auto &c : changed) {
        mark_faces_in_reach(env, c.first.origin, c.first.radius, hit.data());
        mark_faces_in_reach(env, c.second.origin, c.second.radius, hit.data());
    }
    for (int32_t f = 0; f < F; f++)
        if (hit[f]) p.faces.push_back(f);
    return VRG_OK;
}

RelightState &relight_state(vrg_env *env) {
    if (!env->relight) env->relight = new RelightState;
    return *env->relight;
}

// The scene's loop graph, built on first use and rebuilt when a buffer it
// points into has moved.
int loop_graph(vrg_env *env, cudaStream_t st, int sblocks, cudaGraphExec_t *out) {
    vrg_ctx *ctx = env->ctx;
    RelightState &rs = relight_state(env);
    int rc = rs.reserve_loop(ctx);
    if (rc != VRG_OK) return rc;
    const int64_t n = (int64_t)env->patches.leaf_patch.size();
    float4 *B = env->d_total.as<float4>(), *emit = env->d_emit0.as<float4>();
    float4 *x0 = env->d_x.as<float4>(), *x1 = x0 + std::max<int64_t>(n, 1);
    const std::vector<const void *> key = {x0, B, emit, env->d_row_ptr.ptr, env->d_col.ptr, env->d_weight.ptr,
                                           env->d_leaf_info.ptr, rs.ctl, rs.partials,
                                           reinterpret_cast<const void *>((intptr_t)n),
                                           reinterpret_cast<const void *>((intptr_t)sblocks)};
    std::unique_ptr<LoopGraph> &slot = rs.loop;
    if (slot && slot->key == key) {
        *out = slot->exec;
        return VRG_OK;
    }
    slot.reset(new LoopGraph);
    cudaGraph_t g = nullptr;
    VRG_CUDA(ctx, cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wn = nullptr;
    if (e == cudaSuccess) e = cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &cp);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const LeafInfo *info = env->d_leaf_info.as<LeafInfo>();
        const int64_t *rp = env->d_row_ptr.as<int64_t>();
        const int32_t *col = env->d_col.as<int32_t>();
        const float *w = env->d_weight.as<float>();
        k_relight_spmv<<<sblocks, kSpmvThreads, 0, st>>>(rp, col, w, x0, x1, B, emit, info, n, rs.ctl, rs.partials);
        k_relight_reduce<<<1, 256, 0, st>>>(rs.ctl, rs.partials, sblocks, 1, h);
        k_relight_spmv<<<sblocks, kSpmvThreads, 0, st>>>(rp, col, w, x1, x0, B, emit, info, n, rs.ctl, rs.partials);
        k_relight_reduce<<<1, 256, 0, st>>>(rs.ctl, rs.partials, sblocks, 1, h);
        const cudaError_t le = cudaGetLastError();
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(st, &captured);
        if (e == cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&slot->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        slot.reset();
        return cuda_fail(ctx, e, "relight loop graph");
    }
    slot->key = key;
    *out = slot->exec;
    return VRG_OK;
}

// Issues one relight on `st`: table upload, partial re-gather, warm bounce,
// digest.  Nothing here waits on the GPU.
int issue_relight(vrg_env *env, const RelightPlan &p, int32_t max_iters, float tol, cudaStream_t st,
                  RelightScratch &sc, HostStage &stage) {
    vrg_ctx *ctx = env->ctx;
    const int32_t F = env->nfaces;
    const int32_t nf = p.all ? F : (int32_t)p.faces.size();
    int rc = sc.reserve(ctx, (size_t)std::max(nf, 1), p.edited.size());
    if (rc != VRG_OK) return rc;
    // host staging: light table, then the face list and offsets
    const size_t lbytes = 80 * p.table.size();
    const size_t ebytes = 4 * p.edited.size();
    const size_t fbytes = (size_t)(nf + 1) * (8 + 8 + 4 + 4);
    rc = stage.reserve(ctx, lbytes + ebytes + fbytes + 64);
    if (rc != VRG_OK) return rc;
    std::vector<float4> packed;
    pack_lights(p.table, packed);
    char *h = static_cast<char *>(stage.ptr);
    memcpy(h, packed.data(), lbytes);
    uint32_t *he = reinterpret_cast<uint32_t *>(h + lbytes);
    memcpy(he, p.edited.data(), ebytes);
    int64_t *hs = reinterpret_cast<int64_t *>(h + ((lbytes + ebytes + 7) & ~(size_t)7));
    int64_t *hl = hs + (nf + 1);
    int32_t *hf = reinterpret_cast<int32_t *>(hl + (nf + 1));
    int32_t *hb = hf + (nf + 1);
    const int ss = env->relight_ss;
    hs[0] = hl[0] = 0;
    for (int32_t k = 0; k < nf; k++) {
        const int32_t f = p.all ? k : p.faces[k];
        hf[k] = f;
        hb[k] = env->face_leaf_begin[2 * f];
        hs[k + 1] = hs[k] + (env->luxel_offset[f + 1] - env->luxel_offset[f]) * ss;
        hl[k + 1] = hl[k] + (env->face_leaf_begin[2 * f + 1] - env->face_leaf_begin[2 * f]);
    }
    VRG_CUDA(ctx, cudaMemcpyAsync(env->d_lights.ptr, h, lbytes, cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(sc.edited, he, ebytes, cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(sc.samp_off, hs, 8 * (size_t)(nf + 1), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(sc.leaf_off, hl, 8 * (size_t)(nf + 1), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(sc.faces, hf, 4 * (size_t)(nf + 1), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(sc.leaf_beg, hb, 4 * (size_t)(nf + 1), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemsetAsync(sc.work, 0, 16, st));
    RelightList list{sc.faces, sc.samp_off, sc.leaf_off, sc.leaf_beg, nf};
    const int64_t items = hs[nf] + hl[nf];
    if (items > 0) {
        k_relight_gather<kSkyRead><<<persistent_blocks(ctx, (const void *)k_relight_gather<kSkyRead>, items), kThreads, 0, st>>>(
            scene_view(env), env->d_lights.as<DevLight>(), (int)p.table.size(), env->d_faces.as<FaceRec>(),
            env->d_luxel_offset.as<int64_t>(), F, list, ss, env->relight_seed, env->d_bake_rgb.as<float>(),
            env->d_patch_pts.as<float>(), env->d_patch_nrm.as<float>(), env->d_leaf_direct.as<float>(),
            env->d_sky_lux.as<float>(), env->d_sky_pts.as<float>(), env->sky_slots,
            env->d_vis_lux.as<uint32_t>(), env->d_vis_pts.as<uint32_t>(), env->vis_words, sc.edited, sc.work,
            sc.rays);
        VRG_CUDA(ctx, cudaGetLastError());
    }
    const int64_t n = (int64_t)env->patches.leaf_patch.size();
    float4 *B = env->d_total.as<float4>(), *emit = env->d_emit0.as<float4>();
    float4 *x0 = env->d_x.as<float4>(), *x1 = x0 + std::max<int64_t>(n, 1);
    const int ib = (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), (int64_t)ctx->num_sms * 8);
    RelightState &rs = relight_state(env);
    rc = rs.reserve_loop(ctx);
    if (rc != VRG_OK) return rc;
    k_relight_start<<<ib, 256, 0, st>>>(env->d_leaf_info.as<LeafInfo>(), env->d_leaf_direct.as<float>(), B, emit,
                                        x0, n, rs.ctl, max_iters, tol);
    VRG_CUDA(ctx, cudaGetLastError());
    // the loop runs on the device until the control block is done
    cudaGraphExec_t loop = nullptr;
    rc = loop_graph(env, st, spmv_blocks(ctx), &loop);
    if (rc != VRG_OK) return rc;
    VRG_CUDA(ctx, cudaGraphLaunch(loop, st));
    k_digest_partial<<<kDigestBlocks, 256, 0, st>>>(env->d_bake_rgb.as<float>(), 3 * env->luxel_offset.back(), B, n,
                                                     sc.partials);
    k_digest_final<<<1, 32, 0, st>>>(sc.partials, kDigestBlocks, sc.digest);
    VRG_CUDA(ctx, cudaGetLastError());
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->launches += 3 + (items > 0 ? 1 : 0);  // plus the loop graph's kernels
    }
    return VRG_OK;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ------------------------------------------------------------------------
// server

struct Request {
    int64_t ticket;
    int32_t scene;
    std::vector<vrg_light_edit> edits;
    double t_submit = 0, t_start = 0, t_done = 0;
    int32_t status = 1;  // 1 pending, 2 running, 0 done, <0 error
    int32_t bounces = 0;
    float delta = 0;
    double digest[2] = {0, 0};
    uint64_t rays = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    RelightScratch scratch;
    HostStage stage;
    HostStage result;  // pinned: ctl, digest, rays
    Request *req = nullptr;
};

struct vrg_server {
    vrg_ctx *ctx = nullptr;
    std::vector<vrg_env *> scenes;
    std::vector<char> busy;
    std::deque<Slot> slots;  // deque: slots are neither copied nor moved
    std::deque<Request *> pending;
    std::map<int64_t, Request *> reqs;
    std::mutex mu;
    std::condition_variable cv_done;
    std::thread worker;
    std::atomic<bool> stop{false};
    int64_t next_ticket = 1;
    int32_t max_iters = 32;
    float tol = 1e-3f;
    int64_t completed = 0;
};

namespace {

void finish_slot(vrg_server *s, Slot &sl) {
    Request *r = sl.req;
    const char *res = static_cast<const char *>(sl.result.ptr);
    RelightCtl c;
    memcpy(&c, res, sizeof c);
    memcpy(r->digest, res + 64, 16);
    memcpy(&r->rays, res + 128, 8);
    r->bounces = c.iters;
    r->delta = c.last_delta;
    r->t_done = now_s();
    r->status = 0;
    s->busy[r->scene] = 0;
    s->completed++;
    sl.req = nullptr;
}

int start_slot(vrg_server *s, Slot &sl, Request *r) {
    vrg_env *env = s->scenes[r->scene];
    std::lock_guard<std::mutex> lk(env->mu);  // the scene's tables and relight state
    RelightPlan plan;
    int rc = plan_relight(env, r->edits.data(), (int32_t)r->edits.size(), plan);
    if (rc != VRG_OK) return rc;
    rc = issue_relight(env, plan, s->max_iters, s->tol, sl.stream, sl.scratch, sl.stage);
    if (rc != VRG_OK) return rc;
    env->lights = plan.table;
    char *res = static_cast<char *>(sl.result.ptr);
    VRG_CUDA(s->ctx, cudaMemcpyAsync(res, relight_state(env).ctl, sizeof(RelightCtl), cudaMemcpyDeviceToHost,
                                     sl.stream));
    VRG_CUDA(s->ctx, cudaMemcpyAsync(res + 64, sl.scratch.digest, 16, cudaMemcpyDeviceToHost, sl.stream));
    VRG_CUDA(s->ctx, cudaMemcpyAsync(res + 128, sl.scratch.rays, 8, cudaMemcpyDeviceToHost, sl.stream));
    VRG_CUDA(s->ctx, cudaEventRecord(sl.done, sl.stream));
    sl.req = r;
    r->t_start = now_s();
    r->status = 2;
    s->busy[r->scene] = 1;
    return VRG_OK;
}

void worker_main(vrg_server *s) {
    cudaSetDevice(s->ctx->device);
    while (!s->stop.load()) {
        bool progressed = false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Slot &sl : s->slots) {
                if (sl.req && cudaEventQuery(sl.done) == cudaSuccess) {
                    finish_slot(s, sl);
                    progressed = true;
                }
            }
            for (Slot &sl : s->slots) {
                if (sl.req) continue;
                // oldest pending request whose scene is idle
                for (auto it = s->pending.begin(); it != s->pending.end(); ++it) {
                    Request *r = *it;
                    if (s->busy[r->scene]) continue;
                    s->pending.erase(it);
                    const int rc = start_slot(s, sl, r);
                    if (rc != VRG_OK) {
                        r->status = rc;
                        r->t_done = now_s();
                        s->completed++;
                    }
                    progressed = true;
                    break;
                }
            }
        }
        if (progressed) s->cv_done.notify_all();
        else std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

}  // namespace

extern "C" {

int vrg_env_relight_prepare(vrg_env *env, int32_t supersamples, uint64_t seed, int32_t max_bounces, float rel_tol) {
    if (!env) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    return relight_prepare(env, supersamples, seed, max_bounces, rel_tol);
}

int vrg_ctx_set_hbm_reserve(vrg_ctx *ctx, uint64_t bytes) {
    if (!ctx) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->hbm_reserve = bytes;
    return VRG_OK;
}

int vrg_env_relight(vrg_env *env, const vrg_light_edit *edits, int32_t n, int32_t max_iters, float rel_tol,
                    int32_t *out_bounces, float *out_delta) {
    if (!env || n < 0 || (n > 0 && !edits) || max_iters < 0 || !(rel_tol >= 0.0f)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(env->mu);
    vrg_ctx *ctx = env->ctx;
    if (!env->relight_ready) return fail(ctx, VRG_ERR_STATE, "vrg_env_relight_prepare has not run");
    RelightPlan plan;
    int rc = plan_relight(env, edits, n, plan);
    if (rc != VRG_OK) return rc;
    RelightState &rs = relight_state(env);
    RelightScratch &sc = rs.sc;
    rc = issue_relight(env, plan, max_iters, rel_tol, ctx->stream, sc, rs.stage);
    if (rc != VRG_OK) return rc;
    env->lights = plan.table;
    RelightCtl c;
    VRG_CUDA(ctx, cudaMemcpyAsync(&c, rs.ctl, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (out_bounces) *out_bounces = c.iters;
    if (out_delta) *out_delta = c.last_delta;
    env->bake_bounces = c.iters;
    env->bake_delta = c.last_delta;
    return VRG_OK;
}

int vrg_server_create(vrg_ctx *ctx, int32_t slots, int32_t max_iters, float rel_tol, vrg_server **out) {
    if (!ctx || !out || slots < 1 || slots > 64 || max_iters < 1 || !(rel_tol >= 0.0f)) return VRG_ERR_INVALID;
    if (ctx->host_only) return fail(ctx, VRG_ERR_STATE, "host-only context has no device");
    vrg_server *s = new (std::nothrow) vrg_server();
    if (!s) return VRG_ERR_NOMEM;
    s->ctx = ctx;
    s->max_iters = max_iters;
    s->tol = rel_tol;
    for (int32_t i = 0; i < slots; i++) s->slots.emplace_back();
    cudaSetDevice(ctx->device);
    for (Slot &sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
            sl.result.reserve(ctx, 256) != VRG_OK) {
            for (Slot &x : s->slots) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.done) cudaEventDestroy(x.done);
            }
            delete s;
            return VRG_ERR_CUDA;
        }
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return VRG_OK;
}

void vrg_server_destroy(vrg_server *s) {
    if (!s) return;
    s->stop.store(true);
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    for (Slot &sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    for (auto &kv : s->reqs) delete kv.second;
    delete s;
}

int vrg_server_add_scene(vrg_server *s, vrg_env *env, int32_t *scene_id) {
    if (!s || !env || !scene_id) return VRG_ERR_INVALID;
    if (env->ctx != s->ctx) return fail(s->ctx, VRG_ERR_INVALID, "scene belongs to another context");
    if (!env->relight_ready) return fail(s->ctx, VRG_ERR_STATE, "vrg_env_relight_prepare has not run");
    std::lock_guard<std::mutex> lk(s->mu);
    *scene_id = (int32_t)s->scenes.size();
    s->scenes.push_back(env);
    s->busy.push_back(0);
    return VRG_OK;
}

int vrg_server_submit(vrg_server *s, int32_t scene_id, const vrg_light_edit *edits, int32_t n, int64_t *ticket) {
    if (!s || !ticket || n < 0 || (n > 0 && !edits)) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (scene_id < 0 || scene_id >= (int32_t)s->scenes.size()) return fail(s->ctx, VRG_ERR_INVALID, "unknown scene");
    Request *r = new (std::nothrow) Request();
    if (!r) return VRG_ERR_NOMEM;
    r->ticket = s->next_ticket++;
    r->scene = scene_id;
    r->edits.assign(edits, edits + n);
    r->t_submit = now_s();
    s->reqs[r->ticket] = r;
    s->pending.push_back(r);
    *ticket = r->ticket;
    return VRG_OK;
}

int vrg_server_wait(vrg_server *s, int64_t ticket, double timeout_s) {
    if (!s) return VRG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(s->ctx, VRG_ERR_INVALID, "unknown ticket");
    Request *r = it->second;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                         [&] { return r->status <= 0; });
    if (!ok) return VRG_ERR_TIMEOUT;
    return r->status;
}

int vrg_server_drain(vrg_server *s, double timeout_s) {
    if (!s) return VRG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return s->completed == (int64_t)s->reqs.size();
    });
    return ok ? VRG_OK : VRG_ERR_TIMEOUT;
}

int vrg_server_result(vrg_server *s, int64_t ticket, int32_t *status, int32_t *bounces, float *delta,
                      double *times, double *digest) {
    if (!s) return VRG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(s->ctx, VRG_ERR_INVALID, "unknown ticket");
    const Request *r = it->second;
    if (status) *status = r->status;
    if (bounces) *bounces = r->bounces;
    if (delta) *delta = r->delta;
    if (times) {
        times[0] = r->t_submit;
        times[1] = r->t_start;
        times[2] = r->t_done;
    }
    if (digest) {
        digest[0] = r->digest[0];
        digest[1] = r->digest[1];
    }
    return VRG_OK;
}

}  // extern "C"
