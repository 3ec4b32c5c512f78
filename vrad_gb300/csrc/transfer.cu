// transfer.cu -- form-factor transfer lists in CSR.  The reference only
// declares the storage (Transfer{Patch, Transfer}, common/types/transfer.go:3-6;
// Patch.NumTransfers/Transfers, common/types/patch.go:60-61); building them is
// the project's own stage:
//   row i = leaf patch with centre c on face f (normal N, edge U)
//   q = c + N*0.125 ; T1 = U * (1/sqrt(U.U)) ; T2 = N x T1
//   ray r: d = ((lx*T1 + ly*T2) + lz*N) per component, closest hit on
//   [0, MAX_TRACE_LENGTH); a hit on triangle h with tri_face[h] = g >= 0
//   descends g's patch tree at x = q + t*d (coordinate >= dist -> child1)
//   to leaf j.  Row i holds each j once, ascending, with weight hits/k.
#include <algorithm>

#include "vrg_internal.h"
#include "vrg_trace.cuh"

namespace vrg {

namespace {

// One block per row: trace the k rays, sort the k target ids in shared
// memory (bitonic), then a block scan compacts runs into (col, count).  NT
// threads per block (at most k); OPT & kOptStream loads the leaf records without
// allocating in L1.
template <int NT, int OPT>
__global__ void __launch_bounds__(NT) k_transfer_rows(
    DevScene s, const LeafInfo *__restrict__ leaves, const FaceRec *__restrict__ faces,
    const PatchNode *__restrict__ pnodes, const int32_t *__restrict__ face_root,
    const int32_t *__restrict__ tri_face, const float *__restrict__ dirs, int k, int64_t row0,
    int64_t rows, int32_t *__restrict__ stage_col, int32_t *__restrict__ stage_cnt,
    int32_t *__restrict__ nnz) {
    extern __shared__ int32_t sm[];
    int32_t *tg = sm;         // k target ids
    int32_t *starts = sm + k; // k run starts
    __shared__ int32_t warp_sums[NT / 32];
    __shared__ int32_t total_sh;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int64_t rl = blockIdx.x; rl < rows; rl += gridDim.x) {
        const int64_t row = row0 + rl;
        const LeafInfo li = leaves[row];
        const int f = __float_as_int(li.refl.w);
        const FaceRec F = faces[f];
        const float qx = radd(li.center.x, rmul(F.normal.x, kSampleOffset));
        const float qy = radd(li.center.y, rmul(F.normal.y, kSampleOffset));
        const float qz = radd(li.center.z, rmul(F.normal.z, kSampleOffset));
        const float il = rrcp(rsqrt_rn(dot3r(F.u.x, F.u.y, F.u.z, F.u.x, F.u.y, F.u.z)));
        const float t1x = rmul(F.u.x, il), t1y = rmul(F.u.y, il), t1z = rmul(F.u.z, il);
        const float nx = F.normal.x, ny = F.normal.y, nz = F.normal.z;
        const float t2x = rsub(rmul(ny, t1z), rmul(nz, t1y));
        const float t2y = rsub(rmul(nz, t1x), rmul(nx, t1z));
        const float t2z = rsub(rmul(nx, t1y), rmul(ny, t1x));
        for (int r = tid; r < k; r += nt) {
            const float lx = __ldg(dirs + 3 * r), ly = __ldg(dirs + 3 * r + 1), lz = __ldg(dirs + 3 * r + 2);
            const float dx = radd(radd(rmul(lx, t1x), rmul(ly, t2x)), rmul(lz, nx));
            const float dy = radd(radd(rmul(lx, t1y), rmul(ly, t2y)), rmul(lz, ny));
            const float dz = radd(radd(rmul(lx, t1z), rmul(ly, t2z)), rmul(lz, nz));
            float t;
            const int32_t h =
                trace_ray<kClosest, OPT>(s, Ray{qx, qy, qz, dx, dy, dz}, 0.0f, kMaxTraceLength, -1, &t);
            int32_t target = -1;
            if (h >= 0) {
                const int32_t g = __ldg(tri_face + h);
                const int32_t root = g >= 0 ? __ldg(face_root + g) : -1;
                if (root >= 0) {
                    const float x0 = radd(qx, rmul(t, dx)), x1 = radd(qy, rmul(t, dy)), x2 = radd(qz, rmul(t, dz));
                    int32_t node = root;
                    PatchNode pn = pnodes[node];
                    while (pn.axis >= 0) {
                        const float xa = pick3(pn.axis, x0, x1, x2);
                        node = xa >= pn.dist ? pn.child1 : pn.child2;
                        pn = pnodes[node];
                    }
                    target = pn.leaf;
                }
            }
            tg[r] = target;
        }
        __syncthreads();
        // bitonic sort, ascending (misses = -1 first)
        for (int size = 2; size <= k; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = tid; i < (k >> 1); i += nt) {
                    const int lo = 2 * i - (i & (stride - 1));
                    const int hi = lo + stride;
                    const bool asc = (lo & size) == 0;
                    const int32_t a = tg[lo], b = tg[hi];
                    if ((a > b) == asc) {
                        tg[lo] = b;
                        tg[hi] = a;
                    }
                }
                __syncthreads();
            }
        }
        // run starts of valid targets; each thread owns a contiguous segment
        const int per = k / nt;
        const int seg = tid * per;
        int cnt = 0;
        for (int i = seg; i < seg + per; i++)
            cnt += (tg[i] >= 0 && (i == 0 || tg[i] != tg[i - 1])) ? 1 : 0;
        // block exclusive scan of cnt
        int incl = cnt;
        const int lane = tid & 31, wid = tid >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = lane < (nt >> 5) ? warp_sums[lane] : 0;
            int wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += v;
            }
            if (lane < (nt >> 5)) warp_sums[lane] = wi - w;
            if (lane == (nt >> 5) - 1) total_sh = wi;
        }
        __syncthreads();
        int pos = warp_sums[wid] + incl - cnt;
        for (int i = seg; i < seg + per; i++)
            if (tg[i] >= 0 && (i == 0 || tg[i] != tg[i - 1])) starts[pos++] = i;
        __syncthreads();
        const int total = total_sh;
        int32_t *oc = stage_col + rl * (int64_t)k;
        int32_t *on = stage_cnt + rl * (int64_t)k;
        for (int p = tid; p < total; p += nt) {
            const int st = starts[p];
            const int en = p + 1 < total ? starts[p + 1] : k;
            oc[p] = tg[st];
            on[p] = en - st;
        }
        if (tid == 0) nnz[rl] = total;
        __syncthreads();
    }
}

// One warp per row: staged (col, count) -> final CSR (col, count / k).
__global__ void k_transfer_gather(const int32_t *__restrict__ stage_col,
                                  const int32_t *__restrict__ stage_cnt,
                                  const int64_t *__restrict__ row_ptr, int64_t row0, int64_t rows,
                                  int k, int32_t *__restrict__ col, float *__restrict__ w) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float fk = (float)k;
    for (int64_t rl = warp; rl < rows; rl += nwarps) {
        const int64_t b = row_ptr[row0 + rl], e = row_ptr[row0 + rl + 1];
        const int32_t *sc = stage_col + rl * (int64_t)k;
        const int32_t *sn = stage_cnt + rl * (int64_t)k;
        for (int64_t i = lane; i < e - b; i += 32) {
            col[b + i] = sc[i];
            w[b + i] = __fdiv_rn((float)sn[i], fk);
        }
    }
}

int grow(vrg_ctx *ctx, DevBuf &buf, size_t need, size_t keep) {
    if (need <= buf.bytes && buf.ptr) return VRG_OK;
    size_t cap = std::max(need, buf.bytes + buf.bytes / 2);
    void *p = nullptr;
    VRG_CUDA(ctx, cudaMalloc(&p, cap));
    if (keep) VRG_CUDA(ctx, cudaMemcpyAsync(p, buf.ptr, keep, cudaMemcpyDeviceToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    buf.release();
    buf.ptr = p;
    buf.bytes = cap;
    return VRG_OK;
}

}  // namespace

int run_make_transfers(vrg_env *env, const float *dirs_local, int32_t k) {
    vrg_ctx *ctx = env->ctx;
    const int64_t rows = (int64_t)env->patches.leaf_patch.size();
    env->have_transfers = false;
    env->nnz = 0;
    env->transfer_k = k;
    // The rays of a row go out in table order, one per lane.  A row's CSR
    // does not depend on that order (hits are counted per target), so the
    // table is put in 2-D Morton order of its (x, y) disk coordinates: then
    // the 32 rays of a warp leave in neighbouring directions and walk much
    // the same nodes, where the given lattice order sends them all over the
    // hemisphere.
    std::vector<float> dirs(dirs_local, dirs_local + 3 * (size_t)k);
    {
        auto spread = [](uint32_t v) {
            v &= 0xffffu;
            v = (v | (v << 8)) & 0x00ff00ffu;
            v = (v | (v << 4)) & 0x0f0f0f0fu;
            v = (v | (v << 2)) & 0x33333333u;
            v = (v | (v << 1)) & 0x55555555u;
            return v;
        };
        auto q = [](float c) {
            const float u = (c + 1.0f) * 0.5f * 65535.0f;
            return (uint32_t)(u < 0.0f ? 0.0f : (u > 65535.0f ? 65535.0f : u));
        };
        std::vector<std::pair<uint32_t, int32_t>> key(k);
        for (int32_t r = 0; r < k; r++)
            key[r] = {spread(q(dirs_local[3 * r])) | (spread(q(dirs_local[3 * r + 1])) << 1), r};
        std::stable_sort(key.begin(), key.end(),
                         [](const std::pair<uint32_t, int32_t> &a, const std::pair<uint32_t, int32_t> &b) {
                             return a.first < b.first;
                         });
        for (int32_t r = 0; r < k; r++)
            for (int c = 0; c < 3; c++) dirs[3 * r + c] = dirs_local[3 * key[r].second + c];
    }
    DevBuf d_dirs;
    VRG_CUDA(ctx, d_dirs.reserve(12 * (size_t)k));
    VRG_CUDA(ctx, cudaMemcpyAsync(d_dirs.ptr, dirs.data(), 12 * (size_t)k, cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // `dirs` is pageable and goes out of scope
    const size_t smem = 2 * (size_t)k * sizeof(int32_t);
    // variants, picked per (triangles, rows) bucket: 256 or 512 threads per
    // row block, leaf records through L1 or not, children without triangles
    // visited or skipped
    using RowKernel = void (*)(DevScene, const LeafInfo *, const FaceRec *, const PatchNode *, const int32_t *,
                               const int32_t *, const float *, int, int64_t, int64_t, int32_t *, int32_t *,
                               int32_t *);
    constexpr int kRowVariants = 6;
    const RowKernel kvar[kRowVariants] = {k_transfer_rows<256, 0>,          k_transfer_rows<512, 0>,
                                          k_transfer_rows<256, kOptStream>, k_transfer_rows<512, kOptStream>,
                                          k_transfer_rows<256, kOptSkip>,   k_transfer_rows<512, kOptSkip>};
    const int vthreads[kRowVariants] = {256, 512, 256, 512, 256, 512};
    const int twin256[kRowVariants] = {0, 0, 2, 2, 4, 4};  // the 256-thread variant with the same options
    for (int v = 0; v < kRowVariants; v++)
        VRG_CUDA(ctx, cudaFuncSetAttribute(kvar[v], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // rows go through in chunks whose staging stays near 1 GiB
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(rows, ((int64_t)1 << 30) / (8 * (int64_t)k)));
    DevBuf stage_col, stage_cnt, d_nnz, d_rowptr_chunk;
    VRG_CUDA(ctx, stage_col.reserve(4 * (size_t)chunk * k));
    VRG_CUDA(ctx, stage_cnt.reserve(4 * (size_t)chunk * k));
    VRG_CUDA(ctx, d_nnz.reserve(4 * (size_t)chunk));
    std::vector<int64_t> row_ptr(rows + 1, 0);
    std::vector<int32_t> h_nnz(chunk);
    VRG_CUDA(ctx, env->d_row_ptr.reserve(8 * (size_t)(rows + 1)));
    DevScene s = scene_view(env);
    for (int64_t r0 = 0; r0 < rows; r0 += chunk) {
        const int64_t nr = std::min(chunk, rows - r0);
        const int grid = (int)std::min<int64_t>(nr, (int64_t)ctx->num_sms * 8);
        cudaEvent_t ev = nullptr;
        auto launch = [&](int v) -> cudaError_t {
            timing_begin(ctx, "transfer_rows", &ev);
            const int threads = std::min(vthreads[v], k);
            // a row block never has more threads than rays: below 512 rays the
            // 512-thread variants fall back to their 256-thread twin
            const int vv = threads == vthreads[v] ? v : twin256[v];
            kvar[vv]<<<grid, threads, smem, ctx->stream>>>(
                s, env->d_leaf_info.as<LeafInfo>(), env->d_faces.as<FaceRec>(),
                env->d_patch_nodes.as<PatchNode>(), env->d_face_root.as<int32_t>(), env->d_tri_face.as<int32_t>(),
                d_dirs.as<float>(), k, r0, nr, stage_col.as<int32_t>(), stage_cnt.as<int32_t>(),
                d_nnz.as<int32_t>());
            const cudaError_t e = cudaGetLastError();
            timing_end(ctx, "transfer_rows", ev);
            return e;
        };
        const int rc = tune_run(ctx, tune_key("transfer_rows", env->geom.ntris, rows * (int64_t)k), kRowVariants,
                                launch);
        if (rc != VRG_OK) return rc;
        VRG_CUDA(ctx, cudaMemcpyAsync(h_nnz.data(), d_nnz.ptr, 4 * (size_t)nr, cudaMemcpyDeviceToHost, ctx->stream));
        VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t i = 0; i < nr; i++) row_ptr[r0 + i + 1] = row_ptr[r0 + i] + h_nnz[i];
        const int64_t need = row_ptr[r0 + nr];
        if (grow(ctx, env->d_col, 4 * (size_t)std::max<int64_t>(need, 1), 4 * (size_t)row_ptr[r0]) != VRG_OK ||
            grow(ctx, env->d_weight, 4 * (size_t)std::max<int64_t>(need, 1), 4 * (size_t)row_ptr[r0]) != VRG_OK)
            return VRG_ERR_NOMEM;
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_row_ptr.as<int64_t>() + r0, row_ptr.data() + r0, 8 * (size_t)(nr + 1),
                                      cudaMemcpyHostToDevice, ctx->stream));
        timing_begin(ctx, "transfer_gather", &ev);
        k_transfer_gather<<<(int)std::min<int64_t>((nr + 7) / 8, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(
            stage_col.as<int32_t>(), stage_cnt.as<int32_t>(), env->d_row_ptr.as<int64_t>(), r0, nr, k,
            env->d_col.as<int32_t>(), env->d_weight.as<float>());
        VRG_CUDA(ctx, cudaGetLastError());
        timing_end(ctx, "transfer_gather", ev);
    }
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    env->nnz = row_ptr[rows];
    env->have_transfers = true;
    return VRG_OK;
}

}  // namespace vrg
