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

// Row frame and ray directions shared by both row kernels.
struct RowFrame {
    float qx, qy, qz, t1x, t1y, t1z, t2x, t2y, t2z, nx, ny, nz;
};

__device__ __forceinline__ RowFrame row_frame(const LeafInfo &li, const FaceRec &F) {
    RowFrame fr;
    fr.qx = radd(li.center.x, rmul(F.normal.x, kSampleOffset));
    fr.qy = radd(li.center.y, rmul(F.normal.y, kSampleOffset));
    fr.qz = radd(li.center.z, rmul(F.normal.z, kSampleOffset));
    const float il = rrcp(rsqrt_rn(dot3r(F.u.x, F.u.y, F.u.z, F.u.x, F.u.y, F.u.z)));
    fr.t1x = rmul(F.u.x, il);
    fr.t1y = rmul(F.u.y, il);
    fr.t1z = rmul(F.u.z, il);
    fr.nx = F.normal.x;
    fr.ny = F.normal.y;
    fr.nz = F.normal.z;
    fr.t2x = rsub(rmul(fr.ny, fr.t1z), rmul(fr.nz, fr.t1y));
    fr.t2y = rsub(rmul(fr.nz, fr.t1x), rmul(fr.nx, fr.t1z));
    fr.t2z = rsub(rmul(fr.nx, fr.t1y), rmul(fr.ny, fr.t1x));
    return fr;
}

// Target leaf of ray r of a row (-1: no lit face hit).
template <int OPT>
__device__ __forceinline__ int32_t row_ray_target(const DevScene &s, const RowFrame &fr,
                                                  const PatchNode *__restrict__ pnodes,
                                                  const int32_t *__restrict__ face_root,
                                                  const int32_t *__restrict__ tri_face,
                                                  const float *__restrict__ dirs, int r) {
    const float lx = __ldg(dirs + 3 * r), ly = __ldg(dirs + 3 * r + 1), lz = __ldg(dirs + 3 * r + 2);
    const float dx = radd(radd(rmul(lx, fr.t1x), rmul(ly, fr.t2x)), rmul(lz, fr.nx));
    const float dy = radd(radd(rmul(lx, fr.t1y), rmul(ly, fr.t2y)), rmul(lz, fr.ny));
    const float dz = radd(radd(rmul(lx, fr.t1z), rmul(ly, fr.t2z)), rmul(lz, fr.nz));
    float t;
    const int32_t h = trace_ray<kClosest, OPT>(s, Ray{fr.qx, fr.qy, fr.qz, dx, dy, dz}, 0.0f, kMaxTraceLength,
                                               -1, &t);
    if (h < 0) return -1;
    const int32_t g = __ldg(tri_face + h);
    const int32_t root = g >= 0 ? __ldg(face_root + g) : -1;
    if (root < 0) return -1;
    const float x0 = radd(fr.qx, rmul(t, dx)), x1 = radd(fr.qy, rmul(t, dy)), x2 = radd(fr.qz, rmul(t, dz));
    int32_t node = root;
    PatchNode pn = pnodes[node];
    while (pn.axis >= 0) {
        const float xa = pick3(pn.axis, x0, x1, x2);
        node = xa >= pn.dist ? pn.child1 : pn.child2;
        pn = pnodes[node];
    }
    return pn.leaf;
}

// Hash table of a row's targets in shared memory: one 64-bit slot per
// distinct target, (target << 32) | hits, open addressing with linear
// probing.  A row never holds more hits than k <= 65536, so the count word
// never carries into the key.
constexpr int kXferTableMax = 8192;   // slots (64 KiB): rows with k >= 4096
constexpr unsigned long long kSlotEmpty = 0xffffffff00000000ull;

// Adds `cnt` hits of `key` (>= 0).  A new key that takes the table past
// `limit` distinct targets, or finds no free slot, sets *ovf; the row is then
// rebuilt by k_transfer_rows_sorted.
__device__ __forceinline__ void table_add(unsigned long long *table, int tbits, int32_t key, uint32_t cnt,
                                          int *used, int limit, volatile int *ovf) {
    const uint32_t mask = (1u << tbits) - 1u;
    uint32_t slot = ((uint32_t)key * 0x9E3779B1u) >> (32 - tbits);
    const uint32_t want = (uint32_t)key;
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const unsigned long long v = *(volatile unsigned long long *)&table[slot];
        if ((uint32_t)(v >> 32) == want) {
            atomicAdd(&table[slot], (unsigned long long)cnt);
            return;
        }
        if (v == kSlotEmpty) {
            const unsigned long long mine = ((unsigned long long)want << 32) | cnt;
            const unsigned long long old = atomicCAS(&table[slot], kSlotEmpty, mine);
            if (old == kSlotEmpty) {
                if (atomicAdd(used, 1) + 1 > limit) *ovf = 1;
                return;
            }
            if ((uint32_t)(old >> 32) == want) {
                atomicAdd(&table[slot], (unsigned long long)cnt);
                return;
            }
        }
        slot = (slot + 1u) & mask;
    }
    *ovf = 1;
}

// One block per row: trace the k rays; the lanes of a warp that hit the
// same target add their hits with one table update (warp match); then the
// table is sorted in place (bitonic over its 2^tbits slots, ascending as
// 64-bit words, so the occupied slots come first in target order) and its
// first `used` slots are the row: (col, count) into the staging arrays at
// stride 2^tbits.  A row past `limit` distinct targets writes nnz = -1 and
// is rebuilt by k_transfer_rows_sorted.  NT threads per block at most; k is a
// multiple of the block size, so every lane of a warp runs the same rays.
// OPT & kOptStream loads leaf records without allocating in L1; kOptSkip skips
// children without triangles.
template <int NT, int OPT>
__global__ void __launch_bounds__(NT) k_transfer_rows(
    DevScene s, const LeafInfo *__restrict__ leaves, const FaceRec *__restrict__ faces,
    const PatchNode *__restrict__ pnodes, const int32_t *__restrict__ face_root,
    const int32_t *__restrict__ tri_face, const float *__restrict__ dirs, int k, int64_t row0,
    int64_t rows, int tbits, int limit, int32_t *__restrict__ stage_col, int32_t *__restrict__ stage_cnt,
    int32_t *__restrict__ nnz) {
    extern __shared__ unsigned long long table[];
    __shared__ int used_sh;
    __shared__ int ovf_sh;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    const int tsize = 1 << tbits;
    for (int64_t rl = blockIdx.x; rl < rows; rl += gridDim.x) {
        for (int i = tid; i < tsize; i += nt) table[i] = kSlotEmpty;
        if (tid == 0) {
            used_sh = 0;
            ovf_sh = 0;
        }
        __syncthreads();
        const int64_t row = row0 + rl;
        const LeafInfo li = leaves[row];
        const RowFrame fr = row_frame(li, faces[__float_as_int(li.refl.w)]);
        for (int r = tid; r < k; r += nt) {
            const int32_t target = row_ray_target<OPT>(s, fr, pnodes, face_root, tri_face, dirs, r);
            const unsigned peers = __match_any_sync(0xffffffffu, target);
            if (target >= 0 && lane == __ffs(peers) - 1 && !*(volatile int *)&ovf_sh)
                table_add(table, tbits, target, (uint32_t)__popc(peers), &used_sh, limit, &ovf_sh);
        }
        __syncthreads();
        if (ovf_sh) {
            if (tid == 0) nnz[rl] = -1;
            __syncthreads();
            continue;
        }
        for (int size = 2; size <= tsize; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = tid; i < (tsize >> 1); i += nt) {
                    const int lo = 2 * i - (i & (stride - 1));
                    const int hi = lo + stride;
                    const bool asc = (lo & size) == 0;
                    const unsigned long long a = table[lo], b = table[hi];
                    if ((a > b) == asc) {
                        table[lo] = b;
                        table[hi] = a;
                    }
                }
                __syncthreads();
            }
        }
        const int total = used_sh;
        int32_t *oc = stage_col + rl * (int64_t)tsize;
        int32_t *on = stage_cnt + rl * (int64_t)tsize;
        for (int p = tid; p < total; p += nt) {
            const unsigned long long v = table[p];
            oc[p] = (int32_t)(v >> 32);
            on[p] = (int32_t)(uint32_t)v;
        }
        if (tid == 0) nnz[rl] = total;
        __syncthreads();
    }
}

// Rows that overflowed the table: one block per listed row, its k targets
// sorted (bitonic) in a global scratch of 2k int32 per block, then a block
// scan finds the runs.  Without row_ptr it writes each listed row's nnz;
// with row_ptr it writes the row's (col, hits / k) straight into the CSR at
// row_ptr[row].  NT threads per block at most; k is a power of two and a
// multiple of the block size.
template <int NT>
__global__ void __launch_bounds__(NT) k_transfer_rows_sorted(
    DevScene s, const LeafInfo *__restrict__ leaves, const FaceRec *__restrict__ faces,
    const PatchNode *__restrict__ pnodes, const int32_t *__restrict__ face_root,
    const int32_t *__restrict__ tri_face, const float *__restrict__ dirs, int k,
    const int64_t *__restrict__ row_list, int64_t nlist, int32_t *__restrict__ scratch,
    const int64_t *__restrict__ row_ptr, int32_t *__restrict__ col, float *__restrict__ w,
    int32_t *__restrict__ nnz) {
    __shared__ int32_t warp_sums[NT / 32];
    __shared__ int32_t total_sh;
    const int tid = threadIdx.x, nt = blockDim.x;
    int32_t *tg = scratch + (int64_t)blockIdx.x * 2 * k;
    int32_t *starts = tg + k;
    for (int64_t j = blockIdx.x; j < nlist; j += gridDim.x) {
        const int64_t row = row_list[j];
        const LeafInfo li = leaves[row];
        const RowFrame fr = row_frame(li, faces[__float_as_int(li.refl.w)]);
        for (int r = tid; r < k; r += nt) tg[r] = row_ray_target<0>(s, fr, pnodes, face_root, tri_face, dirs, r);
        __syncthreads();
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
        for (int i = seg; i < seg + per; i++) cnt += (tg[i] >= 0 && (i == 0 || tg[i] != tg[i - 1])) ? 1 : 0;
        int incl = cnt;
        const int lane = tid & 31, wid = tid >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            const int w = lane < (nt >> 5) ? warp_sums[lane] : 0;
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
        if (row_ptr) {
            const int64_t b = row_ptr[row];
            const float fk = (float)k;
            for (int p = tid; p < total; p += nt) {
                const int st = starts[p];
                const int en = p + 1 < total ? starts[p + 1] : k;
                col[b + p] = tg[st];
                w[b + p] = __fdiv_rn((float)(en - st), fk);
            }
        } else if (tid == 0) {
            nnz[j] = total;
        }
        __syncthreads();
    }
}

// One warp per row: staged (col, count) at stride `tstride` -> final CSR
// (col, count / k).  Rows with nnz_chunk < 0 overflowed the row table and are
// written by k_transfer_rows_sorted instead.
__global__ void k_transfer_gather(const int32_t *__restrict__ stage_col,
                                  const int32_t *__restrict__ stage_cnt, int tstride,
                                  const int32_t *__restrict__ nnz_chunk,
                                  const int64_t *__restrict__ row_ptr, int64_t row0, int64_t rows,
                                  int k, int32_t *__restrict__ col, float *__restrict__ w) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float fk = (float)k;
    for (int64_t rl = warp; rl < rows; rl += nwarps) {
        if (nnz_chunk[rl] < 0) continue;
        const int64_t b = row_ptr[row0 + rl], e = row_ptr[row0 + rl + 1];
        const int32_t *sc = stage_col + rl * (int64_t)tstride;
        const int32_t *sn = stage_cnt + rl * (int64_t)tstride;
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
    // Table size per row block: 2k slots below k = 4096 (a row has at most k
    // distinct targets, so it never overflows), kXferTableMax from there on.
    int tbits = 6;
    while ((1 << tbits) < std::min(2 * k, kXferTableMax)) tbits++;
    const int tsize = 1 << tbits;
    const int limit = std::min(ctx->xfer_table_limit, tsize - tsize / 8);
    const size_t smem = 8 * (size_t)tsize;
    // variants, picked per (triangles, rows) bucket: 256 or 512 threads per
    // row block, leaf records through L1 or not, children without triangles
    // visited or skipped
    using RowKernel = void (*)(DevScene, const LeafInfo *, const FaceRec *, const PatchNode *, const int32_t *,
                               const int32_t *, const float *, int, int64_t, int64_t, int, int, int32_t *,
                               int32_t *, int32_t *);
    constexpr int kRowVariants = 6;
    const RowKernel kvar[kRowVariants] = {k_transfer_rows<256, 0>,          k_transfer_rows<512, 0>,
                                          k_transfer_rows<256, kOptStream>, k_transfer_rows<512, kOptStream>,
                                          k_transfer_rows<256, kOptSkip>,   k_transfer_rows<512, kOptSkip>};
    const int vthreads[kRowVariants] = {256, 512, 256, 512, 256, 512};
    const int twin256[kRowVariants] = {0, 0, 2, 2, 4, 4};  // the 256-thread variant with the same options
    for (int v = 0; v < kRowVariants; v++)
        VRG_CUDA(ctx, cudaFuncSetAttribute(kvar[v], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // rows go through in chunks whose staging stays near 1 GiB
    const int64_t chunk =
        std::max<int64_t>(1, std::min<int64_t>(rows, ((int64_t)1 << 30) / (8 * (int64_t)tsize)));
    DevBuf stage_col, stage_cnt, d_nnz;
    VRG_CUDA(ctx, stage_col.reserve(4 * (size_t)chunk * tsize));
    VRG_CUDA(ctx, stage_cnt.reserve(4 * (size_t)chunk * tsize));
    VRG_CUDA(ctx, d_nnz.reserve(4 * (size_t)chunk));
    // rows past the table go to the sorting kernel twice: once for their
    // counts, once (after row_ptr is known) to write their entries; its
    // scratch is 2k int32 per block
    const int ovf_threads = std::min(512, k);
    const int ovf_grid_max = ctx->num_sms * 2;
    DevBuf ovf_scratch, ovf_rows, ovf_nnz;
    std::vector<int64_t> row_ptr(rows + 1, 0);
    std::vector<int32_t> h_nnz(chunk);
    std::vector<int64_t> ovf_list;
    VRG_CUDA(ctx, env->d_row_ptr.reserve(8 * (size_t)(rows + 1)));
    DevScene s = scene_view(env);
    env->transfer_overflow_rows = 0;
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
                d_dirs.as<float>(), k, r0, nr, tbits, limit, stage_col.as<int32_t>(), stage_cnt.as<int32_t>(),
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
        ovf_list.clear();
        for (int64_t i = 0; i < nr; i++)
            if (h_nnz[i] < 0) ovf_list.push_back(r0 + i);
        const int64_t novf = (int64_t)ovf_list.size();
        env->transfer_overflow_rows += novf;
        const int ovf_grid = (int)std::min<int64_t>(std::max<int64_t>(novf, 1), ovf_grid_max);
        auto sorted_rows = [&](const int64_t *rp) -> cudaError_t {
            timing_begin(ctx, "transfer_rows_sorted", &ev);
            k_transfer_rows_sorted<512><<<ovf_grid, ovf_threads, 0, ctx->stream>>>(
                s, env->d_leaf_info.as<LeafInfo>(), env->d_faces.as<FaceRec>(), env->d_patch_nodes.as<PatchNode>(),
                env->d_face_root.as<int32_t>(), env->d_tri_face.as<int32_t>(), d_dirs.as<float>(), k,
                ovf_rows.as<int64_t>(), novf, ovf_scratch.as<int32_t>(), rp, env->d_col.as<int32_t>(),
                env->d_weight.as<float>(), ovf_nnz.as<int32_t>());
            const cudaError_t e = cudaGetLastError();
            timing_end(ctx, "transfer_rows_sorted", ev);
            return e;
        };
        if (novf > 0) {
            VRG_CUDA(ctx, ovf_scratch.reserve(8 * (size_t)ovf_grid * k));
            VRG_CUDA(ctx, ovf_rows.reserve(8 * (size_t)novf));
            VRG_CUDA(ctx, ovf_nnz.reserve(4 * (size_t)novf));
            VRG_CUDA(ctx, cudaMemcpyAsync(ovf_rows.ptr, ovf_list.data(), 8 * (size_t)novf, cudaMemcpyHostToDevice,
                                          ctx->stream));
            VRG_CUDA(ctx, sorted_rows(nullptr));
            std::vector<int32_t> onnz(novf);
            VRG_CUDA(ctx, cudaMemcpyAsync(onnz.data(), ovf_nnz.ptr, 4 * (size_t)novf, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int64_t j = 0; j < novf; j++) h_nnz[ovf_list[j] - r0] = onnz[j];
        }
        for (int64_t i = 0; i < nr; i++) row_ptr[r0 + i + 1] = row_ptr[r0 + i] + h_nnz[i];
        const int64_t need = row_ptr[r0 + nr];
        if (grow(ctx, env->d_col, 4 * (size_t)std::max<int64_t>(need, 1), 4 * (size_t)row_ptr[r0]) != VRG_OK ||
            grow(ctx, env->d_weight, 4 * (size_t)std::max<int64_t>(need, 1), 4 * (size_t)row_ptr[r0]) != VRG_OK)
            return VRG_ERR_NOMEM;
        VRG_CUDA(ctx, cudaMemcpyAsync(env->d_row_ptr.as<int64_t>() + r0, row_ptr.data() + r0, 8 * (size_t)(nr + 1),
                                      cudaMemcpyHostToDevice, ctx->stream));
        if (novf > 0) VRG_CUDA(ctx, sorted_rows(env->d_row_ptr.as<int64_t>()));
        timing_begin(ctx, "transfer_gather", &ev);
        k_transfer_gather<<<(int)std::min<int64_t>((nr + 7) / 8, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(
            stage_col.as<int32_t>(), stage_cnt.as<int32_t>(), tsize, d_nnz.as<int32_t>(),
            env->d_row_ptr.as<int64_t>(), r0, nr, k, env->d_col.as<int32_t>(), env->d_weight.as<float>());
        VRG_CUDA(ctx, cudaGetLastError());
        timing_end(ctx, "transfer_gather", ev);
        // the staging and the pageable row_ptr are reused by the next chunk
        VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    VRG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    env->nnz = row_ptr[rows];
    env->have_transfers = true;
    return VRG_OK;
}

}  // namespace vrg
