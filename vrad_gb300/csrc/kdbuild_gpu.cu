// kdbuild_gpu.cu -- the walk tree built on the device (binned SAH), for
// scenes admitted while a GPU is at hand.
//
// Same tree format and the same leaf rule as build_walk_tree (kdbuild.cpp):
// a triangle goes to the left child when its extent, clamped to the node's
// box, starts below the split plane, to the right one when it ends above
// it, and a triangle lying in the plane to the cheaper side; so every leaf holds
// every triangle touching its cell and the walk's answers are those of
// brute force, whatever planes are chosen.  Nodes of up to kSmallNode
// triangles weigh every extent boundary exactly (choose_exact); larger ones,
// per axis and per each of kBins bins of their box, the first start and the
// last end of the clamped extents that fall in the bin, with counts from a
// histogram of the extents (the binned SAH of Wald, "On fast construction of
// SAH-based bounding volume hierarchies", 2007, applied to kd splits, with
// planes kept on extent boundaries as the full sweep keeps them).
//
// Level by level, three launches: (1) one block per node bins its
// triangles, picks a plane or makes it a leaf, and counts the children's
// triangles exactly; (2) one block scans those counts into the next level's
// node and triangle offsets and the leaves' places in the final list, in
// node order, so the tree is the same on every run; (3) one block per node
// writes the node word, the children's boxes and ranges, and partitions its
// triangle list, stably, into the next level's list.  The host reads three
// totals between (2) and (3) to size the next level's buffers.
#include <algorithm>
#include <cstring>
#include <vector>

#include "vrg_internal.h"

namespace vrg {

namespace {

constexpr int kBins = 256;
constexpr int kBuildThreads = 256;

struct LNode {        // a node of the current level
    float mn[3], mx[3];
    int32_t out_id;   // its index in the final node array
    int32_t rbeg, rcnt;
};

struct LDec {         // what a node of the level became
    int32_t axis;     // -1: leaf
    float split;
    int32_t nl, nr;
    int32_t planar_left;  // triangles lying in the plane go left (else right)
};

struct LScan {        // offsets from the scan
    int32_t child;    // rank among the level's split nodes
    int32_t ref_next; // first entry of its children in the next level's list
    int32_t leaf_ref; // first entry of its leaf in the final list (level-relative)
};

// float <-> unsigned key with the same order (for atomicMin / atomicMax)
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ int bin_of(float v, float lo, float inv_w) {
    const int b = (int)((v - lo) * inv_w);
    return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
}

// A small node weighs every extent boundary exactly, as the host sweep
// does: each thread takes candidate planes (the clamped start and end of
// each triangle on each axis) and counts both sides over the node's list;
// the block keeps the cheapest (ties to the lower candidate, so the choice
// is the same on every run).  Triangles lying in the plane go to the side
// that makes the split cheaper, as in the host sweep.
constexpr int kSmallNode = 512;

__device__ void choose_exact(const LNode &nd, const int32_t *__restrict__ refs, const float *__restrict__ lo,
                             const float *__restrict__ hi, int64_t ntri, const WalkTreeCosts &cost,
                             LDec *__restrict__ out) {
    __shared__ double bc_s[kBuildThreads];
    __shared__ int bi_s[kBuildThreads];
    __shared__ float bp_s[kBuildThreads];
    __shared__ int bl_s[kBuildThreads], br_s[kBuildThreads];
    const int n = nd.rcnt, tid = threadIdx.x;
    const double d0 = (double)nd.mx[0] - nd.mn[0], d1 = (double)nd.mx[1] - nd.mn[1],
                 d2 = (double)nd.mx[2] - nd.mn[2];
    const double sa = 2.0 * (d0 * d1 + d0 * d2 + d1 * d2);
    double bc = (double)cost.intersection * n;
    int bi = 0x7fffffff, bl = 0, br = 0;
    float bp = 0.0f;
    for (int c = tid; c < 6 * n && sa > 0.0; c += blockDim.x) {
        const int a = c / (2 * n), r = (c % (2 * n)) >> 1;
        const int32_t t = refs[nd.rbeg + r];
        const float p = (c & 1) ? fminf(hi[a * ntri + t], nd.mx[a]) : fmaxf(lo[a * ntri + t], nd.mn[a]);
        if (!(p > nd.mn[a] && p < nd.mx[a])) continue;
        int cl = 0, cr = 0, np = 0;
        for (int k = 0; k < n; k++) {
            const int32_t u = refs[nd.rbeg + k];
            const float l = fmaxf(lo[a * ntri + u], nd.mn[a]), h = fminf(hi[a * ntri + u], nd.mx[a]);
            if (l == h && l == p) {
                np++;
            } else {
                cl += l < p;
                cr += h > p;
            }
        }
        const double da = a == 0 ? d0 : (a == 1 ? d1 : d2);
        const double db = a == 0 ? d1 : d0, dc = a == 2 ? d1 : d2;
        const double f = ((double)p - nd.mn[a]) / da;
        const double sl = 2.0 * (f * da * db + f * da * dc + db * dc);
        const double sr = 2.0 * ((1.0 - f) * da * db + (1.0 - f) * da * dc + db * dc);
        for (int side = 0; side < 2; side++) {  // the plane's own triangles left, then right
            const int l2 = cl + (side == 0 ? np : 0), r2 = cr + (side == 1 ? np : 0);
            double cst = cost.traversal + cost.intersection * (sl / sa * l2 + sr / sa * r2);
            if (l2 == 0 || r2 == 0) cst *= cost.empty_bonus;
            const int ci = 2 * c + side;
            if (cst < bc || (cst == bc && bi != 0x7fffffff && ci < bi)) {
                bc = cst;
                bi = ci;
                bp = p;
                bl = l2;
                br = r2;
            }
        }
    }
    bc_s[tid] = bc;
    bi_s[tid] = bi;
    bp_s[tid] = bp;
    bl_s[tid] = bl;
    br_s[tid] = br;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (tid < o) {
            const double c2 = bc_s[tid + o];
            const int i2 = bi_s[tid + o];
            if (c2 < bc_s[tid] || (c2 == bc_s[tid] && i2 < bi_s[tid])) {
                bc_s[tid] = c2;
                bi_s[tid] = i2;
                bp_s[tid] = bp_s[tid + o];
                bl_s[tid] = bl_s[tid + o];
                br_s[tid] = br_s[tid + o];
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        const int a = bi_s[0] == 0x7fffffff ? -1 : (bi_s[0] >> 1) / (2 * n);
        *out = a < 0 ? LDec{-1, 0.0f, 0, 0, 0} : LDec{a, bp_s[0], bl_s[0], br_s[0], (bi_s[0] & 1) == 0};
    }
}

// (1) bin, choose, count
__global__ void __launch_bounds__(kBuildThreads) k_kd_choose(
    const LNode *__restrict__ nodes, const int32_t *__restrict__ refs, const float *__restrict__ lo,
    const float *__restrict__ hi, int64_t ntri, int level, WalkTreeCosts cost, LDec *__restrict__ dec) {
    __shared__ int hs[3][kBins], he[3][kBins];
    __shared__ uint32_t kmin[3][kBins], kmax[3][kBins];  // per bin: first start, last end
    __shared__ double best_c[3];
    __shared__ float best_s[3];
    __shared__ int cnt[3];
    const LNode nd = nodes[blockIdx.x];
    const int n = nd.rcnt;
    const int tid = threadIdx.x;
    if (n <= 1 || level + 1 >= cost.max_depth) {
        if (tid == 0) dec[blockIdx.x] = LDec{-1, 0.0f, 0, 0, 0};
        return;
    }
    if (n <= kSmallNode) {
        choose_exact(nd, refs, lo, hi, ntri, cost, dec + blockIdx.x);
        return;
    }
    for (int i = tid; i < 3 * kBins; i += blockDim.x) {
        (&hs[0][0])[i] = 0;
        (&he[0][0])[i] = 0;
        (&kmin[0][0])[i] = 0xffffffffu;
        (&kmax[0][0])[i] = 0u;
    }
    __syncthreads();
    float inv_w[3];
    for (int a = 0; a < 3; a++) {
        const float w = nd.mx[a] - nd.mn[a];
        inv_w[a] = w > 0.0f ? (float)kBins / w : 0.0f;
    }
    for (int r = tid; r < n; r += blockDim.x) {
        const int32_t t = refs[nd.rbeg + r];
        for (int a = 0; a < 3; a++) {
            if (inv_w[a] == 0.0f) continue;
            const float l = fmaxf(lo[a * ntri + t], nd.mn[a]), h = fminf(hi[a * ntri + t], nd.mx[a]);
            const int bl = bin_of(l, nd.mn[a], inv_w[a]), bh = bin_of(h, nd.mn[a], inv_w[a]);
            atomicAdd(&hs[a][bl], 1);
            atomicAdd(&he[a][bh], 1);
            atomicMin(&kmin[a][bl], fkey(l));
            atomicMax(&kmax[a][bh], fkey(h));
        }
    }
    __syncthreads();
    if (tid < 3) {
        const int a = tid;
        double bc = (double)cost.intersection * n;  // the leaf's cost
        float bs = 0.0f;
        const double d0 = (double)nd.mx[0] - nd.mn[0], d1 = (double)nd.mx[1] - nd.mn[1],
                     d2 = (double)nd.mx[2] - nd.mn[2];
        const double sa = 2.0 * (d0 * d1 + d0 * d2 + d1 * d2);
        if (inv_w[a] != 0.0f && sa > 0.0) {
            const double da = a == 0 ? d0 : (a == 1 ? d1 : d2);
            const double db = a == 0 ? d1 : d0, dc = a == 2 ? d1 : d2;
            const float mn = nd.mn[a], w = nd.mx[a] - nd.mn[a];
            // candidate plane p with about nl triangles on the left and nr
            // on the right (the chosen plane is recounted exactly below)
            auto consider = [&](float p, int nl, int nr) {
                if (!(p > nd.mn[a] && p < nd.mx[a])) return;
                const double f = ((double)p - mn) / w;
                const double sl = 2.0 * (f * da * db + f * da * dc + db * dc);
                const double sr = 2.0 * ((1.0 - f) * da * db + (1.0 - f) * da * dc + db * dc);
                double c = cost.traversal + cost.intersection * (sl / sa * nl + sr / sa * nr);
                if (nl == 0 || nr == 0) c *= cost.empty_bonus;
                if (c < bc) {
                    bc = c;
                    bs = p;
                }
            };
            int starts = 0, ends = 0;  // extents starting / ending in the bins below i
            for (int i = 0; i < kBins; i++) {
                // the first start in the bin (a near face): starts below it
                // go left, ends below it are left-only
                if (hs[a][i]) consider(fkey_inv(kmin[a][i]), starts, n - ends);
                // the last end in the bin (a far face): exact counts
                if (he[a][i]) consider(fkey_inv(kmax[a][i]), starts + hs[a][i], n - ends - he[a][i]);
                starts += hs[a][i];
                ends += he[a][i];
            }
        }
        best_c[a] = bc;
        best_s[a] = bs;
    }
    if (tid < 3) cnt[tid] = 0;
    __syncthreads();
    int axis = -1;
    double bc = (double)cost.intersection * n;
    for (int a = 0; a < 3; a++)
        if (best_c[a] < bc && best_s[a] > nd.mn[a] && best_s[a] < nd.mx[a]) {
            bc = best_c[a];
            axis = a;
        }
    if (axis < 0) {
        if (tid == 0) dec[blockIdx.x] = LDec{-1, 0.0f, 0, 0, 0};
        return;
    }
    const float s = best_s[axis];
    int cl = 0, cr = 0, np = 0;
    for (int r = tid; r < n; r += blockDim.x) {
        const int32_t t = refs[nd.rbeg + r];
        const float l = fmaxf(lo[axis * ntri + t], nd.mn[axis]), h = fminf(hi[axis * ntri + t], nd.mx[axis]);
        if (l == h && l == s) {
            np++;
        } else {
            cl += l < s;
            cr += h > s;
        }
    }
    atomicAdd(&cnt[0], cl);
    atomicAdd(&cnt[1], cr);
    atomicAdd(&cnt[2], np);
    __syncthreads();
    if (tid == 0) {
        // the plane was chosen on estimated counts: keep it only if the
        // exact counts still make the split cheaper than the leaf
        const double d0 = (double)nd.mx[0] - nd.mn[0], d1 = (double)nd.mx[1] - nd.mn[1],
                     d2 = (double)nd.mx[2] - nd.mn[2];
        const double sa = 2.0 * (d0 * d1 + d0 * d2 + d1 * d2);
        const double da = axis == 0 ? d0 : (axis == 1 ? d1 : d2);
        const double db = axis == 0 ? d1 : d0, dc = axis == 2 ? d1 : d2;
        const double f = ((double)s - nd.mn[axis]) / ((double)nd.mx[axis] - nd.mn[axis]);
        const double sl = 2.0 * (f * da * db + f * da * dc + db * dc);
        const double sr = 2.0 * ((1.0 - f) * da * db + (1.0 - f) * da * dc + db * dc);
        LDec best{-1, 0.0f, 0, 0, 0};
        double bcost = (double)cost.intersection * n;
        for (int side = 0; side < 2; side++) {  // the plane's own triangles left, then right
            const int l2 = cnt[0] + (side == 0 ? cnt[2] : 0), r2 = cnt[1] + (side == 1 ? cnt[2] : 0);
            double c = cost.traversal + cost.intersection * (sl / sa * l2 + sr / sa * r2);
            if (l2 == 0 || r2 == 0) c *= cost.empty_bonus;
            if (c < bcost) {
                bcost = c;
                best = LDec{axis, s, l2, r2, side == 0};
            }
        }
        dec[blockIdx.x] = best;
    }
}

// (2) scans over the level's nodes, in node order; totals = {split nodes,
// next-level entries, leaf entries}
__global__ void __launch_bounds__(1024) k_kd_scan(const LDec *__restrict__ dec, const LNode *__restrict__ nodes,
                                                  int m, LScan *__restrict__ sc, int64_t *__restrict__ totals) {
    __shared__ int64_t wsum[3][32];
    __shared__ int64_t carry[3];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid < 3) carry[tid] = 0;
    __syncthreads();
    for (int base = 0; base < m; base += blockDim.x) {
        const int i = base + tid;
        int64_t v[3] = {0, 0, 0};
        if (i < m) {
            const LDec d = dec[i];
            if (d.axis >= 0) {
                v[0] = 1;
                v[1] = (int64_t)d.nl + d.nr;
            } else {
                v[2] = nodes[i].rcnt;
            }
        }
        int64_t x[3];
        for (int k = 0; k < 3; k++) {
            x[k] = v[k];
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, x[k], o);
                if (lane >= o) x[k] += y;
            }
            if (lane == 31) wsum[k][wid] = x[k];
        }
        __syncthreads();
        if (wid == 0) {
            for (int k = 0; k < 3; k++) {
                int64_t y = lane < (int)(blockDim.x >> 5) ? wsum[k][lane] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    const int64_t z = __shfl_up_sync(0xffffffffu, y, o);
                    if (lane >= o) y += z;
                }
                wsum[k][lane] = y;  // inclusive over warps
            }
        }
        __syncthreads();
        int64_t ex[3];
        for (int k = 0; k < 3; k++) ex[k] = carry[k] + (wid > 0 ? wsum[k][wid - 1] : 0) + x[k] - v[k];
        if (i < m) sc[i] = LScan{(int32_t)ex[0], (int32_t)ex[1], (int32_t)ex[2]};
        __syncthreads();
        if (tid < 3) carry[tid] += wsum[tid][(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (tid < 3) totals[tid] = carry[tid];
}

// block-wide exclusive scan of one int per thread; returns the prefix and
// sets *total
__device__ __forceinline__ int block_scan(int v, int *buf, int *total) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) buf[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = lane < nw ? buf[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        buf[lane] = y;
    }
    __syncthreads();
    const int pre = (wid > 0 ? buf[wid - 1] : 0) + x - v;
    *total = buf[nw - 1];
    __syncthreads();
    return pre;
}

// (3) write the level: node words, next-level nodes, partitioned lists.
// Every index below is bounded by the scans; the capacities are checked
// anyway and a violation is recorded instead of written.
__global__ void __launch_bounds__(kBuildThreads) k_kd_write(
    const LNode *__restrict__ nodes, const LDec *__restrict__ dec, const LScan *__restrict__ sc,
    const int32_t *__restrict__ refs, const float *__restrict__ lo, const float *__restrict__ hi, int64_t ntri,
    int32_t first_child, int64_t leaf_ref0, uint32_t *__restrict__ children, float *__restrict__ split,
    int64_t node_cap, LNode *__restrict__ next, int64_t next_cap, int32_t *__restrict__ refs_next,
    int64_t refs_next_cap, int32_t *__restrict__ refs_final, int64_t refs_final_cap, int *__restrict__ err) {
    __shared__ int buf[32];
    const LNode nd = nodes[blockIdx.x];
    const LDec d = dec[blockIdx.x];
    const LScan s = sc[blockIdx.x];
    const int tid = threadIdx.x;
    if (nd.out_id < 0 || nd.out_id >= node_cap) {
        if (tid == 0) atomicExch(err, 1);
        return;
    }
    if (d.axis < 0) {
        const int64_t fb = leaf_ref0 + s.leaf_ref;
        if (fb + nd.rcnt > refs_final_cap || fb >= ((int64_t)1 << 30)) {
            if (tid == 0) atomicExch(err, 1);
            return;
        }
        if (tid == 0) {
            children[nd.out_id] = kLeaf | ((uint32_t)fb << 2);
            split[nd.out_id] = (float)nd.rcnt;
        }
        for (int r = tid; r < nd.rcnt; r += blockDim.x) refs_final[fb + r] = refs[nd.rbeg + r];
        return;
    }
    const int32_t left = first_child + 2 * s.child;
    const int64_t li = 2 * (int64_t)s.child;
    if (left + 1 >= node_cap || li + 1 >= next_cap || (int64_t)s.ref_next + d.nl + d.nr > refs_next_cap) {
        if (tid == 0) atomicExch(err, 1);
        return;
    }
    if (tid == 0) {
        children[nd.out_id] = (uint32_t)d.axis | ((uint32_t)left << 2);
        split[nd.out_id] = d.split;
        LNode l = nd, r = nd;
        l.mx[d.axis] = d.split;
        r.mn[d.axis] = d.split;
        l.out_id = left;
        r.out_id = left + 1;
        l.rbeg = s.ref_next;
        l.rcnt = d.nl;
        r.rbeg = s.ref_next + d.nl;
        r.rcnt = d.nr;
        next[li] = l;
        next[li + 1] = r;
    }
    // stable partition in tiles of blockDim.x entries
    int off_l = 0, off_r = 0;
    for (int base = 0; base < nd.rcnt; base += blockDim.x) {
        const int r = base + tid;
        int gl = 0, gr = 0;
        int32_t t = 0;
        if (r < nd.rcnt) {
            t = refs[nd.rbeg + r];
            const float l = fmaxf(lo[d.axis * ntri + t], nd.mn[d.axis]);
            const float h = fminf(hi[d.axis * ntri + t], nd.mx[d.axis]);
            if (l == h && l == d.split) {
                (d.planar_left ? gl : gr) = 1;
            } else {
                gl = l < d.split;
                gr = h > d.split;
            }
        }
        int tl, tr;
        const int pl = block_scan(gl, buf, &tl);
        const int pr = block_scan(gr, buf, &tr);
        if (gl) {
            if (off_l + pl < d.nl) refs_next[s.ref_next + off_l + pl] = t;
            else atomicExch(err, 1);
        }
        if (gr) {
            if (off_r + pr < d.nr) refs_next[s.ref_next + d.nl + off_r + pr] = t;
            else atomicExch(err, 1);
        }
        off_l += tl;
        off_r += tr;
    }
}

// Capacity for n elements, growing geometrically so that the per-level
// buffers are reallocated only a few times per build.
template <class T>
cudaError_t grow_buf(DevBuf &b, int64_t n) {
    const size_t need = sizeof(T) * (size_t)std::max<int64_t>(n, 1);
    if (b.ptr && b.bytes >= need) return cudaSuccess;
    return b.reserve(std::max(need, std::max<size_t>(2 * b.bytes, 64 * 1024)));
}

}  // namespace

// Builds the walk tree on the context's device; the result is copied back
// into `tree` (the host keeps the tree for the upload and for
// vrg_env_get_walk_tree).
int build_walk_tree_device(vrg_env *env, HostTree &tree) {
    vrg_ctx *ctx = env->ctx;
    const int64_t n = (int64_t)env->ids.size();
    cudaStream_t st = ctx->stream;
    tree.children.assign(1, 0);
    tree.split.assign(1, 0.0f);
    tree.refs.clear();
    tree.height = 0;
    if (n == 0) {
        tree.children[0] = kLeaf;
        tree.height = 1;
        return VRG_OK;
    }
    std::vector<float> lo(3 * (size_t)n), hi(3 * (size_t)n);
    for (int64_t t = 0; t < n; t++)
        for (int a = 0; a < 3; a++) {
            const float *v = &env->xyz[9 * t];
            lo[a * n + t] = std::min(v[a], std::min(v[3 + a], v[6 + a]));
            hi[a * n + t] = std::max(v[a], std::max(v[3 + a], v[6 + a]));
        }
    DevBuf d_lo, d_hi, nodes_a, nodes_b, refs_a, refs_b, d_dec, d_sc, d_tot, d_children, d_split, d_final, d_err;
    VRG_CUDA(ctx, d_lo.reserve(4 * lo.size()));
    VRG_CUDA(ctx, d_hi.reserve(4 * hi.size()));
    VRG_CUDA(ctx, cudaMemcpyAsync(d_lo.ptr, lo.data(), 4 * lo.size(), cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(d_hi.ptr, hi.data(), 4 * hi.size(), cudaMemcpyHostToDevice, st));
    LNode root;
    for (int a = 0; a < 3; a++) {
        root.mn[a] = env->min_bound[a];
        root.mx[a] = env->max_bound[a];
    }
    root.out_id = 0;
    root.rbeg = 0;
    root.rcnt = (int32_t)n;
    std::vector<int32_t> all(n);
    for (int64_t t = 0; t < n; t++) all[t] = (int32_t)t;
    VRG_CUDA(ctx, grow_buf<LNode>(nodes_a, 1));
    VRG_CUDA(ctx, grow_buf<int32_t>(refs_a, n));
    VRG_CUDA(ctx, cudaMemcpyAsync(nodes_a.ptr, &root, sizeof root, cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(refs_a.ptr, all.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, st));
    VRG_CUDA(ctx, d_tot.reserve(3 * sizeof(int64_t)));
    VRG_CUDA(ctx, d_err.reserve(sizeof(int)));
    VRG_CUDA(ctx, cudaMemsetAsync(d_err.ptr, 0, sizeof(int), st));
    int64_t node_cap = 1024, final_cap = std::max<int64_t>(2 * n, 1024);
    VRG_CUDA(ctx, grow_buf<uint32_t>(d_children, node_cap));
    VRG_CUDA(ctx, grow_buf<float>(d_split, node_cap));
    VRG_CUDA(ctx, grow_buf<int32_t>(d_final, final_cap));
    int64_t m = 1, nodes_used = 1, final_refs = 0;
    DevBuf *cur_nodes = &nodes_a, *nxt_nodes = &nodes_b, *cur_refs = &refs_a, *nxt_refs = &refs_b;
    int level = 0;
    for (; m > 0; level++) {
        if (m >= ((int64_t)1 << 30)) return fail(ctx, VRG_ERR_UNSUPPORTED, "device kd build: level too wide");
        VRG_CUDA(ctx, grow_buf<LDec>(d_dec, m));
        VRG_CUDA(ctx, grow_buf<LScan>(d_sc, m));
        k_kd_choose<<<(unsigned)m, kBuildThreads, 0, st>>>(cur_nodes->as<LNode>(), cur_refs->as<int32_t>(),
                                                           d_lo.as<float>(), d_hi.as<float>(), n, level,
                                                           env->walk_costs, d_dec.as<LDec>());
        VRG_CUDA(ctx, cudaGetLastError());
        k_kd_scan<<<1, 1024, 0, st>>>(d_dec.as<LDec>(), cur_nodes->as<LNode>(), (int)m, d_sc.as<LScan>(),
                                      d_tot.as<int64_t>());
        VRG_CUDA(ctx, cudaGetLastError());
        int64_t tot[3];
        VRG_CUDA(ctx, cudaMemcpyAsync(tot, d_tot.ptr, sizeof tot, cudaMemcpyDeviceToHost, st));
        VRG_CUDA(ctx, cudaStreamSynchronize(st));
        const int64_t nsplit = tot[0], next_refs = tot[1], leaf_refs = tot[2];
        if (nodes_used + 2 * nsplit >= ((int64_t)1 << 27) || next_refs >= ((int64_t)1 << 31) ||
            final_refs + leaf_refs >= ((int64_t)1 << 30))
            return fail(ctx, VRG_ERR_UNSUPPORTED, "device kd build: tree too large");
        // grow the final arrays (keeping their contents) and the next level's
        if (nodes_used + 2 * nsplit > node_cap) {
            const int64_t cap = std::max(2 * node_cap, nodes_used + 2 * nsplit);
            DevBuf c2, s2;
            VRG_CUDA(ctx, grow_buf<uint32_t>(c2, cap));
            VRG_CUDA(ctx, grow_buf<float>(s2, cap));
            VRG_CUDA(ctx, cudaMemcpyAsync(c2.ptr, d_children.ptr, 4 * (size_t)nodes_used, cudaMemcpyDeviceToDevice, st));
            VRG_CUDA(ctx, cudaMemcpyAsync(s2.ptr, d_split.ptr, 4 * (size_t)nodes_used, cudaMemcpyDeviceToDevice, st));
            VRG_CUDA(ctx, cudaStreamSynchronize(st));
            std::swap(d_children.ptr, c2.ptr);
            std::swap(d_children.bytes, c2.bytes);
            std::swap(d_split.ptr, s2.ptr);
            std::swap(d_split.bytes, s2.bytes);
            node_cap = cap;
        }
        if (final_refs + leaf_refs > final_cap) {
            const int64_t cap = std::max(2 * final_cap, final_refs + leaf_refs);
            DevBuf f2;
            VRG_CUDA(ctx, grow_buf<int32_t>(f2, cap));
            VRG_CUDA(ctx, cudaMemcpyAsync(f2.ptr, d_final.ptr, 4 * (size_t)final_refs, cudaMemcpyDeviceToDevice, st));
            VRG_CUDA(ctx, cudaStreamSynchronize(st));
            std::swap(d_final.ptr, f2.ptr);
            std::swap(d_final.bytes, f2.bytes);
            final_cap = cap;
        }
        VRG_CUDA(ctx, grow_buf<LNode>(*nxt_nodes, 2 * nsplit));
        VRG_CUDA(ctx, grow_buf<int32_t>(*nxt_refs, next_refs));
        k_kd_write<<<(unsigned)m, kBuildThreads, 0, st>>>(
            cur_nodes->as<LNode>(), d_dec.as<LDec>(), d_sc.as<LScan>(), cur_refs->as<int32_t>(), d_lo.as<float>(),
            d_hi.as<float>(), n, (int32_t)nodes_used, final_refs, d_children.as<uint32_t>(), d_split.as<float>(),
            node_cap, nxt_nodes->as<LNode>(), std::max<int64_t>(2 * nsplit, 1), nxt_refs->as<int32_t>(),
            std::max<int64_t>(next_refs, 1), d_final.as<int32_t>(), final_cap, d_err.as<int>());
        VRG_CUDA(ctx, cudaGetLastError());
        nodes_used += 2 * nsplit;
        final_refs += leaf_refs;
        m = 2 * nsplit;
        std::swap(cur_nodes, nxt_nodes);
        std::swap(cur_refs, nxt_refs);
    }
    int err = 0;
    VRG_CUDA(ctx, cudaMemcpyAsync(&err, d_err.ptr, sizeof err, cudaMemcpyDeviceToHost, st));
    tree.children.resize(nodes_used);
    tree.split.resize(nodes_used);
    tree.refs.resize(final_refs);
    VRG_CUDA(ctx, cudaMemcpyAsync(tree.children.data(), d_children.ptr, 4 * (size_t)nodes_used, cudaMemcpyDeviceToHost, st));
    VRG_CUDA(ctx, cudaMemcpyAsync(tree.split.data(), d_split.ptr, 4 * (size_t)nodes_used, cudaMemcpyDeviceToHost, st));
    if (final_refs)
        VRG_CUDA(ctx, cudaMemcpyAsync(tree.refs.data(), d_final.ptr, 4 * (size_t)final_refs, cudaMemcpyDeviceToHost, st));
    VRG_CUDA(ctx, cudaStreamSynchronize(st));
    if (err) return fail(ctx, VRG_ERR_CUDA, "device kd build: an index left its buffer");
    tree.height = level;
    return VRG_OK;
}

}  // namespace vrg
