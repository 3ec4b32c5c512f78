// lightmap.cu -- the lightmap samples of a baked scene.  The reference stops
// before this step: its face extents are computed and then lost
// (rad/world/face.go:14-90, rad/start.go:102-112), its write-out is a stub
// (cmd/tasks/finish/main.go:8-40) and its one call of the sample encoder is a
// line of C++ left in a Go file (compute/leafambient/lighting.go:67).  The
// project's stage:
//   per luxel (face order, row-major nu x nv), light = the luxel's direct
//   light from the last bake + the bounced light (TotalLight,
//   common/types/patch.go:33) of the leaf patch holding the luxel centre
//   (centre + 0.125 N as the gather places it; the face's patch tree is
//   descended with coordinate >= dist -> child1, as the transfer rows do);
//   each light is stored as one 4-byte shared-exponent sample.
//
// Sample encoding (Ward's RGBE, "Real Pixels", Graphics Gems II, with the
// exponent kept as a signed byte -- the r, g, b, exponent layout of the
// lightmap samples Source's ColorRGBExp32 names):
//   channel c -> 0 when c is not > 0 (negatives, NaN), FLT_MAX when +inf;
//   m = largest channel; a zero m gives the all-zero sample; otherwise
//   e = the exponent of m = f * 2^e, 0.5 <= f < 1, x = max(e - 8, -128),
//   byte = floor(c * 2^-x) (<= 255, the largest channel in [128, 255] unless
//   x was clamped), exponent byte = x as int8; decoded c' = byte * 2^x, so
//   0 <= c - c' < 2^x <= m / 128.
// Everything past the float additions is integer work on the bit patterns,
// so the floor is exact and the sample has one answer.
#include <algorithm>

#include "vrg_gather.cuh"
#include "vrg_internal.h"

namespace vrg {

namespace {

constexpr int kThreads = 128;

// Bit pattern of a channel after the clamp to [0, FLT_MAX].
__device__ __forceinline__ uint32_t channel_bits(float c) {
    if (!(c > 0.0f)) return 0u;
    const uint32_t b = __float_as_uint(c);
    return b >= 0x7f800000u ? 0x7f7fffffu : b;
}

// floor(c * 2^-x) for a clamped channel's bits; c <= m keeps it below 256,
// so the shift below is at least 16.
__device__ __forceinline__ uint32_t channel_byte(uint32_t bits, int x) {
    const uint32_t be = bits >> 23;
    const uint32_t mant = (bits & 0x7fffffu) | (be ? 0x800000u : 0u);
    const int sh = x + 150 - (int)(be ? be : 1u);  // c = mant * 2^(-sh + x)
    if (sh <= 0) return 255u;
    if (sh >= 32) return 0u;
    return min(mant >> sh, 255u);
}

__device__ __forceinline__ uint32_t encode_sample(float r, float g, float b) {
    const uint32_t br = channel_bits(r), bg = channel_bits(g), bb = channel_bits(b);
    const uint32_t bm = max(br, max(bg, bb));  // order of non-negative floats
    if (bm == 0u) return 0u;
    const int be = (int)(bm >> 23);
    const int x = be ? max(be - 134, -128) : -128;  // e = be - 126 for a normal m
    return channel_byte(br, x) | (channel_byte(bg, x) << 8) | (channel_byte(bb, x) << 16) |
           ((uint32_t)(uint8_t)(int8_t)x << 24);
}

// A face's patch tree and its leaves' bounced light in shared memory: the
// root and up to kLmNodes - 1 nodes below it, up to kLmLeaves leaves.
constexpr int kLmNodes = 256;
constexpr int kLmLeaves = 128;

// One block per face, faces taken in order from a work counter (zeroed
// before the launch), so that the blocks that draw large faces do not set
// the tail as a static stride over faces did.  Every thread reads the same
// face record (one broadcast); the block copies the face's patch tree and
// its leaves' totals (face_tree: first node below the root, their count,
// first leaf, leaf count) into shared memory with coalesced loads, so that
// each luxel's descent is a chain of shared loads instead of dependent
// global ones; the threads then take the face's luxels in order (coalesced
// 12-byte reads and 4-byte writes).  A face whose tree does not fit, or
// whose ranges the host could not vouch for, is walked in global memory.
// No luxel -> face search.
__global__ void __launch_bounds__(kThreads) k_lightmap(
    const FaceRec *__restrict__ faces, const int64_t *__restrict__ off, int nfaces,
    const float *__restrict__ rgb, const float4 *__restrict__ total, const PatchNode *__restrict__ pnodes,
    const int32_t *__restrict__ face_root, const int4 *__restrict__ face_tree, uint32_t *__restrict__ out,
    unsigned int *__restrict__ work) {
    __shared__ int face_sh;
    __shared__ PatchNode sn[kLmNodes];
    __shared__ float4 sl[kLmLeaves];
    for (;;) {
        __syncthreads();  // every thread is done with the previous face
        if (threadIdx.x == 0) face_sh = (int)atomicAdd(work, 1u);
        __syncthreads();
        const int f = face_sh;
        if (f >= nfaces) break;
        const FaceRec fr = faces[f];
        const int64_t base = __ldg(off + f);
        const int64_t n = __ldg(off + f + 1) - base;
        const int32_t root = __ldg(face_root + f);
        const int4 ft = __ldg(face_tree + f);
        const bool staged = root >= 0 && ft.x >= 0 && ft.y < kLmNodes && ft.z >= 0 && ft.w >= 1 &&
                            ft.w <= kLmLeaves;
        if (staged) {  // block-uniform
            for (int i = threadIdx.x; i <= ft.y; i += blockDim.x) sn[i] = pnodes[i == 0 ? root : ft.x + i - 1];
            for (int i = threadIdx.x; i < ft.w; i += blockDim.x) sl[i] = total[ft.z + i];
        }
        __syncthreads();
        // the luxel centres as luxel_sample places them (one sample, no
        // jitter), with the face's reciprocals taken once
        const float inu = rrcp((float)fr.nu), inv = rrcp((float)fr.nv);
        for (int64_t local = threadIdx.x; local < n; local += blockDim.x) {
            const int64_t lux = base + local;
            int iv, iu;
            if (n <= INT32_MAX) {  // block-uniform: 32-bit division
                iv = (int)local / fr.nu;
                iu = (int)local - iv * fr.nu;
            } else {
                iv = (int)(local / fr.nu);
                iu = (int)(local - (int64_t)iv * fr.nu);
            }
            float r = __ldg(rgb + 3 * lux), g = __ldg(rgb + 3 * lux + 1), b = __ldg(rgb + 3 * lux + 2);
            if (root >= 0) {
                const float su = rmul(radd((float)iu, 0.5f), inu), sv = rmul(radd((float)iv, 0.5f), inv);
                const float px = radd(radd(radd(fr.corner.x, rmul(fr.u.x, su)), rmul(fr.v.x, sv)),
                                      rmul(fr.normal.x, kSampleOffset));
                const float py = radd(radd(radd(fr.corner.y, rmul(fr.u.y, su)), rmul(fr.v.y, sv)),
                                      rmul(fr.normal.y, kSampleOffset));
                const float pz = radd(radd(radd(fr.corner.z, rmul(fr.u.z, su)), rmul(fr.v.z, sv)),
                                      rmul(fr.normal.z, kSampleOffset));
                float4 t;
                if (staged) {
                    PatchNode pn = sn[0];
                    while (pn.axis >= 0)
                        pn = sn[1 + (pick3(pn.axis, px, py, pz) >= pn.dist ? pn.child1 : pn.child2) - ft.x];
                    t = sl[pn.leaf - ft.z];
                } else {
                    PatchNode pn = pnodes[root];
                    while (pn.axis >= 0) pn = pnodes[pick3(pn.axis, px, py, pz) >= pn.dist ? pn.child1 : pn.child2];
                    t = total[pn.leaf];
                }
                r = radd(r, t.x);
                g = radd(g, t.y);
                b = radd(b, t.z);
            }
            out[lux] = encode_sample(r, g, b);
        }
    }
}

}  // namespace

}  // namespace vrg

using namespace vrg;

extern "C" {

int vrg_env_get_lightmap(vrg_env *env, uint8_t *samples, int64_t *face_offset) {
    if (!env) return VRG_ERR_INVALID;
    vrg_ctx *ctx = env->ctx;
    std::lock_guard<std::mutex> lk(env->mu);
    if (!env->have_bake || !env->have_patches)
        return fail(ctx, VRG_ERR_STATE, "no bake of the current faces and patches has run on this scene");
    const int64_t nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    if (face_offset)
        for (int32_t f = 0; f <= env->nfaces; f++) face_offset[f] = 4 * env->luxel_offset[f];
    if (!samples || nlux == 0) return VRG_OK;
    cudaStream_t st = ctx->stream;
    VRG_CUDA(ctx, env->d_out0.reserve(4 * (size_t)nlux));
    VRG_CUDA(ctx, env->d_work.reserve(256));
    // the face counter sits in the scene's work-counter block, apart from the
    // words the gathers use
    unsigned int *work = reinterpret_cast<unsigned int *>(env->d_work.as<char>() + 128);
    VRG_CUDA(ctx, cudaMemsetAsync(work, 0, sizeof(unsigned int), st));
    const int grid = (int)std::min<int64_t>(env->nfaces, (int64_t)ctx->num_sms * 16);
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "lightmap", &ev);
    k_lightmap<<<grid, kThreads, 0, st>>>(env->d_faces.as<FaceRec>(), env->d_luxel_offset.as<int64_t>(),
                                         env->nfaces, env->d_bake_rgb.as<float>(),
                                         env->d_total.as<float4>(), env->d_patch_nodes.as<PatchNode>(),
                                         env->d_face_root.as<int32_t>(), env->d_face_tree.as<int4>(),
                                         env->d_out0.as<uint32_t>(), work);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "lightmap", ev);
    VRG_CUDA(ctx, cudaMemcpyAsync(samples, env->d_out0.ptr, 4 * (size_t)nlux, cudaMemcpyDeviceToHost, st));
    VRG_CUDA(ctx, cudaStreamSynchronize(st));
    return VRG_OK;
}

}  // extern "C"
