// direct.cu -- direct-light gathering into luxels.  The reference leaves
// this stage out (RadWorld_Go is commented out at
// cmd/tasks/computerad/main.go:5-9); the light table it would read comes
// from rad/lightmap/lights.go:38-341 and the sky directions from
// vmath/constants.go:21-184.
#include <cstring>

#include "anorms_table.h"
#include "vrg_internal.h"
#include "vrg_trace.cuh"

#include "vrg_gather.cuh"

namespace vrg {

namespace {

constexpr int kThreads = 128;
static_assert(kThreads <= kShRayLanes, "kOptShRay keeps one slot per thread of a block");


// One thread per supersample; the S = 4 samples of a luxel sit in four
// neighbouring lanes and are summed in sample order by the first of them.
// Persistent warps take FETCH samples at a time from work[0] (zeroed before
// the launch), so faces with many occluders do not leave SMs idle; larger
// claims mean fewer atomics, smaller ones a shorter tail.
// Optional second segment: npts sample points (pts, nrm: 3 floats each)
// after the luxel samples, written to pout -- the leaf-patch points of a
// bake, which alone are too few to fill the GPU.
// TILE walks each face's luxels in 4 x 2 tiles (tile_luxel) instead of row
// order; the output is the same, each luxel written by the lane holding its
// first sample.  WM is the scene's wall layout (slots or cells).
template <int FETCH, int OPT = 0, bool TILE = false, int WM = kWallSlotsOnly, int MINB = 8>
__global__ void __launch_bounds__(kThreads, MINB) k_direct_luxels(
    DevScene s, const DevLight *__restrict__ lights, int nl, const FaceRec *__restrict__ faces,
    const int64_t *__restrict__ off, int nfaces, int64_t nlux, int ss, uint64_t seed,
    float *__restrict__ out, const float *__restrict__ pts, const float *__restrict__ nrm, int64_t npts,
    float *__restrict__ pout, unsigned long long *__restrict__ ray_count,
    unsigned long long *__restrict__ work) {
    if (OPT & kOptTop) stage_top(s);
    const int64_t nsamp = nlux * ss;
    const int64_t total = nsamp + npts;
    const int lane = threadIdx.x & 31;
    uint32_t rays = 0;
    for (;;) {
        unsigned long long wb0 = 0;
        if (lane == 0) wb0 = atomicAdd(work, (unsigned long long)FETCH);
        wb0 = __shfl_sync(0xffffffffu, wb0, 0);
        if (wb0 >= (unsigned long long)total) break;
        for (int sub = 0; sub < FETCH; sub += 32) {
        const unsigned long long wb = wb0 + sub;
        if (wb >= (unsigned long long)total) break;
        const int64_t gi = (int64_t)wb + lane;
        float r = 0.0f, g = 0.0f, b = 0.0f;
        int64_t lux = 0;
        // one sample point per lane: a luxel supersample or an extra point;
        // a single gather_point call site keeps the kernel's code compact
        float px = 0.0f, py = 0.0f, pz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f;
        const bool is_pt = gi >= nsamp && gi < total;
        if (is_pt) {
            const int64_t i = gi - nsamp;
            px = __ldg(pts + 3 * i);
            py = __ldg(pts + 3 * i + 1);
            pz = __ldg(pts + 3 * i + 2);
            nx = __ldg(nrm + 3 * i);
            ny = __ldg(nrm + 3 * i + 1);
            nz = __ldg(nrm + 3 * i + 2);
        } else if (gi < nsamp) {
            lux = gi / ss;
            const int k = (int)(gi - lux * ss);
            const int f = find_face(off, nfaces, lux);
            const FaceRec fr = faces[f];
            int64_t local = lux - __ldg(off + f);
            int iv, iu;
            if (TILE) {
                tile_luxel(local, fr.nu, fr.nv, iu, iv);
                local = (int64_t)iv * fr.nu + iu;
                lux = __ldg(off + f) + local;
            } else {
                iv = (int)(local / fr.nu);
                iu = (int)(local - (int64_t)iv * fr.nu);
            }
            luxel_sample(fr, lux, iu, iv, k, ss, seed, px, py, pz);
            nx = fr.normal.x;
            ny = fr.normal.y;
            nz = fr.normal.z;
        }
        if (gi < total) gather_point<kSkyTrace, OPT, WM>(s, lights, nl, px, py, pz, nx, ny, nz, r, g, b, rays);
        if (is_pt) {
            const int64_t i = gi - nsamp;
            pout[3 * i] = r;
            pout[3 * i + 1] = g;
            pout[3 * i + 2] = b;
        }
        if (ss == 4) {
            const float r1 = __shfl_down_sync(0xffffffffu, r, 1), r2 = __shfl_down_sync(0xffffffffu, r, 2), r3 = __shfl_down_sync(0xffffffffu, r, 3);
            const float g1 = __shfl_down_sync(0xffffffffu, g, 1), g2 = __shfl_down_sync(0xffffffffu, g, 2), g3 = __shfl_down_sync(0xffffffffu, g, 3);
            const float b1 = __shfl_down_sync(0xffffffffu, b, 1), b2 = __shfl_down_sync(0xffffffffu, b, 2), b3 = __shfl_down_sync(0xffffffffu, b, 3);
            if (gi < nsamp && (lane & 3) == 0) {
                out[3 * lux + 0] = rmul(radd(radd(radd(r, r1), r2), r3), 0.25f);
                out[3 * lux + 1] = rmul(radd(radd(radd(g, g1), g2), g3), 0.25f);
                out[3 * lux + 2] = rmul(radd(radd(radd(b, b1), b2), b3), 0.25f);
            }
        } else if (gi < nsamp) {
            out[3 * lux + 0] = r;
            out[3 * lux + 1] = g;
            out[3 * lux + 2] = b;
        }
        }
    }
    // one atomic per warp
    unsigned long long w = rays;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && ray_count) atomicAdd(ray_count, w);
}

__global__ void __launch_bounds__(kThreads, 8) k_direct_points(
    DevScene s, const DevLight *__restrict__ lights, int nl, const float *__restrict__ pts,
    const float *__restrict__ nrm, int64_t n, float *__restrict__ out,
    unsigned long long *__restrict__ ray_count) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    uint32_t rays = 0;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        if (i < n) {
            float r, g, b;
            gather_point<kSkyTrace>(s, lights, nl, __ldg(pts + 3 * i), __ldg(pts + 3 * i + 1), __ldg(pts + 3 * i + 2),
                         __ldg(nrm + 3 * i), __ldg(nrm + 3 * i + 1), __ldg(nrm + 3 * i + 2), r, g, b, rays);
            out[3 * i] = r;
            out[3 * i + 1] = g;
            out[3 * i + 2] = b;
        }
    }
    unsigned long long w = rays;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && ray_count) atomicAdd(ray_count, w);
}

int grid_for(const vrg_ctx *ctx, int64_t n) {
    int64_t blocks = (n + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

}  // namespace

// Packs the host light table into the device layout.
void pack_lights(const std::vector<vrg_light> &src, std::vector<float4> &dst) {
    dst.resize(src.size() * 5);
    for (size_t i = 0; i < src.size(); i++) {
        const vrg_light &l = src[i];
        float tbits;
        int32_t t = l.type;
        memcpy(&tbits, &t, 4);
        dst[5 * i + 0] = make_float4(l.origin[0], l.origin[1], l.origin[2], tbits);
        dst[5 * i + 1] = make_float4(l.intensity[0], l.intensity[1], l.intensity[2], l.radius);
        dst[5 * i + 2] = make_float4(l.normal[0], l.normal[1], l.normal[2], l.exponent);
        dst[5 * i + 3] = make_float4(l.constant_attn, l.linear_attn, l.quadratic_attn, l.cap_distance);
        dst[5 * i + 4] = make_float4(l.stopdot, l.stopdot2, l.start_fade, l.end_fade);
    }
}

// A persistent launch of kernel k: one wave of the blocks k keeps resident
// per SM, or fewer when the work is small.
template <class K>
void launch_direct(K k, int64_t need, int sms, cudaStream_t st, const DevScene &s, const DevLight *lights, int nl,
                   const vrg_env *env, int64_t nlux, int ss, uint64_t seed, float *out_rgb, const float *pts,
                   const float *nrm, int64_t npts, float *pts_out, unsigned long long *d_rays,
                   unsigned long long *work) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 4;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * per_sm));
    k<<<grid, kThreads, 0, st>>>(s, lights, nl, env->d_faces.as<FaceRec>(), env->d_luxel_offset.as<int64_t>(),
                                 env->nfaces, nlux, ss, seed, out_rgb, pts, nrm, npts, pts_out, d_rays, work);
}

// The twelve tuned variants of k_direct_luxels for wall layout WM: samples
// claimed per warp (32, 64, 128), 32 with the leaf records kept out of L1,
// 32 in 4 x 2 luxel tiles without and with the top of the tree in shared
// memory, in tiles skipping children without triangles, in tiles with the
// walk constants in shared memory at 8, 9 or 10 resident blocks per SM (64,
// 56 or 48 registers), in plain tiles at 9 blocks, and in tiles with the
// walk constants and the top of the tree in shared memory at 9 blocks.
template <int WM>
void launch_direct_variant(int v, int64_t need, int sms, cudaStream_t st, const DevScene &s,
                           const DevLight *lights, int nl, const vrg_env *env, int64_t nlux, int ss,
                           uint64_t seed, float *out_rgb, const float *pts, const float *nrm, int64_t npts,
                           float *pts_out, unsigned long long *d_rays, unsigned long long *work) {
#define VRG_DIRECT(...) \
    launch_direct(k_direct_luxels<__VA_ARGS__>, need, sms, st, s, lights, nl, env, nlux, ss, seed, out_rgb, pts, \
                  nrm, npts, pts_out, d_rays, work)
    switch (v) {
    case 0: VRG_DIRECT(32, 0, false, WM); break;
    case 1: VRG_DIRECT(64, 0, false, WM); break;
    case 2: VRG_DIRECT(128, 0, false, WM); break;
    case 3: VRG_DIRECT(32, kOptStream, false, WM); break;
    case 4: VRG_DIRECT(32, 0, true, WM); break;
    case 5: VRG_DIRECT(32, kOptTop, true, WM); break;
    case 6: VRG_DIRECT(32, kOptSkip, true, WM); break;
    case 7: VRG_DIRECT(32, kOptShRay, true, WM); break;
    case 8: VRG_DIRECT(32, kOptShRay, true, WM, 9); break;
    case 9: VRG_DIRECT(32, kOptShRay, true, WM, 10); break;
    case 10: VRG_DIRECT(32, 0, true, WM, 9); break;
    default: VRG_DIRECT(32, kOptShRay | kOptTop, true, WM, 9); break;
    }
#undef VRG_DIRECT
}

int launch_gather_luxels(vrg_env *env, int ss, uint64_t seed, float *out_rgb,
                         unsigned long long *d_rays, const float *pts, const float *nrm, int64_t npts,
                         float *pts_out) {
    vrg_ctx *ctx = env->ctx;
    const int64_t nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    if (nlux == 0 && npts == 0) return VRG_OK;
    VRG_CUDA(ctx, env->d_work.reserve(256));
    unsigned long long *work = env->d_work.as<unsigned long long>() + 1;
    const int64_t need = (nlux * ss + npts + kThreads - 1) / kThreads;
    const DevScene s = scene_view(env);
    const DevLight *lights = env->d_lights.as<DevLight>();
    const int nl = (int)env->lights.size();
    // the variants of launch_direct_variant, picked per bucket, built for the
    // scene's wall layout
    auto launch = [&](int v) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(work, 0, 8, ctx->stream);
        if (e == cudaSuccess && d_rays) e = cudaMemsetAsync(d_rays, 0, 8, ctx->stream);
        if (e != cudaSuccess) return e;
        cudaEvent_t ev = nullptr;
        timing_begin(ctx, "direct_luxels", &ev);
        if (env->wall_layout == 0)
            launch_direct_variant<kWallSlotsOnly>(v, need, ctx->num_sms, ctx->stream, s, lights, nl, env, nlux, ss,
                                                  seed, out_rgb, pts, nrm, npts, pts_out, d_rays, work);
        else
            launch_direct_variant<kWallCellsOnly>(v, need, ctx->num_sms, ctx->stream, s, lights, nl, env, nlux, ss,
                                                  seed, out_rgb, pts, nrm, npts, pts_out, d_rays, work);
        e = cudaGetLastError();
        timing_end(ctx, "direct_luxels", ev);
        return e;
    };
    return tune_run(ctx, tune_key("direct_luxels", env->geom.ntris, nlux * ss + npts), 12, launch);
}

int launch_gather_points(vrg_env *env, const float *pts, const float *nrm, int64_t n,
                         float *out_rgb, unsigned long long *d_rays) {
    vrg_ctx *ctx = env->ctx;
    if (n <= 0) return VRG_OK;
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "direct_points", &ev);
    k_direct_points<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(
        scene_view(env), env->d_lights.as<DevLight>(), (int)env->lights.size(), pts, nrm, n,
        out_rgb, d_rays);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "direct_points", ev);
    return VRG_OK;
}

}  // namespace vrg
