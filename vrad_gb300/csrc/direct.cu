// direct.cu -- direct-light gathering into luxels.  The reference leaves
// this stage out (RadWorld_Go is commented out at
// cmd/tasks/computerad/main.go:5-9); the light table it would read comes
// from rad/lightmap/lights.go:38-341 and the sky directions from
// vmath/constants.go:21-184.
#include <cstring>

#include "anorms_table.h"
#include "vrg_internal.h"
#include "vrg_trace.cuh"

namespace vrg {

__constant__ float c_anorms[kNumAnorms * 3] = VRG_ANORMS_INIT;

namespace {

constexpr int kThreads = 128;

// Device copy of a light: five 16-byte words.
struct alignas(16) DevLight {
    float4 origin;     // xyz, w = type (as int bits)
    float4 intensity;  // xyz, w = radius
    float4 normal;     // xyz, w = exponent
    float4 attn;       // constant, linear, quadratic, cap_distance
    float4 cone;       // stopdot, stopdot2, start_fade, end_fade
};

__device__ __forceinline__ uint64_t splitmix(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Irradiance at p with normal n, summed over the lights in table order.
// Point / spot: distance cull by radius, cosine at the receiver, falloff
// 1 / ((c + b*d) + a*d*d) with d capped at cap_distance, smoothstep fade
// between start_fade and end_fade, spot cone ramp and exponent, and a
// shadow line to the light.  Sky light: direction -normal.  Sky ambient:
// cosine-weighted fraction of the 162 directions whose line reaches sky.
__device__ void gather_point(const DevScene &s, const DevLight *__restrict__ lights, int nl,
                             float px, float py, float pz, float nx, float ny, float nz, float &r,
                             float &g, float &b, uint32_t &rays) {
    float ar = 0.0f, ag = 0.0f, ab = 0.0f;
    for (int li = 0; li < nl; li++) {
        const float4 lo = __ldg(&lights[li].origin);
        const int type = __float_as_int(lo.w);
        const float4 li_i = __ldg(&lights[li].intensity);
        if (type == VRG_EMIT_POINT || type == VRG_EMIT_SPOTLIGHT) {
            const float dlx = rsub(lo.x, px), dly = rsub(lo.y, py), dlz = rsub(lo.z, pz);
            const float dist2 = dot3r(dlx, dly, dlz, dlx, dly, dlz);
            const float radius = li_i.w;
            if (radius > 0.0f && dist2 > rmul(radius, radius)) continue;
            if (dist2 == 0.0f) continue;
            const float dist = rsqrt_rn(dist2);
            const float inv = rdiv(1.0f, dist);
            const float Lx = rmul(dlx, inv), Ly = rmul(dly, inv), Lz = rmul(dlz, inv);
            const float cosr = dot3r(nx, ny, nz, Lx, Ly, Lz);
            if (!(cosr > 0.0f)) continue;
            const float4 at = __ldg(&lights[li].attn);
            float dc = dist, dc2 = dist2;
            if (dist > at.w) {
                dc = at.w;
                dc2 = rmul(at.w, at.w);
            }
            const float denom = radd(radd(at.x, rmul(at.y, dc)), rmul(at.z, dc2));
            if (!(denom > 0.0f)) continue;
            float f = rdiv(1.0f, denom);
            const float4 cn = __ldg(&lights[li].cone);
            if (cn.w > cn.z && dist > cn.z) {
                if (dist >= cn.w) continue;
                const float sfr = rdiv(rsub(dist, cn.z), rsub(cn.w, cn.z));
                const float om = rsub(1.0f, sfr);
                f = rmul(f, rmul(rmul(om, om), radd(1.0f, rmul(2.0f, sfr))));
            }
            if (type == VRG_EMIT_SPOTLIGHT) {
                const float4 ln = __ldg(&lights[li].normal);
                const float dot2 = -dot3r(Lx, Ly, Lz, ln.x, ln.y, ln.z);
                if (!(dot2 > cn.y)) continue;
                if (dot2 < cn.x) f = rmul(f, rdiv(rsub(dot2, cn.y), rsub(cn.x, cn.y)));
                if (ln.w == 1.0f) f = rmul(f, dot2);
                else if (ln.w != 0.0f) f = rmul(f, powf(dot2, ln.w));
            }
            rays++;
            if (line_occluded(s, make_line(px, py, pz, lo.x, lo.y, lo.z), -1)) continue;
            const float sc = rmul(f, cosr);
            ar = radd(ar, rmul(li_i.x, sc));
            ag = radd(ag, rmul(li_i.y, sc));
            ab = radd(ab, rmul(li_i.z, sc));
        } else if (type == VRG_EMIT_SKYLIGHT) {
            const float4 ln = __ldg(&lights[li].normal);
            const float dx = -ln.x, dy = -ln.y, dz = -ln.z;
            const float cosr = dot3r(nx, ny, nz, dx, dy, dz);
            if (!(cosr > 0.0f)) continue;
            rays++;
            const Line L = make_line(px, py, pz, radd(px, rmul(dx, kMaxTraceLength)),
                                     radd(py, rmul(dy, kMaxTraceLength)),
                                     radd(pz, rmul(dz, kMaxTraceLength)));
            if (line_occluded(s, L, -1)) continue;
            ar = radd(ar, rmul(li_i.x, cosr));
            ag = radd(ag, rmul(li_i.y, cosr));
            ab = radd(ab, rmul(li_i.z, cosr));
        } else if (type == VRG_EMIT_SKYAMBIENT) {
            float sw = 0.0f, sv = 0.0f;
            for (int j = 0; j < kNumAnorms; j++) {
                const float ax = c_anorms[3 * j], ay = c_anorms[3 * j + 1], az = c_anorms[3 * j + 2];
                const float w = dot3r(nx, ny, nz, ax, ay, az);
                if (!(w > 0.0f)) continue;
                sw = radd(sw, w);
                rays++;
                const Line L = make_line(px, py, pz, radd(px, rmul(ax, kMaxTraceLength)),
                                         radd(py, rmul(ay, kMaxTraceLength)),
                                         radd(pz, rmul(az, kMaxTraceLength)));
                if (!line_occluded(s, L, -1)) sv = radd(sv, w);
            }
            if (sw > 0.0f) {
                const float fr = rdiv(sv, sw);
                ar = radd(ar, rmul(li_i.x, fr));
                ag = radd(ag, rmul(li_i.y, fr));
                ab = radd(ab, rmul(li_i.z, fr));
            }
        }
    }
    r = ar;
    g = ag;
    b = ab;
}

// Luxel supersample position: face f spans corner + U*su + V*sv; sample k of
// luxel (iu, iv) with global luxel index lux uses h = splitmix(seed, 4*lux+k),
// r1 = (h >> 40) * 2^-24, r2 = ((h >> 16) & 0xffffff) * 2^-24 and
// su = (iu + ((k & 1) + r1) * 0.5) * (1/nu), sv = (iv + ((k >> 1) + r2) * 0.5) * (1/nv)
// (S = 1: the luxel centre), then p = ((corner + U*su) + V*sv) + N*0.125.
__device__ __forceinline__ void luxel_sample(const FaceRec &f, int64_t lux, int iu, int iv, int k,
                                             int ss, uint64_t seed, float &px, float &py,
                                             float &pz) {
    const float inu = rdiv(1.0f, (float)f.nu), inv = rdiv(1.0f, (float)f.nv);
    float su, sv;
    if (ss == 4) {
        const uint64_t h = splitmix(seed, (uint64_t)(lux * 4 + k));
        const float r1 = rmul((float)(uint32_t)(h >> 40), 5.9604644775390625e-08f);
        const float r2 = rmul((float)(uint32_t)((h >> 16) & 0xffffffu), 5.9604644775390625e-08f);
        su = rmul(radd((float)iu, rmul(radd((float)(k & 1), r1), 0.5f)), inu);
        sv = rmul(radd((float)iv, rmul(radd((float)(k >> 1), r2), 0.5f)), inv);
    } else {
        su = rmul(radd((float)iu, 0.5f), inu);
        sv = rmul(radd((float)iv, 0.5f), inv);
    }
    px = radd(radd(radd(f.corner.x, rmul(f.u.x, su)), rmul(f.v.x, sv)), rmul(f.normal.x, kSampleOffset));
    py = radd(radd(radd(f.corner.y, rmul(f.u.y, su)), rmul(f.v.y, sv)), rmul(f.normal.y, kSampleOffset));
    pz = radd(radd(radd(f.corner.z, rmul(f.u.z, su)), rmul(f.v.z, sv)), rmul(f.normal.z, kSampleOffset));
}

__device__ __forceinline__ int find_face(const int64_t *__restrict__ off, int nfaces, int64_t lux) {
    int lo = 0, hi = nfaces - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= lux) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One thread per supersample; the S = 4 samples of a luxel sit in four
// neighbouring lanes and are summed in sample order by the first of them.
// Persistent warps take 32 samples at a time from work[0] (zeroed before
// the launch), so faces with many occluders do not leave SMs idle.
__global__ void __launch_bounds__(kThreads, 8) k_direct_luxels(
    DevScene s, const DevLight *__restrict__ lights, int nl, const FaceRec *__restrict__ faces,
    const int64_t *__restrict__ off, int nfaces, int64_t nlux, int ss, uint64_t seed,
    float *__restrict__ out, unsigned long long *__restrict__ ray_count,
    unsigned long long *__restrict__ work) {
    const int64_t nsamp = nlux * ss;
    const int lane = threadIdx.x & 31;
    uint32_t rays = 0;
    for (;;) {
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(work, 32ull);
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (wb >= (unsigned long long)nsamp) break;
        const int64_t gi = (int64_t)wb + lane;
        float r = 0.0f, g = 0.0f, b = 0.0f;
        int64_t lux = 0;
        if (gi < nsamp) {
            lux = gi / ss;
            const int k = (int)(gi - lux * ss);
            const int f = find_face(off, nfaces, lux);
            const FaceRec fr = faces[f];
            const int64_t local = lux - __ldg(off + f);
            const int iv = (int)(local / fr.nu), iu = (int)(local - (int64_t)iv * fr.nu);
            float px, py, pz;
            luxel_sample(fr, lux, iu, iv, k, ss, seed, px, py, pz);
            gather_point(s, lights, nl, px, py, pz, fr.normal.x, fr.normal.y, fr.normal.z, r, g, b, rays);
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
            gather_point(s, lights, nl, __ldg(pts + 3 * i), __ldg(pts + 3 * i + 1), __ldg(pts + 3 * i + 2),
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

int launch_gather_luxels(vrg_env *env, int ss, uint64_t seed, float *out_rgb,
                         unsigned long long *d_rays) {
    vrg_ctx *ctx = env->ctx;
    const int64_t nlux = env->luxel_offset.empty() ? 0 : env->luxel_offset.back();
    if (nlux == 0) return VRG_OK;
    VRG_CUDA(ctx, env->d_work.reserve(256));
    unsigned long long *work = env->d_work.as<unsigned long long>() + 1;
    VRG_CUDA(ctx, cudaMemsetAsync(work, 0, 8, ctx->stream));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_direct_luxels, kThreads, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 4;
    const int64_t need = (nlux * ss + kThreads - 1) / kThreads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)ctx->num_sms * per_sm));
    cudaEvent_t ev = nullptr;
    timing_begin(ctx, "direct_luxels", &ev);
    k_direct_luxels<<<grid, kThreads, 0, ctx->stream>>>(
        scene_view(env), env->d_lights.as<DevLight>(), (int)env->lights.size(),
        env->d_faces.as<FaceRec>(), env->d_luxel_offset.as<int64_t>(), env->nfaces, nlux, ss, seed,
        out_rgb, d_rays, work);
    VRG_CUDA(ctx, cudaGetLastError());
    timing_end(ctx, "direct_luxels", ev);
    return VRG_OK;
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
