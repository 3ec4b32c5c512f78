// vrg_gather.cuh -- direct-light evaluation at one sample point, shared by the
// single-scene and batched gather kernels.
#pragma once

#include <cstdint>

#include "../../include/vradgpu.h"
#include "anorms_table.h"
#include "vrg_device.h"
#include "vrg_trace.cuh"

namespace vrg {

// The 162 sky directions (one copy per translation unit).
static __constant__ float c_anorms[kNumAnorms * 3] = VRG_ANORMS_INIT;




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
//
// SKY selects what happens to the sky-type lights (sky light, sky ambient),
// which do not depend on any light position: 0 traces them; 1 traces them
// and stores each one's multiplier (cosine or visible fraction, -1 when it
// adds nothing) in sky[0..]; 2 reads those multipliers instead of tracing.
// With a visibility cache vis (one bit per light, bit li of word li/32),
// mode 1 also stores whether each traced point/spot shadow line reached its
// light, and mode 2 traces only the lights flagged in `edited` (refreshing
// their bits) and takes every other light's visibility from the cache.
// The accumulation order and arithmetic are the same in all modes, so a
// relight that re-traces only edited lights is bit-identical to a full
// gather with the edited table.
enum SkyMode { kSkyTrace = 0, kSkyWrite = 1, kSkyRead = 2 };

template <int SKY, int OPT = 0, int WM = kWallAny>
static __device__ void gather_point(const DevScene &s, const DevLight *__restrict__ lights, int nl,
                                    float px, float py, float pz, float nx, float ny, float nz,
                                    float &r, float &g, float &b, uint32_t &rays,
                                    float *__restrict__ sky = nullptr, uint32_t *__restrict__ vis = nullptr,
                                    const uint32_t *__restrict__ edited = nullptr) {
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
            const float inv = rrcp(dist);
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
            float f = rrcp(denom);
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
            bool occ;
            const uint32_t bit = 1u << (li & 31);
            if (SKY == kSkyRead && vis && !(__ldg(edited + (li >> 5)) & bit)) {
                occ = !(vis[li >> 5] & bit);
            } else {
                rays++;
                occ = line_occluded<OPT, WM>(s, make_line(px, py, pz, lo.x, lo.y, lo.z), -1);
                if (SKY != kSkyTrace && vis) {
                    if (occ) vis[li >> 5] &= ~bit;
                    else vis[li >> 5] |= bit;
                }
            }
            if (occ) continue;
            const float sc = rmul(f, cosr);
            ar = radd(ar, rmul(li_i.x, sc));
            ag = radd(ag, rmul(li_i.y, sc));
            ab = radd(ab, rmul(li_i.z, sc));
        } else if (type == VRG_EMIT_SKYLIGHT || type == VRG_EMIT_SKYAMBIENT) {
            float m = -1.0f;  // multiplier of the intensity; -1: adds nothing
            if (SKY == kSkyRead) {
                m = *sky++;
            } else if (type == VRG_EMIT_SKYLIGHT) {
                const float4 ln = __ldg(&lights[li].normal);
                const float dx = -ln.x, dy = -ln.y, dz = -ln.z;
                const float cosr = dot3r(nx, ny, nz, dx, dy, dz);
                if (cosr > 0.0f) {
                    rays++;
                    const Line L = make_line(px, py, pz, radd(px, rmul(dx, kMaxTraceLength)),
                                             radd(py, rmul(dy, kMaxTraceLength)),
                                             radd(pz, rmul(dz, kMaxTraceLength)));
                    if (!line_occluded<OPT, WM>(s, L, -1)) m = cosr;
                }
            } else {
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
                    if (!line_occluded<OPT, WM>(s, L, -1)) sv = radd(sv, w);
                }
                if (sw > 0.0f) m = rdiv(sv, sw);
            }
            if (SKY == kSkyWrite) *sky++ = m;
            if (m >= 0.0f) {
                ar = radd(ar, rmul(li_i.x, m));
                ag = radd(ag, rmul(li_i.y, m));
                ab = radd(ab, rmul(li_i.z, m));
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
    const float inu = rrcp((float)f.nu), inv = rrcp((float)f.nv);
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

// Walk order of a face's luxels in 4 x 2 tiles: ordinal o (0 .. nu*nv-1)
// -> (iu, iv), tiles left to right within bands of two rows (one row in the
// last band of a face with odd nv), the last tile of a band narrower when
// nu is not a multiple of 4.  A bijection, so every luxel is visited once;
// a warp's 8 consecutive luxels then cover a 64 x 32-unit patch of the face
// instead of a 128-unit strip, and its lanes' shadow lines stay together
// longer.
__device__ __forceinline__ void tile_luxel(int64_t o, int nu, int nv, int &iu, int &iv) {
    const int band = (int)(o / (2 * (int64_t)nu));
    const int h = (2 * band + 1 < nv) ? 2 : 1;
    const int r = (int)(o - (int64_t)band * 2 * nu);
    const int c = r / (4 * h);
    const int q = r - c * 4 * h;
    const int w = min(4, nu - 4 * c);
    iu = 4 * c + q % w;
    iv = 2 * band + q / w;
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

}  // namespace vrg
