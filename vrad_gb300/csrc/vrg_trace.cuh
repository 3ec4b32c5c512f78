// vrg_trace.cuh -- kd-tree traversal and shadow-line visibility on the device.
//
// Every float operation on the bit-exact path (the ray/triangle test, the
// shadow-line setup) goes through the __f*_rn intrinsics, which are never
// fused into FMAs whatever the compiler flags, so results match the float32
// CPU restatement bit for bit.  The slab walk that only decides which leaves
// to visit uses faster approximate arithmetic inside a conservative margin.
#pragma once

#include <cuda_runtime.h>

#include "vrg_device.h"

namespace vrg {

__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
// 1 / b rounded to nearest: the same float as rdiv(1.0f, b) (both are the
// correctly rounded quotient), with a shorter instruction sequence
__device__ __forceinline__ float rrcp(float b) { return __frcp_rn(b); }
__device__ __forceinline__ float rsqrt_rn(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ float dot3r(float ax, float ay, float az, float bx, float by, float bz) {
    return radd(radd(rmul(ax, bx), rmul(ay, by)), rmul(az, bz));
}
__device__ __forceinline__ float pick3(int a, float x, float y, float z) {
    return a == 0 ? x : (a == 1 ? y : z);
}

constexpr int32_t kTraceIdSky = 0x01000000;

// Walk options (template bits): kOptStream loads leaf records without
// allocating in L1; kOptTop reads the top levels of the tree from a copy in
// shared memory (stage_top).
constexpr int kOptStream = 1;
constexpr int kOptTop = 2;
constexpr int kOptPipe = 8;    // unit rounds: the next triangle's plane loads during this test
constexpr int kOptSkip = 16;   // children flagged as leaves without triangles are not visited
// kOptShRay: the walk constants of each lane's ray are kept in shared memory,
// one float4 (inv, A, B, neg) per axis and lane, and an inner step reads its
// axis's with one load instead of selecting three of nine registers.  For
// blocks of at most kShRayLanes threads.
constexpr int kOptShRay = 32;
constexpr int kShRayLanes = 128;
// kOptOneVote (unit-round walks): the idle lanes follow from the busy ballot
// and a warp-wide mask of the lanes out of work, one ballot per round
// instead of two.
constexpr int kOptOneVote = 64;

// Shared-memory copy of the scene's top table, for kernels walking with
// kOptTop (allocated only in kernels that use it).
static __shared__ uint2 g_top_nodes[kTopNodes];

// Per-lane copy of the walk constants for kOptShRay (allocated only in kernels
// that use it).
static __shared__ float4 g_ray_axes[3 * kShRayLanes];

// Every thread of the block calls this once, before its first walk.
__device__ __forceinline__ void stage_top(const DevScene &s) {
    for (uint32_t i = threadIdx.x; i < s.ntop; i += blockDim.x) g_top_nodes[i] = __ldg(&s.top[i]);
    __syncthreads();
}

// The node a walk starts from, and a node record by reference: with kOptTop
// a reference carrying kTopRef is read from the shared copy.
template <int OPT>
__device__ __forceinline__ uint32_t root_ref(const DevScene &s) {
    return ((OPT & kOptTop) && s.ntop > 0) ? kTopRef : 0u;
}

template <int OPT>
__device__ __forceinline__ uint2 fetch_node(const DevScene &s, uint32_t ref) {
    if ((OPT & kOptTop) && (ref & kTopRef)) return g_top_nodes[ref & (kTopRef - 1u)];
    return __ldg(&s.nodes[ref]);
}
constexpr float kInf = __builtin_huge_valf();

// Conservative slab half-thickness for split planes: a computed hit lies
// within a few float32 roundings of its triangle, and treating each split
// plane as a slab 2^-17 * (scale + |origin| + 1) thick guarantees that no
// leaf holding such a triangle is skipped.
__device__ __forceinline__ float ray_slack(const SceneGeom &g, float ox, float oy, float oz) {
    float om = fmaxf(fabsf(ox), fmaxf(fabsf(oy), fabsf(oz)));
    return rmul(7.62939453125e-06f, radd(radd(g.scale, om), 1.0f));
}

// Approximate reciprocal for traversal decisions only.  A zero or tiny
// direction component is replaced by +-1e-30 first, so the result is finite
// and the slab arithmetic below never forms inf - inf.
__device__ __forceinline__ float trav_rcp(float d) {
    float dd = fabsf(d) < 1e-30f ? copysignf(1e-30f, d) : d;
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(dd));
    return r;
}

struct Ray {
    float ox, oy, oz, dx, dy, dz;
};

// Per-ray constants of the slab walk.  For axis a with the ray moving
// toward +a (neg = 0) the near child is the left one; a split plane s is
// treated as the slab [s - slack, s + slack]:
//   near child exits at  t = (s + sd - o) / d = fma(s, inv, A)
//   far child enters at  t = (s - sd - o) / d = fma(s, inv, B)
// with sd = +-slack toward the far side.  The rounding of these forms moves
// a crossing by about 2^-22 * (|s| + |o|) along the axis, far inside the
// slack, so the walk stays conservative.
struct RayPre {
    float inv[3], A[3], B[3];
    uint32_t neg;  // bit a set when the direction's a component is negative
};

__device__ __forceinline__ RayPre ray_pre(const Ray &ray, float slack) {
    RayPre r;
    const float o[3] = {ray.ox, ray.oy, ray.oz}, d[3] = {ray.dx, ray.dy, ray.dz};
    r.neg = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool neg = signbit(d[a]);
        r.neg |= (neg ? 1u : 0u) << a;
        r.inv[a] = trav_rcp(d[a]);
        const float sd = neg ? -slack : slack;
        r.A[a] = (sd - o[a]) * r.inv[a];
        r.B[a] = (-sd - o[a]) * r.inv[a];
    }
    return r;
}

// Clip [t0, t1] to the box [mn - pad, mx + pad] (approximate arithmetic,
// padded far beyond its error).
__device__ __forceinline__ void clip_box(const float *mn, const float *mx, float pad,
                                         const Ray &ray, const RayPre &r, float &t0, float &t1) {
    const float o[3] = {ray.ox, ray.oy, ray.oz};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float ta = ((mn[a] - pad) - o[a]) * r.inv[a];
        const float tb = ((mx[a] + pad) - o[a]) * r.inv[a];
        const bool neg = (r.neg >> a) & 1u;
        t0 = fmaxf(t0, neg ? tb : ta);
        t1 = fminf(t1, neg ? ta : tb);
    }
}

// Modes of a walk:
//   kAny      stop at the first accepted triangle;
//   kClosest  minimum t, ties to the lower triangle index -- the same answer
//             as testing every triangle;
//   kSkyOcc   closest-hit, except that a hit with t < any_limit stops at
//             once (the caller guarantees no sky triangle can be hit there).
enum TraceMode { kAny = 0, kClosest = 1, kSkyOcc = 2 };

// Resumable state of one walk: the current subtree and its t interval, the
// stack of far subtrees, and the best hit so far.
struct TraceState {
    uint32_t node;
    float t0, t1;
    int sp;
    int32_t best;
    float best_t;
    uint4 stk[kStackMax];  // (node, t0 bits, t1 bits, unused): one 16-byte access
};

// Starts a walk; returns false when the ray misses the scene's padded box
// (st.best = -1 then).
__device__ __forceinline__ bool trace_init(const DevScene &s, const Ray &ray, const RayPre &rp,
                                           float slack, float tmin, float tmax, TraceState &st,
                                           uint32_t root = 0u) {
    st.best = -1;
    st.best_t = kInf;
    st.sp = 0;
    st.node = root;
    if (s.g.ntris == 0 || !(tmin <= tmax)) return false;
    st.t0 = tmin;
    st.t1 = tmax;
    clip_box(s.g.bmin, s.g.bmax, slack, ray, rp, st.t0, st.t1);
    return st.t0 <= st.t1;
}

// One step through an inner node: sets `next` to the child that holds the
// first part of [t0, t1] and narrows the interval to it; the other child is
// pushed (with its part of the interval) when the ray reaches it too.  With
// kOptSkip children without triangles are neither entered nor pushed, and
// the step returns false when no child is left to visit (without it, it
// always returns true).  The stack never overflows: it holds at most one
// entry per tree level.
template <int OPT>
__device__ __forceinline__ bool inner_step(const RayPre &rp, uint2 nd, float &t0, float &t1,
                                           uint4 *stk, int &sp, uint32_t &next) {
    const uint32_t type = nd.x & 3u;
    const float sv = __uint_as_float(nd.y);
    const uint32_t left = (nd.x >> 2) & kChildIndexMask;
    float inv, A, B;
    uint32_t neg;
    if (OPT & kOptShRay) {
        const float4 c = g_ray_axes[type * kShRayLanes + threadIdx.x];
        inv = c.x;
        A = c.y;
        B = c.z;
        neg = __float_as_uint(c.w);
    } else {
        inv = pick3((int)type, rp.inv[0], rp.inv[1], rp.inv[2]);
        A = pick3((int)type, rp.A[0], rp.A[1], rp.A[2]);
        B = pick3((int)type, rp.B[0], rp.B[1], rp.B[2]);
        neg = (rp.neg >> type) & 1u;
    }
    const uint32_t nearc = left + neg, farc = left + 1u - neg;
    const bool near_empty = (OPT & kOptSkip) && (nd.x & (neg ? kRightEmpty : kLeftEmpty)) != 0u;
    const bool far_empty = (OPT & kOptSkip) && (nd.x & (neg ? kLeftEmpty : kRightEmpty)) != 0u;
    const float tne = __fmaf_rn(sv, inv, A);
    const float tfe = __fmaf_rn(sv, inv, B);
    const bool vn = !(tne < t0) && !near_empty, vf = !(tfe > t1) && !far_empty;
    if (vn) {
        if (vf && sp < kStackMax) {
            stk[sp] = make_uint4(farc, __float_as_uint(fmaxf(t0, tfe)), __float_as_uint(t1), 0u);
            sp++;
        }
        t1 = fminf(t1, tne);
        next = nearc;
        return true;
    }
    t0 = fmaxf(t0, tfe);
    next = farc;
    return (OPT & kOptSkip) ? vf : true;
}

// Ray/triangle test (project semantics, in this operation order):
//   den = (Nx*dx + Ny*dy) + Nz*dz ; t = (D - ((Nx*ox + Ny*oy) + Nz*oz)) / den
//   tmin <= t < tmax ; h = o + t*d on the two kept axes
//   b0 = (e0*h0 + e1*h1) + e2 ; b1 = (e3*h0 + e4*h1) + e5 ; b2 = (1 - b0) - b1
//   hit iff all three are >= 0.
// Tests TriangleIndexList entry k, whose plane w0 the caller has loaded, and
// updates best / best_t (minimum t, ties to the lower index).  Returns true
// when the walk ends here: any accepted hit in kAny mode, a hit before
// any_limit in kSkyOcc mode.  The edge part is fetched only when the plane
// hit is in range.
// Leaf-record load; kOptStream asks L1 not to keep the line (the leaf records
// of a large scene stream past L1, where they would evict the nodes and the
// traversal stacks that are reused).
template <int OPT>
__device__ __forceinline__ float4 leaf_load(const float4 *p) {
    if (!(OPT & kOptStream)) return __ldg(p);
    float4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

template <int MODE, int OPT = 0>
__device__ __forceinline__ bool tri_test(const DevScene &s, const Ray &ray, float tmin, float tmax,
                                         int32_t skip, float any_limit, const float4 w0, size_t k,
                                         int32_t &best, float &best_t) {
    const float den = dot3r(w0.x, w0.y, w0.z, ray.dx, ray.dy, ray.dz);
    const float on = dot3r(w0.x, w0.y, w0.z, ray.ox, ray.oy, ray.oz);
    const float t = rdiv(rsub(w0.w, on), den);
    if (!(t >= tmin && t < tmax)) return false;
    if (MODE != kAny && !(t <= best_t)) return false;
    const float4 *ed = s.leaf_edges + 2 * k;
    const float4 w2 = leaf_load<OPT>(ed + 1);
    if (__float_as_int(w2.z) == skip) return false;
    const float4 w1 = leaf_load<OPT>(ed);
    const uint32_t idx_drop = __float_as_uint(w2.w);
    const int drop = (int)(idx_drop & 3u);
    // kept axes (drop+1)%3, (drop+2)%3
    const float o0 = drop == 0 ? ray.oy : (drop == 1 ? ray.oz : ray.ox);
    const float o1 = drop == 0 ? ray.oz : (drop == 1 ? ray.ox : ray.oy);
    const float d0 = drop == 0 ? ray.dy : (drop == 1 ? ray.dz : ray.dx);
    const float d1 = drop == 0 ? ray.dz : (drop == 1 ? ray.dx : ray.dy);
    // edge words: w1 = (e0, e3, e1, e4), w2 = (e2, e5, id, index << 2 | drop)
    const float h0 = radd(o0, rmul(t, d0));
    const float h1 = radd(o1, rmul(t, d1));
    const float b0 = radd(radd(rmul(w1.x, h0), rmul(w1.z, h1)), w2.x);
    const float b1 = radd(radd(rmul(w1.y, h0), rmul(w1.w, h1)), w2.y);
    const float b2 = rsub(rsub(1.0f, b0), b1);
    if (b0 >= 0.0f && b1 >= 0.0f && b2 >= 0.0f) {
        const int32_t ti = (int32_t)(idx_drop >> 2);
        if (MODE == kAny || (MODE == kSkyOcc && t < any_limit)) {
            best = ti;
            best_t = t;
            return true;
        }
        if (t < best_t || ti < best) {
            best = ti;
            best_t = t;
        }
    }
    return false;
}

// Tests the cnt triangles of a leaf (TriangleIndexList[start .. start+cnt))
// with tri_test; true when the walk ends here.  LB triangle planes are
// fetched at a time so their loads overlap.
template <int MODE, int LB, int OPT = 0>
__device__ __forceinline__ bool leaf_test(const DevScene &s, const Ray &ray, float tmin, float tmax,
                                          int32_t skip, float any_limit, uint32_t start, int cnt,
                                          int32_t &best, float &best_t) {
    const float4 *pl = s.leaf_planes + start;
    for (int k0 = 0; k0 < cnt; k0 += LB) {
        float4 P[LB];
#pragma unroll
        for (int j = 0; j < LB; j++)
            if (k0 + j < cnt) P[j] = leaf_load<OPT>(pl + k0 + j);
#pragma unroll
        for (int j = 0; j < LB; j++) {
            if (k0 + j >= cnt) break;
            if (tri_test<MODE, OPT>(s, ray, tmin, tmax, skip, any_limit, P[j], (size_t)start + k0 + j,
                                       best, best_t))
                return true;
        }
    }
    return false;
}

// Pops the next stacked subtree whose interval can still hold the answer
// (kAny: every one); false when the stack is empty.
template <int MODE>
__device__ __forceinline__ bool pop_next(const uint4 *stk, int &sp, float best_t,
                                         uint32_t &node, float &t0, float &t1) {
    while (sp > 0) {
        --sp;
        const uint4 e = stk[sp];
        if (MODE != kAny && __uint_as_float(e.y) > best_t) continue;
        node = e.x;
        t0 = __uint_as_float(e.y);
        t1 = __uint_as_float(e.z);
        return true;
    }
    return false;
}

// One step of the walk: descend to a leaf, test its triangles, pop the next
// subtree that can still hold the answer.  Returns true when the walk is
// over; the answer is st.best / st.best_t.
template <int MODE, int LB = 1, int OPT = 0>
__device__ __forceinline__ bool trace_step(const DevScene &s, const Ray &ray, const RayPre &rp,
                                           float tmin, float tmax, int32_t skip, float any_limit,
                                           TraceState &st) {
    uint32_t node = st.node;
    float t0 = st.t0, t1 = st.t1;
    int sp = st.sp;
    uint2 nd = fetch_node<OPT>(s, node);
    bool reached = true;
    while ((nd.x & 3u) != 3u) {
        if (!inner_step<OPT>(rp, nd, t0, t1, st.stk, sp, node)) {
            reached = false;
            break;
        }
        nd = fetch_node<OPT>(s, node);
    }
    if (reached && leaf_test<MODE, LB, OPT>(s, ray, tmin, tmax, skip, any_limit, nd.x >> 2,
                                            (int)__uint_as_float(nd.y), st.best, st.best_t))
        return true;
    if (!pop_next<MODE>(st.stk, sp, st.best_t, st.node, st.t0, st.t1))
        return true;
    st.sp = sp;
    return false;
}

// A whole walk; returns the hit triangle index (-1 for none) and its t.
template <int MODE, int OPT = 0>
__device__ int32_t kd_trace(const DevScene &s, const Ray &ray, const RayPre &rp, float slack,
                            float tmin, float tmax, int32_t skip, float any_limit, float *t_out) {
    TraceState st;
    if (OPT & kOptShRay) {
#pragma unroll
        for (int a = 0; a < 3; a++)
            g_ray_axes[a * kShRayLanes + threadIdx.x] =
                make_float4(rp.inv[a], rp.A[a], rp.B[a], __uint_as_float((rp.neg >> a) & 1u));
    }
    if (trace_init(s, ray, rp, slack, tmin, tmax, st, root_ref<OPT>(s)))
        while (!trace_step<MODE, 1, OPT>(s, ray, rp, tmin, tmax, skip, any_limit, st)) {
        }
    *t_out = st.best_t;
    return st.best;
}

// Closest or first hit of one ray with its own setup.
template <int MODE, int OPT = 0>
__device__ __forceinline__ int32_t trace_ray(const DevScene &s, const Ray &ray, float tmin,
                                             float tmax, int32_t skip, float *t_out) {
    const float slack = ray_slack(s.g, ray.ox, ray.oy, ray.oz);
    const RayPre rp = ray_pre(ray, slack);
    return kd_trace<MODE, OPT>(s, ray, rp, slack, tmin, tmax, skip, 0.0f, t_out);
}

// Shadow-line setup of TestLineDoesHitSky (raytracer/trace/testline.go:22-27):
// dir = stop - start ; len = sqrt((x*x + y*y) + z*z) ; dir = dir * (1/len).
struct Line {
    float ox, oy, oz, dx, dy, dz, len;
};
__device__ __forceinline__ Line make_line(float sx, float sy, float sz, float ex, float ey,
                                          float ez) {
    Line L;
    L.ox = sx;
    L.oy = sy;
    L.oz = sz;
    float dx = rsub(ex, sx), dy = rsub(ey, sy), dz = rsub(ez, sz);
    L.len = rsqrt_rn(dot3r(dx, dy, dz, dx, dy, dz));
    const float r = rrcp(L.len);
    L.dx = rmul(dx, r);
    L.dy = rmul(dy, r);
    L.dz = rmul(dz, r);
    return L;
}

// How a shadow line is walked (semantics of testline.go:36-51: the closest
// hit on [0, len) that is not skipped occludes unless it carries
// TRACE_ID_SKY).  The walk is closest-hit, but any hit before the line first
// comes within 2*slack of the box of the sky triangles stops at once: no sky
// triangle can be hit there, so that hit is opaque and occludes.  Without
// sky triangles near the line every hit stops the walk (any-hit).
struct LinePlan {
    Ray ray;
    RayPre rp;
    float slack, len;
    float any_limit;  // hits before this t occlude at once (+inf: every hit)
    bool trivial;     // zero length: not occluded, nothing to walk
};

__device__ __forceinline__ LinePlan plan_line(const DevScene &s, const Line &L) {
    LinePlan p;
    p.ray = Ray{L.ox, L.oy, L.oz, L.dx, L.dy, L.dz};
    p.len = L.len;
    p.trivial = !(L.len > 0.0f);
    p.slack = ray_slack(s.g, L.ox, L.oy, L.oz);
    p.rp = ray_pre(p.ray, p.slack);
    p.any_limit = kInf;
    if (s.g.has_sky) {
        float ts0 = -kInf, ts1 = kInf;
        clip_box(s.g.smin, s.g.smax, 2.0f * p.slack, p.ray, p.rp, ts0, ts1);
        if (ts0 <= ts1 && ts0 < L.len) p.any_limit = ts0;
    }
    return p;
}

// Occlusion verdict from a finished kSkyOcc walk of a planned line.
__device__ __forceinline__ bool line_verdict(const DevScene &s, const LinePlan &p, int32_t h,
                                             float th) {
    if (h < 0) return false;
    if (th < p.any_limit) return true;
    return (__ldg(&s.tri_ids[h]) & kTraceIdSky) == 0;
}

// Face of the scene box (padded by `pad`) through which the ray leaves it,
// 2 * axis + 1 for a max side, and the t there (approximate arithmetic).
__device__ __forceinline__ int exit_face(const SceneGeom &g, const Ray &ray, const RayPre &rp, float pad,
                                         float &tex) {
    const float o[3] = {ray.ox, ray.oy, ray.oz};
    int f = 0;
    tex = kInf;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool neg = (rp.neg >> a) & 1u;
        const float t = ((neg ? g.bmin[a] - pad : g.bmax[a] + pad) - o[a]) * rp.inv[a];
        if (t < tex) {
            tex = t;
            f = 2 * a + (neg ? 0 : 1);
        }
    }
    return f;
}

// Which wall layouts a wall test handles: a scene has either slots (every
// face of its box at most kWallSlots triangles) or cells; kernels built for
// one layout carry only its code (the direct-light kernel measured 4-10 %
// slower with both paths in it), the others handle both.
constexpr int kWallSlotsOnly = 0;
constexpr int kWallCellsOnly = 1;
constexpr int kWallAny = 2;

// True when an opaque triangle lying in the face of the scene box through
// which the line leaves (a closed room's wall or floor in the face's slots,
// or a brush side of a map's wall in the cell holding the exit point) is hit
// before any_limit by the exact triangle test.  The walk's verdict is then
// "occluded" whatever lies in front of that wall: the walk would find this
// hit or stop at an earlier one before any_limit, and no sky triangle can be
// hit before any_limit.  False says nothing (the line is walked), so which
// cell the approximate exit point picks decides only how often the test
// answers, never the answer.
template <int OPT = 0, int WM = kWallAny>
__device__ __forceinline__ bool wall_occludes(const DevScene &s, const LinePlan &p, int32_t skip) {
    if (WM == kWallSlotsOnly && s.g.wall_count == 0) return false;
    if (WM == kWallCellsOnly && s.g.wall_cell_mask == 0) return false;
    if (WM == kWallAny && (s.g.wall_count | s.g.wall_cell_mask) == 0) return false;
    float tex;
    const int f = exit_face(s.g, p.ray, p.rp, p.slack, tex);
    if (!(tex < 2.0f * p.len)) return false;  // the line ends well inside the box
    int32_t best = -1;
    float best_t = kInf;
    if (WM != kWallCellsOnly) {
        const uint32_t cnt = (s.g.wall_count >> (3 * f)) & 7u;
        for (uint32_t i = 0; i < cnt; i++) {
            const size_t k = (size_t)s.g.wall_base + (size_t)kWallSlots * f + i;
            if (tri_test<kSkyOcc, OPT>(s, p.ray, 0.0f, p.len, skip, p.any_limit, __ldg(s.leaf_planes + k), k,
                                       best, best_t))
                return true;
        }
        if (WM == kWallSlotsOnly || cnt) return false;
    }
    if (!((s.g.wall_cell_mask >> f) & 1u)) return false;
    const uint32_t *cells = wall_table(s);
    const uint32_t *wf = cells + kWallFaceWords * f;
    const uint4 d0 = __ldg(reinterpret_cast<const uint4 *>(wf));
    const uint4 d1 = __ldg(reinterpret_cast<const uint4 *>(wf) + 1);
    const int a = f >> 1;
    // exit point in the face's in-plane axes (a+1)%3, (a+2)%3
    const float ou = pick3((a + 1) % 3, p.ray.ox, p.ray.oy, p.ray.oz);
    const float ov = pick3((a + 2) % 3, p.ray.ox, p.ray.oy, p.ray.oz);
    const float du = pick3((a + 1) % 3, p.ray.dx, p.ray.dy, p.ray.dz);
    const float dv = pick3((a + 2) % 3, p.ray.dx, p.ray.dy, p.ray.dz);
    const int gu = (int)d1.x, gv = (int)d1.y;
    const float cu = fminf(fmaxf((ou + tex * du - __uint_as_float(d0.x)) * __uint_as_float(d0.z), 0.0f),
                           (float)(gu - 1));
    const float cv = fminf(fmaxf((ov + tex * dv - __uint_as_float(d0.y)) * __uint_as_float(d0.w), 0.0f),
                           (float)(gv - 1));
    const uint32_t cell = d1.z + (uint32_t)((int)cu * gv + (int)cv);
    const uint32_t b = __ldg(cells + cell), e = __ldg(cells + cell + 1);
    for (uint32_t i = b; i < e; i++) {
        const size_t k = __ldg(cells + i);
        if (tri_test<kSkyOcc, OPT>(s, p.ray, 0.0f, p.len, skip, p.any_limit, __ldg(s.leaf_planes + k), k,
                                   best, best_t))
            return true;
    }
    return false;
}

template <int OPT = 0, int WM = kWallAny>
__device__ __forceinline__ bool line_occluded(const DevScene &s, const Line &L, int32_t skip) {
    const LinePlan p = plan_line(s, L);
    if (p.trivial) return false;
    if (wall_occludes<OPT, WM>(s, p, skip)) return true;
    float th;
    const int32_t h =
        kd_trace<kSkyOcc, OPT>(s, p.ray, p.rp, p.slack, 0.0f, p.len, skip, p.any_limit, &th);
    return line_verdict(s, p, h, th);
}

}  // namespace vrg
