// vrg_spmv.cuh -- one CSR row of the transfer matrix times the emission
// vector, shared by the bounce, batched-bounce and relight kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace vrg {

// Column / weight stream loads; NA loads them without allocating in L1, so
// that L1 keeps the gathered emission entries.
template <bool NA>
__device__ __forceinline__ int32_t csr_col(const int32_t *p) {
    if (!NA) return __ldg(p);
    int32_t v;
    asm volatile("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
template <bool NA>
__device__ __forceinline__ float csr_w(const float *p) {
    if (!NA) return __ldg(p);
    float v;
    asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

// sum_j w_j * x[col_j] over the row's entries [b, e) for one warp: lane l
// takes entries b+l, b+l+32, ... in that order, each added with one fused
// multiply-add (so every U gives the same per-lane sums), U of them per round, with the next round's column and
// weight loads in flight while this round's x entries are gathered (the
// gathers wait on the column loads; without the overlap every round pays
// both latencies back to back).  Returns the lane's partial sums; the
// caller reduces across the warp.
template <int U, bool NA = false>
__device__ __forceinline__ float3 row_gather(const int32_t *__restrict__ col,
                                             const float *__restrict__ w,
                                             const float4 *__restrict__ x, int64_t b, int64_t e,
                                             int lane) {
    float ar = 0.0f, ag = 0.0f, ab = 0.0f;
    int64_t i = b + lane;
    int32_t c[U];
    float wv[U];
    if (i + 32 * (U - 1) < e) {
#pragma unroll
        for (int k = 0; k < U; k++) {
            c[k] = csr_col<NA>(col + i + 32 * k);
            wv[k] = csr_w<NA>(w + i + 32 * k);
        }
    }
    for (; i + 32 * (U - 1) < e; i += 32 * U) {
        const int64_t in = i + 32 * U;
        int32_t cn[U];
        float wn[U];
        if (in + 32 * (U - 1) < e) {
#pragma unroll
            for (int k = 0; k < U; k++) {
                cn[k] = csr_col<NA>(col + in + 32 * k);
                wn[k] = csr_w<NA>(w + in + 32 * k);
            }
        }
        float4 xv[U];
#pragma unroll
        for (int k = 0; k < U; k++) xv[k] = __ldg(x + c[k]);
#pragma unroll
        for (int k = 0; k < U; k++) {
            ar = __fmaf_rn(wv[k], xv[k].x, ar);
            ag = __fmaf_rn(wv[k], xv[k].y, ag);
            ab = __fmaf_rn(wv[k], xv[k].z, ab);
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            c[k] = cn[k];
            wv[k] = wn[k];
        }
    }
    for (; i < e; i += 32) {
        const float wk = csr_w<NA>(w + i);
        const float4 xk = __ldg(x + csr_col<NA>(col + i));
        ar = __fmaf_rn(wk, xk.x, ar);
        ag = __fmaf_rn(wk, xk.y, ag);
        ab = __fmaf_rn(wk, xk.z, ab);
    }
    return make_float3(ar, ag, ab);
}

__device__ __forceinline__ float3 warp_sum3(float3 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
    }
    return v;
}

}  // namespace vrg
