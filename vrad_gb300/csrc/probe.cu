// probe.cu -- L2 read bandwidth probe used by bench.py to put the trace
// kernels' L2-served bytes beside a measured L2 figure.  Built into its own
// small library (libvrgprobe.so); the product library does not contain it.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

// Each thread strides over the buffer `reps` times with 16-byte loads; the
// buffer is small enough to stay in L2, so after the first pass every load
// is an L2 (or L1) hit.  The sum is written so the loads are not removed.
__global__ void k_l2_read(const float4 *__restrict__ buf, int64_t n4, int reps,
                          float *__restrict__ sink) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    float acc = 0.0f;
    for (int r = 0; r < reps; r++) {
        // rotate the start so one thread does not reread its own lines
        const int64_t shift = ((int64_t)r * 4099) % n4;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
            int64_t j = i + shift;
            if (j >= n4) j -= n4;
            const float4 v = __ldcg(buf + j);  // cache in L2 only, not L1
            acc += v.x + v.y + v.z + v.w;
        }
    }
    sink[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace

extern "C" int vrg_probe_l2_read_gbs(int device, int64_t bytes, int reps, double *gbs) {
    if (!gbs || bytes < (1 << 20) || reps < 1) return -1;
    if (cudaSetDevice(device) != cudaSuccess) return -3;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 512, blocks = sms * 4;
    const int64_t n4 = bytes / 16;
    float4 *buf = nullptr;
    float *sink = nullptr;
    if (cudaMalloc(&buf, n4 * 16) != cudaSuccess) return -2;
    if (cudaMalloc(&sink, (size_t)threads * blocks * 4) != cudaSuccess) {
        cudaFree(buf);
        return -2;
    }
    cudaMemset(buf, 0, n4 * 16);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_l2_read<<<blocks, threads>>>(buf, n4, 2, sink);  // warm L2
    cudaEventRecord(a);
    k_l2_read<<<blocks, threads>>>(buf, n4, reps, sink);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return -3;
    *gbs = (double)n4 * 16.0 * reps / (ms * 1e-3) / 1e9;
    return 0;
}
