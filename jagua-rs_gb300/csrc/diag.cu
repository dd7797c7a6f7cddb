// Measurement helpers of the C ABI (no counterpart in the reference): the L2 read bandwidth this
// GPU sustains for a buffer that stays L2-resident, the ceiling for the query kernels, whose
// layout (a few MB) lives in L2 while the query batch streams from HBM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/jcde.h"

namespace {

// Every thread reads 16-byte words of the buffer with ld.global.cg (cached in L2 only, so that
// repeated passes are not served by L1), `reps` passes in a grid-stride order that differs per
// pass, so a pass never finds its lines in another SM's L1 either.  The sum is kept live by a
// store that happens only for an impossible value.
__global__ void __launch_bounds__(512) k_l2_read(const float4* __restrict__ buf, uint64_t n, uint32_t reps,
                                                 float* __restrict__ sink) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    for (uint32_t r = 0; r < reps; r++) {
        const uint64_t shift = ((uint64_t)r * 7919u * blockDim.x) % n;
        for (uint64_t i = t; i < n; i += stride) {
            uint64_t j = i + shift;
            if (j >= n) j -= n;
            const float4 v = __ldcg(&buf[j]);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == -1.2345678e30f) sink[0] = acc;
}

__global__ void k_fill(float4* buf, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        buf[i] = make_float4(1.0f, 2.0f, 3.0f, 4.0f);
}

}  // namespace

extern "C" jcde_status jcde_l2_read_peak(uint64_t bytes, uint32_t reps, double* out_gbs) {
    if (!out_gbs || bytes < (1u << 20) || reps == 0) return JCDE_ERR_ARG;
    int dev = 0, n_sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return JCDE_ERR_CUDA;
    if (cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return JCDE_ERR_CUDA;
    const uint64_t n = bytes / sizeof(float4);
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    jcde_status st = JCDE_ERR_CUDA;
    if (cudaMalloc(&buf, n * sizeof(float4)) != cudaSuccess) return JCDE_ERR_CUDA;
    if (cudaMalloc(&sink, 4) != cudaSuccess) goto done;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) goto done;
    {
        const uint32_t grid = (uint32_t)n_sms * 4;
        k_fill<<<grid, 512>>>(buf, n);
        k_l2_read<<<grid, 512>>>(buf, n, 2, sink);   // warm: the buffer now sits in L2
        cudaEventRecord(a);
        k_l2_read<<<grid, 512>>>(buf, n, reps, sink);
        cudaEventRecord(b);
        if (cudaEventSynchronize(b) != cudaSuccess || cudaGetLastError() != cudaSuccess) goto done;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess || ms <= 0.0f) goto done;
        *out_gbs = (double)n * sizeof(float4) * reps / (ms * 1e-3) / 1e9;
        st = JCDE_OK;
    }
done:
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(sink);
    cudaFree(buf);
    return st;
}
