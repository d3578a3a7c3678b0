// Measured FP32 FMA rate of the device: the compute denominator for the list
// pass, whose pair arithmetic runs on the FP32 pipe (no tensor-core form).
// Every thread runs eight independent FMA chains, so the pipe, not the
// dependency latency, bounds the rate; the grid fills every SM with 2048
// threads.  Two FLOPs per FMA.
#include <cuda_runtime.h>

#include "timothy_gb300.h"

#define PEAK_CHAINS 8

__global__ void __launch_bounds__(256) k_fma_peak(float *out, int iters, float b, float c)
{
    float acc[PEAK_CHAINS];
#pragma unroll
    for (int k = 0; k < PEAK_CHAINS; k++) acc[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int k = 0; k < PEAK_CHAINS; k++) acc[k] = fmaf(acc[k], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < PEAK_CHAINS; k++) s += acc[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" int tm_measure_fp32_peak(int device, double *tflops)
{
    if (!tflops) return TM_EINVAL;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return TM_ECUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        return TM_ECUDA;
    const int block = 256, grid = sms * 8, iters = 16384;
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = TM_OK;
    if (cudaMalloc((void **)&out, (size_t)grid * block * sizeof(float)) != cudaSuccess) return TM_ENOMEM;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = TM_ECUDA;
    float best = 0.0f;
    for (int rep = 0; rc == TM_OK && rep < 3; rep++) {
        cudaEventRecord(e0);
        k_fma_peak<<<grid, block>>>(out, iters, 0.9999999f, 1e-7f);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = TM_ECUDA;
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.0f && (best == 0.0f || ms < best)) best = ms;
    }
    if (rc == TM_OK && best > 0.0f) {
        const double flops = 2.0 * 4.0 * PEAK_CHAINS * (double)iters * (double)grid * block;
        *tflops = flops / (best * 1e-3) / 1e12;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}
