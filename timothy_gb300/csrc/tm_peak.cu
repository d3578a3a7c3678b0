// Measured FP32 FMA rate of the device: the compute denominator for the list
// pass, whose pair arithmetic runs on the FP32 pipe (no tensor-core form).
// Every thread runs eight independent FMA chains, so the pipe, not the
// dependency latency, bounds the rate; the grid fills every SM with 2048
// threads.  Two FLOPs per FMA.
#include <cuda_runtime.h>

#include "timothy_gb300.h"
#include "tm_core.cuh"

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

// Self-check of the arithmetic the kernels form themselves instead of calling
// the CUDA library: the FMA-based quotient against the correctly rounded
// division, the integer rounding of a double to float against the hardware
// conversion, and the integer float -> double conversion against the
// hardware one, on `n` pseudo-random inputs per check (counter-based, seed).

__device__ __forceinline__ unsigned long long mix64_peak(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void k_numerics_check(long long n, unsigned long long seed, unsigned long long *bad)
{
    unsigned long long nb[3] = {0, 0, 0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r0 = mix64_peak(seed ^ (unsigned long long)k), r1 = mix64_peak(r0), r2 = mix64_peak(r1);
        // quotient: b a cutoff-like length in [0.25, 16), a in [0, b] (near b for a quarter of the draws)
        const double b = ldexp(1.0 + (double)(r0 >> 11) * 0x1.0p-53, (int)(r1 & 7) - 2);
        double t = (double)(r2 >> 11) * 0x1.0p-53;
        if ((r1 >> 8 & 3) == 0) t = 1.0 - t * 1e-6;
        const double a = __dmul_rn(b, t);
        const double y = __drcp_rn(b);
        if (div_by_recip(a, b, y) != __ddiv_rn(a, b)) nb[0]++;
        // double -> float rounding: random bit patterns over the float range and halfway cases
        unsigned long long wb = (r0 & 0x800fffffffffffffull) | ((unsigned long long)(860 + (r1 % 330)) << 52);
        if ((r2 & 3) == 0) wb = (wb & ~0x1fffffffull) | 0x10000000ull;
        const double w = __longlong_as_double((long long)wb);
        const double want = (double)__double2float_rn(w);
        const double got = tm_round_to_float(w);
        if (__double_as_longlong(got) != __double_as_longlong(want)) nb[1]++;
        // float -> double: every class of float bit pattern
        const float f = __uint_as_float((unsigned)(r2 >> 32));
        const double fd = (double)f;
        const double fg = tm_f2d(f);
        if (!(fd != fd && fg != fg) && __double_as_longlong(fd) != __double_as_longlong(fg)) nb[2]++;
    }
    for (int q = 0; q < 3; q++)
        if (nb[q]) atomicAdd(&bad[q], nb[q]);
}

extern "C" int tm_check_numerics(int device, int64_t n, uint64_t seed, int64_t *mismatches)
{
    if (!mismatches || n < 0) return TM_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return TM_ECUDA;
    unsigned long long *d = nullptr;
    if (cudaMalloc((void **)&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return TM_ENOMEM;
    int rc = TM_OK;
    unsigned long long h[3] = {0, 0, 0};
    if (cudaMemset(d, 0, sizeof h) != cudaSuccess) rc = TM_ECUDA;
    if (rc == TM_OK) {
        k_numerics_check<<<1024, 256>>>((long long)n, (unsigned long long)seed, d);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = TM_ECUDA;
    }
    cudaFree(d);
    for (int q = 0; q < 3; q++) mismatches[q] = (int64_t)h[q];
    return rc;
}
