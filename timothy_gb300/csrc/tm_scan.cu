// Device-wide exclusive prefix sum over uint32 (the bin table), three passes:
// per-tile totals, a scan of the totals in one block, then per-tile scans.
#include "tm_kernels.cuh"

#define SCAN_THREADS 256
#define SCAN_ITEMS 8
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t &total)
{
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = t;
    }
    __syncthreads();
    uint32_t before = w > 0 ? warp_tot[w - 1] : 0u;
    total = warp_tot[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const uint32_t *in, long long n, uint32_t *sums)
{
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_exclusive_scan(s, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(uint32_t *sums, long long nt)
{
    uint32_t carry = 0;
    for (long long base = 0; base < nt; base += SCAN_THREADS) {
        long long i = base + threadIdx.x;
        uint32_t v = i < nt ? sums[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, tot);
        if (i < nt) sums[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t *in, uint32_t *out, long long n,
                                                             const uint32_t *sums)
{
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(s, tot) + sums[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
}

long long tm_scan_tmp_words(long long n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

cudaError_t tm_scan_exclusive(const uint32_t *in, uint32_t *out, long long n, uint32_t *tmp, cudaStream_t st)
{
    long long nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nt == 0) return cudaSuccess;
    k_scan_tiles<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, n, tmp);
    k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(tmp, nt);
    k_scan_apply<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, out, n, tmp);
    return cudaGetLastError();
}
