// Device-wide exclusive prefix sum over uint32 (the bin table), three passes:
// per-tile totals, a scan of the totals in one block (8192 totals per round),
// then per-tile scans.
#include "tm_kernels.cuh"

#define SCAN_THREADS 256
#define SCAN_ITEMS 8
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)
#define SUMS_THREADS 1024

template <int THREADS>
__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t &total)
{
    __shared__ uint32_t warp_tot[THREADS / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < THREADS / 32 ? warp_tot[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < THREADS / 32) warp_tot[lane] = t;
    }
    __syncthreads();
    uint32_t before = w > 0 ? warp_tot[w - 1] : 0u;
    total = warp_tot[THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// a thread's SCAN_ITEMS consecutive words: two 16-byte loads when the run is
// whole and aligned, word by word at the end of the array
template <bool VEC>
__device__ __forceinline__ void load_items(const uint32_t *in, long long base, long long n, uint32_t (&v)[SCAN_ITEMS])
{
    if (VEC && base + SCAN_ITEMS <= n) {
        const uint4 p = *(const uint4 *)(in + base), q = *(const uint4 *)(in + base + 4);
        v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w;
        v[4] = q.x; v[5] = q.y; v[6] = q.z; v[7] = q.w;
        return;
    }
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = base + k < n ? in[base + k] : 0u;
}

template <bool VEC>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const uint32_t *in, long long n, uint32_t *sums)
{
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    load_items<VEC>(in, base, n, v);
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
    uint32_t tot;
    block_exclusive_scan<SCAN_THREADS>(s, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// one block: the exclusive scan of the tile totals, SCAN_ITEMS per thread
__global__ void __launch_bounds__(SUMS_THREADS) k_scan_sums(uint32_t *sums, long long nt)
{
    uint32_t carry = 0;
    for (long long base = 0; base < nt; base += (long long)SUMS_THREADS * SCAN_ITEMS) {
        const long long i0 = base + (long long)threadIdx.x * SCAN_ITEMS;
        uint32_t v[SCAN_ITEMS];
        load_items<false>(sums, i0, nt, v);
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
        uint32_t tot;
        uint32_t ex = carry + block_exclusive_scan<SUMS_THREADS>(s, tot);
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            if (i0 + k < nt) sums[i0 + k] = ex;
            ex += v[k];
        }
        carry += tot;
    }
}

template <bool VEC>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t *in, uint32_t *out, long long n,
                                                             const uint32_t *sums)
{
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    load_items<VEC>(in, base, n, v);
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) s += v[k];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan<SCAN_THREADS>(s, tot) + sums[blockIdx.x];
    if (VEC && base + SCAN_ITEMS <= n) {
        uint32_t o[SCAN_ITEMS];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            o[k] = ex;
            ex += v[k];
        }
        *(uint4 *)(out + base) = make_uint4(o[0], o[1], o[2], o[3]);
        *(uint4 *)(out + base + 4) = make_uint4(o[4], o[5], o[6], o[7]);
        return;
    }
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
    const bool vec = (((uintptr_t)in | (uintptr_t)out) & 15u) == 0;
    if (vec) k_scan_tiles<true><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, n, tmp);
    else k_scan_tiles<false><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, n, tmp);
    k_scan_sums<<<1, SUMS_THREADS, 0, st>>>(tmp, nt);
    if (vec) k_scan_apply<true><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, out, n, tmp);
    else k_scan_apply<false><<<(unsigned)nt, SCAN_THREADS, 0, st>>>(in, out, n, tmp);
    return cudaGetLastError();
}
