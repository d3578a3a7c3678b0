// CIC deposit that allocates no device memory (tm_cic_deposit_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured, host programs that hand the library a fixed device-memory
// budget and forbid further allocation, or real-time loops where an
// allocation may block.  This entry point takes every input and output from
// the caller and keeps its only scratch -- the per-block partial bounding
// boxes of the touched grid nodes (patches.c:81-132) -- in a file-scope
// device array of fixed size, reserved in every GPU that loads the library
// until the process exits.
#include "tm_core.cuh"
#include "timothy_gb300.h"

#include <cstdio>
#include <mutex>

#define NOALLOC_BLOCK 256
#define NOALLOC_MAX_CELLS (1ll << 24)                          // 16,777,216 cells per call
#define NOALLOC_MAX_BLOCKS (NOALLOC_MAX_CELLS / NOALLOC_BLOCK)  // 65,536 partial boxes

// 6 int64 per block (lower x,y,z, upper x,y,z) = 3 MiB per GPU
static __device__ __align__(256) long long g_cic_scratch[NOALLOC_MAX_BLOCKS * 6];

// Host-side table of the scratch's device address, filled once per device
// and CUDA context.  The symbol itself is only a host-side stand-in for the
// device array and must never be passed to a kernel.  A context that is
// destroyed and created again (cudaDeviceReset, or a caller switching to
// another context on the same device) loads the module anew, possibly at
// another address, so each entry remembers the context it was taken in and is
// looked up again when the current context differs.
struct scratch_slot {
    unsigned long long ctx_id;   // 0: no context identity (looked up on every call)
    long long *ptr;
};
static std::mutex g_setup_mutex;
static scratch_slot g_scratch_dev[64];

typedef int (*ctx_get_current_fn)(void **);
typedef int (*ctx_get_id_fn)(void *, unsigned long long *);

// identity of the calling thread's current context, 0 when the driver does not
// provide one (cuCtxGetCurrent / cuCtxGetId through the runtime's entry-point
// query, so the library need not link the driver library)
static unsigned long long current_context_id()
{
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    static bool queried = false;
    if (!queried) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) ==
                cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = (ctx_get_current_fn)f1;
            get_id = (ctx_get_id_fn)f2;
        }
        queried = true;
    }
    if (!get_current || !get_id) return 0;
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

static int scratch_for_current_device(long long **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TM_ENODEV;
    // cudaSetDevice makes the device's context current, creating it if needed
    if (cudaSetDevice(dev) != cudaSuccess) return TM_ECUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    scratch_slot &slot = g_scratch_dev[dev];
    if (!slot.ptr || ctx == 0 || slot.ctx_id != ctx) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cic_scratch);
        if (e != cudaSuccess || !p) return TM_ECUDA;
        slot.ptr = (long long *)p;
        slot.ctx_id = ctx;
    }
    *out = slot.ptr;
    return TM_OK;
}

// deposit (same arithmetic as the session's CIC kernel) + per-block box
__global__ void __launch_bounds__(NOALLOC_BLOCK)
k_cic_noalloc(const double *x, const double *y, const double *z, const int *phase, long long n, int dim,
              double lx, double ly, double lz, float res, int gx, int gy, int gz, double *grid, long long *part)
{
    const unsigned FULLM = 0xffffffffu;
    __shared__ long long red[NOALLOC_BLOCK / 32][6];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool live = i < n;
    const double lower[3] = {lx, ly, lz};
    long long ci[3] = {0, 0, 0};
    double dd[3] = {0, 0, 0}, tt[3] = {0, 0, 0};
    int ph = 5;
    if (live) {
        const double pos[3] = {x[i], y[i], z[i]};
        for (int k = 0; k < 3; k++) {
            ci[k] = (long long)tm_div_res(sub64(pos[k], lower[k]), res);
            const double cic = add64(lower[k], (double)__fmul_rn((float)ci[k], res));
            dd[k] = tm_div_res(sub64(pos[k], cic), res);
            tt[k] = sub64(1.0, dd[k]);
        }
        ph = phase[i];
    }
    const long long up[3] = {gx - 1, gy - 1, dim == 3 ? gz - 1 : 0};
    const double wph = ph == 0 ? 0.75 : 1.0;
    long long lo[3] = {0x7fffffffll, 0x7fffffffll, 0x7fffffffll};
    long long hi[3] = {-0x7fffffffll - 1, -0x7fffffffll - 1, -0x7fffffffll - 1};
    // ((wphase * wx) * wy) * wz in the reference's order, partial products shared
    const double wx0 = mul64(wph, tt[0]), wx1 = mul64(wph, dd[0]);
    double wxy = 0.0;
    for (int corner = 0; corner < 8; corner++) {
        const int ax = corner >> 2, ay = (corner >> 1) & 1, az = corner & 1;
        if (az == 0) wxy = mul64(ax ? wx1 : wx0, ay ? dd[1] : tt[1]);
        const long long px = ci[0] + ax, py = ci[1] + ay, pz = ci[2] + az;
        const bool inb = live && px >= 0 && py >= 0 && pz >= 0 && px <= up[0] && py <= up[1] && pz <= up[2];
        if (inb) {
            lo[0] = min(lo[0], px);
            lo[1] = min(lo[1], py);
            lo[2] = min(lo[2], pz);
            hi[0] = max(hi[0], px);
            hi[1] = max(hi[1], py);
            hi[2] = max(hi[2], pz);
        }
        const bool dep = inb && ph != 5;
        const double wgt = dep ? mul64(wxy, az ? dd[2] : tt[2]) : 0.0;
        const long long gi = dep ? ((long long)gy * px + py) * gz + pz : -1;
        tm_warp_deposit(grid, gi, wgt, dep, lane);
    }
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = min(lo[k], __shfl_xor_sync(FULLM, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(FULLM, hi[k], o));
        }
    }
    if (lane == 0)
        for (int k = 0; k < 3; k++) {
            red[w][k] = lo[k];
            red[w][3 + k] = hi[k];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        long long v = red[0][threadIdx.x];
        for (int u = 1; u < NOALLOC_BLOCK / 32; u++)
            v = threadIdx.x < 3 ? min(v, red[u][threadIdx.x]) : max(v, red[u][threadIdx.x]);
        part[(long long)blockIdx.x * 6 + threadIdx.x] = v;   // every partial is rewritten each call
    }
}

// reduce the partial boxes into the caller's 6 corners; 2-D grids keep z at 0
// as patches_alloc does (patches.c:68-77)
__global__ void __launch_bounds__(256) k_cic_noalloc_box(const long long *part, int nblocks, int dim,
                                                         long long *corners)
{
    __shared__ long long red[256][6];
    long long v[6] = {0x7fffffffll, 0x7fffffffll, 0x7fffffffll, -0x7fffffffll - 1, -0x7fffffffll - 1,
                      -0x7fffffffll - 1};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        for (int k = 0; k < 6; k++) v[k] = k < 3 ? min(v[k], part[b * 6ll + k]) : max(v[k], part[b * 6ll + k]);
    for (int k = 0; k < 6; k++) red[threadIdx.x][k] = v[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 6; k++)
                red[threadIdx.x][k] = k < 3 ? min(red[threadIdx.x][k], red[threadIdx.x + s][k])
                                            : max(red[threadIdx.x][k], red[threadIdx.x + s][k]);
        __syncthreads();
    }
    if (threadIdx.x < 6) {
        long long r = red[0][threadIdx.x];
        if (dim != 3 && (threadIdx.x == 2 || threadIdx.x == 5)) r = 0;
        corners[threadIdx.x] = r;
    }
}

extern "C" int tm_cic_deposit_noalloc(const double *x, const double *y, const double *z, const int *phase,
                                      int64_t n, int dimension, const double lower[3], float resolution,
                                      const int64_t gsize[3], double *grid, int64_t *corners, void *stream)
{
    if (n < 0 || !lower || !gsize || !grid || !corners || (dimension != 2 && dimension != 3)) return TM_EINVAL;
    if (n > 0 && (!x || !y || !z || !phase)) return TM_EINVAL;
    if (n > NOALLOC_MAX_CELLS) {
        fprintf(stderr, "tm_cic_deposit_noalloc: %lld cells exceed the fixed scratch limit of %lld\n", (long long)n,
                (long long)NOALLOC_MAX_CELLS);
        return TM_EINVAL;
    }
    if (!(resolution > 0.0f) || gsize[0] <= 0 || gsize[1] <= 0 || gsize[2] <= 0) return TM_EINVAL;
    long long *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != TM_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t gbytes = (size_t)(gsize[0] * gsize[1] * gsize[2]) * sizeof(double);
    // Every step's own return code is checked, not the thread's last-error
    // state: an error left there by earlier, unrelated work is neither
    // reported as this call's failure nor cleared.
    // patches_cells2envinfo zeroes the patch before depositing (patches.c:165-170)
    if (cudaMemsetAsync(grid, 0, gbytes, st) != cudaSuccess) return TM_ECUDA;
    int nblocks = n > 0 ? (int)((n + NOALLOC_BLOCK - 1) / NOALLOC_BLOCK) : 0;
    if (nblocks > 0) {
        long long nn = (long long)n;
        int dim = dimension;
        double lx = lower[0], ly = lower[1], lz = lower[2];
        float res = resolution;
        int gx = (int)gsize[0], gy = (int)gsize[1], gz = (int)gsize[2];
        void *args[] = {(void *)&x, (void *)&y, (void *)&z, (void *)&phase, &nn, &dim, &lx, &ly, &lz, &res,
                        &gx, &gy, &gz, (void *)&grid, (void *)&scratch};
        if (cudaLaunchKernel((const void *)k_cic_noalloc, dim3((unsigned)nblocks), dim3(NOALLOC_BLOCK), args, 0,
                             st) != cudaSuccess)
            return TM_ECUDA;
    }
    {
        int dim = dimension;
        long long *cor = (long long *)corners;
        void *args[] = {(void *)&scratch, &nblocks, &dim, (void *)&cor};
        if (cudaLaunchKernel((const void *)k_cic_noalloc_box, dim3(1), dim3(256), args, 0, st) != cudaSuccess)
            return TM_ECUDA;
    }
    return TM_OK;
}
