// Grid -> cell gather (patches_applyenv2cells, patches.c:512-593) and the
// field gradient (fieldgradient_compute, fieldgradient.c:149-225) at one rank.
//
// Gather: every cell takes the 8 grid nodes of its CIC cell that lie inside
// the grid, in the corner order ax, ay, az, and adds data * wx * wy * wz
// (weights t = 1 - d or d, exactly as the reference forms them) to its field
// value and the same weights times the three gradient components to gx, gy,
// gz.  Gradient: (u[i+1] - u[i-1]) / resolution inside (no factor 1/2, as in
// the reference), one-sided differences on the faces; an axis of one node
// (the z axis of a 2-D grid) gets 0, where the reference reads outside the
// row.  Both are FP64 with the reference's roundings: a division by the
// resolution becomes a scaling by its reciprocal only when that is a power of
// two (then both round the same real number).
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"
#include "timothy_gb300.h"

#include <algorithm>
#include <cmath>

// x * 2^e for a power-of-two scale: the exponent field moves by e, which is
// the exactly rounded product whenever x and the result are normal numbers
// (integer work: the FP64 pipe of this GPU is narrow); other cases multiply
__device__ __forceinline__ double scale_pow2(double x, int e, double factor)
{
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0 || ex == 0x7ff || ex + e <= 0 || ex + e >= 0x7ff) return mul64(x, factor);
    return __longlong_as_double(b + ((long long)e << 52));
}

// x / res with the reference's rounding
__device__ __forceinline__ double div_res(double x, const tm_envgeom &g)
{
    return g.pow2 ? scale_pow2(x, g.inv_exp, g.inv) : div64(x, g.res);
}

// gather for one cell at pos; out[(f * out_n + c) * 4 + k]
__device__ __forceinline__ void env_gather(const tm_envgeom &g, const double pos[3], const double *data,
                                           const double *grad, double *out, long long out_n, long long c)
{
    long long ci[3];
    double d[3], t[3];
    for (int k = 0; k < 3; k++) {
        ci[k] = (long long)div_res(sub64(pos[k], g.lower[k]), g);
        // grid->lowercorner + cellIdx * resolution: an int64 * float product is a float
        const double cic = add64(g.lower[k], (double)__fmul_rn((float)ci[k], g.resf));
        d[k] = div_res(sub64(pos[k], cic), g);
        t[k] = sub64(1.0, d[k]);
    }
    const long long vol = g.bsz[0] * g.bsz[1] * g.bsz[2];
    for (int f = 0; f < g.nfields; f++) {
        double v = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
        for (int corner = 0; corner < 8; corner++) {
            const int ax = corner >> 2, ay = (corner >> 1) & 1, az = corner & 1;
            const long long a0 = ci[0] + ax, a1 = ci[1] + ay, a2 = ci[2] + az;
            if (a0 < 0 || a1 < 0 || a2 < 0 || a0 > g.hi[0] || a1 > g.hi[1] || a2 > g.hi[2]) continue;
            const long long b0 = a0 - g.blo[0], b1 = a1 - g.blo[1], b2 = a2 - g.blo[2];
            // nodes outside the supplied box are never touched by a cell of it
            if (b0 < 0 || b1 < 0 || b2 < 0 || b0 >= g.bsz[0] || b1 >= g.bsz[1] || b2 >= g.bsz[2]) continue;
            const long long node = (b0 * g.bsz[1] + b1) * g.bsz[2] + b2;
            const double wx = ax ? d[0] : t[0], wy = ay ? d[1] : t[1], wz = az ? d[2] : t[2];
            v = add64(v, mul64(mul64(mul64(data[f * vol + node], wx), wy), wz));
            const double *gr = grad + (f * vol + node) * 3;
            gx = add64(gx, mul64(mul64(mul64(gr[0], wx), wy), wz));
            gy = add64(gy, mul64(mul64(mul64(gr[1], wx), wy), wz));
            gz = add64(gz, mul64(mul64(mul64(gr[2], wx), wy), wz));
        }
        double *o = out + (f * out_n + c) * 4;
        o[0] = v;
        o[1] = gx;
        o[2] = gy;
        o[3] = gz;
    }
}

__global__ void __launch_bounds__(256) k_env2cells(tm_envgeom g, const double *x, const double *y, const double *z,
                                                   long long n, const double *data, const double *grad, double *out)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double pos[3] = {x[c], y[c], z[c]};
        env_gather(g, pos, data, grad, out, n, c);
    }
}

// the cells of one session colony, written in the caller's order (perm)
__global__ void __launch_bounds__(256) k_env2cells_colony(tm_envgeom g, tm_arrays a, long long off, long long n,
                                                          const double *data, const double *grad, double *out)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long s = off + k;
        const double pos[3] = {a.x[s], a.y[s], a.z[s]};
        env_gather(g, pos, data, grad, out, n, (long long)a.perm[s]);
    }
}

// one field per blockIdx.y; node indices fit in 32 bits (checked by the host)
__global__ void __launch_bounds__(256) k_field_gradient(tm_envgeom g, unsigned nx, unsigned ny, unsigned nz,
                                                        const double *data, double *grad)
{
    const unsigned G = nx * ny * nz, nyz = ny * nz;
    const long long f = blockIdx.y;
    const double *u = data + f * (long long)G;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        const unsigned i = o / nyz, r = o - i * nyz, j = r / nz, k = r - j * nz;
        const unsigned n3[3] = {nx, ny, nz}, ix[3] = {i, j, k}, st[3] = {nyz, nz, 1u};
        double *out = grad + (f * (long long)G + o) * 3;
        for (int c = 0; c < 3; c++) {
            double v;
            if (n3[c] < 2) v = 0.0;
            else if (ix[c] == 0) v = div_res(sub64(u[o + st[c]], u[o]), g);
            else if (ix[c] == n3[c] - 1) v = div_res(sub64(u[o], u[o - st[c]]), g);
            else v = div_res(sub64(u[o + st[c]], u[o - st[c]]), g);
            out[c] = v;
        }
    }
}

// geometry of a gather or gradient on a box of the grid
tm_envgeom tm_make_envgeom(const double lower[3], float res, const int64_t grid_hi[3], const int64_t box_lo[3],
                           const int64_t box_size[3], int nfields)
{
    tm_envgeom g;
    for (int k = 0; k < 3; k++) {
        g.lower[k] = lower ? lower[k] : 0.0;
        g.hi[k] = grid_hi ? grid_hi[k] : 0;
        g.blo[k] = box_lo ? box_lo[k] : 0;
        g.bsz[k] = box_size ? box_size[k] : 1;
    }
    g.resf = res;
    g.res = (double)res;
    int e = 0;
    const double m = std::frexp(g.res, &e);
    g.pow2 = (m == 0.5) ? 1 : 0;             // res = 2^(e-1): its reciprocal is exact
    g.inv = g.pow2 ? std::ldexp(1.0, 1 - e) : 0.0;
    g.inv_exp = 1 - e;
    g.nfields = nfields;
    return g;
}

static unsigned grid_for(long long work)
{
    const long long b = (work + 255) / 256;
    return (unsigned)std::max(1ll, std::min(b, 152ll * 64));
}

cudaError_t tm_launch_env2cells(const tm_envgeom &g, const double *x, const double *y, const double *z, long long n,
                                const double *data, const double *grad, double *out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_env2cells<<<grid_for(n), 256, 0, st>>>(g, x, y, z, n, data, grad, out);
    return cudaGetLastError();
}

cudaError_t tm_launch_env2cells_colony(const tm_envgeom &g, const tm_arrays &a, long long off, long long n,
                                       const double *data, const double *grad, double *out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_env2cells_colony<<<grid_for(n), 256, 0, st>>>(g, a, off, n, data, grad, out);
    return cudaGetLastError();
}

cudaError_t tm_launch_field_gradient(const tm_envgeom &g, const int64_t gsize[3], const double *data, double *grad,
                                     cudaStream_t st)
{
    const long long G = (long long)gsize[0] * gsize[1] * gsize[2];
    if (G <= 0 || g.nfields <= 0) return cudaSuccess;
    if (G >= (1ll << 31) || g.nfields > 65535) return cudaErrorInvalidValue;
    const dim3 blocks(grid_for(G), (unsigned)g.nfields);
    k_field_gradient<<<blocks, 256, 0, st>>>(g, (unsigned)gsize[0], (unsigned)gsize[1], (unsigned)gsize[2], data,
                                             grad);
    return cudaGetLastError();
}

static bool geom_ok(int dimension, float resolution, const int64_t gsize[3], int nfields)
{
    if ((dimension != 2 && dimension != 3) || !(resolution > 0.0f) || !gsize || nfields < 1) return false;
    if (gsize[0] < 1 || gsize[1] < 1 || gsize[2] < 1) return false;
    if (dimension == 2 && gsize[2] != 1) return false;
    return true;
}

extern "C" int tm_env2cells(const double *x, const double *y, const double *z, int64_t n, int dimension,
                            const double lower[3], float resolution, const int64_t gsize[3], int nfields,
                            const double *data, const double *gradient, double *cellenv, void *stream)
{
    if (n < 0 || !lower || !geom_ok(dimension, resolution, gsize, nfields) || !data || !gradient || !cellenv)
        return TM_EINVAL;
    if (n > 0 && (!x || !y || !z)) return TM_EINVAL;
    const int64_t hi[3] = {gsize[0] - 1, gsize[1] - 1, dimension == 3 ? gsize[2] - 1 : 0};
    const int64_t lo[3] = {0, 0, 0};
    const tm_envgeom g = tm_make_envgeom(lower, resolution, hi, lo, gsize, nfields);
    return tm_launch_env2cells(g, x, y, z, n, data, gradient, cellenv, (cudaStream_t)stream) == cudaSuccess
               ? TM_OK
               : TM_ECUDA;
}

extern "C" int tm_field_gradient(const double *data, const int64_t gsize[3], float resolution, int nfields,
                                 double *gradient, void *stream)
{
    if (!data || !gradient || !geom_ok(gsize && gsize[2] == 1 ? 2 : 3, resolution, gsize, nfields))
        return TM_EINVAL;
    const tm_envgeom g = tm_make_envgeom(nullptr, resolution, nullptr, nullptr, gsize, nfields);
    return tm_launch_field_gradient(g, gsize, data, gradient, (cudaStream_t)stream) == cudaSuccess ? TM_OK
                                                                                                     : TM_ECUDA;
}
