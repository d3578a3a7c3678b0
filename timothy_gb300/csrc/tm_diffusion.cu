// Implicit diffusion step of environment_compute (environment.c:131-523) at
// one rank, on device fields (x-major, z fastest, FP64).
//
// Per field: z = dc * gfdt / (res * res) (the product res * res in float),
// the operator A u = (1 + 6 z + lambda dt) u_i - z * (sum of the in-grid
// neighbours), and numberofiters solves A u = u + faces + source per call,
// "faces" adding z * bc once for each grid face the node lies on, in the
// reference's order x-, x+, y-, y+, z-, z+ (a one-layer grid lies on both z
// faces).  The reference hands the system to Hypre's PCG with a BoomerAMG
// preconditioner (tolerance 1e-12, at most 50 iterations); here each solve
// reaches a relative FP64 residual |b - A u| / |b| <= tol.
//
// The FP64 pipe of this GPU is narrow, so a solve is iterative refinement:
// the residual r = b - A u and the update u += |r| d are FP64, and the
// correction d solves A d = r / |r| in FP32 by preconditioned conjugate
// gradients to a relative residual of 1e-5 (each refinement gains about five
// digits; the FP64 residual is the stopping test).  The inner preconditioner
// is a geometric multigrid V(1,1)-cycle in FP32 when the operator is stiff
// (condition bound (1 + 12 z + lambda dt) / (1 + lambda dt) above 30), the
// constant diagonal otherwise.
//
// Multigrid: coarsening n -> n / 2 along every axis with more than 3 nodes,
// coarse node I on fine node 2I + 1, so that the coarse grid's Dirichlet
// ghost below node 0 is the fine grid's (and, for odd n, the one above the
// last node too); the operator rediscretised per level (z_d / 4 along
// a coarsened axis), full weighting (the transpose of trilinear interpolation
// over 2^dc), red-black Gauss-Seidel (red then black before the coarse
// correction, black then red after it, so the cycle is symmetric), and on the
// coarsest grid (at most 3 nodes per axis) 64 Jacobi sweeps in one block.
// Errors live on homogeneous Dirichlet ghosts, as the fine operator's
// couplings to nodes outside the grid are absent.
//
// Reductions are deterministic: every reduction kernel runs on a fixed grid
// and writes one FP64 partial per block, and one block adds the partials in
// a fixed order; the CG scalars stay on the device.  The host reads a norm
// once per iteration for the stopping tests.
#include "tm_kernels.cuh"
#include "timothy_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

int tm_report(int code, const char *msg);

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 152 * 8;      // reduction grid (8 blocks of 256 per SM): partials per reduction
constexpr int kCoarseMax = 27;           // at most 3 nodes per axis on the coarsest grid
constexpr int kCoarseSweeps = 64;
constexpr double kInnerTol = 1e-5;       // relative residual of one FP32 correction solve
constexpr int kMaxRefine = 40;

struct level {
    unsigned nx, ny, nz;
    double zx, zy, zz;      // couplings along x, y, z
    double diag;
    float zxf, zyf, zzf, diagf, invf;   // FP32 copies for the FP32 kernels (set on the host: no FP64 per node)
    __host__ __device__ unsigned size() const { return nx * ny * nz; }
};

// scalars on the device: outer (FP64 residual) and inner (FP32 CG)
struct scalars {
    double bb, rr;                            // |b|^2, |b - A u|^2
    double rho, pq, alpha, beta, ss;          // inner CG
};

__device__ __forceinline__ void coords(const level &L, unsigned o, unsigned &i, unsigned &j, unsigned &k)
{
    const unsigned nyz = L.ny * L.nz;
    i = o / nyz;
    const unsigned r = o - i * nyz;
    j = r / L.nz;
    k = r - j * L.nz;
}

// in-grid neighbour sums along x, y, z
template <typename T>
__device__ __forceinline__ void nbsums(const level &L, const T *u, unsigned o, unsigned i, unsigned j, unsigned k,
                                       T &sx, T &sy, T &sz)
{
    const unsigned nyz = L.ny * L.nz;
    sx = T(0);
    sy = T(0);
    sz = T(0);
    if (i > 0) sx += u[o - nyz];
    if (i + 1 < L.nx) sx += u[o + nyz];
    if (j > 0) sy += u[o - L.nz];
    if (j + 1 < L.ny) sy += u[o + L.nz];
    if (k > 0) sz += u[o - 1];
    if (k + 1 < L.nz) sz += u[o + 1];
}

__device__ __forceinline__ float neighbours(const level &L, const float *u, unsigned o, unsigned i, unsigned j,
                                            unsigned k)
{
    float sx, sy, sz;
    nbsums(L, u, o, i, j, k, sx, sy, sz);
    return L.zxf * sx + L.zyf * sy + L.zzf * sz;
}

// block sum into partial[linear block index] (fixed order for a fixed
// launch; blocks of kThreads threads, of any 1-, 2- or 3-D shape)
__device__ __forceinline__ void block_partial(double v, double *partial)
{
    __shared__ double sh[kThreads / 32];
    const unsigned t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        v = t < kThreads / 32 ? sh[t] : 0.0;
        for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if (t == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = v;
    }
}

// FP32 sums of one thread, then FP64 across the block
__device__ __forceinline__ void block_partial32(float v, double *partial) { block_partial((double)v, partial); }

// ------------------------------------------------------------ FP64 outer

// b = u + faces + source; partials of b.b
__global__ void __launch_bounds__(kThreads) k_rhs(level L, const double *u, const double *src, double zb, double *b,
                                                  double *partial)
{
    double acc = 0.0;
    const unsigned G = L.size();
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(L, o, i, j, k);
        double v = u[o];
        if (i == 0) v += zb;
        if (i == L.nx - 1) v += zb;
        if (j == 0) v += zb;
        if (j == L.ny - 1) v += zb;
        if (k == 0) v += zb;
        if (k == L.nz - 1) v += zb;
        if (src) v += src[o];
        b[o] = v;
        acc += v * v;
    }
    block_partial(acc, partial);
}

// r = b - A u (the fine operator has one coupling z for every axis); partials
// of r.r.  FP64 instructions are the cost here: the neighbours outside the
// grid are selected away, not added as zeros (5 adds for the six), and the
// rest is two fused multiply-adds.
__global__ void __launch_bounds__(kThreads) k_residual64(level L, const double *u, const double *b, double *r,
                                                         double *partial)
{
    double acc = 0.0;
    const unsigned G = L.size(), nyz = L.ny * L.nz;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(L, o, i, j, k);
        const double xm = i > 0 ? u[o - nyz] : 0.0, xp = i + 1 < L.nx ? u[o + nyz] : 0.0;
        const double ym = j > 0 ? u[o - L.nz] : 0.0, yp = j + 1 < L.ny ? u[o + L.nz] : 0.0;
        const double zm = k > 0 ? u[o - 1] : 0.0, zp = k + 1 < L.nz ? u[o + 1] : 0.0;
        const double sn = ((xm + xp) + (ym + yp)) + (zm + zp);
        const double v = fma(-L.diag, u[o], fma(L.zx, sn, b[o]));
        r[o] = v;
        acc = fma(v, v, acc);
    }
    block_partial(acc, partial);
}

// s = r / |r| in FP32, d = 0
__global__ void __launch_bounds__(kThreads) k_scale32(unsigned G, const double *r, const scalars *sc, float *s,
                                                      float *d)
{
    const double inv = sc->rr > 0.0 ? 1.0 / sqrt(sc->rr) : 0.0;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        s[o] = (float)(r[o] * inv);
        d[o] = 0.0f;
    }
}

// u += |r| d
__global__ void __launch_bounds__(kThreads) k_correct64(unsigned G, double *u, const float *d, const scalars *sc)
{
    const double nr = sqrt(sc->rr);
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x)
        u[o] += nr * (double)d[o];
}

// ------------------------------------------------------------ FP32 inner CG

// q = A p; partials of p.q; blocks over (z, y), each thread walks x in
// steps of gridDim.z (no coordinate division; a fixed number of partials)
__global__ void __launch_bounds__(kThreads) k_apply_dot32(level L, const float *p, float *q, double *partial)
{
    float acc = 0.0f;
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (k < L.nz && j < L.ny)
        for (unsigned i = blockIdx.z; i < L.nx; i += gridDim.z) {
            const unsigned o = (i * L.ny + j) * L.nz + k;
            const float v = L.diagf * p[o] - neighbours(L, p, o, i, j, k);
            q[o] = v;
            acc = fmaf(p[o], v, acc);
        }
    block_partial32(acc, partial);
}

// d += alpha p; s -= alpha q; partials of s.s
__global__ void __launch_bounds__(kThreads) k_update32(unsigned G, float *d, float *s, const float *p, const float *q,
                                                       const scalars *sc, double *partial)
{
    const float a = (float)sc->alpha;
    float acc = 0.0f;
    // four nodes per access (the vectors are 256-byte aligned), the tail singly
    const unsigned G4 = G / 4, stride = gridDim.x * blockDim.x;
    float4 *d4 = (float4 *)d, *s4 = (float4 *)s;
    const float4 *p4 = (const float4 *)p, *q4 = (const float4 *)q;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G4; o += stride) {
        float4 dv = d4[o], sv = s4[o];
        const float4 pv = p4[o], qv = q4[o];
        dv.x = fmaf(a, pv.x, dv.x);
        dv.y = fmaf(a, pv.y, dv.y);
        dv.z = fmaf(a, pv.z, dv.z);
        dv.w = fmaf(a, pv.w, dv.w);
        sv.x = fmaf(-a, qv.x, sv.x);
        sv.y = fmaf(-a, qv.y, sv.y);
        sv.z = fmaf(-a, qv.z, sv.z);
        sv.w = fmaf(-a, qv.w, sv.w);
        d4[o] = dv;
        s4[o] = sv;
        acc = fmaf(sv.x, sv.x, fmaf(sv.y, sv.y, fmaf(sv.z, sv.z, fmaf(sv.w, sv.w, acc))));
    }
    for (unsigned o = 4 * G4 + blockIdx.x * blockDim.x + threadIdx.x; o < G; o += stride) {
        d[o] = fmaf(a, p[o], d[o]);
        const float v = fmaf(-a, q[o], s[o]);
        s[o] = v;
        acc = fmaf(v, v, acc);
    }
    block_partial32(acc, partial);
}

// p = zv + beta p (first: p = zv); four nodes per access, the tail singly
__global__ void __launch_bounds__(kThreads) k_direction32(unsigned G, float *p, const float *zv, const scalars *sc,
                                                          int first)
{
    const float be = first ? 0.0f : (float)sc->beta;
    const unsigned G4 = G / 4, stride = gridDim.x * blockDim.x;
    float4 *p4 = (float4 *)p;
    const float4 *z4 = (const float4 *)zv;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G4; o += stride) {
        const float4 z = z4[o];
        if (first) {
            p4[o] = z;
        } else {
            float4 v = p4[o];
            v.x = fmaf(be, v.x, z.x);
            v.y = fmaf(be, v.y, z.y);
            v.z = fmaf(be, v.z, z.z);
            v.w = fmaf(be, v.w, z.w);
            p4[o] = v;
        }
    }
    for (unsigned o = 4 * G4 + blockIdx.x * blockDim.x + threadIdx.x; o < G; o += stride)
        p[o] = first ? zv[o] : fmaf(be, p[o], zv[o]);
}

// zv = s / diag; partials of s.zv
__global__ void __launch_bounds__(kThreads) k_jacobi_dot32(unsigned G, const float *s, float *zv, float inv_diag,
                                                           double *partial)
{
    float acc = 0.0f;
    const unsigned G4 = G / 4, stride = gridDim.x * blockDim.x;
    const float4 *s4 = (const float4 *)s;
    float4 *z4 = (float4 *)zv;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G4; o += stride) {
        const float4 a = s4[o];
        const float4 v = make_float4(a.x * inv_diag, a.y * inv_diag, a.z * inv_diag, a.w * inv_diag);
        z4[o] = v;
        acc = fmaf(a.x, v.x, fmaf(a.y, v.y, fmaf(a.z, v.z, fmaf(a.w, v.w, acc))));
    }
    for (unsigned o = 4 * G4 + blockIdx.x * blockDim.x + threadIdx.x; o < G; o += stride) {
        const float v = s[o] * inv_diag;
        zv[o] = v;
        acc = fmaf(s[o], v, acc);
    }
    block_partial32(acc, partial);
}

// partials of x.y (FP32 vectors)
__global__ void __launch_bounds__(kThreads) k_dot32(unsigned G, const float *x, const float *y, double *partial)
{
    float acc = 0.0f;
    const unsigned G4 = G / 4, stride = gridDim.x * blockDim.x;
    const float4 *x4 = (const float4 *)x, *y4 = (const float4 *)y;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G4; o += stride) {
        const float4 a = x4[o], b = y4[o];
        acc = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc))));
    }
    for (unsigned o = 4 * G4 + blockIdx.x * blockDim.x + threadIdx.x; o < G; o += stride) acc = fmaf(x[o], y[o], acc);
    block_partial32(acc, partial);
}

// one block adds the partials in a fixed order and updates the scalars:
// 0: bb; 1: rr; 2: pq -> alpha; 3: ss; 4: rho (first); 5: rho -> beta
__global__ void __launch_bounds__(kThreads) k_finish(const double *partial, int n, scalars *sc, int what)
{
    double v = 0.0;
    for (int b = threadIdx.x; b < n; b += blockDim.x) v += partial[b];
    __shared__ double sh[kThreads];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double t = sh[0];
    switch (what) {
    case 0: sc->bb = t; break;
    case 1: sc->rr = t; break;
    case 2:
        sc->pq = t;
        sc->alpha = t != 0.0 ? sc->rho / t : 0.0;
        break;
    case 3: sc->ss = t; break;
    case 4: sc->rho = t; break;
    case 5:
        sc->beta = sc->rho != 0.0 ? t / sc->rho : 0.0;
        sc->rho = t;
        break;
    }
}

// ---------------------------------------------------------------- multigrid (FP32)

// The stencil kernels of the V-cycle run one thread per node on a 3-D grid:
// blocks of 256 threads over (z, y), blockIdx.z = x, so no thread divides
// to find its node (see shape3).
__device__ __forceinline__ bool node3(const level &L, unsigned &i, unsigned &j, unsigned &k)
{
    k = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    i = blockIdx.z;
    return k < L.nz && j < L.ny;
}

// Gauss-Seidel on the nodes of one colour ((i + j + k) & 1 == colour): a
// thread per node of the colour, two z positions per thread index
__global__ void __launch_bounds__(kThreads) k_rbgs(level L, float *e, const float *f, int colour)
{
    const unsigned kk = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y,
                   i = blockIdx.z;
    const unsigned k = 2 * kk + ((i + j + (unsigned)colour) & 1u);
    if (k >= L.nz || j >= L.ny) return;
    const unsigned o = (i * L.ny + j) * L.nz + k;
    e[o] = (f[o] + neighbours(L, e, o, i, j, k)) * L.invf;
}

// the first half-sweep from e = 0: red nodes e = f / diag (their neighbours
// are zero), black nodes 0
__global__ void __launch_bounds__(kThreads) k_rbgs_first(level L, float *e, const float *f)
{
    unsigned i, j, k;
    if (!node3(L, i, j, k)) return;
    const unsigned o = (i * L.ny + j) * L.nz + k;
    e[o] = ((i + j + k) & 1u) ? 0.0f : f[o] * L.invf;
}

// res = f - A e
__global__ void __launch_bounds__(kThreads) k_residual32(level L, const float *e, const float *f, float *res)
{
    unsigned i, j, k;
    if (!node3(L, i, j, k)) return;
    const unsigned o = (i * L.ny + j) * L.nz + k;
    res[o] = f[o] - (L.diagf * e[o] - neighbours(L, e, o, i, j, k));
}

// Restriction taps of coarse index I along an axis: the coarse node sits on
// fine node 2I + 1 (weight 1) with its fine neighbours 2I and 2I + 2 at half
// weight; the last one is a Dirichlet ghost on a grid of odd size (weight 0,
// index clamped).  An axis that is not coarsened has the single tap I.
__device__ __forceinline__ void rtaps(unsigned I, unsigned nf, bool coarse, unsigned t[3], float w[3])
{
    if (!coarse) {
        t[0] = t[1] = t[2] = I;
        w[0] = 1.0f;
        w[1] = w[2] = 0.0f;
        return;
    }
    const unsigned c = 2 * I + 1;        // < nf: I < nf / 2
    t[0] = c;
    w[0] = 1.0f;
    t[1] = c - 1;
    w[1] = 0.5f;
    const bool has = c + 1 < nf;
    t[2] = has ? c + 1 : c;
    w[2] = has ? 0.5f : 0.0f;
}

// f_c = R res_f (the transpose of interpolation over 2^dc); one thread per
// coarse node, 27 fixed taps (absent ones weigh 0)
__global__ void __launch_bounds__(kThreads) k_restrict(level Lf, level Lc, const float *res, float *fc, float scale)
{
    unsigned I, J, K;
    if (!node3(Lc, I, J, K)) return;
    unsigned tx[3], ty[3], tz[3];
    float wx[3], wy[3], wz[3];
    rtaps(I, Lf.nx, Lc.nx != Lf.nx, tx, wx);
    rtaps(J, Lf.ny, Lc.ny != Lf.ny, ty, wy);
    rtaps(K, Lf.nz, Lc.nz != Lf.nz, tz, wz);
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const float wab = wx[a] * wy[b];
            const float *row = res + (tx[a] * Lf.ny + ty[b]) * Lf.nz;
#pragma unroll
            for (int c = 0; c < 3; c++) s = fmaf(wab * wz[c], row[tz[c]], s);
        }
    fc[(I * Lc.ny + J) * Lc.nz + K] = s * scale;
}

// Interpolation taps of fine index f along an axis (the transpose of rtaps):
// an odd f is coarse node (f - 1) / 2; an even f lies between coarse nodes
// f / 2 - 1 and f / 2, each at half weight, either of which may be a ghost
// (weight 0, index clamped)
__device__ __forceinline__ void ptaps(unsigned f, unsigned nc, bool coarse, unsigned t[2], float w[2])
{
    if (!coarse) {
        t[0] = t[1] = f;
        w[0] = 1.0f;
        w[1] = 0.0f;
        return;
    }
    if (f & 1u) {
        t[0] = t[1] = f >> 1;            // < nc
        w[0] = 1.0f;
        w[1] = 0.0f;
        return;
    }
    const unsigned hi = f >> 1;
    const bool has_lo = hi >= 1, has_hi = hi < nc;
    t[0] = has_lo ? hi - 1 : 0;
    w[0] = has_lo ? 0.5f : 0.0f;
    t[1] = has_hi ? hi : (has_lo ? hi - 1 : 0);
    w[1] = has_hi ? 0.5f : 0.0f;
}

// e_f += P e_c; one thread per fine node, 8 fixed taps
__global__ void __launch_bounds__(kThreads) k_prolong(level Lf, level Lc, const float *ec, float *ef)
{
    unsigned i, j, k;
    if (!node3(Lf, i, j, k)) return;
    unsigned tx[2], ty[2], tz[2];
    float wx[2], wy[2], wz[2];
    ptaps(i, Lc.nx, Lc.nx != Lf.nx, tx, wx);
    ptaps(j, Lc.ny, Lc.ny != Lf.ny, ty, wy);
    ptaps(k, Lc.nz, Lc.nz != Lf.nz, tz, wz);
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
            const float wab = wx[a] * wy[b];
            const float *row = ec + (tx[a] * Lc.ny + ty[b]) * Lc.nz;
#pragma unroll
            for (int c = 0; c < 2; c++) s = fmaf(wab * wz[c], row[tz[c]], s);
        }
    ef[(i * Lf.ny + j) * Lf.nz + k] += s;
}

// the coarsest grid (at most kCoarseMax nodes): Jacobi sweeps from zero in one block
__global__ void __launch_bounds__(32) k_coarse(level L, float *e, const float *f)
{
    __shared__ float a[kCoarseMax], b[kCoarseMax];
    const unsigned G = L.size();
    const unsigned o = threadIdx.x;
    if (o < G) a[o] = 0.0f;
    __syncthreads();
    float *cur = a, *nxt = b;
    const float inv = L.invf;
    for (int s = 0; s < kCoarseSweeps; s++) {
        if (o < G) {
            unsigned i, j, k;
            coords(L, o, i, j, k);
            nxt[o] = (f[o] + neighbours(L, (const float *)cur, o, i, j, k)) * inv;
        }
        __syncthreads();
        float *t = cur;
        cur = nxt;
        nxt = t;
    }
    if (o < G) e[o] = cur[o];
}

unsigned blocks_for(unsigned G)
{
    const unsigned b = (G + kThreads - 1) / kThreads;
    return b < 152u * 8u ? (b ? b : 1u) : 152u * 8u;
}

// launch shape of a 3-D stencil kernel over nx x ny x nzw threads: blocks
// of 256 threads over (z, y), z-width the power of two covering nzw (at most
// 32), blockIdx.z = x
struct shape3 {
    dim3 grid, block;
};

shape3 shape_of(unsigned nx, unsigned ny, unsigned nzw)
{
    unsigned bx = 1;
    while (bx < nzw && bx < 32) bx <<= 1;
    const unsigned by = kThreads / bx;
    return {dim3((nzw + bx - 1) / bx, (ny + by - 1) / by, nx), dim3(bx, by, 1)};
}

// column kernel (k_apply_dot32): the (z, y) blocks of
// shape_of, and as many x-slices as keep the blocks near kRedBlocks
shape3 column_shape(unsigned nx, unsigned ny, unsigned nz)
{
    shape3 sh = shape_of(nx, ny, nz);
    const unsigned plane = sh.grid.x * sh.grid.y;
    unsigned gz = plane >= (unsigned)kRedBlocks ? 1u : (unsigned)kRedBlocks / plane;
    sh.grid.z = gz < nx ? gz : nx;
    return sh;
}

// partials a reduction over level L0 writes at most
size_t partial_count(const level &L0)
{
    const shape3 cs = column_shape(L0.nx, L0.ny, L0.nz);
    const size_t cn = (size_t)cs.grid.x * cs.grid.y * cs.grid.z;
    return cn > (size_t)kRedBlocks ? cn : (size_t)kRedBlocks;
}

unsigned red_blocks(unsigned G)
{
    const unsigned b = blocks_for(G);
    return b < (unsigned)kRedBlocks ? b : (unsigned)kRedBlocks;
}

}  // namespace

struct tm_diffusion {
    int device = 0;
    int64_t gsize[3] = {0, 0, 0};
    std::vector<level> lv;              // geometry of the levels (couplings set per solve)
    std::vector<float *> e, f, res;     // per level (level 0: the inner CG's vectors)
    double *b = nullptr, *r = nullptr;  // FP64 right-hand side and residual
    float *s = nullptr, *d = nullptr, *p = nullptr, *q = nullptr, *zv = nullptr;   // FP32 inner CG
    double *partial = nullptr;
    scalars *sc = nullptr;
    scalars *h_sc = nullptr;            // page-locked copy for the stopping tests
    double *field = nullptr;            // the drop-in's fields and source (nfields x G)
    double *src = nullptr;
    int field_n = 0;
};

#define DK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            char m_[256];                                                                         \
            snprintf(m_, sizeof m_, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return tm_report(TM_ECUDA, m_);                                                       \
        }                                                                                         \
    } while (0)

static void diffusion_free(tm_diffusion *d)
{
    for (float *v : d->e) cudaFree(v);
    for (float *v : d->f) cudaFree(v);
    for (float *v : d->res) cudaFree(v);
    cudaFree(d->b);
    cudaFree(d->r);
    cudaFree(d->s);
    cudaFree(d->d);
    cudaFree(d->p);
    cudaFree(d->q);
    cudaFree(d->zv);
    cudaFree(d->partial);
    cudaFree(d->sc);
    cudaFree(d->field);
    cudaFree(d->src);
    if (d->h_sc) cudaFreeHost(d->h_sc);
}

extern "C" int tm_diffusion_create(tm_diffusion **out, const int64_t gsize[3], int device)
{
    if (!out || !gsize) return tm_report(TM_EINVAL, "null argument");
    *out = nullptr;
    if (gsize[0] < 1 || gsize[1] < 1 || gsize[2] < 1) return tm_report(TM_EINVAL, "grid sizes must be >= 1");
    const long long G = (long long)gsize[0] * gsize[1] * gsize[2];
    if (G >= (1ll << 31)) return tm_report(TM_EINVAL, "grid above 2^31 nodes");
    if (gsize[0] > 65535 || gsize[1] > 65535 * 8) return tm_report(TM_EINVAL, "grid axis too long for the launch shape");
    DK(cudaSetDevice(device));
    tm_diffusion *d = new tm_diffusion();
    d->device = device;
    for (int a = 0; a < 3; a++) d->gsize[a] = gsize[a];
    level L{(unsigned)gsize[0], (unsigned)gsize[1], (unsigned)gsize[2], 0, 0, 0, 0};
    d->lv.push_back(L);
    while (L.nx > 3 || L.ny > 3 || L.nz > 3) {
        L.nx = L.nx > 3 ? L.nx / 2 : L.nx;
        L.ny = L.ny > 3 ? L.ny / 2 : L.ny;
        L.nz = L.nz > 3 ? L.nz / 2 : L.nz;
        d->lv.push_back(L);
    }
    auto a64 = [&](double **p, size_t n) { return cudaMalloc((void **)p, n * sizeof(double)) == cudaSuccess; };
    auto a32 = [&](float **p, size_t n) { return cudaMalloc((void **)p, n * sizeof(float)) == cudaSuccess; };
    bool ok = true;
    const size_t n0 = (size_t)G;
    ok = ok && a64(&d->b, n0) && a64(&d->r, n0);
    ok = ok && a32(&d->s, n0) && a32(&d->d, n0) && a32(&d->p, n0) && a32(&d->q, n0) && a32(&d->zv, n0);
    ok = ok && a64(&d->partial, partial_count(d->lv[0]));
    ok = ok && cudaMalloc((void **)&d->sc, sizeof(scalars)) == cudaSuccess;
    ok = ok && cudaMallocHost((void **)&d->h_sc, sizeof(scalars)) == cudaSuccess;
    d->e.assign(d->lv.size(), nullptr);
    d->f.assign(d->lv.size(), nullptr);
    d->res.assign(d->lv.size(), nullptr);
    for (size_t l = 0; ok && l < d->lv.size(); l++) {
        const size_t n = d->lv[l].size();
        if (l > 0) ok = a32(&d->e[l], n) && a32(&d->f[l], n);
        if (ok && l + 1 < d->lv.size()) ok = a32(&d->res[l], n);
    }
    if (!ok) {
        diffusion_free(d);
        delete d;
        cudaGetLastError();
        return tm_report(TM_ENOMEM, "device allocation for the diffusion solver failed");
    }
    *out = d;
    return TM_OK;
}

extern "C" int tm_diffusion_destroy(tm_diffusion *d)
{
    if (!d) return TM_OK;
    cudaSetDevice(d->device);
    diffusion_free(d);
    delete d;
    return TM_OK;
}

extern "C" int tm_diffusion_levels(const tm_diffusion *d) { return d ? (int)d->lv.size() : 0; }

// the V-cycle applied to the inner residual s (level 0) into zv
static int vcycle(tm_diffusion *d, const std::vector<level> &lv, cudaStream_t st)
{
    const int nl = (int)lv.size();
    std::vector<float *> E(nl), F(nl);
    E[0] = d->zv;
    F[0] = d->s;
    for (int l = 1; l < nl; l++) {
        E[l] = d->e[l];
        F[l] = d->f[l];
    }
    for (int l = 0; l + 1 < nl; l++) {
        const level &L = lv[l];
        const shape3 full = shape_of(L.nx, L.ny, L.nz), half = shape_of(L.nx, L.ny, (L.nz + 1) / 2);
        k_rbgs_first<<<full.grid, full.block, 0, st>>>(L, E[l], F[l]);
        k_rbgs<<<half.grid, half.block, 0, st>>>(L, E[l], F[l], 1);
        k_residual32<<<full.grid, full.block, 0, st>>>(L, E[l], F[l], d->res[l]);
        const level &C = lv[l + 1];
        const int dc = (C.nx != L.nx) + (C.ny != L.ny) + (C.nz != L.nz);
        const shape3 cs = shape_of(C.nx, C.ny, C.nz);
        k_restrict<<<cs.grid, cs.block, 0, st>>>(L, C, d->res[l], F[l + 1], 1.0f / (float)(1 << dc));
    }
    k_coarse<<<1, 32, 0, st>>>(lv[nl - 1], E[nl - 1], F[nl - 1]);
    for (int l = nl - 2; l >= 0; l--) {
        const level &L = lv[l];
        const shape3 full = shape_of(L.nx, L.ny, L.nz), half = shape_of(L.nx, L.ny, (L.nz + 1) / 2);
        k_prolong<<<full.grid, full.block, 0, st>>>(L, lv[l + 1], E[l + 1], E[l]);
        k_rbgs<<<half.grid, half.block, 0, st>>>(L, E[l], F[l], 1);
        k_rbgs<<<half.grid, half.block, 0, st>>>(L, E[l], F[l], 0);
    }
    DK(cudaGetLastError());
    return TM_OK;
}

static int read_scalars(tm_diffusion *d, cudaStream_t st)
{
    DK(cudaMemcpyAsync(d->h_sc, d->sc, sizeof(scalars), cudaMemcpyDeviceToHost, st));
    DK(cudaStreamSynchronize(st));
    return TM_OK;
}

// A d = s (|s| = 1) in FP32 by PCG to a relative residual of kInnerTol; returns iterations
static int inner_pcg(tm_diffusion *d, const std::vector<level> &lv, bool mg, int max_iter, cudaStream_t st,
                     int *iters)
{
    const level &L0 = lv[0];
    const unsigned G = L0.size(), rb = red_blocks(G), gb = blocks_for(G);
    const shape3 cs = column_shape(L0.nx, L0.ny, L0.nz);
    const int cn = (int)(cs.grid.x * cs.grid.y * cs.grid.z);
    const float inv_diag = (float)(1.0 / L0.diag);
    int rc, it = 0;
    for (; it < max_iter; it++) {
        if (mg) {
            if ((rc = vcycle(d, lv, st))) return rc;
            k_dot32<<<rb, kThreads, 0, st>>>(G, d->s, d->zv, d->partial);
        } else {
            k_jacobi_dot32<<<rb, kThreads, 0, st>>>(G, d->s, d->zv, inv_diag, d->partial);
        }
        k_finish<<<1, kThreads, 0, st>>>(d->partial, rb, d->sc, it == 0 ? 4 : 5);
        k_direction32<<<gb, kThreads, 0, st>>>(G, d->p, d->zv, d->sc, it == 0);
        k_apply_dot32<<<cs.grid, cs.block, 0, st>>>(L0, d->p, d->q, d->partial);
        k_finish<<<1, kThreads, 0, st>>>(d->partial, cn, d->sc, 2);
        k_update32<<<rb, kThreads, 0, st>>>(G, d->d, d->s, d->p, d->q, d->sc, d->partial);
        k_finish<<<1, kThreads, 0, st>>>(d->partial, rb, d->sc, 3);
        DK(cudaGetLastError());
        if ((rc = read_scalars(d, st))) return rc;
        if (!(d->h_sc->ss > kInnerTol * kInnerTol)) {      // also stops on a NaN
            it++;
            break;
        }
    }
    *iters = it;
    return TM_OK;
}

// one solve A u = b (b in d->b) by iterative refinement
static int solve(tm_diffusion *d, const std::vector<level> &lv, double *u, double tol, bool mg, cudaStream_t st,
                 int *inner, int *refinements, double *relres)
{
    const level &L0 = lv[0];
    const unsigned G = L0.size(), rb = red_blocks(G), gb = blocks_for(G);
    int rc;
    *inner = 0;
    *refinements = 0;
    double rel = 0.0;
    for (int k = 0; k <= kMaxRefine; k++) {
        k_residual64<<<rb, kThreads, 0, st>>>(L0, u, d->b, d->r, d->partial);
        k_finish<<<1, kThreads, 0, st>>>(d->partial, rb, d->sc, 1);
        DK(cudaGetLastError());
        if ((rc = read_scalars(d, st))) return rc;
        const double bb = d->h_sc->bb, rr = d->h_sc->rr;
        rel = bb > 0.0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (rr <= tol * tol * bb || rr == 0.0 || k == kMaxRefine) break;
        k_scale32<<<gb, kThreads, 0, st>>>(G, d->r, d->sc, d->s, d->d);
        int n = 0;
        if ((rc = inner_pcg(d, lv, mg, mg ? 60 : 400, st, &n))) return rc;
        k_correct64<<<gb, kThreads, 0, st>>>(G, u, d->d, d->sc);
        *inner += n;
        (*refinements)++;
    }
    *relres = rel;
    return TM_OK;
}

extern "C" int tm_diffusion_step(tm_diffusion *d, double *data, float resolution, int nfields, const double *dc,
                                 const double *bc, const double *lambda, float secondsperstep, float gfdt,
                                 const double *source, double tol, tm_diffusion_stats *stats, void *stream)
{
    if (!d || !data || !dc || !bc || !lambda || nfields < 1) return tm_report(TM_EINVAL, "null argument or no field");
    if (!(resolution > 0.0f) || !(gfdt > 0.0f) || !(tol > 0.0)) return tm_report(TM_EINVAL, "bad step parameters");
    DK(cudaSetDevice(d->device));
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned G = d->lv[0].size();
    // solves per step (environment.c:144-164, float arithmetic as there)
    int iters = 1;
    if ((secondsperstep / gfdt) > 1) {
        const int intdiv = (int)(secondsperstep / gfdt) + 1;
        const float a1 = secondsperstep / intdiv;
        const float a2 = secondsperstep / (intdiv - 1);
        iters = (gfdt - a1) < (a2 - gfdt) ? intdiv : intdiv - 1;
    }
    tm_diffusion_stats S;
    memset(&S, 0, sizeof S);
    S.solves_per_field = iters;
    S.levels = (int)d->lv.size();
    const double dt = gfdt;
    const float r2 = resolution * resolution;
    for (int fi = 0; fi < nfields; fi++) {
        const double z = dc[fi] * dt / r2;
        const double diag = 1 + 6.0 * z + lambda[fi] * dt, zb = z * bc[fi];
        const double c0 = diag - 6.0 * z;
        const bool mg = !(c0 > 0.0) || (diag + 6.0 * z) > 30.0 * c0;
        std::vector<level> lv = d->lv;
        for (size_t l = 0; l < lv.size(); l++) {
            level &L = lv[l];
            if (l == 0) {
                L.zx = L.zy = L.zz = z;
                L.diag = diag;
            } else {
                const level &P = lv[l - 1];
                L.zx = P.zx * (L.nx != P.nx ? 0.25 : 1.0);
                L.zy = P.zy * (L.ny != P.ny ? 0.25 : 1.0);
                L.zz = P.zz * (L.nz != P.nz ? 0.25 : 1.0);
                L.diag = c0 + 2.0 * (L.zx + L.zy + L.zz);
            }
            L.zxf = (float)L.zx;
            L.zyf = (float)L.zy;
            L.zzf = (float)L.zz;
            L.diagf = (float)L.diag;
            L.invf = (float)(1.0 / L.diag);
        }
        if (mg) S.multigrid_fields++;
        double *u = data + (size_t)fi * G;
        const double *src = source ? source + (size_t)fi * G : nullptr;
        const unsigned rb = red_blocks(G);
        for (int s = 0; s < iters; s++) {
            k_rhs<<<rb, kThreads, 0, st>>>(lv[0], u, src, zb, d->b, d->partial);
            k_finish<<<1, kThreads, 0, st>>>(d->partial, rb, d->sc, 0);
            DK(cudaGetLastError());
            int n = 0, nref = 0;
            double rel = 0.0;
            int rc = solve(d, lv, u, tol, mg, st, &n, &nref, &rel);
            if (rc) return rc;
            S.iterations += n;
            S.refinements += nref;
            if (n > S.max_iterations) S.max_iterations = n;
            if (rel > S.max_relative_residual) S.max_relative_residual = rel;
        }
    }
    if (stats) *stats = S;
    return TM_OK;
}

extern "C" int tm_field_diffuse(double *data, const int64_t gsize[3], float resolution, int nfields, const double *dc,
                                const double *bc, const double *lambda, float secondsperstep, float gfdt,
                                const double *source, double tol, tm_diffusion_stats *stats, void *stream)
{
    int dev = 0;
    DK(cudaGetDevice(&dev));
    tm_diffusion *d = nullptr;
    int rc = tm_diffusion_create(&d, gsize, dev);
    if (rc) return rc;
    rc = tm_diffusion_step(d, data, resolution, nfields, dc, bc, lambda, secondsperstep, gfdt, source, tol, stats,
                           stream);
    if (rc == TM_OK) {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess) rc = tm_report(TM_ECUDA, cudaGetErrorString(e));
    }
    tm_diffusion_destroy(d);
    return rc;
}

// ---------------------------------------------------------------------------
// drop-in environment_compute at one rank: every field starts from its
// initialconditionmean (a new solution vector per call, environment.c:298-316)
// with the point source of environment_pcfunction (100 at node (5, 5, 5) from
// step 1 on, environment.c:251-266); the solution stays on the device

__global__ void k_env_start(unsigned G, int nf, const double *mean, double *u)
{
    const long long n = (long long)G * nf;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x)
        u[o] = mean[o / G];
}

extern "C" int tmi_env_compute(tm_diffusion *d, int nfields, const double *mean, const double *dc, const double *bc,
                               const double *lambda, float resolution, float secondsperstep, float gfdt, int step,
                               tm_diffusion_stats *stats)
{
    if (!d || nfields < 1 || nfields > 64) return tm_report(TM_EINVAL, "bad field count");
    DK(cudaSetDevice(d->device));
    const unsigned G = d->lv[0].size();
    if (d->field_n < nfields) {
        cudaFree(d->field);
        cudaFree(d->src);
        d->field = d->src = nullptr;
        d->field_n = 0;
        DK(cudaMalloc((void **)&d->field, (size_t)nfields * G * sizeof(double)));
        DK(cudaMalloc((void **)&d->src, (size_t)nfields * G * sizeof(double) + 64 * sizeof(double)));
        d->field_n = nfields;
    }
    double *dmean = d->src + (size_t)nfields * G;      // 64 doubles after the source
    DK(cudaMemcpy(dmean, mean, (size_t)nfields * sizeof(double), cudaMemcpyHostToDevice));
    k_env_start<<<blocks_for(G), kThreads>>>(G, nfields, dmean, d->field);
    DK(cudaGetLastError());
    DK(cudaMemset(d->src, 0, (size_t)nfields * G * sizeof(double)));
    const level &L = d->lv[0];
    if (step != 0 && L.nx > 5 && L.ny > 5 && L.nz > 5) {
        const double v = 100.0;
        const size_t node = ((size_t)5 * L.ny + 5) * L.nz + 5;
        for (int f = 0; f < nfields; f++)
            DK(cudaMemcpy(d->src + (size_t)f * G + node, &v, sizeof v, cudaMemcpyHostToDevice));
    }
    DK(cudaDeviceSynchronize());
    int rc = tm_diffusion_step(d, d->field, resolution, nfields, dc, bc, lambda, secondsperstep, gfdt, d->src, 1e-12,
                               stats, nullptr);
    if (rc) return rc;
    DK(cudaStreamSynchronize(nullptr));
    return TM_OK;
}

// field f of the last tmi_env_compute into host memory (G values, z fastest)
extern "C" int tmi_env_solution(tm_diffusion *d, int f, double *host)
{
    if (!d || !d->field || f < 0 || f >= d->field_n || !host) return tm_report(TM_EINVAL, "no such field");
    DK(cudaSetDevice(d->device));
    const size_t G = d->lv[0].size();
    DK(cudaMemcpy(host, d->field + (size_t)f * G, G * sizeof(double), cudaMemcpyDeviceToHost));
    return TM_OK;
}
