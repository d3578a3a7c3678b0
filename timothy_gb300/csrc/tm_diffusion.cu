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
constexpr int kRedBlocks = 152 * 4;      // reduction grid: partials per reduction
constexpr int kCoarseMax = 27;           // at most 3 nodes per axis on the coarsest grid
constexpr int kCoarseSweeps = 64;
constexpr double kInnerTol = 1e-5;       // relative residual of one FP32 correction solve
constexpr int kMaxRefine = 40;

struct level {
    unsigned nx, ny, nz;
    double zx, zy, zz;      // couplings along x, y, z
    double diag;
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

template <typename T>
__device__ __forceinline__ T neighbours(const level &L, const T *u, unsigned o, unsigned i, unsigned j, unsigned k)
{
    T sx, sy, sz;
    nbsums(L, u, o, i, j, k, sx, sy, sz);
    return T(L.zx) * sx + T(L.zy) * sy + T(L.zz) * sz;
}

// block sum into partial[blockIdx.x] (fixed order for a fixed launch)
__device__ __forceinline__ void block_partial(double v, double *partial)
{
    __shared__ double sh[kThreads / 32];
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
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
        const double s = ((xm + xp) + (ym + yp)) + (zm + zp);
        const double v = fma(-L.diag, u[o], fma(L.zx, s, b[o]));
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

// q = A p; partials of p.q
__global__ void __launch_bounds__(kThreads) k_apply_dot32(level L, const float *p, float *q, double *partial)
{
    float acc = 0.0f;
    const unsigned G = L.size();
    const float dg = (float)L.diag;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(L, o, i, j, k);
        const float v = dg * p[o] - neighbours(L, p, o, i, j, k);
        q[o] = v;
        acc += p[o] * v;
    }
    block_partial32(acc, partial);
}

// d += alpha p; s -= alpha q; partials of s.s
__global__ void __launch_bounds__(kThreads) k_update32(unsigned G, float *d, float *s, const float *p, const float *q,
                                                       const scalars *sc, double *partial)
{
    const float a = (float)sc->alpha;
    float acc = 0.0f;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        d[o] += a * p[o];
        const float v = s[o] - a * q[o];
        s[o] = v;
        acc += v * v;
    }
    block_partial32(acc, partial);
}

// p = zv + beta p (first: p = zv)
__global__ void __launch_bounds__(kThreads) k_direction32(unsigned G, float *p, const float *zv, const scalars *sc,
                                                          int first)
{
    const float be = first ? 0.0f : (float)sc->beta;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x)
        p[o] = first ? zv[o] : zv[o] + be * p[o];
}

// zv = s / diag; partials of s.zv
__global__ void __launch_bounds__(kThreads) k_jacobi_dot32(unsigned G, const float *s, float *zv, float inv_diag,
                                                           double *partial)
{
    float acc = 0.0f;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        const float v = s[o] * inv_diag;
        zv[o] = v;
        acc += s[o] * v;
    }
    block_partial32(acc, partial);
}

// partials of x.y (FP32 vectors)
__global__ void __launch_bounds__(kThreads) k_dot32(unsigned G, const float *x, const float *y, double *partial)
{
    float acc = 0.0f;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) acc += x[o] * y[o];
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

__global__ void __launch_bounds__(kThreads) k_zero(unsigned G, float *e)
{
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) e[o] = 0.0f;
}

// Gauss-Seidel on the nodes of one colour ((i + j + k) & 1 == colour)
__global__ void __launch_bounds__(kThreads) k_rbgs(level L, float *e, const float *f, int colour)
{
    const unsigned G = L.size();
    const float inv = (float)(1.0 / L.diag);
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(L, o, i, j, k);
        if (((i + j + k) & 1u) != (unsigned)colour) continue;
        e[o] = (f[o] + neighbours(L, e, o, i, j, k)) * inv;
    }
}

// res = f - A e
__global__ void __launch_bounds__(kThreads) k_residual32(level L, const float *e, const float *f, float *res)
{
    const unsigned G = L.size();
    const float dg = (float)L.diag;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(L, o, i, j, k);
        res[o] = f[o] - (dg * e[o] - neighbours(L, e, o, i, j, k));
    }
}

// fine indices and weights restricting to coarse index I along an axis: the
// coarse node sits on fine node 2I + 1 and takes its two fine neighbours at
// half weight (the first fine node's other coarse neighbour, and the last's
// on a grid of odd size, are the Dirichlet ghosts)
__device__ __forceinline__ void axis_taps(unsigned I, unsigned nf, bool coarse, unsigned *idx, float *w, int &n)
{
    if (!coarse) {
        idx[0] = I;
        w[0] = 1.0f;
        n = 1;
        return;
    }
    const unsigned c = 2 * I + 1;       // < nf: I < nf / 2
    idx[0] = c;
    w[0] = 1.0f;
    idx[1] = c - 1;
    w[1] = 0.5f;
    n = 2;
    if (c + 1 < nf) {
        idx[2] = c + 1;
        w[2] = 0.5f;
        n = 3;
    }
}

// f_c = R res_f (the transpose of interpolation over 2^dc)
__global__ void __launch_bounds__(kThreads) k_restrict(level Lf, level Lc, const float *res, float *fc, float scale)
{
    const unsigned G = Lc.size();
    const bool cx = Lc.nx != Lf.nx, cy = Lc.ny != Lf.ny, cz = Lc.nz != Lf.nz;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned I, J, K;
        coords(Lc, o, I, J, K);
        unsigned ix[3], iy[3], iz[3];
        float wx[3], wy[3], wz[3];
        int nx, ny, nz;
        axis_taps(I, Lf.nx, cx, ix, wx, nx);
        axis_taps(J, Lf.ny, cy, iy, wy, ny);
        axis_taps(K, Lf.nz, cz, iz, wz, nz);
        float s = 0.0f;
        for (int a = 0; a < nx; a++)
            for (int b = 0; b < ny; b++)
                for (int c = 0; c < nz; c++)
                    s += wx[a] * wy[b] * wz[c] * res[(ix[a] * Lf.ny + iy[b]) * Lf.nz + iz[c]];
        fc[o] = s * scale;
    }
}

// coarse indices and weights interpolating fine index fi along an axis (the
// transpose of axis_taps)
__device__ __forceinline__ void axis_from(unsigned fi, unsigned nc, bool coarse, unsigned *idx, float *w, int &n)
{
    if (!coarse) {
        idx[0] = fi;
        w[0] = 1.0f;
        n = 1;
        return;
    }
    n = 0;
    if (fi & 1u) {
        idx[0] = fi >> 1;               // (fi - 1) / 2 < nc
        w[0] = 1.0f;
        n = 1;
        return;
    }
    const unsigned hi = fi >> 1;         // coarse neighbours hi - 1 and hi
    if (hi >= 1) {
        idx[n] = hi - 1;
        w[n++] = 0.5f;
    }
    if (hi < nc) {
        idx[n] = hi;
        w[n++] = 0.5f;
    }
}

// e_f += P e_c
__global__ void __launch_bounds__(kThreads) k_prolong(level Lf, level Lc, const float *ec, float *ef)
{
    const unsigned G = Lf.size();
    const bool cx = Lc.nx != Lf.nx, cy = Lc.ny != Lf.ny, cz = Lc.nz != Lf.nz;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < G; o += gridDim.x * blockDim.x) {
        unsigned i, j, k;
        coords(Lf, o, i, j, k);
        unsigned ix[2], iy[2], iz[2];
        float wx[2], wy[2], wz[2];
        int nx, ny, nz;
        axis_from(i, Lc.nx, cx, ix, wx, nx);
        axis_from(j, Lc.ny, cy, iy, wy, ny);
        axis_from(k, Lc.nz, cz, iz, wz, nz);
        float s = 0.0f;
        for (int a = 0; a < nx; a++)
            for (int b = 0; b < ny; b++)
                for (int c = 0; c < nz; c++) s += wx[a] * wy[b] * wz[c] * ec[(ix[a] * Lc.ny + iy[b]) * Lc.nz + iz[c]];
        ef[o] += s;
    }
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
    const float inv = (float)(1.0 / L.diag);
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
    ok = ok && a64(&d->partial, kRedBlocks);
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
        const unsigned G = L.size(), gb = blocks_for(G);
        k_zero<<<gb, kThreads, 0, st>>>(G, E[l]);
        k_rbgs<<<gb, kThreads, 0, st>>>(L, E[l], F[l], 0);
        k_rbgs<<<gb, kThreads, 0, st>>>(L, E[l], F[l], 1);
        k_residual32<<<gb, kThreads, 0, st>>>(L, E[l], F[l], d->res[l]);
        const level &C = lv[l + 1];
        const int dc = (C.nx != L.nx) + (C.ny != L.ny) + (C.nz != L.nz);
        k_restrict<<<blocks_for(C.size()), kThreads, 0, st>>>(L, C, d->res[l], F[l + 1], 1.0f / (float)(1 << dc));
    }
    k_coarse<<<1, 32, 0, st>>>(lv[nl - 1], E[nl - 1], F[nl - 1]);
    for (int l = nl - 2; l >= 0; l--) {
        const level &L = lv[l];
        const unsigned gb = blocks_for(L.size());
        k_prolong<<<gb, kThreads, 0, st>>>(L, lv[l + 1], E[l + 1], E[l]);
        k_rbgs<<<gb, kThreads, 0, st>>>(L, E[l], F[l], 1);
        k_rbgs<<<gb, kThreads, 0, st>>>(L, E[l], F[l], 0);
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
        k_apply_dot32<<<rb, kThreads, 0, st>>>(L0, d->p, d->q, d->partial);
        k_finish<<<1, kThreads, 0, st>>>(d->partial, rb, d->sc, 2);
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
