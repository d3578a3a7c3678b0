// Position update (updatepositions + outsidethebox, cells.c:41-58, 342-365)
// and the Cloud-In-Cell deposit of cells onto field 0 of the grid
// (patches_alloc / patches_cells2envinfo / patches_applycells2env at one rank,
// patches.c:47-234, 321-367; grid geometry grid.c:37-136).
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

#include <algorithm>

// uniform float in [0, 1] from a counter (stands in for (float)rand()/RAND_MAX)
__device__ inline float tm_uniform(unsigned long long step, unsigned long long cell, int axis)
{
    unsigned long long z = tm_mix64(step * 0x9e3779b97f4a7c15ull ^ (cell * 3ull + (unsigned long long)axis));
    return (float)(uint32_t)(z >> 40) * (1.0f / 16777215.0f);
}

__device__ inline bool tm_outside(double x, double y, double z, double r, int dim)
{
    // x - r <= -BOXSIZEX/2.0 || x + r >= BOXSIZEX/2.0 (global.h:59-61)
    if (sub64(x, r) <= -1024.0 || add64(x, r) >= 1024.0) return true;
    if (sub64(y, r) <= -1024.0 || add64(y, r) >= 1024.0) return true;
    if (dim == 3 && (sub64(z, r) <= -1024.0 || add64(z, r) >= 1024.0)) return true;
    return false;
}

// True when the cell surely lies inside the box: |x| + r < 1023.99 on every
// axis in FP32 from the split (truncated) position, where the truncation and
// float errors stay below 2e-4.  Then tm_outside would find every test false;
// otherwise (near a wall, or a huge, negative or non-finite value, whose
// split is not valid) the FP64 test decides.  FP64 operations cost this GPU
// about 16 cycles per warp instruction, and the update is bound by them.
__device__ __forceinline__ bool tm_surely_inside(double x, double y, double z, double r, int dim, float hx, float hy,
                                                 float hz)
{
    const long long rb = __double_as_longlong(r);
    if (rb < 0 || (int)((rb >> 52) & 0x7ff) >= 1033) return false;
    float rh, rl;
    tm_split(r, rh, rl);
    const float lim = 1023.99f - rh;
    const auto ok = [lim](double v, float h) {
        return (int)((__double_as_longlong(v) >> 52) & 0x7ff) < 1033 && fabsf(h) < lim;
    };
    return ok(x, hx) && ok(y, hy) && (dim != 3 || ok(z, hz));
}

__global__ void k_update(tm_arrays a, const tm_consts *K)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nslots_total) return;
    const int c = a.col[i];
    const tm_desc &d = a.desc[c];
    if (!d.active || !tm_live(i, d) || d.update_mode == 2) return;
    const int dim = K->dim;
    double x = a.x[i], y = a.y[i], z = a.z[i];
    const double fx = a.fx[i], fy = a.fy[i], fz = a.fz[i];
    if (d.update_mode == 0) {
        x = add64(x, fx);
        y = add64(y, fy);
        if (dim == 3) z = add64(z, fz);
        const float rm = K->t[a.ctype[i]].randommove;
        if (a.move_draws) {
            // the reference's own draws (cells.c:353-355), dim per cell in caller order
            const int *r = a.move_draws + (long long)dim * a.perm[i];
            x = add64(x, mul64((double)rm, sub64(mul64((double)tm_frand(r[0]), 2.0), 1.0)));
            y = add64(y, mul64((double)rm, sub64(mul64((double)tm_frand(r[1]), 2.0), 1.0)));
            if (dim == 3) z = add64(z, mul64((double)rm, sub64(mul64((double)tm_frand(r[2]), 2.0), 1.0)));
        } else if (rm != 0.0f) {
            const unsigned long long id = (unsigned long long)a.perm[i];
            x = add64(x, mul64((double)rm, sub64(mul64((double)tm_uniform(a.frame[c].step_counter, id, 0), 2.0), 1.0)));
            y = add64(y, mul64((double)rm, sub64(mul64((double)tm_uniform(a.frame[c].step_counter, id, 1), 2.0), 1.0)));
            if (dim == 3) z = add64(z, mul64((double)rm, sub64(mul64((double)tm_uniform(a.frame[c].step_counter, id, 2), 2.0), 1.0)));
        }
    } else {
        x = add64(x, mul64(d.dt, fx));
        y = add64(y, mul64(d.dt, fy));
        if (dim == 3) z = add64(z, mul64(d.dt, fz));
    }
    a.x[i] = x;
    a.y[i] = y;
    a.z[i] = z;
    float hx, hy, hz, lx, ly, lz;
    tm_split(x, hx, lx);
    tm_split(y, hy, ly);
    tm_split(z, hz, lz);
    const double r = a.size[i];
    if (!tm_surely_inside(x, y, z, r, dim, hx, hy, hz) && tm_outside(x, y, z, r, dim) && a.rem[i] == 0) {
        a.rem[i] = 1;
        atomicAdd(&a.frame[c].removecount, 1ull);
    }
    if (d.verlet) {
        // displacement since the lists were built, in FP32 from the split
        // positions (the rebuild test adds a margin for this rounding)
        const float4 o = a.x0[i];
        const float ex = hx - o.x, ey = hy - o.y, ez = hz - o.z;
        const unsigned bits = __float_as_uint(sqrtf(fmaf(ex, ex, fmaf(ey, ey, ez * ez))));
        const unsigned m = __reduce_max_sync(__activemask(), bits);
        // one word per colony: only warps past its current value post (it only grows)
        if (bits == m && m > __ldcg(&a.frame[c].maxdisp)) atomicMax(&a.frame[c].maxdisp, m);
    }
}

// CIC weights onto field 0; the patch bounding box (patches.c:81-132) is
// reduced alongside for the drop-in's patches_alloc.  Morton-ordered cells of
// one warp mostly share grid nodes, so each run of cells on one node gets
// one atomic carrying the sum of their weights (tm_warp_deposit).
__global__ void __launch_bounds__(256) k_cic(tm_arrays a, const tm_consts *K)
{
    const unsigned FULLM = 0xffffffffu;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (((i >> 5) << 5) >= a.nslots_total) return;            // whole warp beyond the slots
    const int c = a.col[(i >> 5) << 5];
    const tm_desc &d = a.desc[c];
    if (!d.active || d.gridoff < 0) return;                    // uniform per warp
    const bool live = tm_live(i, d);
    const int dim = K->dim;
    const int lane = threadIdx.x & 31;
    long long ci[3] = {0, 0, 0};
    double dd[3] = {0, 0, 0}, tt[3] = {0, 0, 0};
    int ph = 5;
    if (live) {
        const double pos[3] = {a.x[i], a.y[i], a.z[i]};
        for (int k = 0; k < 3; k++) {
            ci[k] = (long long)tm_div_res(sub64(pos[k], d.glower[k]), d.gres);
            // grid->lowercorner + cellIdx * resolution: an int64 * float product is a float
            const double cic = add64(d.glower[k], (double)__fmul_rn((float)ci[k], d.gres));
            dd[k] = tm_div_res(sub64(pos[k], cic), d.gres);
            tt[k] = sub64(1.0, dd[k]);
        }
        ph = a.phase[i];
    }
    const long long up[3] = {d.gsize[0] - 1, d.gsize[1] - 1, dim == 3 ? d.gsize[2] - 1 : 0};
    const double wph = ph == 0 ? 0.75 : 1.0;
    long long lo[3] = {0x7fffffffll, 0x7fffffffll, 0x7fffffffll}, hi[3] = {-0x7fffffffll - 1, -0x7fffffffll - 1, -0x7fffffffll - 1};
    // the weight ((wphase * wx) * wy) * wz in the reference's order, its
    // partial products shared between corners
    const double wx0 = mul64(wph, tt[0]), wx1 = mul64(wph, dd[0]);
    double wxy = 0.0;
    for (int corner = 0; corner < 8; corner++) {
        const int ax = corner >> 2, ay = (corner >> 1) & 1, az = corner & 1;
        if (az == 0) wxy = mul64(ax ? wx1 : wx0, ay ? dd[1] : tt[1]);
        const long long gx = ci[0] + ax, gy = ci[1] + ay, gz = ci[2] + az;
        const bool inb = live && gx >= 0 && gy >= 0 && gz >= 0 && gx <= up[0] && gy <= up[1] && gz <= up[2];
        if (inb) {
            lo[0] = gx < lo[0] ? gx : lo[0];
            lo[1] = gy < lo[1] ? gy : lo[1];
            lo[2] = gz < lo[2] ? gz : lo[2];
            hi[0] = gx > hi[0] ? gx : hi[0];
            hi[1] = gy > hi[1] ? gy : hi[1];
            hi[2] = gz > hi[2] ? gz : hi[2];
        }
        const bool dep = inb && ph != 5;                       // necrotic cells deposit nothing
        const double w = dep ? mul64(wxy, az ? dd[2] : tt[2]) : 0.0;
        const long long gi = dep ? d.gridoff + ((long long)d.gsize[1] * gx + gy) * d.gsize[2] + gz : -1;
        tm_warp_deposit(a.grid, gi, w, dep, lane);
    }
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            const long long ql = __shfl_xor_sync(FULLM, lo[k], o), qh = __shfl_xor_sync(FULLM, hi[k], o);
            lo[k] = ql < lo[k] ? ql : lo[k];
            hi[k] = qh > hi[k] ? qh : hi[k];
        }
    }
    if (lane == 0 && hi[0] >= lo[0]) {
        tm_frame &f = a.frame[c];
        const int nd = dim == 3 ? 3 : 2;
        // one address per corner for the whole colony: read it first and
        // touch it only when this warp's box reaches past it (a stale read
        // only costs an atomic; the corners move one way)
        for (int k = 0; k < nd; k++) {
            if (lo[k] < __ldcg(&f.patch_lo[k])) atomicMin(&f.patch_lo[k], lo[k]);
            if (hi[k] > __ldcg(&f.patch_hi[k])) atomicMax(&f.patch_hi[k], hi[k]);
        }
    }
}

cudaError_t tm_launch_update(const tm_arrays &a, const tm_consts *K, cudaStream_t st)
{
    unsigned grid = (unsigned)((a.nslots_total + 255) / 256);
    if (grid == 0) return cudaSuccess;
    k_update<<<grid, 256, 0, st>>>(a, K);
    return cudaGetLastError();
}

cudaError_t tm_launch_cic(const tm_arrays &a, const tm_consts *K, cudaStream_t st)
{
    unsigned grid = (unsigned)((a.nslots_total + 255) / 256);
    if (grid == 0) return cudaSuccess;
    k_cic<<<grid, 256, 0, st>>>(a, K);
    return cudaGetLastError();
}
