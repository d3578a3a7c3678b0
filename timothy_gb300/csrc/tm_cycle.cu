// Cell cycle of resident colonies (updatecellcycles, cells.c:370-523, with
// mitosis, cells.c:124-205).  Per cell: the phase time advances, the phase
// machine G0 -> G1 -> S -> G2 -> M -> G1 (or necrotic, or death) steps once,
// G1 cells grow, and M cells divide, appending a daughter.
//
// The reference draws its random numbers with rand() cell by cell, in cell
// order.  Here a first pass decides every cell's transition and how many
// draws it takes (1 for the death test at G1->S and G2->M, 12 (11 in 2-D)
// for a division, 0 otherwise); scans over the caller's cell order give each
// cell its first draw and each dividing cell its daughter's index; the host
// produces that many values from the caller's generator (the C library's
// rand() unless given another) in order; a second pass applies the
// transitions.  A cell's result is the reference's whenever the generator
// yields the reference's stream.  The velocity that mitosis reads
// (cells.c:134) is not used: the reference overwrites the value before use.
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

#define TM_RAND_MAX_I 2147483647

__device__ __forceinline__ float frand(int r) { return tm_frand(r); }

struct cycle_decision {
    int next_phase;       // phase after this step
    int draws;            // random values the cell takes
    bool grow, to_s, to_m, divide, reset_time;
    float phasetime;      // after the increment of this step
};

// the transition of one cell (both passes), without its draws
__device__ __forceinline__ cycle_decision cycle_decide(const tm_cycle_dev &P, const tm_arrays &a, long long s,
                                                      long long cidx, long long n, int dim)
{
    cycle_decision r;
    r.grow = r.to_s = r.to_m = r.divide = r.reset_time = false;
    r.draws = 0;
    const int phase = a.phase[s];
    r.next_phase = phase;
    float pt = a.cy_pt[cidx];
    r.phasetime = pt;
    if (a.rem[s]) return r;                          // cells.c:383
    const int t = a.ctype[s];
    const tm_cycle_type &T = P.types[t];
    const double eps = (double)T.criticaldensity;
    bool low1 = false, low2 = false;
    for (int f = 0; f < P.nfields; f++) {
        const double val = P.cellenv[((long long)f * n + (cidx - P.off)) * 4];
        if (val < (double)P.cl1[t * P.nfields + f]) { low1 = true; break; }
        if (val < (double)P.cl2[t * P.nfields + f]) { low2 = true; break; }
    }
    if (!P.simulationstart) return r;
    const double dens = a.density[s];
    if (phase != 0 && dens <= eps)
        pt = __double2float_rn(add64((double)pt, div64((double)P.sps, 3600.0)));
    r.phasetime = pt;
    switch (phase) {
    case 0:
        if (low2) { r.next_phase = 5; r.reset_time = true; break; }
        if (dens <= eps || n == 1 || !low1) r.next_phase = 1;
        break;
    case 1:
        if (dens > eps || low1) {
            if (low2) { r.next_phase = 5; r.reset_time = true; }
            else r.next_phase = 0;
            break;
        }
        r.grow = true;
        if (pt >= a.cy_g1[cidx]) { r.next_phase = 2; r.reset_time = true; r.to_s = true; r.draws = 1; }
        break;
    case 2:
        if (low2) { r.next_phase = 5; r.reset_time = true; break; }
        if (pt >= a.cy_s[cidx]) { r.next_phase = 3; r.reset_time = true; }
        break;
    case 3:
        if (low2) { r.next_phase = 5; r.reset_time = true; break; }
        if (pt >= a.cy_g2[cidx]) { r.next_phase = 4; r.reset_time = true; r.to_m = true; r.draws = 1; }
        break;
    case 4:
        if (low2) { r.next_phase = 5; r.reset_time = true; }
        else if (pt >= a.cy_m[cidx]) {
            r.divide = true;
            r.next_phase = 1;
            r.reset_time = true;
            r.draws = dim == 3 ? 12 : 11;
        }
        break;
    }
    return r;
}

__global__ void __launch_bounds__(256) k_cycle_count(tm_cycle_dev P, tm_arrays a, long long off, long long n, int dim,
                                                     uint32_t *draws, uint32_t *divs)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
    if (k == n) {                                    // one past the end: the scans' totals
        draws[n] = 0;
        divs[n] = 0;
        return;
    }
    const long long s = off + k;
    const long long c = a.perm[s];
    const cycle_decision d = cycle_decide(P, a, s, off + c, n, dim);
    draws[c] = (uint32_t)d.draws;
    divs[c] = d.divide ? 1u : 0u;
}

// g * (1 + ((float)r/RAND_MAX*2.0 - 1.0) * v), as cells.c:171-174 and 192-195
__device__ __forceinline__ float cycle_length(float g, int r, float v)
{
    const double u = sub64(mul64((double)frand(r), 2.0), 1.0);
    return __double2float_rn(mul64((double)g, add64(1.0, mul64(u, (double)v))));
}

__global__ void __launch_bounds__(256) k_cycle_apply(tm_cycle_dev P, tm_arrays a, long long off, long long n, int dim,
                                                     const uint32_t *draw_off, const uint32_t *div_off,
                                                     const int *stream, unsigned long long *marked,
                                                     uint32_t *divlist)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long s = off + k;
    const long long c = a.perm[s];
    const long long ci = off + c;
    const cycle_decision d = cycle_decide(P, a, s, ci, n, dim);
    if (a.rem[s]) return;
    const int t = a.ctype[s];
    const tm_cycle_type &T = P.types[t];
    const int *dr = stream + draw_off[c];
    a.cy_pt[ci] = d.reset_time ? 0.0f : d.phasetime;
    a.phase[s] = d.next_phase;
    if (d.grow) {
        const double csize = P.csize[t];
        double sz = a.size[s];
        if (sz < csize)
            sz = add64(sz, div64(mul64(sub64(csize, mul64(P.shrink, csize)), (double)P.sps),
                                 mul64(3600.0, (double)a.cy_g1[ci])));
        if (sz > csize) sz = csize;
        a.size[s] = sz;
    }
    if (d.to_s || d.to_m) {
        if ((double)frand(dr[0]) < (double)T.rd) {
            a.rem[s] = 1;
            atomicAdd(marked, 1ull);
        }
    }
    if (d.divide) divlist[div_off[c]] = (uint32_t)s;   // k_cycle_divide does the rest
}

// the divisions (cells.c:175-201), one thread per dividing cell from the list
// k_cycle_apply leaves in daughter order: their FP64 work (draw scaling,
// sqrt, divisions) runs in full warps instead of in every warp that holds
// one dividing cell
__global__ void __launch_bounds__(256) k_cycle_divide(tm_cycle_dev P, tm_arrays a, long long off, long long n, int dim,
                                                      long long ndiv, const uint32_t *divlist,
                                                      const uint32_t *draw_off, const uint32_t *div_off,
                                                      const int *stream)
{
    const long long jj = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (jj >= ndiv) return;
    const long long s = divlist[jj];
    const long long c = a.perm[s];
    const long long ci = off + c;
    const int t = a.ctype[s];
    const tm_cycle_type &T = P.types[t];
    const int *dr = stream + draw_off[c];
    double sh[3];
    sh[0] = sub64(mul64(div64((double)dr[0], (double)TM_RAND_MAX_I), 2.0), 1.0);
    sh[1] = sub64(mul64(div64((double)dr[1], (double)TM_RAND_MAX_I), 2.0), 1.0);
    int q = 2;
    if (dim == 3) sh[2] = sub64(mul64(div64((double)dr[q++], (double)TM_RAND_MAX_I), 2.0), 1.0);
    else sh[2] = 0.0;
    double sc = __dsqrt_rn(add64(add64(mul64(sh[0], sh[0]), mul64(sh[1], sh[1])), mul64(sh[2], sh[2])));
    const double psize = a.size[s];
    sc = div64(psize, mul64(2.0, sc));
    for (int e = 0; e < 3; e++) sh[e] = mul64(sc, sh[e]);
    const long long j = div_off[c];
    const long long ds = off + n + j, dc = off + n + j;   // daughter slot and caller index (n + j)
    const double dsize = mul64(P.shrink, psize);
    a.x[ds] = add64(a.x[s], sh[0]);
    a.y[ds] = add64(a.y[s], sh[1]);
    a.z[ds] = add64(a.z[s], sh[2]);
    a.size[ds] = dsize;
    a.ctype[ds] = t;
    a.cy_age[dc] = a.cy_age[ci] + 1;
    a.x[s] = sub64(a.x[s], sh[0]);
    a.y[s] = sub64(a.y[s], sh[1]);
    a.z[s] = sub64(a.z[s], sh[2]);
    a.size[s] = dsize;
    a.cy_age[ci] = a.cy_age[ci] + 1;
    a.cy_g1[ci] = cycle_length(T.g1, dr[q], T.v);
    a.cy_g2[ci] = cycle_length(T.g2, dr[q + 1], T.v);
    a.cy_s[ci] = cycle_length(T.s, dr[q + 2], T.v);
    a.cy_m[ci] = cycle_length(T.m, dr[q + 3], T.v);
    a.density[ds] = a.density[s];
    a.young[ds] = __double2float_rn(add64(2100.0, mul64(sub64(mul64((double)frand(dr[q + 4]), 2.0), 1.0), 100.0)));
    a.phase[ds] = 1;
    a.cy_pt[dc] = 0.0f;
    // the daughter's own v is 0 (cells.c:184): its draws leave the type's lengths
    a.cy_g1[dc] = cycle_length(T.g1, dr[q + 5], 0.0f);
    a.cy_g2[dc] = cycle_length(T.g2, dr[q + 6], 0.0f);
    a.cy_s[dc] = cycle_length(T.s, dr[q + 7], 0.0f);
    a.cy_m[dc] = cycle_length(T.m, dr[q + 8], 0.0f);
    a.perm[ds] = (int)(n + j);
    a.rem[ds] = 0;
    a.v[ds] = 0.0;
    a.mindist[ds] = 0.0;
    a.fx[ds] = 0.0;
    a.fy[ds] = 0.0;
    a.fz[ds] = 0.0;
    a.nbcount[ds] = 0;
    a.nbmin[ds] = -1;
}

cudaError_t tm_launch_cycle_count(const tm_cycle_dev &P, const tm_arrays &a, long long off, long long n, int dim,
                                  uint32_t *draws, uint32_t *divs, cudaStream_t st)
{
    k_cycle_count<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(P, a, off, n, dim, draws, divs);
    return cudaGetLastError();
}

cudaError_t tm_launch_cycle_apply(const tm_cycle_dev &P, const tm_arrays &a, long long off, long long n, int dim,
                                  const uint32_t *draw_off, const uint32_t *div_off, const int *stream,
                                  unsigned long long *marked, uint32_t *divlist, long long ndiv, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_cycle_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P, a, off, n, dim, draw_off, div_off, stream, marked,
                                                               divlist);
    if (ndiv > 0)
        k_cycle_divide<<<(unsigned)((ndiv + 255) / 256), 256, 0, st>>>(P, a, off, n, dim, ndiv, divlist, draw_off,
                                                                       div_off, stream);
    return cudaGetLastError();
}
