// Pair kernel: SPH density, nearest distance and SPH-gradient force of every
// cell (computepotential potential.c:87-138 with potential() :39-78 and
// sphkernel inline.h:40-51; computegradient potential.c:209-259 with
// sphgradient inline.h:59-83), fused into one pass because the force does not
// depend on the density.  v (the potential of the last walked candidate) is
// produced by the octree kernel.
//
// Work decomposition: a warp owns 8 Morton-consecutive slots of one colony,
// four lanes per cell.
//  1. stage: the Morton bins covering the union of the 8 query spheres are
//     enumerated 32 at a time (one bin per lane), their cell runs are copied
//     into a shared-memory tile as group-relative FP32 coordinates;
//  2. test: the four lanes of a cell take every fourth tile entry and test it
//     against their cell with a conservative FP32 squared-distance bound,
//     appending hits to their own list in shared memory (predicated append);
//  3. drain: each lane walks its own list with the exact pair maths, so the
//     expensive part runs with all lanes busy; the four partial sums of a
//     cell are combined with shuffles at the end.
// PREC 0 is the plain FP64 path: every reference expression is evaluated in
// the same order with separate roundings (no contraction), the cutoff test is
// fl(sqrt(.)) <= h and the kernel value is rounded to float (inline.h:40).
// PREC 1 is the FP32 path: distances from double-float group-relative
// coordinates, kernel and gradient in FP32, Kahan-compensated sums, and an
// FP64 recheck of the cutoff for pairs within 1e-5 h of h, so the neighbour
// sets equal the FP64 ones.
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

#include <algorithm>

#define FULL 0xffffffffu
#define PAIR_TILE 256
#define PAIR_LCAP 64
#define PAIR_LPC 4                      // lanes per cell
#define PAIR_CPW (32 / PAIR_LPC)        // cells per warp

template <int PREC>
struct pair_acc;

template <>
struct pair_acc<0> {
    double dens, fx, fy, fz;
    unsigned long long mind2;         // least squared distance (its bits: non-negative doubles order as integers)
    __device__ void init() { dens = 0.0; mind2 = 0x7fefffffffffffffull; fx = fy = fz = 0.0; }
};

template <>
struct pair_acc<1> {
    kahan dens, fx, fy, fz;
    float mins, err2;
    __device__ void init() { dens.init(); fx.init(); fy.init(); fz.init(); mins = 3.0e38f; err2 = 0.0f; }
};

// FP64 pair of potential.c:39-78 / inline.h:40-83 (density and force parts;
// v comes from the octree walk).  The squared distance has the reference's
// association and roundings, and the cutoff is decided on it exactly:
// sqrt(d2) <= h (the reference's test, with a correctly rounded square root,
// which is monotone) holds exactly for d2 <= h2cut, the largest double whose
// square root rounds to h or below (formed on the host), so entries beyond h
// take no square root, and the least distance is the square root of the
// least d2.  Within h the reference's expressions follow in FP64 with
// separate roundings: dist is the correctly rounded square root and u =
// dist / h the correctly rounded quotient (div_by_recip), so the kernel
// value, rounded to float as the reference does, is the reference's bit for
// bit (a one-ulp change of u could round it to the neighbouring float, 6e-8
// of the term).  Only the force's three divisions by dist are taken as
// products with one correctly rounded reciprocal, a few ulps from the
// reference's quotients against the path's 1e-12 bound (divisions are a
// software sequence on this part's slow FP64 pipe).  The comparisons of non-negative
// values run on their bit patterns, the rounding of the kernel value to float
// with integer operations (tm_round_to_float), and x_j - x_i is the negated
// x_i - x_j (exact), so the FP64 pipe does only the arithmetic.
__device__ __forceinline__ void pair64(const tm_type &T, int dim, double xi, double yi, double zi, double xj,
                                       double yj, double zj, double mj, pair_acc<0> &acc, bool &in)
{
    const double dx = sub64(xi, xj), dy = sub64(yi, yj), dz = sub64(zi, zj);
    const double d2 = add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz));
    const unsigned long long b2 = (unsigned long long)__double_as_longlong(d2);
    acc.mind2 = b2 < acc.mind2 ? b2 : acc.mind2;
    in = b2 <= (unsigned long long)__double_as_longlong(T.h2cut);
    if (in) {
        const double dist = __dsqrt_rn(d2);
        const double u = div_by_recip(dist, T.h, T.inv_h);
        const double omu = sub64(1.0, u);
        double wk, wg;
        if ((unsigned long long)__double_as_longlong(u) <= 0x3fe0000000000000ull) {   // u <= 0.5
            const double six_uu = mul64(mul64(6.0, u), u);
            wk = mul64(T.cW, add64(sub64(1.0, six_uu), mul64(six_uu, u)));
            wg = add64(mul64(-2.0, u), mul64(mul64(3.0, u), u));
        } else {
            wk = mul64(T.cW, mul64(mul64(mul64(2.0, omu), omu), omu));
            wg = mul64(-omu, omu);
        }
        acc.dens = add64(acc.dens, mul64(mj, tm_round_to_float(wk)));
        const double wc = mul64(wg, T.cG);
        const double rd = __drcp_rn(dist);
        acc.fx = add64(acc.fx, mul64(mul64(wc, -dx), rd));
        acc.fy = add64(acc.fy, mul64(mul64(wc, -dy), rd));
        if (dim == 3) acc.fz = add64(acc.fz, mul64(mul64(wc, -dz), rd));
    }
}

// FP32 cutoff decision for squared distance s: FP64 only in the band
// |r - h| < 1e-5 h, so the neighbour set equals the FP64 one
__device__ __forceinline__ bool within32(const tm_type &T, float s, double xi, double yi, double zi, double xj,
                                        double yj, double zj)
{
    if (s <= T.thr_lo) return true;
    if (s > T.thr_hi) return false;
    const double dx = sub64(xi, xj), dy = sub64(yi, yj), dz = sub64(zi, zj);
    return __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz))) <= T.h;
}

// FP64 density term of cell j at distance dist <= h from a cell of type T
// (potential.c:60-62 with sphkernel inline.h:40-51, W rounded to float)
__device__ __forceinline__ double dens_term64(const tm_type &T, double dist, double sizej)
{
    const double u = div64(dist, T.h);
    double wk;
    if (u <= 0.5) {
        const double six_uu = mul64(mul64(6.0, u), u);
        wk = mul64(T.cW, add64(sub64(1.0, six_uu), mul64(six_uu, u)));
    } else {
        const double omu = sub64(1.0, u);
        wk = mul64(T.cW, mul64(mul64(mul64(2.0, omu), omu), omu));
    }
    const double mj = mul64(T.sc, div64(sizej, T.csize));
    return mul64(mj, (double)__double2float_rn(wk));
}

// The same term for the FP32 path's FP64 re-do of a flagged cell: u and the
// density weight by multiplications with 1 / h and sc / csize formed on the
// host (the FP32 path's contract is 1e-6; the re-do removes the FP32
// cancellation in 1 - u, which these one-ulp differences do not bring back).
__device__ __forceinline__ double dens_term64_fast(const tm_type &T, double dist, double sizej)
{
    const double u = dist * T.inv_h;
    double wk;
    if (u <= 0.5) {
        const double six_uu = 6.0 * u * u;
        wk = T.cW * ((1.0 - six_uu) + six_uu * u);
    } else {
        const double omu = 1.0 - u;
        wk = T.cW * (2.0 * omu * omu * omu);
    }
    return (T.kmass * sizej) * (double)__double2float_rn(wk);
}

__device__ __forceinline__ double dist64(const tm_arrays &a, long long i, long long j)
{
    const double dx = sub64(a.x[i], a.x[j]), dy = sub64(a.y[i], a.y[j]), dz = sub64(a.z[i], a.z[j]);
    return __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz)));
}

// within32 with both cells' FP64 positions read only inside the band
__device__ __forceinline__ bool within32_at(const tm_type &T, float s, const tm_arrays &a, long long i, long long j)
{
    if (s <= T.thr_lo) return true;
    if (s > T.thr_hi) return false;
    return dist64(a, i, j) <= T.h;
}

// FP32 + compensated pair (caller decided it is within h).  The kernel
// value's error estimate is term / (1 - u) (W ~ (1-u)^3 amplifies the FP32
// error of 1 - u near the cutoff), formed without a division: outside
// u = 1/2 it is ms * 2 cW (1-u)^2 exactly; inside, where 1 - u lies in
// [1/2, 1], 1 / (1 - u) is bounded by the chord 3 - 2 (1 - u) (at most 12.5 %
// above it), so cells are flagged for the FP64 density a little early,
// never late.
__device__ __forceinline__ void pair32(const tm_type &T, int dim, float dx, float dy, float dz, float s,
                                       float sizej, pair_acc<1> &acc)
{
    acc.mins = fminf(acc.mins, s);
    const float rs = s > 0.0f ? rsqrtf(s) : 0.0f;
    // dist = sqrt(s): s * rsqrt(s) and one Newton step on dist^2 = s
    float dist = s * rs;
    dist = fmaf(0.5f * rs, fmaf(-dist, dist, s), dist);
    const float u = dist * T.inv_hf;
    // 1 - u as (h - dist) / h: the subtraction is exact near the cutoff
    const float omu = (T.hf - dist) * T.inv_hf;
    // both branches of the cubic spline, selected (no divergence)
    const bool inner = u <= 0.5f;
    const float o2 = omu * omu;
    const float q2 = (2.0f * T.cWf) * o2;                  // 2 cW (1-u)^2
    const float w_in = T.cWf * fmaf(6.0f * u * u, u - 1.0f, 1.0f);
    const float wk = inner ? w_in : q2 * omu;
    const float ms = T.kmassf * sizej;
    acc.dens.add(ms * wk);
    const float ek = ms * (inner ? w_in * fmaf(-2.0f, omu, 3.0f) : q2);
    acc.err2 = fmaf(ek, ek, acc.err2);
    const float wg = inner ? u * fmaf(3.0f, u, -2.0f) : -o2;
    const float g = wg * T.cGf * rs;
    acc.fx.add(g * dx);
    acc.fy.add(g * dy);
    if (dim == 3) acc.fz.add(g * dz);
}

// The terms of one pair within h, without the accumulation (pair32 above):
// density term, its error estimate and the gradient factor g (force = g * d).
__device__ __forceinline__ void pair32_terms(const tm_type &T, float s, float sizej, float &term, float &ek,
                                             float &g)
{
    const float rs = rsqrtf(fmaxf(s, 1.0e-30f));
    float dist = s * rs;
    dist = fmaf(0.5f * rs, fmaf(-dist, dist, s), dist);
    const float u = dist * T.inv_hf;
    const float omu = (T.hf - dist) * T.inv_hf;
    const bool inner = u <= 0.5f;
    const float o2 = omu * omu;
    const float q2 = (2.0f * T.cWf) * o2;
    const float w_in = T.cWf * fmaf(6.0f * u * u, u - 1.0f, 1.0f);
    const float wk = inner ? w_in : q2 * omu;
    const float ms = T.kmassf * sizej;
    term = ms * wk;
    ek = ms * (inner ? w_in * fmaf(-2.0f, omu, 3.0f) : q2);
    const float wg = inner ? u * fmaf(3.0f, u, -2.0f) : -o2;
    g = wg * T.cGf * rs;
}

// write one cell's results (both pair kernels)
// Cells whose estimated relative FP32 density error exceeds 3e-7 (almost
// only cells whose neighbours all sit near the cutoff) are redone in FP64.
// Per term the error is about term * (1e-7 / (1-u) + 1.2e-7); err2 sums
// (term / (1-u))^2, and (a + b)^2 <= 2a^2 + 2b^2 with sum(term^2) <= rho^2
// turns the 3e-7 bound into err2 * 1e-14 * 2 + 2.88e-14 rho^2 > 9e-14 rho^2.
__device__ __forceinline__ bool needs_fix64(const pair_acc<1> &acc)
{
    const float rho = acc.dens.value();
    return acc.err2 * 2.0e-14f > 6.12e-14f * rho * rho;
}

// queue: flagged cells go to the FP64 fix-up kernel (otherwise the caller
// redoes them)
template <int PREC>
__device__ __forceinline__ void pair_store(const tm_arrays &a, long long i, pair_acc<PREC> &acc, int cnt_nb,
                                           int nbmin, unsigned long long hash, bool queue = true)
{
    if constexpr (PREC == 0) {
        a.density[i] = acc.dens;
        a.mindist[i] = acc.mind2 < 0x7fefffffffffffffull ? __dsqrt_rn(__longlong_as_double((long long)acc.mind2))
                                                          : 1.7976931348623157e308;
        a.fx[i] = acc.fx;
        a.fy[i] = acc.fy;
        a.fz[i] = acc.fz;
    } else {
        const float rho = acc.dens.value();
        a.density[i] = (double)rho;
        if (queue && needs_fix64(acc)) {
            const int q = atomicAdd(a.fix_count, 1);
            a.fix_list[q] = (int)i;
            atomicAdd(&a.frame[a.col[i]].fix64, 1ull);
        }
        a.mindist[i] = cnt_nb ? (double)sqrtf(acc.mins) : 1.7976931348623157e308;
        a.fx[i] = (double)acc.fx.value();
        a.fy[i] = (double)acc.fy.value();
        a.fz[i] = (double)acc.fz.value();
    }
    a.nbcount[i] = cnt_nb;
    a.nbmin[i] = cnt_nb ? nbmin : -1;
    if (a.want_diag) a.nbhash[i] = hash;
}

// Diagnostics of one pair within h: the set's fingerprint and, for a sampled
// cell (row >= 0), the neighbour's caller index in the cell's list.
__device__ __forceinline__ void diag_pair(const tm_arrays &a, int row, long long j, unsigned long long &hash)
{
    const unsigned long long pj = (unsigned long long)a.perm[j];
    hash += tm_mix64(pj + 1ull);
    if (row >= 0) {
        const int q = atomicAdd(a.diag_cnt + row, 1);
        if (q < a.diag_lcap) a.diag_nb[(long long)row * a.diag_lcap + q] = (int)pj;
    }
}

// sample row of cell i of colony d (diagnostics), -1 if none
__device__ __forceinline__ int diag_row_of(const tm_arrays &a, const tm_desc &d, long long i)
{
    return (a.want_diag && a.diag_row) ? a.diag_row[d.off + a.perm[i]] : -1;
}

// one warp, one group of PAIR_CPW Morton-consecutive slots starting at base
template <int PREC>
__device__ __forceinline__ void pair_group(const tm_arrays &a, const tm_consts *K, int fallback, int lshift,
                                           long long base, int lane, float4 *tA, float4 *tB,
                                           unsigned short (*list)[32])
{
    if (base >= a.nslots_total) return;
    const int c = a.col[base];             // colonies are 32-aligned, so a group stays in one
    const tm_desc &d = a.desc[c];
    if (!d.active || d.precision != PREC || d.n <= 1) return;   // potential.c:89
    const tm_frame &f = a.frame[c];
    if (!f.rebuild) return;                 // the list kernel handles this step
    // first pass: colonies without lists; second pass (fallback): colonies
    // whose lists overflowed
    if (fallback ? (!d.verlet || f.list_ok) : d.verlet) return;
    if (!tm_live(base, d)) return;      // group beyond the colony's cells
    const int dim = K->dim;

    const int quarter = lane % PAIR_LPC;   // this lane's share of the cell's candidates
    const long long i = base + lane / PAIR_LPC;
    const bool live = tm_live(i, d);
    const int t = live ? a.ctype[i] : 0;
    const tm_type &T = K->t[t];

    // Subgroups: cells sharing a Morton node two levels above the bins.
    // Morton-consecutive cells can straddle a high-level boundary (the last
    // cell of one octant and the first of the next), and one union box would
    // then span much of the colony; the subgroup node bounds every box.
    const int L = f.L;
    const int Lg = L >= 2 ? L - 2 : 0;
    // candidate ranges come from nodes lshift levels above the bins: each is
    // one contiguous run of 8^lshift bins in Morton order
    const int ls = L > lshift ? lshift : 0;
    const int Lp = L - ls;
    const uint32_t key = live ? tm_prefix(a.codes[i], Lg) : 0xffffffffu;
    const unsigned live_mask = __ballot_sync(FULL, live);
    int my_leader = 0;
    {
        unsigned rem = live_mask;
        while (rem) {
            const int ldr = __ffs(rem) - 1;
            const uint32_t kg = __shfl_sync(FULL, key, ldr);
            const bool member = live && key == kg;
            if (member) my_leader = ldr;
            rem &= ~__ballot_sync(FULL, member);
        }
    }
    const float4 hi_i = live ? a.hi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 lo_i = live ? a.lo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // origin: the float position of the subgroup's first cell
    const float ox = __shfl_sync(FULL, hi_i.x, my_leader), oy = __shfl_sync(FULL, hi_i.y, my_leader),
                oz = __shfl_sync(FULL, hi_i.z, my_leader);
    // double-float origin-relative position: s (exact sum) + e (its error + lo part)
    float sx, sy, sz, ex, ey, ez;
    two_sum(hi_i.x, -ox, sx, ex);
    two_sum(hi_i.y, -oy, sy, ey);
    two_sum(hi_i.z, -oz, sz, ez);
    ex += lo_i.x;
    ey += lo_i.y;
    ez += lo_i.z;
    // conservative test radius (the test uses s only, |e| < 1e-5 here)
    const float hr = T.hf * 1.00002f + 1e-4f;
    const int nside = 1 << Lp;
    const float bs = f.binscale * (1.0f / (float)(1 << ls));
    auto binof = [&](float g, float o, float sh, float eps) {
        float v = (o - sh + g) * bs + eps;
        int b = (int)floorf(v);
        return b < 0 ? 0 : (b >= nside ? nside - 1 : b);
    };
    const uint32_t *bstart = a.bin_start + d.binoff;
    const long long bbase = f.bin_base;

    // FP64 data of the own cell (plain path and band rechecks)
    const double xi = live ? a.x[i] : 0.0, yi = live ? a.y[i] : 0.0, zi = live ? a.z[i] : 0.0;
    const int drow = live ? diag_row_of(a, d, i) : -1;
    pair_acc<PREC> acc;
    acc.init();
    int cnt_nb = 0;
    int nbmin = 0x7fffffff;   // first Morton position within h (slots are positions here)
    unsigned long long hash = 0;
    int nl = 0;

    // exact pair maths over this lane's hit list (tile indices)
    auto drain = [&]() {
        int m = nl;
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
        for (int q = 0; q < m; q++) {
            if (q >= nl) continue;
            const int ti = list[q][lane];
            const float4 A = tA[ti];
            const int j = __float_as_int(A.w);
            if constexpr (PREC == 0) {
                bool in;
                pair64(T, dim, xi, yi, zi, a.x[j], a.y[j], a.z[j], a.mass[(long long)t * a.nslots_total + j], acc,
                       in);
                if (in) {
                    cnt_nb++;
                    nbmin = min(nbmin, j);
                    if (a.want_diag) diag_pair(a, drow, j, hash);
                }
            } else {
                const float4 B = tB[ti];
                const float dx = (A.x - sx) + (B.x - ex);
                const float dy = (A.y - sy) + (B.y - ey);
                const float dz = (A.z - sz) + (B.z - ez);
                const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (s <= T.thr_hi && within32(T, s, xi, yi, zi, a.x[j], a.y[j], a.z[j])) {
                    pair32(T, dim, dx, dy, dz, s, B.w, acc);
                    cnt_nb++;
                    nbmin = min(nbmin, j);
                    if (a.want_diag) diag_pair(a, drow, j, hash);
                }
            }
        }
        nl = 0;
    };

    // test the staged tile [0, fill) and drain; the tile is refilled afterwards
    auto test_tile = [&](int fill, float thr) {
        for (int tb = 0; tb < fill; tb += 32 * PAIR_LPC) {
            const int te = min(fill, tb + 32 * PAIR_LPC);
#pragma unroll 8
            for (int tt = tb + quarter; tt < te; tt += PAIR_LPC) {
                const float4 cc = tA[tt];
                const float dx = cc.x - sx, dy = cc.y - sy, dz = cc.z - sz;
                const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (s <= thr && (long long)__float_as_int(cc.w) != i) {
                    list[nl][lane] = (unsigned short)tt;
                    nl++;
                }
            }
            if (__any_sync(FULL, nl > PAIR_LCAP - 32)) drain();
        }
        drain();
        __syncwarp();
    };

    unsigned pending = live_mask;
    while (pending) {
        const int ldr = __ffs(pending) - 1;
        const bool member = live && my_leader == ldr;
        pending &= ~__ballot_sync(FULL, member);
        const float gox = __shfl_sync(FULL, ox, ldr), goy = __shfl_sync(FULL, oy, ldr), goz = __shfl_sync(FULL, oz, ldr);
        const float thr = member ? hr * hr : -1.0f;
        // union of the members' query boxes, relative to the subgroup origin
        float mnx = member ? sx - hr : 3e38f, mny = member ? sy - hr : 3e38f, mnz = member ? sz - hr : 3e38f;
        float mxx = member ? sx + hr : -3e38f, mxy = member ? sy + hr : -3e38f, mxz = member ? sz + hr : -3e38f;
        for (int o = 16; o > 0; o >>= 1) {
            mnx = fminf(mnx, __shfl_xor_sync(FULL, mnx, o));
            mny = fminf(mny, __shfl_xor_sync(FULL, mny, o));
            mnz = fminf(mnz, __shfl_xor_sync(FULL, mnz, o));
            mxx = fmaxf(mxx, __shfl_xor_sync(FULL, mxx, o));
            mxy = fmaxf(mxy, __shfl_xor_sync(FULL, mxy, o));
            mxz = fmaxf(mxz, __shfl_xor_sync(FULL, mxz, o));
        }
        const int bx0 = binof(mnx, gox, f.shiftf[0], -0.01f), bx1 = binof(mxx, gox, f.shiftf[0], 0.01f);
        const int by0 = binof(mny, goy, f.shiftf[1], -0.01f), by1 = binof(mxy, goy, f.shiftf[1], 0.01f);
        const int bz0 = binof(mnz, goz, f.shiftf[2], -0.01f), bz1 = binof(mxz, goz, f.shiftf[2], 0.01f);
        const int nbx = bx1 - bx0 + 1, nby = by1 - by0 + 1, nbz = bz1 - bz0 + 1;
        int fill = 0;   // entries staged in the tile
        // lanes cover whole rows of nbx bins (nbx <= 32; wider boxes use one
        // row per chunk pass over bx in steps of 32)
        const int rowlen = min(nbx, 32);
        const int rows_per = 32 / rowlen;
        const int my_row = lane / rowlen, my_col = lane % rowlen;
        const int nrows = nby * nbz;
        const int xpasses = (nbx + 31) / 32;
        const float inv_nby = 1.0f / (float)nby;
        for (int chunk = 0; chunk < nrows * xpasses; chunk += rows_per) {
            const int rr = chunk + my_row;               // row-pass index
            const int xp = xpasses == 1 ? 0 : rr % xpasses;
            const int row = xpasses == 1 ? rr : rr / xpasses;
            const int bxo = xp * 32 + my_col;
            long long st = 0;
            uint32_t cnt = 0;
            if (my_row < rows_per && row < nrows && bxo < nbx) {
                const int bz = bz0 + (int)(((float)row + 0.5f) * inv_nby);
                const int by = by0 + row - (bz - bz0) * nby;
                const int bx = bx0 + bxo;
                const uint32_t m = tm_morton((uint32_t)bx, (uint32_t)by, (uint32_t)bz) << (3 * ls);
                const uint32_t s0 = bstart[m];
                st = bbase + s0;
                cnt = bstart[m + (1u << (3 * ls))] - s0;
            }
            uint32_t incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t total = __shfl_sync(FULL, incl, 31);
            const uint32_t off = incl - cnt;
            // copy the chunk's candidates [0, total) into the tile with parallel,
            // coalesced loads: candidate k lives in the bin of the first lane whose
            // inclusive count exceeds k
            for (uint32_t k0 = 0; k0 < total; k0 += 32) {
                const uint32_t k = min(k0 + lane, total - 1);
                int b = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const uint32_t v = __shfl_sync(FULL, incl, b + step - 1);
                    if (v <= k) b += step;
                }
                const long long stb = __shfl_sync(FULL, st, b);
                const uint32_t offb = __shfl_sync(FULL, off, b);
                const int slot = fill + lane;
                const bool valid = k0 + lane < total;
                if (valid) {
                    const long long j = stb + (k - offb);
                    const float4 hj = a.hi[j], lj = a.lo[j];
                    float s1, e1, s2, e2, s3, e3;
                    two_sum(hj.x, -gox, s1, e1);
                    two_sum(hj.y, -goy, s2, e2);
                    two_sum(hj.z, -goz, s3, e3);
                    tA[slot] = make_float4(s1, s2, s3, __int_as_float((int)j));
                    tB[slot] = make_float4(e1 + lj.x, e2 + lj.y, e3 + lj.z, hj.w);
                }
                fill += min(32u, total - k0);
                if (fill > PAIR_TILE - 32) {
                    __syncwarp();
                    test_tile(fill, thr);
                    fill = 0;
                }
            }
        }
        if (fill > 0) {
            __syncwarp();
            test_tile(fill, thr);
        }
    }

    // combine the partial results of the four lanes of each cell
    for (int o = 1; o < PAIR_LPC; o <<= 1) {
        if constexpr (PREC == 0) {
            acc.dens = add64(acc.dens, __shfl_xor_sync(FULL, acc.dens, o));
            acc.fx = add64(acc.fx, __shfl_xor_sync(FULL, acc.fx, o));
            acc.fy = add64(acc.fy, __shfl_xor_sync(FULL, acc.fy, o));
            acc.fz = add64(acc.fz, __shfl_xor_sync(FULL, acc.fz, o));
            const unsigned long long om = __shfl_xor_sync(FULL, acc.mind2, o);
            acc.mind2 = om < acc.mind2 ? om : acc.mind2;
        } else {
            acc.dens.merge(__shfl_xor_sync(FULL, acc.dens.s, o), __shfl_xor_sync(FULL, acc.dens.c, o));
            acc.fx.merge(__shfl_xor_sync(FULL, acc.fx.s, o), __shfl_xor_sync(FULL, acc.fx.c, o));
            acc.fy.merge(__shfl_xor_sync(FULL, acc.fy.s, o), __shfl_xor_sync(FULL, acc.fy.c, o));
            acc.fz.merge(__shfl_xor_sync(FULL, acc.fz.s, o), __shfl_xor_sync(FULL, acc.fz.c, o));
            acc.mins = fminf(acc.mins, __shfl_xor_sync(FULL, acc.mins, o));
            acc.err2 += __shfl_xor_sync(FULL, acc.err2, o);
        }
        cnt_nb += __shfl_xor_sync(FULL, cnt_nb, o);
        nbmin = min(nbmin, __shfl_xor_sync(FULL, nbmin, o));
        hash += __shfl_xor_sync(FULL, hash, o);
    }
    if (!live || quarter != 0) return;
    pair_store<PREC>(a, i, acc, cnt_nb, nbmin, hash);
}

// Grid-stride over the groups: the grid is sized to the resident blocks, and
// on a step where no colony searches (all evaluate their lists) or no list
// overflowed (fallback pass) every block leaves after one load.
template <int PREC>
__global__ void __launch_bounds__(TM_WARPS_PER_BLOCK * 32) k_pair(tm_arrays a, const tm_consts *K, int fallback,
                                                                   int lshift)
{
    // per warp: tile of staged candidates (A: hi part of the origin-relative
    // position + slot, B: lo part + radius) and one hit list per lane holding
    // tile indices
    __shared__ float4 tA_s[TM_WARPS_PER_BLOCK][PAIR_TILE];
    __shared__ float4 tB_s[TM_WARPS_PER_BLOCK][PAIR_TILE];
    __shared__ unsigned short list_s[TM_WARPS_PER_BLOCK][PAIR_LCAP][32];
    if (a.work[fallback ? 1 : 0] == 0) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long long ngroups = (a.nslots_total + PAIR_CPW - 1) / PAIR_CPW;
    const long long stride = (long long)gridDim.x * TM_WARPS_PER_BLOCK;
    for (long long w = (long long)blockIdx.x * TM_WARPS_PER_BLOCK + wib; w < ngroups; w += stride) {
        pair_group<PREC>(a, K, fallback, lshift, w * PAIR_CPW, lane, tA_s[wib], tB_s[wib], list_s[wib]);
        __syncwarp();
    }
}

// Pair kernel on the neighbour lists (every step of a colony with lists): one
// thread per cell walks its list with the same exact maths; the cutoff is
// decided each step, so the neighbour sets are those of this step.
// Entries are taken two at a time with both gathers issued before either is
// used (the walk is bound by the latency of the dependent index -> position
// loads, not by arithmetic).
// List build (rebuild steps of colonies with lists): one thread per cell,
// positions are Morton positions here (the state was just reordered).  The
// bins covering the cell's box [x - r, x + r] (r = h + skin with a float
// margin) are visited row by row and every cell in them within r of the cell
// (double-float distance) is appended to its list; the list kernel then
// decides the cutoff exactly.  The list order (bins z, y, x, then Morton order
// inside a bin) depends on the colony's own cells only.
__device__ __forceinline__ void listbuild_cell(const tm_arrays &a, const tm_consts *K, int c, long long i)
{
    const tm_desc &d = a.desc[c];
    if (d.n <= 1 || !d.verlet || !tm_live(i, d)) return;
    const tm_frame &f = a.frame[c];
    const tm_type &T = K->t[a.ctype[i]];
    const float rlist = T.hf + d.skin;
    const float hr = rlist * 1.00002f + 1e-4f;
    const float thr = hr * hr;
    const float4 hi_i = a.hi[i], lo_i = a.lo[i];
    const int nside = 1 << f.L;
    const float bs = f.binscale;
    auto bin_lo = [&](float x, float sh) {
        const int b = (int)floorf((x - sh - hr) * bs - 0.01f);
        return b < 0 ? 0 : (b >= nside ? nside - 1 : b);
    };
    auto bin_hi = [&](float x, float sh) {
        const int b = (int)floorf((x - sh + hr) * bs + 0.01f);
        return b < 0 ? 0 : (b >= nside ? nside - 1 : b);
    };
    const int bx0 = bin_lo(hi_i.x, f.shiftf[0]), bx1 = bin_hi(hi_i.x, f.shiftf[0]);
    const int by0 = bin_lo(hi_i.y, f.shiftf[1]), by1 = bin_hi(hi_i.y, f.shiftf[1]);
    const int bz0 = bin_lo(hi_i.z, f.shiftf[2]), bz1 = bin_hi(hi_i.z, f.shiftf[2]);
    const uint32_t *bst = a.bin_start + d.binoff;
    const long long bbase = f.bin_base;
    const float4 *__restrict__ hi = a.hi;
    const float4 *__restrict__ lo = a.lo;
    const long long ls = a.lstride;
    // Rows of bins whose y/z gap to the cell already exceeds the radius hold
    // no cell within it, and the rest are cut to the x range the remaining
    // radius reaches: the corners of the box are skipped, the lists are the
    // same.  A bin's extent is widened by the 0.01-bin margin of bin_lo/bin_hi.
    const float mrg = 0.01f / bs;
    auto gap = [&](int b, float x, float sh) {
        const float e0 = sh + (float)b / bs - mrg, e1 = sh + (float)(b + 1) / bs + mrg;
        return x < e0 ? e0 - x : (x > e1 ? x - e1 : 0.0f);
    };
    int vc = 0;
    for (int bz = bz0; bz <= bz1; bz++) {
        const float gz = gap(bz, hi_i.z, f.shiftf[2]);
        if (gz * gz > thr) continue;
        for (int by = by0; by <= by1; by++) {
            const float gy = gap(by, hi_i.y, f.shiftf[1]);
            const float r2 = thr - gz * gz - gy * gy;
            if (r2 < 0.0f) continue;
            const float rx = sqrtf(r2) * 1.00002f + 1e-4f;
            int xa = (int)floorf((hi_i.x - f.shiftf[0] - rx) * bs - 0.01f);
            int xb = (int)floorf((hi_i.x - f.shiftf[0] + rx) * bs + 0.01f);
            xa = xa < bx0 ? bx0 : xa;
            xb = xb > bx1 ? bx1 : xb;
            const uint32_t yz = tm_morton(0u, (uint32_t)by, (uint32_t)bz);
            for (int bx = xa; bx <= xb;) {
                // x is the lowest Morton bit: an even bin and the next one are
                // one contiguous range, visited in the same order
                const uint32_t m = yz | tm_morton((uint32_t)bx, 0u, 0u);
                const int w = ((bx & 1) == 0 && bx < xb) ? 2 : 1;
                bx += w;
                const long long j0 = bbase + __ldg(bst + m), j1 = bbase + __ldg(bst + m + w);
                auto test = [&](long long j, float4 hj, float4 lj) {
                    const float dx = (hj.x - hi_i.x) + (lj.x - lo_i.x);
                    const float dy = (hj.y - hi_i.y) + (lj.y - lo_i.y);
                    const float dz = (hj.z - hi_i.z) + (lj.z - lo_i.z);
                    const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    if (s <= thr && j != i) {
                        if (vc < a.vcap) a.vlist[(long long)vc * ls + i] = (int)j;
                        vc++;
                    }
                };
                // two candidates' loads in flight, appended in order
                long long j = j0;
                for (; j + 1 < j1; j += 2) {
                    const float4 h0 = __ldg(hi + j), l0 = __ldg(lo + j), h1 = __ldg(hi + j + 1), l1 = __ldg(lo + j + 1);
                    test(j, h0, l0);
                    test(j + 1, h1, l1);
                }
                if (j < j1) test(j, __ldg(hi + j), __ldg(lo + j));
            }
        }
    }
    a.vcount[i] = min(vc, a.vcap);
    a.x0[i] = hi_i;
    // an overflowing list cannot serve this step: flag the colony, whose
    // results the fallback search pass then computes
    if (vc > a.vcap)
        if (atomicExch(&a.frame[c].list_ok, 0) == 1) atomicAdd(&a.work[1], 1);
}

// the cells of the colonies that rebuild this step (worklist 0), a warp per
// 32-slot group; warps take the next group from a counter (work[4]) as they
// finish one, since groups differ widely in cost (dense regions hold more
// candidates), and consecutive groups run at about the same time (their
// bins and positions share the caches)
__global__ void __launch_bounds__(256) k_listbuild(tm_arrays a, const tm_consts *K)
{
    const uint32_t *wl = a.wl;
    const uint32_t total = wl[a.ncol];
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd((unsigned *)&a.work[4], 1u);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= total) break;
        int c;
        const long long i = tm_wl_slot(a, wl, q, c) + lane;
        listbuild_cell(a, K, c, i);
    }
}

template <int PREC>
__device__ __forceinline__ void plist_one(const tm_arrays &a, const tm_type &T, int dim, int t, long long i,
                                          float4 hi_i, float4 lo_i, int j, float4 hj, float4 lj, pair_acc<PREC> &acc,
                                          int &cnt_nb, int &nbmin, unsigned long long &hash, int drow)
{
    bool in;
    if constexpr (PREC == 0) {
        pair64(T, dim, a.x[i], a.y[i], a.z[i], a.x[j], a.y[j], a.z[j], a.mass[(long long)t * a.nslots_total + j],
               acc, in);
    } else {
        const float dx = (hj.x - hi_i.x) + (lj.x - lo_i.x);
        const float dy = (hj.y - hi_i.y) + (lj.y - lo_i.y);
        const float dz = (hj.z - hi_i.z) + (lj.z - lo_i.z);
        const float s = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        in = within32_at(T, s, a, i, j);
        if (in) pair32(T, dim, dx, dy, dz, s, hj.w, acc);
    }
    if (in) {
        cnt_nb++;
        nbmin = min(nbmin, PREC == 0 ? a.rank[j] : __float_as_int(lj.w));
        if (a.want_diag) diag_pair(a, drow, j, hash);
    }
}

template <int PREC, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_plist(tm_arrays a, const tm_consts *K)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (((i >> 5) << 5) >= a.nslots_total) return;
    const int c = a.col[(i >> 5) << 5];
    const tm_desc &d = a.desc[c];
    if (!d.active || d.precision != PREC || d.n <= 1 || !d.verlet) return;
    const tm_frame &f = a.frame[c];
    if (!f.list_ok) return;                 // overflowed: the search pass evaluates
    if (!tm_live(i, d)) return;
    const int dim = K->dim;
    const int t = a.ctype[i];
    const tm_type &T = K->t[t];
    const float4 hi_i = a.hi[i], lo_i = a.lo[i];
    const float4 *__restrict__ hi = a.hi;
    const float4 *__restrict__ lo = a.lo;
    pair_acc<PREC> acc;
    acc.init();
    int cnt_nb = 0, nbmin = 0x7fffffff;
    unsigned long long hash = 0;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const int cnt = __ldg(a.vcount + i);
    const long long ls = a.lstride;
    const int drow = diag_row_of(a, d, i);
    const int *__restrict__ lst = a.vlist + i;
    int k = 0;
    for (; k + 1 < cnt; k += 2, lst += 2 * ls) {
        const int j0 = __ldg(lst);
        const int j1 = __ldg(lst + ls);
        const float4 h0 = PREC ? __ldg(hi + j0) : z4, l0 = PREC ? __ldg(lo + j0) : z4;
        const float4 h1 = PREC ? __ldg(hi + j1) : z4, l1 = PREC ? __ldg(lo + j1) : z4;
        plist_one<PREC>(a, T, dim, t, i, hi_i, lo_i, j0, h0, l0, acc, cnt_nb, nbmin, hash, drow);
        plist_one<PREC>(a, T, dim, t, i, hi_i, lo_i, j1, h1, l1, acc, cnt_nb, nbmin, hash, drow);
    }
    if (k < cnt) {
        const int j0 = __ldg(lst);
        const float4 h0 = PREC ? __ldg(hi + j0) : z4, l0 = PREC ? __ldg(lo + j0) : z4;
        plist_one<PREC>(a, T, dim, t, i, hi_i, lo_i, j0, h0, l0, acc, cnt_nb, nbmin, hash, drow);
    }
    pair_store<PREC>(a, i, acc, cnt_nb, nbmin, hash, false);
    // the octree walk's first pass for this cell (see k_octree_mark): walk if
    // the first within-h neighbour in Morton order may overlap it
    bool walk = cnt_nb == 0 || a.want_diag;
    if (!walk) {
        const long long m = f.ident ? (long long)nbmin : (long long)a.tmp[nbmin];
        const float4 hm = hi[m], lm = lo[m];
        const float dx = (hi_i.x - hm.x) + (lo_i.x - lm.x), dy = (hi_i.y - hm.y) + (lo_i.y - lm.y),
                    dz = (hi_i.z - hm.z) + (lo_i.z - lm.z);
        const float rs = (hi_i.w + hm.w) * 1.0001f + 1e-5f;
        walk = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < rs * rs;
    }
    tm_queue_walk(a, c, i, cnt_nb == 0, walk);
    if constexpr (PREC == 1) {
        if (needs_fix64(acc)) {
            // FP64 density over the same list, the cutoff decided in FP64
            double dens = 0.0;
            for (int kk = 0; kk < cnt; kk++) {
                const int j = a.vlist[(long long)kk * ls + i];
                const double dist = dist64(a, i, j);
                if (dist <= T.h) dens = add64(dens, dens_term64(T, dist, a.size[j]));
            }
            a.density[i] = dens;
        }
    }
}

// List pass of the FP32 + compensated path: LPC lanes share a cell, lane q
// evaluating the cell's entries q, q + LPC, ... with two entries in flight
// and the next two list indices already loading; the lanes' compensated
// partial sums are merged by shuffles in a fixed order, so a colony's
// results do not depend on the block shape.  With LPC = 4 a warp holds 8
// Morton-consecutive cells, whose list lengths differ less than those of 32.
#define PLIST_LPC 4

// Each lane takes two entries per iteration (its entries q, q + LPC, then
// q + 2 LPC, ...) with the next two list indices already loading, and forms
// both entries' terms without branches on the cutoff: those of an entry
// beyond h (or absent) are zeroed, and each accumulator takes the pair's sum
// in one compensated add.  The pre-add rounds once per pair, an error of the
// same order as the compensated sum's own (eps times the sum of the
// magnitudes), and halves the compensated adds.
//
// v needs the octree walk only when no candidate precedes the first within-h
// neighbour m in Morton order (then j* = m, see tm_octree.cu).  A list entry
// j whose position lies inside p's query box [x - h, x + h) on every axis is
// a candidate: its own lattice code lies in the box, so its leaf meets it.
// The box test is taken with a margin (1e-4 h, two lattice units and the
// float error of the split distance), so an entry that passes is inside the
// box in the reference's FP64 lattice arithmetic too; boxmin is the least
// Morton position of such entries, and boxmin < m means j* precedes m: j* is
// not within h and v = 0 without a walk.  Both minima travel in one key,
// 2 pos + 1 for an entry within h and 2 pos for one only inside the box: the
// least key is m's (odd) unless a box entry precedes m (even).
template <int BLOCK, int MINB, bool DIAG>
__global__ void __launch_bounds__(BLOCK, MINB) k_plist32(tm_arrays a, const tm_consts *K)
{
    constexpr int LPC = PLIST_LPC;
    constexpr int CPW = 32 / LPC;
    const int lane = threadIdx.x & 31;
    const long long base = (((long long)blockIdx.x * BLOCK + threadIdx.x) >> 5) * CPW;
    if (base >= a.nslots_total) return;            // whole warps leave together
    const int c = a.col[base];                      // colonies are 32-aligned: one colony per warp
    const tm_desc &d = a.desc[c];
    if (!d.active || d.precision != 1 || d.n <= 1 || !d.verlet) return;
    const tm_frame &f = a.frame[c];
    if (!f.list_ok) return;                         // overflowed: the search pass evaluates
    const long long i = base + lane / LPC;
    const int q = lane % LPC;
    const bool live = tm_live(i, d);
    if (!__any_sync(FULL, live)) return;
    const int dim = K->dim;
    const tm_type &T = K->t[live ? a.ctype[i] : 0];
    const float thr_lo = T.thr_lo, thr_hi = T.thr_hi;
    const float4 hi_i = live ? a.hi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 lo_i = live ? a.lo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 *__restrict__ hi = a.hi;
    const float4 *__restrict__ lo = a.lo;
    // query-box half width with the margin (a lattice unit is scale / 2^29)
    const float hbox = T.hf * (1.0f - 1e-4f) - f.units2;
    pair_acc<1> acc;
    acc.init();
    int cnt_nb = 0;
    unsigned key = 0xffffffffu;
    unsigned long long hash = 0;
    const int cnt = live ? __ldg(a.vcount + i) : 0;
    const long long ls = a.lstride;
    const int drow = (DIAG && live) ? diag_row_of(a, d, i) : -1;
    const int *__restrict__ lst = a.vlist + i;
    int k = q;
    int ja = k < cnt ? __ldg(lst + k * ls) : 0;
    int jb = k + LPC < cnt ? __ldg(lst + (k + LPC) * ls) : 0;
    for (; k < cnt; k += 2 * LPC) {
        const int kn = k + 2 * LPC;
        const int na = kn < cnt ? __ldg(lst + kn * ls) : 0;
        const int nb = kn + LPC < cnt ? __ldg(lst + (kn + LPC) * ls) : 0;
        const bool hasb = k + LPC < cnt;
        const float4 ha = __ldg(hi + ja), la = __ldg(lo + ja);
        const float4 hb = __ldg(hi + jb), lb = __ldg(lo + jb);   // jb = 0 (a valid slot) when absent
        const float dxa = (ha.x - hi_i.x) + (la.x - lo_i.x), dya = (ha.y - hi_i.y) + (la.y - lo_i.y),
                    dza = (ha.z - hi_i.z) + (la.z - lo_i.z);
        const float dxb = (hb.x - hi_i.x) + (lb.x - lo_i.x), dyb = (hb.y - hi_i.y) + (lb.y - lo_i.y),
                    dzb = (hb.z - hi_i.z) + (lb.z - lo_i.z);
        const float sa = fmaf(dxa, dxa, fmaf(dya, dya, dza * dza));
        const float sb = fmaf(dxb, dxb, fmaf(dyb, dyb, dzb * dzb));
        bool ina = sa <= thr_lo, inb = hasb && sb <= thr_lo;
        if (!ina && sa <= thr_hi) ina = dist64(a, i, ja) <= T.h;            // FP64 only in the band
        if (hasb && !inb && sb <= thr_hi) inb = dist64(a, i, jb) <= T.h;
        float ta, ea, ga, tb, eb, gb;
        pair32_terms(T, sa, ha.w, ta, ea, ga);
        pair32_terms(T, sb, hb.w, tb, eb, gb);
        ta = ina ? ta : 0.0f;
        ea = ina ? ea : 0.0f;
        ga = ina ? ga : 0.0f;
        tb = inb ? tb : 0.0f;
        eb = inb ? eb : 0.0f;
        gb = inb ? gb : 0.0f;
        acc.dens.add(ta + tb);
        acc.err2 = fmaf(ea, ea, fmaf(eb, eb, acc.err2));
        acc.fx.add(fmaf(ga, dxa, gb * dxb));
        acc.fy.add(fmaf(ga, dya, gb * dyb));
        if (dim == 3) acc.fz.add(fmaf(ga, dza, gb * dzb));
        // over every entry: with a neighbour within h the minimum is one of
        // them (an entry beyond h is farther); a cell with none takes its
        // mindist from the octree walk
        acc.mins = fminf(acc.mins, fminf(sa, hasb ? sb : 3.0e38f));
        cnt_nb += (ina ? 1 : 0) + (inb ? 1 : 0);
        const unsigned pa = 2u * (unsigned)__float_as_int(la.w), pb = 2u * (unsigned)__float_as_int(lb.w);
        const bool bxa = fmaxf(fabsf(dxa), fmaxf(fabsf(dya), fabsf(dza))) < hbox;
        const bool bxb = hasb && fmaxf(fabsf(dxb), fmaxf(fabsf(dyb), fabsf(dzb))) < hbox;
        key = min(key, min(ina ? pa + 1u : (bxa ? pa : 0xffffffffu), inb ? pb + 1u : (bxb ? pb : 0xffffffffu)));
        if (DIAG) {
            if (ina) diag_pair(a, drow, ja, hash);
            if (inb) diag_pair(a, drow, jb, hash);
        }
        ja = na;
        jb = nb;
    }
    // merge the LPC partial results of each cell (fixed butterfly order)
    for (int o = 1; o < LPC; o <<= 1) {
        acc.dens.merge(__shfl_xor_sync(FULL, acc.dens.s, o), __shfl_xor_sync(FULL, acc.dens.c, o));
        acc.fx.merge(__shfl_xor_sync(FULL, acc.fx.s, o), __shfl_xor_sync(FULL, acc.fx.c, o));
        acc.fy.merge(__shfl_xor_sync(FULL, acc.fy.s, o), __shfl_xor_sync(FULL, acc.fy.c, o));
        acc.fz.merge(__shfl_xor_sync(FULL, acc.fz.s, o), __shfl_xor_sync(FULL, acc.fz.c, o));
        acc.mins = fminf(acc.mins, __shfl_xor_sync(FULL, acc.mins, o));
        acc.err2 += __shfl_xor_sync(FULL, acc.err2, o);
        cnt_nb += __shfl_xor_sync(FULL, cnt_nb, o);
        key = min(key, __shfl_xor_sync(FULL, key, o));
        if (DIAG) hash += __shfl_xor_sync(FULL, hash, o);
    }
    // with cnt_nb > 0 an odd key is m's, an even one a box entry's before m
    // (nbmin is read by the walk only, which then does not run)
    const int nbmin = (int)(key >> 1);
    // the merged results are the same in the cell's four lanes; lane 0 owns them
    const bool owner = live && q == 0;
    bool walk = false;
    if (owner) {
        pair_store<1>(a, i, acc, cnt_nb, nbmin, hash, false);
        // the octree walk's first pass for this cell (see k_octree_mark): walk
        // if the first within-h neighbour in Morton order may overlap it and
        // no list entry shows a candidate before it (diagnostics walk every
        // cell: they record j*)
        walk = cnt_nb == 0 || DIAG;
        if (!walk && (key & 1u)) {
            const long long m = f.ident ? (long long)nbmin : (long long)a.tmp[nbmin];
            const float4 hm = hi[m], lm = lo[m];
            const float dx = (hi_i.x - hm.x) + (lo_i.x - lm.x), dy = (hi_i.y - hm.y) + (lo_i.y - lm.y),
                        dz = (hi_i.z - hm.z) + (lo_i.z - lm.z);
            const float rs = (hi_i.w + hm.w) * 1.0001f + 1e-5f;
            walk = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < rs * rs;
        }
    }
    // one queue append per warp: every lane takes part, the owners carry the cells
    tm_queue_walk_owned(a, c, i, owner, cnt_nb == 0, walk);
    if (live && needs_fix64(acc)) {
        // FP64 density over the same list, the cutoff decided in FP64, the
        // list split over the cell's lanes and the partial sums added in a
        // fixed order
        const unsigned gmask = 0xfu << (lane & ~(LPC - 1));
        if (q == 0) atomicAdd(&a.frame[c].fix64, 1ull);
        double dens = 0.0;
        for (int kk = q; kk < cnt; kk += LPC) {
            const int j = a.vlist[(long long)kk * ls + i];
            const double dist = dist64(a, i, j);
            if (dist <= T.h) dens += dens_term64_fast(T, dist, a.size[j]);
        }
        for (int o = 1; o < LPC; o <<= 1) dens = add64(dens, __shfl_xor_sync(gmask, dens, o));
        if (q == 0) a.density[i] = dens;
    }
}

// FP64 density of the cells flagged by the FP32 path: the same neighbour set
// (exact FP64 cutoff) and the reference expression of potential.c:62.
__global__ void __launch_bounds__(128) k_density_fix64(tm_arrays a, const tm_consts *K)
{
    const int nfix = *a.fix_count;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nfix; q += gridDim.x * blockDim.x) {
        const long long i = a.fix_list[q];
        const int c = a.col[i];
        const tm_desc &d = a.desc[c];
        const tm_frame &f = a.frame[c];
        const tm_type &T = K->t[a.ctype[i]];
        const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
        const int nside = 1 << f.L;
        int lo[3], hi[3];
        const double pos[3] = {xi, yi, zi};
        for (int k = 0; k < 3; k++) {
            const float v0 = ((float)pos[k] - f.shiftf[k] - (float)T.h) * f.binscale - 0.01f;
            const float v1 = ((float)pos[k] - f.shiftf[k] + (float)T.h) * f.binscale + 0.01f;
            lo[k] = max(0, min(nside - 1, (int)floorf(v0)));
            hi[k] = max(0, min(nside - 1, (int)floorf(v1)));
        }
        const uint32_t *bst = a.bin_start + d.binoff;
        const bool ident = f.ident != 0;
        double dens = 0.0;
        for (int bz = lo[2]; bz <= hi[2]; bz++)
            for (int by = lo[1]; by <= hi[1]; by++)
                for (int bx = lo[0]; bx <= hi[0]; bx++) {
                    const uint32_t m = tm_morton((uint32_t)bx, (uint32_t)by, (uint32_t)bz);
                    const long long j0 = f.bin_base + bst[m], j1 = f.bin_base + bst[m + 1];
                    for (long long jk = j0; jk < j1; jk++) {
                        const long long j = ident ? jk : (long long)a.tmp[jk];   // slot of position jk
                        if (j == i) continue;
                        const double dist = dist64(a, i, j);
                        if (!(dist <= T.h)) continue;
                        dens = add64(dens, dens_term64(T, dist, a.size[j]));
                    }
                }
        a.density[i] = dens;
    }
}

// resident blocks of the pair kernel on the current device (all SMs)
static unsigned pair_grid_cap(int prec)
{
    static int cached[2][64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1024;
    if (!cached[prec][dev]) {
        int sms = 0, per = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (prec == 0)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pair<0>, TM_WARPS_PER_BLOCK * 32, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pair<1>, TM_WARPS_PER_BLOCK * 32, 0);
        cached[prec][dev] = std::max(1, sms) * std::max(1, per);
    }
    return (unsigned)cached[prec][dev];
}

template <bool DIAG>
static void launch_plist32(const tm_arrays &a, const tm_consts *K, int variant, cudaStream_t st)
{
    // PLIST_LPC threads per slot (a warp holds 32 / PLIST_LPC cells)
    const long long nt = a.nslots_total * PLIST_LPC;
    switch (variant) {
    // every variant accumulates alike (the paired form), so the block shape
    // changes no result bit
    case 2: k_plist32<64, 16, DIAG><<<(unsigned)((nt + 63) / 64), 64, 0, st>>>(a, K); break;
    case 3: k_plist32<64, 14, DIAG><<<(unsigned)((nt + 63) / 64), 64, 0, st>>>(a, K); break;
    case 4: k_plist32<256, 3, DIAG><<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(a, K); break;
    default: k_plist32<128, 7, DIAG><<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(a, K); break;
    }
}

template <int PREC>
static void launch_plist(const tm_arrays &a, const tm_consts *K, int variant, cudaStream_t st)
{
    const long long n = a.nslots_total;
    switch (variant) {
    case 2: k_plist<PREC, 128, 8><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a, K); break;
    case 3: k_plist<PREC, 256, 3><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, K); break;
    case 4: k_plist<PREC, 512, 2><<<(unsigned)((n + 511) / 512), 512, 0, st>>>(a, K); break;
    default: k_plist<PREC, 256, 4><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, K); break;
    }
}

static unsigned pair_grid(const tm_arrays &a, int prec)
{
    const long long groups = (a.nslots_total + PAIR_CPW - 1) / PAIR_CPW;
    const long long need = (groups + TM_WARPS_PER_BLOCK - 1) / TM_WARPS_PER_BLOCK;
    return (unsigned)std::min<long long>(need, pair_grid_cap(prec != 0));
}

// search pass (fallback 0: searches of colonies without lists; fallback 1:
// searches of colonies whose lists overflowed)
cudaError_t tm_launch_search(const tm_arrays &a, const tm_consts *K, int prec, const tm_shapes &sh, int fallback,
                             cudaStream_t st)
{
    const unsigned grid = pair_grid(a, prec);
    if (grid == 0) return cudaSuccess;
    if (fallback && a.vcap == 0) return cudaSuccess;
    const int bt = TM_WARPS_PER_BLOCK * 32;
    if (prec == 0) k_pair<0><<<grid, bt, 0, st>>>(a, K, fallback, sh.pair_lshift);
    else k_pair<1><<<grid, bt, 0, st>>>(a, K, fallback, sh.pair_lshift);
    return cudaGetLastError();
}

// list build of the colonies that rebuild their lists this step (both precisions)
cudaError_t tm_launch_listbuild(const tm_arrays &a, const tm_consts *K, cudaStream_t st)
{
    if (a.vcap == 0 || a.nslots_total == 0) return cudaSuccess;
    k_listbuild<<<tm_stream_grid(256, 16), 256, 0, st>>>(a, K);
    return cudaGetLastError();
}

// list pass (colonies with valid lists)
cudaError_t tm_launch_list(const tm_arrays &a, const tm_consts *K, int prec, const tm_shapes &sh, cudaStream_t st)
{
    if (a.vcap == 0 || a.nslots_total == 0) return cudaSuccess;
    if (prec == 0) launch_plist<0>(a, K, sh.list_variant, st);
    else if (a.want_diag) launch_plist32<true>(a, K, sh.list_variant, st);
    else launch_plist32<false>(a, K, sh.list_variant, st);
    return cudaGetLastError();
}

// FP64 density of the FP32 cells the search passes flagged
cudaError_t tm_launch_fix(const tm_arrays &a, const tm_consts *K, cudaStream_t st)
{
    k_density_fix64<<<256, 128, 0, st>>>(a, K);
    return cudaGetLastError();
}
