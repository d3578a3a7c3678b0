// Build phase of one step: bounding box and affine map, lattice codes, Morton
// bins, counting sort into Morton order, gather of the cell state.
//
// Replaces octbuild (octree.c:145-207).  The reference inserts cells one by one
// into a pointer octree; here the same octree is implicit in the Morton order
// of the same lattice codes: a node is a contiguous run of sorted cells that
// share a prefix, and a cell's leaf is the largest node holding only it.
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

#include <algorithm>

#define FULL 0xffffffffu

// ---------------------------------------------------------------------------
// per-step reset of the frames and the bin table's padding entries

__global__ void k_step_init(tm_arrays a)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncol) return;
    tm_frame &f = a.frame[c];
    for (int t = 0; t < TM_MAX_TYPES; t++) {
        for (int k = 0; k < 3; k++) {
            f.bbox[t][k] = 0xffffffffffffffffull;
            f.bbox[t][3 + k] = 0ull;
        }
    }
    f.error = 0;
    f.nbig = 0;
    f.boundary_pairs = 0;
    f.codes_slow = 0;
    f.fix64 = 0;
    f.walks = 0;
    f.walks_isolated = 0;
    // Neighbour lists stay valid while no pair can have come from beyond
    // h + skin to within h: every cell moved less than skin/2 since the lists
    // were built (maxdisp carries a float-rounding margin).
    const tm_desc &d = a.desc[c];
    const bool rb = !d.verlet || f.force_rebuild || !f.list_ok || f.age + 1 >= d.rmax ||
                    2.0f * __uint_as_float(f.maxdisp) + 1e-3f >= d.skin;
    f.rebuild = rb ? 1 : 0;
    f.ident = f.rebuild;
    if (rb) {
        f.age = 0;
        f.rebuilds++;
        f.list_ok = d.verlet;      // cleared again if a list overflows
    } else {
        f.age++;
    }
    if (rb && d.active && d.n > 1 && !d.verlet) atomicAdd(&a.work[0], 1);   // colonies the search pass serves
    f.force_rebuild = 0;
    f.disp = rb ? 0u : f.maxdisp;
    f.maxdisp = 0u;
    for (int k = 0; k < 3; k++) {
        f.patch_lo[k] = 2147483647ll;
        f.patch_hi[k] = -2147483648ll;
    }
    f.step_counter++;
}

// slot of the colony's first bin (after the scan)
__global__ void k_binbase(tm_arrays a)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncol) return;
    const tm_desc &d = a.desc[c];
    a.frame[c].bin_base = d.off - (long long)a.bin_start[d.binoff];
}

// ---------------------------------------------------------------------------
// bounding box with the per-type pad h + 0.01 (octree.c:155-174).
// min over cells of fl(x - e) equals fl(min x - e) because rounding is
// monotone, so per-type minima/maxima of x suffice; they are reduced on the
// order-preserving integer image of the doubles (no FP64 instructions).

// Each warp streams BBOX_GROUPS groups of 32 slots (a group lies in one
// colony: colonies are 32-aligned) and keeps running per-type minima and
// maxima in registers; it reduces them across the lanes and posts them only
// when the colony changes and at the end of its groups.  The positions, types
// and colonies of BBOX_BATCH groups are loaded before any of them is used, so
// a warp waits for memory once per batch rather than once per group.
#define BBOX_GROUPS 16
#define BBOX_BATCH 4

template <int NT>
__device__ __forceinline__ void bbox_post(tm_arrays &a, int c, unsigned long long (&r)[NT][6], int lane)
{
#pragma unroll
    for (int tt = 0; tt < NT; tt++) {
#pragma unroll
        for (int q = 0; q < 6; q++) {
            unsigned long long v = r[tt][q];
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long u = __shfl_xor_sync(FULL, v, o);
                v = q < 3 ? (u < v ? u : v) : (u > v ? u : v);
            }
            // the box only widens during the pass: post only what reaches past its current value
            if (lane == 0 && (q < 3 ? v != 0xffffffffffffffffull : v != 0ull)) {
                unsigned long long *t = &a.frame[c].bbox[tt][q];
                if (q < 3 && v < __ldcg(t)) atomicMin(t, v);
                else if (q >= 3 && v > __ldcg(t)) atomicMax(t, v);
            }
            r[tt][q] = q < 3 ? 0xffffffffffffffffull : 0ull;
        }
    }
}

template <int NT>
__device__ __forceinline__ void bbox_take(unsigned long long (&r)[NT][6], int t, double x, double y, double z)
{
    const unsigned long long v0 = tm_ordered(x), v1 = tm_ordered(y), v2 = tm_ordered(z);
#pragma unroll
    for (int tt = 0; tt < NT; tt++) {
        if (t != tt) continue;
        r[tt][0] = v0 < r[tt][0] ? v0 : r[tt][0];
        r[tt][1] = v1 < r[tt][1] ? v1 : r[tt][1];
        r[tt][2] = v2 < r[tt][2] ? v2 : r[tt][2];
        r[tt][3] = v0 > r[tt][3] ? v0 : r[tt][3];
        r[tt][4] = v1 > r[tt][4] ? v1 : r[tt][4];
        r[tt][5] = v2 > r[tt][5] ? v2 : r[tt][5];
    }
}

template <int NT>
__global__ void __launch_bounds__(256) k_bbox(tm_arrays a, int ntypes)
{
    const int lane = threadIdx.x & 31;
    const long long ngroups = (a.nslots_total + 31) >> 5;
    const long long g0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * BBOX_GROUPS;
    if (g0 >= ngroups) return;                      // whole warp
    const long long g1 = g0 + BBOX_GROUPS < ngroups ? g0 + BBOX_GROUPS : ngroups;
    unsigned long long r[NT][6];
#pragma unroll
    for (int tt = 0; tt < NT; tt++)
#pragma unroll
        for (int q = 0; q < 6; q++) r[tt][q] = q < 3 ? 0xffffffffffffffffull : 0ull;
    int cur = -1;                                   // the colony being reduced
    for (long long gb = g0; gb < g1; gb += BBOX_BATCH) {
        double px[BBOX_BATCH], py[BBOX_BATCH], pz[BBOX_BATCH];
        int pt[BBOX_BATCH], pc[BBOX_BATCH];
#pragma unroll
        for (int u = 0; u < BBOX_BATCH; u++) {
            const long long g = gb + u, s = (g << 5) + lane;
            const bool in = g < g1 && s < a.nslots_total;
            pc[u] = g < g1 ? a.col[g << 5] : -1;    // uniform over the group
            px[u] = in ? a.x[s] : 0.0;
            py[u] = in ? a.y[s] : 0.0;
            pz[u] = in ? a.z[s] : 0.0;
            pt[u] = in ? a.ctype[s] : -1;
        }
        bool one = true;                            // the batch lies in one colony
#pragma unroll
        for (int u = 1; u < BBOX_BATCH; u++) one = one && (pc[u] == pc[0] || pc[u] < 0);
        if (one) {
            const int c = pc[0];
            const tm_desc &d = a.desc[c];
            if (!d.active) continue;
            if (c != cur) {
                if (cur >= 0) bbox_post<NT>(a, cur, r, lane);
                cur = c;
            }
#pragma unroll
            for (int u = 0; u < BBOX_BATCH; u++) {
                const long long s = ((gb + u) << 5) + lane;
                if (pc[u] >= 0 && s < a.nslots_total && tm_live(s, d)) bbox_take<NT>(r, pt[u], px[u], py[u], pz[u]);
            }
        } else {
            // a colony boundary inside the batch: group by group
#pragma unroll 1
            for (long long g = gb; g < gb + BBOX_BATCH && g < g1; g++) {
                const int c = a.col[g << 5];
                const tm_desc &d = a.desc[c];
                if (!d.active) continue;
                if (c != cur) {
                    if (cur >= 0) bbox_post<NT>(a, cur, r, lane);
                    cur = c;
                }
                const long long s = (g << 5) + lane;
                if (s < a.nslots_total && tm_live(s, d)) bbox_take<NT>(r, a.ctype[s], a.x[s], a.y[s], a.z[s]);
            }
        }
    }
    if (cur >= 0) bbox_post<NT>(a, cur, r, lane);
    (void)ntypes;
}

cudaError_t tm_launch_bbox(const tm_arrays &a, int ntypes, cudaStream_t st)
{
    const long long ngroups = (a.nslots_total + 31) >> 5;
    const long long warps = (ngroups + BBOX_GROUPS - 1) / BBOX_GROUPS;
    const unsigned grid = (unsigned)std::max(1ll, (warps + 7) / 8);
    if (ntypes <= 1) k_bbox<1><<<grid, 256, 0, st>>>(a, ntypes);
    else if (ntypes <= 2) k_bbox<2><<<grid, 256, 0, st>>>(a, ntypes);
    else if (ntypes <= 4) k_bbox<4><<<grid, 256, 0, st>>>(a, ntypes);
    else k_bbox<TM_MAX_TYPES><<<grid, 256, 0, st>>>(a, ntypes);
    return cudaGetLastError();
}

// affShift / affScale (octree.c:175-180) and the bin depth of each colony
__global__ void k_frame(tm_arrays a, const tm_consts *K)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncol) return;
    tm_frame &f = a.frame[c];
    const tm_desc &d = a.desc[c];
    f.n = d.n;
    if (!d.active || d.n == 0) return;   // octbuild returns early: the previous map stays
    double bmin[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double bmax[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    double hmax = 0.0;
    for (int t = 0; t < K->ntypes; t++) {
        if (f.bbox[t][3] == 0ull) continue;   // no cell of this type
        double e = K->t[t].e;
        hmax = K->t[t].h > hmax ? K->t[t].h : hmax;
        for (int k = 0; k < 3; k++) {
            double lo = sub64(tm_unordered(f.bbox[t][k]), e);
            double hi = add64(tm_unordered(f.bbox[t][3 + k]), e);
            bmin[k] = lo < bmin[k] ? lo : bmin[k];
            bmax[k] = hi > bmax[k] ? hi : bmax[k];
        }
    }
    double sc = sub64(bmax[0], bmin[0]);
    sc = (sc > sub64(bmax[1], bmin[1]) ? sc : sub64(bmax[1], bmin[1]));
    sc = (sc > sub64(bmax[2], bmin[2]) ? sc : sub64(bmax[2], bmin[2]));
    f.scale = sc;
    for (int k = 0; k < 3; k++) {
        f.shift[k] = bmin[k];
        f.shiftf[k] = (float)bmin[k];
    }
    // deepest level whose bins are at least h/2 wide
    int L = 1;
    while (L < d.Lcap && sc / (double)(1 << (L + 1)) >= 0.5 * hmax) L++;
    f.L = L;
    f.nbins = 1u << (3 * L);
    f.binscale = (float)((double)(1 << L) / sc);
    f.units2 = (float)(sc * 3.7252902984619141e-9);
    // integer lattice path: cmul = 2^(78-ck)/scale in [2^62, 2^63)
    int es = 0;
    frexp(sc, &es);                       // sc in [2^(es-1), 2^es)
    const int ck = 16 - es;
    const bool small_shift = fabs(f.shift[0]) < 16384.0 && fabs(f.shift[1]) < 16384.0 && fabs(f.shift[2]) < 16384.0;
    if (ck >= 1 && ck <= 40 && small_shift) {
        f.ck = ck;
        f.cmul = (unsigned long long)ldexp(1.0 / sc, 78 - ck);
        for (int k = 0; k < 3; k++) f.sh_fx[k] = (long long)ldexp(f.shift[k], 47);
        // bound of |integer value - FP64 value| in lattice units, doubled:
        // FP64 roundings of x -+ h and - shift on values below 2^15 (2^-37 each
        // after two operations) and of the division (2^-24), plus the three
        // fixed-point truncations (2^-47 each) and the product (2^-31)
        const double eps = 2.0 * (ldexp(1.0, -8) / sc + 3.0 * ldexp(1.0, -18) / sc + ldexp(1.0, -23));
        f.ceps = eps >= 0.25 ? 0x40000000u : (uint32_t)ldexp(eps, 32) + 1u;
    } else {
        f.ck = 1;
        f.cmul = 0;
        f.ceps = 0xffffffffu;             // never accept: exact FP64 path for every code
    }
}

// exact lattice codes (octree.c:187-191) and bin occupancy
__global__ void k_codes(tm_arrays a)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.nslots_total) return;
    // the position loads go out with the colony's, not after it
    const double px = a.x[s], py = a.y[s], pz = a.z[s];
    int c = a.col[s];
    const tm_desc &d = a.desc[c];
    if (!d.active || !tm_live(s, d)) return;
    const tm_frame &f = a.frame[c];
    uint4 q;
    long long X, Y, Z;
    const bool okx = tm_fix47(px, X), oky = tm_fix47(py, Y), okz = tm_fix47(pz, Z);
    unsigned slow = 0;
    q.x = tm_lattice_fast(px, X, okx, 0, 0.0, f, 0, slow);
    q.y = tm_lattice_fast(py, Y, oky, 0, 0.0, f, 1, slow);
    q.z = tm_lattice_fast(pz, Z, okz, 0, 0.0, f, 2, slow);
    q.w = 0;
    if (slow) atomicAdd(&a.frame[c].codes_slow, (unsigned long long)slow);
    a.code[s] = q;
    uint32_t b = (uint32_t)(d.binoff) + tm_prefix(q, f.L);
    a.bin[s] = b;
    // one atomic per distinct bin in the warp
    unsigned peers = __match_any_sync(__activemask(), b);
    int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&a.bin_count[b], (uint32_t)__popc(peers));
}

// Group each colony's live slots by bin (grp holds the slots of bin b at the
// bin's Morton positions, in no particular order): the count k_codes left in
// bin_count is taken down as the cursor, and the slot that takes the last
// place of a bin of more than 32 cells queues it for k_binsort_big.
__global__ void k_scatter(tm_arrays a)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.nslots_total) return;
    int c = a.col[s];
    const tm_desc &d = a.desc[c];
    if (!d.active || !tm_live(s, d)) return;
    const uint32_t b = a.bin[s];
    const uint32_t k = atomicSub(&a.bin_count[b], 1u) - 1u;
    const uint32_t b0 = a.bin_start[b];
    a.grp[a.frame[c].bin_base + b0 + k] = (int)s;
    if (k == 0 && a.bin_start[b + 1] - b0 > 32) {
        atomicAdd(&a.frame[c].nbig, 1);
        const int q = atomicAdd(&a.bigbins[0], 1);
        a.bigbins[1 + 2 * q] = (int)b;
        a.bigbins[2 + 2 * q] = c;
    }
}

// Morton order bookkeeping of every step for the cell in slot r, whose
// Morton position is i, and for colonies that rebuild their neighbour lists
// the move of its state into Morton order (into the scratch buffers;
// k_copyback brings it back).  Positions are split for the FP32 path and the
// FP64 density weights sc_t * (size_j / csize_t) of potential.c:62 are
// precomputed for every query type t.
__device__ __forceinline__ void place_one(const tm_arrays &a, const tm_consts *K, const tm_desc &d, bool rebuild,
                                          long long r, long long i, uint4 key, double x, double y, double z,
                                          double sz)
{
    a.tmp[i] = (int)r;
    a.codes[i] = key;
    long long s;                            // slot the split positions go to
    if (rebuild) {
        a.x2[i] = x;
        a.y2[i] = y;
        a.z2[i] = z;
        a.size2[i] = sz;
        a.young2[i] = a.young[r];
        a.ctype2[i] = a.ctype[r];
        a.phase2[i] = a.phase[r];
        a.perm2[i] = a.perm[r];
        a.rem2[i] = a.rem[r];
        a.rank[i] = (int)i;
        s = i;
        if (d.precision == 0) {
            for (int t = 0; t < K->ntypes; t++)
                a.mass[(long long)t * a.nslots_total + i] = mul64(K->t[t].sc, div64(sz, K->t[t].csize));
        }
    } else {
        a.rank[r] = (int)i;
        s = r;
    }
    float hx, hy, hz, lx, ly, lz;
    tm_split(x, hx, lx);
    tm_split(y, hy, ly);
    tm_split(z, hz, lz);
    a.hi[s] = make_float4(hx, hy, hz, (float)sz);
    // .w carries the Morton position of this step (what rank[s] holds)
    a.lo[s] = make_float4(lx, ly, lz, __int_as_float((int)i));
}

// One thread per slot: the cell's Morton position is its bin's first
// position plus the number of the bin's cells whose codes sort before its own
// (ties, an error, by slot); then the cell is placed there.  The cell's own
// data are read in slot order; only the bin's members (up to 32, grouped by
// k_scatter) are gathered.  Cells of larger bins are left to k_binsort_big.
__global__ void __launch_bounds__(256) k_place(tm_arrays a, const tm_consts *K)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nslots_total) return;
    const double x = a.x[r], y = a.y[r], z = a.z[r], sz = a.size[r];
    const uint4 key = a.code[r];
    const uint32_t b = a.bin[r];
    const int c = a.col[r];
    const tm_desc &d = a.desc[c];
    if (!d.active || !tm_live(r, d)) return;
    const tm_frame &f = a.frame[c];
    const uint32_t b0 = a.bin_start[b];
    const uint32_t cnt = a.bin_start[b + 1] - b0;
    if (cnt > 32) return;
    const long long st = f.bin_base + b0;
    uint32_t rk = 0;
    bool dup = false;
    // a bin of one cell (most of them) needs no member read
    for (uint32_t k = 0; cnt > 1 && k < cnt; k++) {
        const int j = a.grp[st + k];
        if (j == (int)r) continue;
        const uint4 kj = a.code[j];
        if (tm_morton_less(kj, key)) rk++;
        else if (tm_code_eq(kj, key)) {
            dup = true;
            if (j < (int)r) rk++;
        }
    }
    if (dup) atomicOr(&a.frame[c].error, TM_ERR_CODES);
    place_one(a, K, d, f.rebuild != 0, r, st + rk, key, x, y, z, sz);
}

// one block per large bin: bitonic sort of up to TM_BIG_BIN cells in shared
// memory, then the cells are placed at their Morton positions
__global__ void k_binsort_big(tm_arrays a, const tm_consts *K)
{
    __shared__ uint4 key[TM_BIG_BIN];
    __shared__ int idx[TM_BIG_BIN];
    int nbig = a.bigbins[0];
    for (int q = blockIdx.x; q < nbig; q += gridDim.x) {
        uint32_t b = (uint32_t)a.bigbins[1 + 2 * q];
        int c = a.bigbins[2 + 2 * q];
        const tm_desc &d = a.desc[c];
        const tm_frame &f = a.frame[c];
        long long st = f.bin_base + a.bin_start[b];
        uint32_t cnt = a.bin_start[b + 1] - a.bin_start[b];
        if (cnt > TM_BIG_BIN) {
            if (threadIdx.x == 0) atomicOr(&a.frame[c].error, TM_ERR_BIGBIN);
            continue;
        }
        uint32_t p2 = 1;
        while (p2 < cnt) p2 <<= 1;
        for (uint32_t k = threadIdx.x; k < p2; k += blockDim.x) {
            if (k < cnt) {
                idx[k] = a.grp[st + k];       // grouped by k_scatter
                key[k] = a.code[idx[k]];
            } else {
                idx[k] = -1;
                key[k] = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
            }
        }
        __syncthreads();
        for (uint32_t size = 2; size <= p2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t k = threadIdx.x; k < p2; k += blockDim.x) {
                    uint32_t m = k ^ stride;
                    if (m > k) {
                        bool up = (k & size) == 0;
                        uint4 ka = key[k], kb = key[m];
                        // padding keys (idx -1) sort last; equal codes by slot
                        bool a_pad = idx[k] < 0, b_pad = idx[m] < 0;
                        bool gt = a_pad ? !b_pad
                                        : (b_pad ? false
                                                 : (tm_morton_less(kb, ka) || (tm_code_eq(kb, ka) && idx[m] < idx[k])));
                        if (gt == up) {
                            key[k] = kb;
                            key[m] = ka;
                            int t = idx[k];
                            idx[k] = idx[m];
                            idx[m] = t;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
            if (k > 0 && tm_code_eq(key[k], key[k - 1])) atomicOr(&a.frame[c].error, TM_ERR_CODES);
            const long long r = idx[k];
            place_one(a, K, d, f.rebuild != 0, r, st + k, key[k], a.x[r], a.y[r], a.z[r], a.size[r]);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void copyback_one(const tm_arrays &a, long long i)
{
    a.x[i] = a.x2[i];
    a.y[i] = a.y2[i];
    a.z[i] = a.z2[i];
    a.size[i] = a.size2[i];
    a.young[i] = a.young2[i];
    a.ctype[i] = a.ctype2[i];
    a.phase[i] = a.phase2[i];
    a.perm[i] = a.perm2[i];
    a.rem[i] = a.rem2[i];
}

// 32-slot groups of the colonies a worklist holds (see tm_arrays.wl)
__device__ __forceinline__ uint32_t wl_groups(const tm_arrays &a, int c, int which)
{
    const tm_desc &d = a.desc[c];
    const tm_frame &f = a.frame[c];
    if (!d.active || d.n == 0) return 0;
    const bool in = which == 0 ? f.rebuild != 0 : (d.n > 1 && (!d.verlet || !f.list_ok));
    return in ? (uint32_t)((d.n + 31) >> 5) : 0u;
}

// One block: worklist `which` as an exclusive prefix over the colonies.  The
// kernels that serve only some colonies in a step (the copy back and the list
// build on rebuild steps, the walk's first pass for colonies without lists)
// stride over the list's groups with a small grid, so a step where no colony
// needs them costs one launch that reads the list's length, not a pass over
// every slot.
__global__ void __launch_bounds__(1024) k_worklist(tm_arrays a, int which)
{
    __shared__ uint32_t part[1024];
    uint32_t *wl = a.wl + (long long)which * a.wl_stride;
    const int nc = a.ncol;
    const int per = (nc + 1023) >> 10;
    const int c0 = (int)threadIdx.x * per;
    const int c1 = min(c0 + per, nc);
    uint32_t sum = 0;
    for (int c = c0; c < c1; c++) sum += wl_groups(a, c, which);
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int c = c0; c < c1; c++) {
        wl[c] = run;
        run += wl_groups(a, c, which);
    }
    if (threadIdx.x == 1023) wl[nc] = part[1023];
}

unsigned tm_stream_grid(int block, int per_sm)
{
    static int sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    const int nsm = (dev >= 0 && dev < 64 && sms[dev] > 0) ? sms[dev] : 152;
    (void)block;
    return (unsigned)(nsm * per_sm);
}

// state of the rebuilding colonies back from the gather target (worklist 0)
__global__ void __launch_bounds__(256) k_copyback(tm_arrays a)
{
    const uint32_t *wl = a.wl;
    const uint32_t total = wl[a.ncol];
    const int lane = threadIdx.x & 31;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < total;
         q += (gridDim.x * blockDim.x) >> 5) {
        int c;
        const long long i = tm_wl_slot(a, wl, q, c) + lane;
        if (!tm_live(i, a.desc[c])) continue;
        copyback_one(a, i);
    }
}

// ---------------------------------------------------------------------------
// node count of the reference octree, for cellsinfo->octsize:
// 1 + sum_k (leafdepth_k - lcp(k-1, k)) over the Morton-sorted cells, where
// leafdepth_k = 1 + max(lcp(k-1,k), lcp(k,k+1)) and lcp counts shared levels.

__global__ void k_octsize(tm_arrays a, unsigned long long *out)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long term = 0;
    int c = 0;
    if (i < a.nslots_total) {
        c = a.col[i];
        const tm_desc &d = a.desc[c];
        long long k = i - d.off;
        if (d.active && k >= 0 && k < d.n && d.n >= 2) {
            uint4 me = a.codes[i];
            int lp = k > 0 ? tm_lcp(a.codes[i - 1], me) : 0;
            int ln = (k + 1 < d.n) ? tm_lcp(me, a.codes[i + 1]) : 0;
            int leaf = 1 + (lp > ln ? lp : ln);
            term = (unsigned long long)(leaf - lp);
        }
    }
    for (int o = 16; o > 0; o >>= 1) term += __shfl_xor_sync(FULL, term, o);
    if ((threadIdx.x & 31) == 0 && term) atomicAdd(&out[c], term);
}
