// Octree-walk quantities that depend on the reference's tree, not only on
// distances:
//   v        potential.c:118-125 assigns (not adds) potential() of every
//            candidate, so v is potential(p, j*) for the LAST candidate the
//            walk visits.  The walk pops child 7 first (LIFO over children
//            pushed 0..7), so j* is the candidate first in Morton order.
//   mindist  potential.c:49 takes the minimum over all candidates, within h or
//            not.  With a neighbour within h that is the nearest-neighbour
//            distance (the pair kernel's value); for a cell with no neighbour
//            within h it is the minimum over the candidates of the walk.
// A candidate is a cell j != p whose octree leaf intersects p's query box
// (octcomputebox octree.c:246-266, octnodeintersection inline.h:26-32).  The
// octree is implicit in the Morton-sorted codes: a node is a run of cells
// sharing a prefix, a leaf is a node holding one cell, and the walk starts at
// the node of octlocateregion (octree.c:295-316), the smallest node holding
// the box.
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

#include <algorithm>

#define WALK_STACK 32

struct walk_frame {
    uint32_t end, cur;
    int depth;
};

// first slot in [lo, hi) whose depth-d prefix differs from that of `ref`;
// every slot before it shares the prefix (sorted order)
__device__ inline uint32_t run_end(const uint4 *codes, uint32_t lo, uint32_t hi, uint4 ref, int d)
{
    const int s = TM_ROOT_LEVEL - d;
    const uint32_t rx = ref.x >> s, ry = ref.y >> s, rz = ref.z >> s;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        uint4 c = codes[mid];
        if ((c.x >> s) == rx && (c.y >> s) == ry && (c.z >> s) == rz) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// first slot in [lo, hi) whose depth-d prefix is not Morton-below that of `ref`
__device__ inline uint32_t prefix_lower_bound(const uint4 *codes, uint32_t lo, uint32_t hi, uint4 ref, int d)
{
    const int s = TM_ROOT_LEVEL - d;
    const uint4 r = make_uint4(ref.x >> s, ref.y >> s, ref.z >> s, 0);
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        uint4 c = codes[mid];
        uint4 cp = make_uint4(c.x >> s, c.y >> s, c.z >> s, 0);
        if (tm_morton_less(cp, r)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// potential(), potential.c:39-78, for one pair in FP64 (returns v's value)
__device__ double pair_potential64(double xi, double yi, double zi, double s1, float y1,
                                   double xj, double yj, double zj, double s2, float y2, double h)
{
    const double dx = sub64(xi, xj), dy = sub64(yi, yj), dz = sub64(zi, zj);
    const double dist = __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz)));
    if (!(dist <= h)) return 0.0;
    const double xc = sub64(add64(s1, s2), dist);
    if (xc <= 0.0) return 0.0;
    const double pp = mul64(0.33, 0.33);
    const double D = mul64(0.75, add64(div64(sub64(1.0, pp), (double)y1), sub64(1.0, div64(pp, (double)y2))));
    const double r01 = div64(add64(sub64(mul64(s1, s1), mul64(s2, s2)), mul64(dist, dist)), mul64(2.0, dist));
    const double r02 = sub64(dist, r01);
    const double s11 = mul64(s1, s1), s22 = mul64(s2, s2);
    const double cap1 = sub64(mul64(s11, sub64(s1, r01)), div64(sub64(mul64(s11, s1), mul64(mul64(r01, r01), r01)), 3.0));
    const double cap2 = sub64(mul64(s22, sub64(s2, r02)), div64(sub64(mul64(s22, s2), mul64(mul64(r02, r02), r02)), 3.0));
    const double area = mul64(3.141592653589793, add64(cap1, cap2));
    const double hertz = div64(mul64(2.0, mul64(xc, xc)), mul64(5.0, D));
    return add64(mul64(hertz, __dsqrt_rn(div64(mul64(s1, s2), add64(s1, s2)))), mul64(area, 0.1));
}

// the same in FP32 for the compensated path (the cutoff decided in FP64)
__device__ float pair_potential32(float dist, float s1, float y1, float s2, float y2)
{
    const float xc = (s1 + s2) - dist;
    if (xc <= 0.0f) return 0.0f;
    const float pp = 0.33f * 0.33f;
    const float D = 0.75f * ((1.0f - pp) / y1 + (1.0f - pp / y2));
    const float r01 = (s1 * s1 - s2 * s2 + dist * dist) / (2.0f * dist);
    const float r02 = dist - r01;
    const float cap1 = s1 * s1 * (s1 - r01) - (s1 * s1 * s1 - r01 * r01 * r01) * (1.0f / 3.0f);
    const float cap2 = s2 * s2 * (s2 - r02) - (s2 * s2 * s2 - r02 * r02 * r02) * (1.0f / 3.0f);
    const float area = 3.14159265f * (cap1 + cap2);
    return (2.0f * xc * xc / (5.0f * D)) * sqrtf((s1 * s2) / (s1 + s2)) + area * 0.1f;
}

// squared distance of two cells from their split (hi + lo) positions
__device__ __forceinline__ float dist2_split(const tm_arrays &a, long long p, long long j)
{
    const float4 hp = a.hi[p], lp = a.lo[p], hj = a.hi[j], lj = a.lo[j];
    const float dx = (hp.x - hj.x) + (lp.x - lj.x), dy = (hp.y - hj.y) + (lp.y - lj.y),
                dz = (hp.z - hj.z) + (lp.z - lj.z);
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// The walk of one cell p (octlocateregion + the DFS of computepotential),
// split into a start, single DFS steps and an end.  The kernel runs it as a
// loop in which a lane whose walk is over takes its next queued cell while
// the other lanes of the warp keep walking: walks differ in length by a wide
// margin, and a warp that waited for its longest one kept a third of its
// lanes busy on average.
struct walk_state {
    long long p, ps, mpos, jstar;   // the cell, its Morton position, m's position, j*
    double mind;                    // mindist of an isolated cell
    uint32_t bmin[3], bmax[3];      // query box, half-open
    uint32_t base;                  // the colony's first Morton position
    int L, c, sp;                   // bin depth, colony, frames (the top one in top)
    walk_frame top;                 // the frame being walked; the ones below it in the stack
    bool isolated, ident, fp64;
    const uint32_t *bst;            // the colony's bin starts
};

// distance of p to the cell in slot j as the walk takes it for mindist: FP64
// on the plain path, from the split positions (FP32) on the compensated one
__device__ __forceinline__ double walk_dist(const tm_arrays &a, bool fp64, long long p, long long j)
{
    if (fp64) {
        const double dx = sub64(a.x[p], a.x[j]), dy = sub64(a.y[p], a.y[j]), dz = sub64(a.z[p], a.z[j]);
        return __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz)));
    }
    return tm_f2d(sqrtf(dist2_split(a, p, j)));   // FP32 path: no FP64 work
}

// An isolated cell (no neighbour within h) walks for its mindist, the least
// distance over the walk's candidates.  With neighbour lists in use its list
// holds every cell nearer than R = h + skin - 2 max displacement since the
// build: when the nearest entry is nearer than R and its lattice code lies in
// the query box (so its leaf meets the box and it is a candidate), no
// candidate is nearer and its distance is mindist; v = 0 (no candidate is
// within h).  True with w.mind set; the walk is then not needed.
__device__ __forceinline__ bool isolated_from_list(const tm_arrays &a, const tm_desc &d, const tm_frame &f,
                                                   const tm_type &T, walk_state &w)
{
    const long long p = w.p;
    const float R = (T.hf + d.skin - 2.0f * __uint_as_float(f.disp) - 2e-3f) * (1.0f - 1e-5f);
    const int cnt = a.vcount[p];
    double best = 1.7976931348623157e308;
    bool cand = false;
    for (int k = 0; k < cnt; k++) {
        const long long j = a.vlist[(long long)k * a.lstride + p];
        const double dist = walk_dist(a, w.fp64, p, j);
        if (dist > best) continue;
        const uint4 cj = a.codes[w.ident ? j : (long long)a.rank[j]];
        const bool in = cj.x >= w.bmin[0] && cj.x < w.bmax[0] && cj.y >= w.bmin[1] && cj.y < w.bmax[1] &&
                        cj.z >= w.bmin[2] && cj.z < w.bmax[2];
        cand = dist < best ? in : (cand || in);
        best = dist;
    }
    if (!cand || !(best < (double)R)) return false;
    w.mind = best;
    // queued as a walk, settled without one: the colony's walk counts drop
    atomicAdd(&a.frame[w.c].walks, ~0ull);
    atomicAdd(&a.frame[w.c].walks_isolated, ~0ull);
    return true;
}

// octlocateregion and the first stack frame; false when there is nothing to
// walk (fewer than two cells in the start node, or an isolated cell settled
// from its list)
__device__ __forceinline__ bool walk_begin(const tm_arrays &a, const tm_consts *K, long long p, walk_state &w,
                                           walk_frame *stk)
{
    const int c = a.col[p];
    const tm_desc &d = a.desc[c];
    const tm_frame &f = a.frame[c];
    const tm_type &T = K->t[a.ctype[p]];
    w.p = p;
    w.c = c;
    w.isolated = a.nbcount[p] == 0;
    w.ident = f.ident != 0;
    w.fp64 = d.precision == 0;
    w.ps = w.ident ? p : (long long)a.rank[p];
    w.jstar = -1;
    w.mind = 1.7976931348623157e308;
    w.mpos = -1;
    w.sp = 0;

    // query box in lattice codes, octree.c:251-263; half-open [bmin, bmax)
    {
        const double pos[3] = {a.x[p], a.y[p], a.z[p]};
        unsigned slow = 0;
        for (int k = 0; k < 3; k++) {
            long long P;
            const bool ok = tm_fix47(pos[k], P) && T.h < 8192.0;
            w.bmin[k] = tm_lattice_fast(pos[k], P, ok, -T.h_fx, -T.h, f, k, slow);
            w.bmax[k] = tm_lattice_fast(pos[k], P, ok, T.h_fx, T.h, f, k, slow);
        }
        if (slow) atomicAdd(&a.frame[c].codes_slow, (unsigned long long)slow);
    }
    if (w.isolated && !a.want_diag && d.verlet && f.list_ok && isolated_from_list(a, d, f, T, w)) return false;

    // octlocateregion: the highest differing bit over the three axes
    const uint32_t diff = (w.bmin[0] ^ w.bmax[0]) | (w.bmin[1] ^ w.bmax[1]) | (w.bmin[2] ^ w.bmax[2]);
    int lm = diff ? 31 - __clz(diff) : 0;
    lm++;
    const int dT = TM_ROOT_LEVEL - lm;       // depth of the start node
    const uint4 mcode = make_uint4(w.bmin[0], w.bmin[1], w.bmin[2], 0);
    const uint4 *codes = a.codes;
    w.bst = a.bin_start + d.binoff;
    w.base = (uint32_t)f.bin_base;   // slots fit in 32 bits; wraps consistently
    w.L = f.L;
    uint32_t a0, a1;
    if (dT <= w.L) {
        const uint32_t P = tm_prefix(mcode, dT);
        const int sh = 3 * (w.L - dT);
        a0 = w.base + w.bst[P << sh];
        a1 = w.base + w.bst[(P + 1) << sh];
    } else {
        const uint32_t b = tm_prefix(mcode, w.L);
        const uint32_t lo = w.base + w.bst[b], hi = w.base + w.bst[b + 1];
        a0 = prefix_lower_bound(codes, lo, hi, mcode, dT);
        a1 = run_end(codes, a0, hi, mcode, dT);
        if (a0 < hi) {
            // a0 may hold a larger prefix (empty node): then nothing matches
            const int s = TM_ROOT_LEVEL - dT;
            const uint4 c0 = codes[a0];
            if ((c0.x >> s) != (mcode.x >> s) || (c0.y >> s) != (mcode.y >> s) || (c0.z >> s) != (mcode.z >> s))
                a1 = a0;
        }
    }

    // The walk visits candidates in Morton order, and the first within-h
    // neighbour m is itself a candidate when its leaf meets the box; then no
    // candidate after position m can be j*, and the walk stops on reaching it.
    if (!w.isolated) {
        const long long m = a.nbmin[p];
        if (m >= (long long)a0 && m < (long long)a1) {
            const uint4 cm = codes[m];
            const int lp = m > d.off ? tm_lcp(codes[m - 1], cm) : 0;
            const int ln = m + 1 < d.off + d.n ? tm_lcp(cm, codes[m + 1]) : 0;
            const int dl = 1 + (lp > ln ? lp : ln);         // m's leaf depth
            const int s = TM_ROOT_LEVEL - dl;
            const uint32_t len = 1u << s;
            const uint32_t lx = (cm.x >> s) << s, ly = (cm.y >> s) << s, lz = (cm.z >> s) << s;
            const bool meets = !(w.bmax[0] <= lx || w.bmin[0] >= lx + len || w.bmax[1] <= ly ||
                                 w.bmin[1] >= ly + len || w.bmax[2] <= lz || w.bmin[2] >= lz + len);
            if (meets && dl > dT && m != w.ps) w.mpos = m;
        }
    }
    if (a1 > a0 && a1 - a0 >= 2) {
        w.top = {a1, a0, dT};
        w.sp = 1;
        return true;
    }
    return false;
}

// one DFS step (the child pop order of computepotential); true when the walk is over
__device__ __forceinline__ bool walk_step(const tm_arrays &a, walk_state &w, walk_frame *stk)
{
    walk_frame &top = w.top;
    if (top.cur >= top.end) {
        if (--w.sp == 0) return true;
        top = stk[w.sp - 1];
        return false;
    }
    const uint32_t k = top.cur;
    if (w.mpos >= 0 && (long long)k >= w.mpos) {
        w.jstar = w.mpos;                   // every later candidate follows m
        return true;
    }
    const uint4 *codes = a.codes;
    const uint4 ck = codes[k];
    const int dc = top.depth + 1;
    uint32_t e;
    if (dc <= w.L) {
        const uint32_t P = tm_prefix(ck, dc);
        e = w.base + w.bst[(P + 1) << (3 * (w.L - dc))];
        if (e > top.end) e = top.end;
    } else {
        e = run_end(codes, k + 1, top.end, ck, dc);
    }
    if (e <= k) {                           // inconsistent bins: never loop in place
        atomicOr(&a.frame[w.c].error, TM_ERR_STACK);
        e = k + 1;
    }
    top.cur = e;
    // child node box, tested as octnodeintersection does
    const int s = TM_ROOT_LEVEL - dc;
    const uint32_t lx = (ck.x >> s) << s, ly = (ck.y >> s) << s, lz = (ck.z >> s) << s;
    const uint32_t len = 1u << s;
    if (w.bmax[0] <= lx || w.bmin[0] >= lx + len) return false;
    if (w.bmax[1] <= ly || w.bmin[1] >= ly + len) return false;
    if (w.bmax[2] <= lz || w.bmin[2] >= lz + len) return false;
    if (e - k == 1) {
        if ((long long)k == w.ps) return false;
        if (w.jstar < 0) w.jstar = k;
        if (!w.isolated) return true;
        const long long sk = w.ident ? (long long)k : (long long)a.tmp[k];
        const double dist = walk_dist(a, w.fp64, w.p, sk);
        w.mind = (dist < w.mind ? dist : w.mind);
        return false;
    }
    if (w.sp == WALK_STACK) {
        atomicOr(&a.frame[w.c].error, TM_ERR_STACK);
        return true;
    }
    stk[w.sp - 1] = top;                // keep the parent (its cursor already past this child)
    top = {e, k, dc};
    w.sp++;
    return false;
}

// v from j*, mindist of an isolated cell, the diagnostics' candidate
__device__ __forceinline__ void walk_end(const tm_arrays &a, const tm_consts *K, const walk_state &w)
{
    const long long p = w.p;
    long long jstar = w.jstar;
    if (jstar >= 0 && !w.ident) jstar = (long long)a.tmp[jstar];
    double vv = 0.0;
    if (jstar >= 0) {
        const tm_type &T = K->t[a.ctype[p]];
        if (w.fp64) {
            vv = pair_potential64(a.x[p], a.y[p], a.z[p], a.size[p], a.young[p], a.x[jstar], a.y[jstar], a.z[jstar],
                                  a.size[jstar], a.young[jstar], T.h);
        } else {
            // distance from the split positions; the cutoff in FP64 only within
            // 1e-5 h of h
            const float dist = sqrtf(dist2_split(a, p, jstar));
            bool in = dist <= T.hf;
            if (fabsf(dist - T.hf) <= 1.0e-5f * T.hf) {
                const double dx = sub64(a.x[p], a.x[jstar]), dy = sub64(a.y[p], a.y[jstar]),
                             dz = sub64(a.z[p], a.z[jstar]);
                in = __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz))) <= T.h;
            }
            if (in)
                vv = tm_f2d(pair_potential32(dist, (float)a.size[p], a.young[p], (float)a.size[jstar],
                                             a.young[jstar]));
        }
    }
    a.v[p] = vv;
    if (w.isolated) a.mindist[p] = w.mind;
    if (a.want_diag) a.vcand[p] = jstar >= 0 ? a.perm[jstar] : -1;
}

// Pass 1 over the cells of colonies the list kernel did not evaluate (it
// does this pass itself).  v is potential(p, j*) and j* precedes every
// within-h neighbour in Morton order, so v can only be non-zero when j* is
// the first within-h neighbour m and m overlaps p (xc > 0, potential.c:63-65);
// otherwise v = 0 without walking (the overlap is excluded with a margin in
// FP32).  Cells that must walk -- those, isolated cells (mindist comes from
// the walk) and every cell in diagnostics mode -- are queued, so the walk
// runs with full warps.
__device__ __forceinline__ void octree_mark_cell(const tm_arrays &a, int c, long long p)
{
    const tm_desc &d = a.desc[c];
    const tm_frame &f = a.frame[c];
    if (!tm_live(p, d)) return;
    const bool isolated = a.nbcount[p] == 0;
    bool walk = isolated || a.want_diag;
    if (!walk) {
        // slots and Morton positions coincide on rebuild steps; otherwise tmp
        // translates a position to its slot
        const long long m = f.ident ? (long long)a.nbmin[p] : (long long)a.tmp[a.nbmin[p]];
        const float4 hp = a.hi[p], lp = a.lo[p], hm = a.hi[m], lm = a.lo[m];
        const float dx = (hp.x - hm.x) + (lp.x - lm.x), dy = (hp.y - hm.y) + (lp.y - lm.y),
                    dz = (hp.z - hm.z) + (lp.z - lm.z);
        const float rs = (hp.w + hm.w) * 1.0001f + 1e-5f;
        walk = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < rs * rs;
    }
    tm_queue_walk(a, c, p, isolated, walk);
}

// the cells of the colonies without lists in use this step (worklist 1), a
// warp per 32-slot group
__global__ void __launch_bounds__(256) k_octree_mark(tm_arrays a)
{
    const uint32_t *wl = a.wl + a.wl_stride;
    const uint32_t total = wl[a.ncol];
    const int lane = threadIdx.x & 31;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < total;
         q += (gridDim.x * blockDim.x) >> 5) {
        int c;
        const long long p = tm_wl_slot(a, wl, q, c) + lane;
        octree_mark_cell(a, c, p);
    }
}

// Pass 2: the walk of every queued cell (grid-stride over both queues).  Each
// lane runs its own sequence of walks: in one iteration it either takes one
// step of its current walk or starts its next cell, so the warp's lanes stay
// busy until their sequences run out.
__global__ void __launch_bounds__(256, 4) k_octree(tm_arrays a, const tm_consts *K)
{
    const int nf = a.work[2], nq = nf + a.work[3];
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    walk_state w;
    walk_frame stk[WALK_STACK];   // the DFS stack (local memory)
    bool busy = false;
    for (;;) {
        bool over;
        if (busy) {
            over = walk_step(a, w, stk);
        } else if (q < nq) {
            const long long p = q < nf ? a.walk_list[q] : a.walk_list[a.nslots_total - 1 - (q - nf)];
            q += stride;
            busy = walk_begin(a, K, p, w, stk);
            over = !busy;
        } else {
            break;
        }
        if (over) {
            walk_end(a, K, w);
            busy = false;
        }
    }
}

cudaError_t tm_launch_octree(const tm_arrays &a, const tm_consts *K, int block, cudaStream_t st)
{
    if (block != 64 && block != 256) block = 128;
    if (a.nslots_total == 0 || a.ncol == 0) return cudaSuccess;
    k_worklist<<<1, 1024, 0, st>>>(a, 1);
    k_octree_mark<<<tm_stream_grid(256, 8), 256, 0, st>>>(a);
    // the queue length is known on the device only: a grid of resident size
    static int sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    const int nsm = (dev >= 0 && dev < 64 && sms[dev] > 0) ? sms[dev] : 152;
    const long long cap = (long long)nsm * (2048 / block);
    const unsigned wgrid = (unsigned)std::min<long long>(cap, (a.nslots_total + block - 1) / block);
    k_octree<<<wgrid, block, 0, st>>>(a, K);
    return cudaGetLastError();
}
