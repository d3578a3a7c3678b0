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

// the walk of one cell p (octlocateregion + the DFS of computepotential)
__device__ __noinline__ void octree_walk(const tm_arrays &a, const tm_consts *K, long long p)
{
    const int c = a.col[p];
    const tm_desc &d = a.desc[c];
    const tm_frame &f = a.frame[c];
    const tm_type &T = K->t[a.ctype[p]];
    const double xp = a.x[p], yp = a.y[p], zp = a.z[p];
    const bool isolated = a.nbcount[p] == 0;
    const bool ident = f.ident != 0;
    const long long ps = ident ? p : (long long)a.rank[p];   // p's Morton position
    auto slot_of = [&](long long k) -> long long { return ident ? k : (long long)a.tmp[k]; };

    // query box in lattice codes, octree.c:251-263; half-open [bmin, bmax)
    uint32_t bmin[3], bmax[3];
    {
        const double pos[3] = {xp, yp, zp};
        unsigned slow = 0;
        for (int k = 0; k < 3; k++) {
            long long P;
            const bool ok = tm_fix47(pos[k], P) && T.h < 8192.0;
            bmin[k] = tm_lattice_fast(pos[k], P, ok, -T.h_fx, -T.h, f, k, slow);
            bmax[k] = tm_lattice_fast(pos[k], P, ok, T.h_fx, T.h, f, k, slow);
        }
        if (slow) atomicAdd(&a.frame[c].codes_slow, (unsigned long long)slow);
    }

    // octlocateregion: the highest differing bit over the three axes
    uint32_t diff = (bmin[0] ^ bmax[0]) | (bmin[1] ^ bmax[1]) | (bmin[2] ^ bmax[2]);
    int lm = diff ? 31 - __clz(diff) : 0;
    lm++;
    const int dT = TM_ROOT_LEVEL - lm;       // depth of the start node
    const uint4 mcode = make_uint4(bmin[0], bmin[1], bmin[2], 0);
    const uint4 *codes = a.codes;
    const uint32_t *bst = a.bin_start + d.binoff;
    const uint32_t base = (uint32_t)f.bin_base;   // slots fit in 32 bits; wraps consistently
    const int L = f.L;
    uint32_t a0, a1;
    if (dT <= L) {
        const uint32_t P = tm_prefix(mcode, dT);
        const int sh = 3 * (L - dT);
        a0 = base + bst[P << sh];
        a1 = base + bst[(P + 1) << sh];
    } else {
        const uint32_t b = tm_prefix(mcode, L);
        const uint32_t lo = base + bst[b], hi = base + bst[b + 1];
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
    long long mpos = -1;
    if (!isolated) {
        const long long m = a.nbmin[p];
        if (m >= (long long)a0 && m < (long long)a1) {
            const uint4 cm = codes[m];
            const int lp = m > d.off ? tm_lcp(codes[m - 1], cm) : 0;
            const int ln = m + 1 < d.off + d.n ? tm_lcp(cm, codes[m + 1]) : 0;
            const int dl = 1 + (lp > ln ? lp : ln);         // m's leaf depth
            const int s = TM_ROOT_LEVEL - dl;
            const uint32_t len = 1u << s;
            const uint32_t lx = (cm.x >> s) << s, ly = (cm.y >> s) << s, lz = (cm.z >> s) << s;
            const bool meets = !(bmax[0] <= lx || bmin[0] >= lx + len || bmax[1] <= ly || bmin[1] >= ly + len ||
                                 bmax[2] <= lz || bmin[2] >= lz + len);
            if (meets && dl > dT && m != ps) mpos = m;
        }
    }

    long long jstar = -1;
    double mind = 1.7976931348623157e308;
    if (a1 > a0 && a1 - a0 >= 2) {
        walk_frame stk[WALK_STACK];
        int sp = 0;
        stk[sp++] = {a1, a0, dT};
        bool done = false;
        while (sp > 0 && !done) {
            walk_frame &top = stk[sp - 1];
            if (top.cur >= top.end) {
                sp--;
                continue;
            }
            const uint32_t k = top.cur;
            if (mpos >= 0 && (long long)k >= mpos) {
                jstar = mpos;                   // every later candidate follows m
                done = true;
                continue;
            }
            const uint4 ck = codes[k];
            const int dc = top.depth + 1;
            uint32_t e;
            if (dc <= L) {
                const uint32_t P = tm_prefix(ck, dc);
                e = base + bst[(P + 1) << (3 * (L - dc))];
                if (e > top.end) e = top.end;
            } else {
                e = run_end(codes, k + 1, top.end, ck, dc);
            }
            if (e <= k) {                       // inconsistent bins: never loop in place
                atomicOr(&a.frame[c].error, TM_ERR_STACK);
                e = k + 1;
            }
            top.cur = e;
            // child node box, tested as octnodeintersection does
            const int s = TM_ROOT_LEVEL - dc;
            const uint32_t lx = (ck.x >> s) << s, ly = (ck.y >> s) << s, lz = (ck.z >> s) << s;
            const uint32_t len = 1u << s;
            if (bmax[0] <= lx || bmin[0] >= lx + len) continue;
            if (bmax[1] <= ly || bmin[1] >= ly + len) continue;
            if (bmax[2] <= lz || bmin[2] >= lz + len) continue;
            if (e - k == 1) {
                if ((long long)k == ps) continue;
                if (jstar < 0) jstar = k;
                if (!isolated) {
                    done = true;
                } else {
                    const long long sk = slot_of(k);
                    double dist;
                    if (d.precision == 0) {
                        const double dx = sub64(xp, a.x[sk]), dy = sub64(yp, a.y[sk]), dz = sub64(zp, a.z[sk]);
                        dist = __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz)));
                    } else {
                        dist = (double)sqrtf(dist2_split(a, p, sk));   // FP32 path: no FP64 work
                    }
                    mind = (dist < mind ? dist : mind);
                }
                continue;
            }
            if (sp == WALK_STACK) {
                atomicOr(&a.frame[c].error, TM_ERR_STACK);
                done = true;
                continue;
            }
            stk[sp++] = {e, k, dc};
        }
    }

    double vv = 0.0;
    if (jstar >= 0) jstar = slot_of(jstar);
    if (jstar >= 0) {
        if (d.precision == 0) {
            vv = pair_potential64(xp, yp, zp, a.size[p], a.young[p], a.x[jstar], a.y[jstar], a.z[jstar],
                                  a.size[jstar], a.young[jstar], T.h);
        } else {
            // distance from the split positions; the cutoff in FP64 only within
            // 1e-5 h of h
            const float dist = sqrtf(dist2_split(a, p, jstar));
            bool in = dist <= T.hf;
            if (fabsf(dist - T.hf) <= 1.0e-5f * T.hf) {
                const double dx = sub64(xp, a.x[jstar]), dy = sub64(yp, a.y[jstar]), dz = sub64(zp, a.z[jstar]);
                in = __dsqrt_rn(add64(add64(mul64(dx, dx), mul64(dy, dy)), mul64(dz, dz))) <= T.h;
            }
            if (in)
                vv = (double)pair_potential32(dist, (float)a.size[p], a.young[p], (float)a.size[jstar],
                                              a.young[jstar]);
        }
    }
    a.v[p] = vv;
    if (isolated) a.mindist[p] = mind;
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
__global__ void __launch_bounds__(256) k_octree_mark(tm_arrays a)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (((p >> 5) << 5) >= a.nslots_total) return;
    const int c = a.col[(p >> 5) << 5];                  // colonies are 32-aligned
    const tm_desc &d = a.desc[c];
    if (!d.active || d.n <= 1) return;
    const tm_frame &f = a.frame[c];
    if (d.verlet && f.list_ok) return;                   // done by the list kernel
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
    tm_queue_walk(a, p, isolated, walk);
}

// Pass 2: the walk of every queued cell (grid-stride over both queues)
__global__ void __launch_bounds__(256) k_octree(tm_arrays a, const tm_consts *K)
{
    const int nf = a.work[2], nq = nf + a.work[3];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq;
         q += (long long)gridDim.x * blockDim.x) {
        const long long p = q < nf ? a.walk_list[q] : a.walk_list[a.nslots_total - 1 - (q - nf)];
        octree_walk(a, K, p);
    }
}

cudaError_t tm_launch_octree(const tm_arrays &a, const tm_consts *K, int block, cudaStream_t st)
{
    if (block != 64 && block != 256) block = 128;
    unsigned grid = (unsigned)((a.nslots_total + 255) / 256);
    if (grid == 0) return cudaSuccess;
    k_octree_mark<<<grid, 256, 0, st>>>(a);
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
