// Shared device-side definitions for the GB300 cell-mechanics path.
//
// Data layout in HBM (one colony; every array indexed by "slot", the cell's
// position in the current Morton order unless stated otherwise):
//   x, y, z, size          FP64 positions and radii (celldata_t, global.h:100-120)
//   young                  FP32;  ctype, phase  int32;  perm  caller index
//   hi[slot], lo[slot]     float4 split of (x, y, z): hi = x rounded to 24 bits,
//                          lo = x - hi; hi.w = size as float
//   code[slot]             uint4 (cx, cy, cz, 0) lattice codes of octree.c:187-191
//   bin_start[b]           first slot of Morton bin b (depth-L octree node), b in
//                          [0, 8^L]; bin_start[8^L] = n
// Outputs (same slot order): density, v, mindist, fx, fy, fz, nbcount, nbhash.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define TM_MAX_TYPES 8
#define TM_ROOT_LEVEL 29          // global.h:65-66: codes are 29-bit
#define TM_LMAX 8                 // deepest bin level: 8^8 bins
#define TM_WARPS_PER_BLOCK 4
#define TM_BIG_BIN 2048           // largest bin the in-bin sort handles

// error bits written by kernels into tm_frame::error
#define TM_ERR_BIGBIN 1u          // a bin held more than TM_BIG_BIN cells
#define TM_ERR_STACK 2u           // octree walk deeper than its stack
#define TM_ERR_CODES 4u           // two cells share a lattice code
#define TM_ERR_TYPES 8u           // an asynchronous upload carried a cell type outside the table
#define TM_ERR_LIST 8u            // pair list overflow (internal)

// Per-type constants, computed on the host with the reference's expressions
// (inline.h:45-46, 71-72; potential.c:60) so the FP64 values are bit-identical.
struct tm_type {
    double h, h2, h3, h4, csize;
    double sc;       // density scale: h3 (3-D) or h2 (2-D)
    double cW;       // sphkernel constant 8/(pi h3) or 40/(7 pi h2)
    double cG;       // sphgradient constant 48/(pi h4) or 320/(7 pi h3)
    double e;        // bounding-box pad h + 0.01 (octree.c:167)
    float randommove;
    long long h_fx;  // h * 2^47, truncated
    // FP32 forms for the compensated path
    float hf, h2f, inv_hf, cWf, cGf, kmassf;   // kmassf = sc / csize
    float thr_lo, thr_hi;                      // squared-distance band around h^2
    double inv_h, kmass;                       // 1 / h and sc / csize for the FP32 path's FP64 re-do
    double h2cut;                              // largest double d2 with sqrt(d2) <= h (the FP64 cutoff)
};

struct tm_consts {
    int ntypes;
    int dim;
    tm_type t[TM_MAX_TYPES];
};

// Per-step frame, written on the device (no host round trip inside a step).
struct tm_frame {
    double shift[3];     // affShift (octree.c:178-180)
    double scale;        // affScale (octree.c:175-177)
    unsigned long long bbox[TM_MAX_TYPES][6];   // order-preserving min x,y,z / max x,y,z
    int L;               // bin depth
    uint32_t nbins;      // 8^L
    float shiftf[3];     // FP32 copies for culling
    float binscale;      // 2^L / scale
    float units2;        // two lattice units, 2 scale / 2^29 (the list pass's box margin)
    int n;               // cells in this colony
    uint32_t error;      // TM_ERR_* bits
    unsigned long long removecount;
    unsigned long long boundary_pairs;   // within-h pairs outside the lattice box (diagnostic)
    int nbig;            // bins needing the block sort
    int pad_;
    long long bin_base;      // slot of a bin = bin_base + bin_start[bin]
    // fixed-point form of the affine map for the integer lattice-code path
    long long sh_fx[3];      // shift * 2^47, truncated
    unsigned long long cmul; // ~ 2^(78-ck) / scale
    int ck;                  // left shift restoring 2^32 * code
    uint32_t ceps;           // 2^32 * error bound of the integer path
    unsigned long long codes_slow;   // codes that took the FP64 path (diagnostic)
    // neighbour lists (Verlet): built when cells may have moved half the skin
    int rebuild;             // this step searches bins and rebuilds the lists
    int age;                 // steps since the last rebuild
    int list_ok;             // 0: the lists are missing or overflowed
    int force_rebuild;       // set by uploads
    int ident;               // 1: slots are in this step's Morton order
    unsigned maxdisp;        // float bits of max |x - x_build| after the last update
    unsigned disp;           // the same for the positions this step evaluates (0 on rebuild steps)
    unsigned long long rebuilds;     // rebuild steps so far (diagnostic)
    unsigned long long step_counter;
    long long patch_lo[3];   // CIC patch corners (patches.c:61-132); INT_MAX/INT_MIN when empty
    long long patch_hi[3];
    unsigned long long fix64;        // FP32 cells whose density this step was redone in FP64 (diagnostic)
    unsigned long long walks;        // cells of this step that took the octree walk (diagnostic)
    unsigned long long walks_isolated;   // those of them without a neighbour within h
};

// ---------------------------------------------------------------------------
// small helpers

__host__ __device__ inline unsigned long long tm_ordered(double d)
{
    unsigned long long b;
#ifdef __CUDA_ARCH__
    b = (unsigned long long)__double_as_longlong(d);
#else
    union { double d; unsigned long long u; } c; c.d = d; b = c.u;
#endif
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__host__ __device__ inline double tm_unordered(unsigned long long o)
{
    unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    union { double d; unsigned long long u; } c; c.u = b; return c.d;
#endif
}

__host__ __device__ inline uint64_t tm_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// spread the low 10 bits of v so that bit i lands at bit 3i
__host__ __device__ inline uint32_t tm_spread3(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton index of a node at depth d (d <= 10) from its per-axis prefixes;
// the child digit is x + 2y + 4z (octree.c:105-107), so z is the most
// significant bit of every level.
__host__ __device__ inline uint32_t tm_morton(uint32_t px, uint32_t py, uint32_t pz)
{
    return tm_spread3(px) | (tm_spread3(py) << 1) | (tm_spread3(pz) << 2);
}

// Morton prefix of depth d (<= 10) of a cell's lattice codes
__host__ __device__ inline uint32_t tm_prefix(uint4 c, int d)
{
    int s = TM_ROOT_LEVEL - d;
    return tm_morton(c.x >> s, c.y >> s, c.z >> s);
}

// digit of a cell at depth d (1..29): the bits at position 29 - d
__device__ inline int tm_digit(uint4 c, int d)
{
    int s = TM_ROOT_LEVEL - d;
    return (int)(((c.x >> s) & 1u) | (((c.y >> s) & 1u) << 1) | (((c.z >> s) & 1u) << 2));
}

__device__ inline bool tm_less_msb(uint32_t a, uint32_t b) { return a < b && a < (a ^ b); }

// true when code a precedes code b in Morton order (z, then y, then x at each level)
__device__ inline bool tm_morton_less(uint4 a, uint4 b)
{
    uint32_t xz = a.z ^ b.z, xy = a.y ^ b.y, xx = a.x ^ b.x;
    uint32_t best = xz;
    int dim = 2;
    if (tm_less_msb(best, xy)) { best = xy; dim = 1; }
    if (tm_less_msb(best, xx)) { best = xx; dim = 0; }
    if (dim == 2) return a.z < b.z;
    if (dim == 1) return a.y < b.y;
    return a.x < b.x;
}

__device__ inline bool tm_code_eq(uint4 a, uint4 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// FP64 arithmetic without contraction, so every product and sum rounds
// separately as in the reference's C expressions.
__device__ __forceinline__ double mul64(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add64(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub64(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double div64(double a, double b) { return __ddiv_rn(a, b); }

// x / r (r the grid's float resolution) with the rounding of an FP64
// division.  When r is a power of two the quotient is x scaled by 2^-e,
// exact for a normal result, and is made by moving x's exponent field
// (integer work: this GPU's FP64 pipe is narrow); zero, subnormal or
// non-finite x, a result leaving the normal range, or any other r take the
// FP64 division.
__device__ __forceinline__ double tm_div_res(double x, float r)
{
    const unsigned rb = __float_as_uint(r);
    const unsigned ex = (rb >> 23) & 0xffu;
    if ((rb & 0x807fffffu) == 0u && ex != 0u && ex != 0xffu) {
        const int e = (int)ex - 127;                    // r = 2^e
        const long long b = __double_as_longlong(x);
        const int xe = (int)((b >> 52) & 0x7ff);
        if (xe != 0 && xe != 0x7ff && xe - e > 0 && xe - e < 0x7ff) return __longlong_as_double(b - ((long long)e << 52));
    }
    return div64(x, (double)r);
}

// Adds w to grid[gi] for every lane with dep set.  Lanes in a row holding
// the same node (a run; Morton-ordered cells give long ones) are summed by a
// segmented scan, ceil(log2(longest run)) shuffle-and-add steps for the whole
// warp, and the run's last lane issues one atomic.  No FP64 add is spent when
// every run is one lane long.  All 32 lanes of the warp call it.
__device__ __forceinline__ void tm_warp_deposit(double *grid, long long gi, double w, bool dep, int lane)
{
    const unsigned FULLM = 0xffffffffu;
    if (!__any_sync(FULLM, dep)) return;
    const long long prev = __shfl_up_sync(FULLM, gi, 1);
    const unsigned heads = __ballot_sync(FULLM, lane == 0 || gi != prev);
    const int span = lane - (31 - __clz(heads & (FULLM >> (31 - lane))));   // lanes before this one in its run
    const int longest = __reduce_max_sync(FULLM, span);
    double v = w;
    for (int d = 1; d <= longest; d <<= 1) {
        const double u = __shfl_up_sync(FULLM, v, d);
        if (span >= d) v = add64(v, u);
    }
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (dep && tail) atomicAdd(grid + gi, v);
}

// (unsigned int)(((x - shift) / scale) * 2^29), octree.c:188-190
__device__ inline uint32_t tm_lattice(double x, double shift, double scale)
{
    double q = div64(sub64(x, shift), scale);
    return (uint32_t)mul64(q, 536870912.0);
}

// query-box corners of octcomputebox, octree.c:251-263: ((x -/+ h) - shift) / scale
__device__ inline uint32_t tm_lattice_off(double x, double off, double shift, double scale)
{
    double q = div64(sub64(add64(x, off), shift), scale);
    return (uint32_t)mul64(q, 536870912.0);
}

// Lattice codes without FP64 arithmetic in the common case.
//
// A position x (|x| < 2^13) becomes the 2^-47 fixed-point integer X by bit
// manipulation (truncation).  With D = X + OFF - SHIFT (OFF = 0 or +-h, all
// truncated the same way) the real code value is D * 2^-18 / scale; it is
// formed as the 128-bit product D * cmul, cmul ~ 2^(78-ck) / scale, giving
// 2^32 * code.  Its distance to the value the reference computes,
// (unsigned)(((x - h - shift) / scale) * 2^29) in FP64 (octree.c:188-190,
// 251-263), is bounded in k_frame (ceps); when the fraction lies farther than
// that from an integer the truncations agree, otherwise the exact FP64
// expression decides.
__device__ __forceinline__ bool tm_fix47(double x, long long &X)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e > 1035) return false;                              // |x| >= 2^13, inf, nan
    const unsigned long long m = (b & 0xfffffffffffffull) | (e ? 0x10000000000000ull : 0ull);
    const int sh = e - 1028;                                  // x * 2^47 = m * 2^(e - 1075 + 47)
    unsigned long long v = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> (-sh)) : 0ull);
    X = (b >> 63) ? -(long long)v : (long long)v;
    return true;
}

// 2^32 * code from D (D >= 0); ok = false when the integer path cannot decide
__device__ __forceinline__ uint32_t tm_code_fix(long long D, unsigned long long cmul, int ck, uint32_t ceps,
                                                bool &ok)
{
    if (D < 0) { ok = false; return 0; }
    const unsigned long long lo = (unsigned long long)D * cmul;
    const unsigned long long hi = __umul64hi((unsigned long long)D, cmul);
    const unsigned long long q = (hi << ck) | (lo >> (64 - ck));
    const uint32_t frac = (uint32_t)q;
    ok = (hi >> (64 - ck)) == 0 && (q >> 61) == 0 && frac > ceps && frac < 0xffffffffu - ceps;
    return (uint32_t)(q >> 32);
}

// the code of x + off (off in {0, -h, +h}) with the exact FP64 fallback
__device__ __forceinline__ uint32_t tm_lattice_fast(double x, long long Xfx, bool xok, long long offfx, double off,
                                                    const tm_frame &f, int k, unsigned &slow)
{
    bool ok = xok;
    uint32_t c = 0;
    if (ok) c = tm_code_fix(Xfx + offfx - f.sh_fx[k], f.cmul, f.ck, f.ceps, ok);
    if (ok) return c;
    slow++;
    return off == 0.0 ? tm_lattice(x, f.shift[k], f.scale) : tm_lattice_off(x, off, f.shift[k], f.scale);
}

// float -> double, exact, with integer operations only: on this part a
// conversion issues on the FP64 pipe, which runs at a small fraction of the
// FP32 rate; the octree walk, a chain of dependent steps, converts its FP32
// distances this way.  (The list pass keeps the hardware conversion: there
// the dozen integer instructions cost more than the pipe time, measured.)
// The fields are moved into the binary64 layout (exponent rebiased by
// 1023 - 127); subnormal floats are normalised; infinities and NaNs keep
// their payload bits.
__device__ __forceinline__ double tm_f2d(float f)
{
    const uint32_t u = __float_as_uint(f);
    const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
    const uint32_t e = (u >> 23) & 0xffu;
    const unsigned long long m = u & 0x7fffffu;
    if (e == 0u) {
        if (m == 0ull) return __longlong_as_double((long long)sgn);
        const int p = 31 - __clz((int)m);                       // leading one of m, value m * 2^-149
        const unsigned long long mant = (m << (52 - p)) & 0xfffffffffffffull;
        return __longlong_as_double((long long)(sgn | ((unsigned long long)(p + 874) << 52) | mant));
    }
    const unsigned long long ex = e == 255u ? 2047ull : (unsigned long long)e + 896ull;
    return __longlong_as_double((long long)(sgn | (ex << 52) | (m << 29)));
}

// a / b rounded to nearest, given y = RN(1 / b): q = RN(a y) is within an
// ulp of a / b, so the remainder a - b q is exact in one FMA, and
// RN(q + (a - b q) y) is the correctly rounded quotient (Markstein's
// correction, the division by an FMA-based reciprocal).  Three FP64
// operations instead of a division's software sequence; the result is the
// reference's own u = dist / h, so the kernel value rounds to the same float.
__device__ __forceinline__ double div_by_recip(double a, double b, double y)
{
    const double q = __dmul_rn(a, y);
    const double r = __fma_rn(-q, b, a);
    return __fma_rn(r, y, q);
}

// (double)(float)w, round to nearest even, with integer operations for a w
// whose float is normal (the hardware conversions otherwise): the 29 low
// mantissa bits are dropped with the round-half-even carry, which runs into
// the exponent field as it should.
__device__ __forceinline__ double tm_round_to_float(double w)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(w);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 126 || e > 1023 + 126) return (double)__double2float_rn(w);
    const unsigned long long low = b & 0x1fffffffull, half = 0x10000000ull;
    unsigned long long r = b & ~0x1fffffffull;
    if (low > half || (low == half && (b & 0x20000000ull))) r += 0x20000000ull;
    return __longlong_as_double((long long)r);
}

// Split a double into hi (x truncated to 24 significant bits) + lo (float of
// the remainder) with integer operations only, so no FP64 instruction runs.
// |x| < 2^-70 flushes to zero; |x| must stay below 2^100.
__device__ inline void tm_split(double x, float &hi, float &lo)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
    int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 70) { hi = 0.0f; lo = 0.0f; return; }
    unsigned long long m = b & 0xfffffffffffffull;               // 52 fraction bits
    uint32_t fb = sgn | ((uint32_t)(e - 1023 + 127) << 23) | (uint32_t)(m >> 29);
    hi = __uint_as_float(fb);
    uint32_t ml = (uint32_t)(m & ((1ull << 29) - 1));              // remainder = ml * 2^(e-1075)
    float r = __uint2float_rn(ml);                                 // 24 of 29 bits kept
    float p2 = __int_as_float((e - 1075 + 127) << 23);             // 2^(e-1075), normal for e >= 953
    lo = __fmul_rn(r, p2);
    if (sgn) lo = -lo;
}

// Knuth's TwoSum: s + err == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Kahan-compensated accumulation in FP32
struct kahan {
    float s, c;
    __device__ void init() { s = 0.0f; c = 0.0f; }
    __device__ __forceinline__ void add(float v)
    {
        float y = __fsub_rn(v, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float value() const { return __fsub_rn(s, c); }
    // add another compensated sum (s2 - c2): TwoSum keeps the rounding of s + s2
    __device__ __forceinline__ void merge(float s2, float c2)
    {
        float t, e;
        two_sum(s, s2, t, e);
        c = __fsub_rn(__fadd_rn(c, c2), e);
        s = t;
    }
};

// levels two lattice codes share (the depth of their deepest common octree
// node; TM_ROOT_LEVEL when equal)
__device__ inline int tm_lcp(uint4 a, uint4 b)
{
    uint32_t x = (a.x ^ b.x) | (a.y ^ b.y) | (a.z ^ b.z);
    if (x == 0) return TM_ROOT_LEVEL;
    return 28 - (31 - __clz(x));
}

// (float)rand()/RAND_MAX for a value r of the C library's rand() (RAND_MAX
// = 2^31 - 1 with glibc), as the reference forms its random numbers
__device__ __forceinline__ float tm_frand(int r) { return __fdiv_rn(__int2float_rn(r), (float)2147483647); }
