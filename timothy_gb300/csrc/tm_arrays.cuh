// Packed multi-colony state shared by all kernels.
//
// Colony c owns the slot range [desc[c].off, desc[c].off + desc[c].nslots),
// nslots = n rounded up to a multiple of 32, so a warp never straddles two
// colonies; slots past n are padding that every kernel skips.  Its bins live
// at [desc[c].binoff, desc[c].binoff + 8^Lcap + 1) of the shared bin table.
// One exclusive scan runs over the whole table; a colony turns the scanned
// value of its bin b into a slot as frame.bin_base + bin_start[b], so slot
// ranges and bin ranges can be allocated independently.
#pragma once
#include "tm_core.cuh"

struct tm_desc {
    long long off;       // first slot
    long long binoff;    // first bin-table entry
    long long gridoff;   // first CIC grid entry (-1: no deposit)
    int n;               // live cells
    int nslots;          // padded slot count
    int Lcap;            // deepest bin level this colony's table holds
    int precision;       // 0 plain FP64, 1 FP32 + compensated
    int update_mode;     // 0 reference x += F (+ random move), 1 x += dt*F, 2 none
    int active;          // 0: skipped by every kernel
    int verlet;          // 1: reuse neighbour lists between rebuilds
    float skin;          // list radius is h + skin
    int rmax;            // rebuild at least every rmax steps
    double dt;
    // CIC grid geometry (grid.c:37-136 at one rank)
    double glower[3];
    float gres;
    int gsize[3];
};

struct tm_arrays {
    // state, current order (double-buffered by the host)
    double *x, *y, *z, *size;
    float *young;
    int *ctype, *phase, *perm;
    unsigned char *rem;  // removal marks (cells.c:80-83)
    // state, the other buffer (gather target)
    double *x2, *y2, *z2, *size2;
    float *young2;
    int *ctype2, *phase2, *perm2;
    unsigned char *rem2;
    // per slot, constant after upload
    int *col;
    // build scratch
    uint4 *code;         // lattice codes in the pre-sort order
    uint4 *codes;        // lattice codes in Morton order
    uint32_t *bin;       // global bin-table index of each pre-sort slot
    int *grp;            // slots grouped by bin at their bins' Morton positions (build scratch)
    int *tmp;            // Morton position -> slot
    int *rank;           // slot -> Morton position
    float4 *hi, *lo;     // FP32 split positions (hi.w = size)
    double *mass;        // FP64 density weights sc_t * (size / csize_t), [type][slot]
    // bin table
    uint32_t *bin_count, *bin_start;   // bin_count: occupancy, then the scatter's cursor
    long long nbin_total;
    int *bigbins;
    int *fix_count;      // cells whose FP32 density is redone in FP64
    int *fix_list;
    // per step: work[0] colonies that search (no lists), work[1] colonies
    // whose lists overflowed; lets the search grid leave at once
    // cell-cycle state, indexed by colony offset + the caller's cell index
    // (allocated when a colony first runs the cell cycle)
    float *cy_pt, *cy_g1, *cy_s, *cy_g2, *cy_m;
    int *cy_age;
    // the C library's rand() values of updatepositions' random move, dim per
    // cell in the caller's order (drop-in only; null: a counter-based stream)
    const int *move_draws;
    int *work;           // work[2], work[3]: cells queued for the octree walk; work[4]: list build's next group
    int *walk_list;
    // worklists of 32-slot groups, wl_stride words each: entry c is the first
    // group of colony c in the list (an exclusive prefix over the colonies),
    // entry ncol the list's length.  List 0: colonies that rebuild this step;
    // list 1: colonies the octree walk's first pass serves (no lists in use)
    uint32_t *wl;
    int wl_stride;
    // outputs (Morton order)
    double *density, *v, *mindist, *fx, *fy, *fz;
    int *nbcount;
    int *nbmin;          // first Morton position within h, -1 if none
    // neighbour lists: cell `slot` holds vcount[slot] entries
    // vlist[k*lstride + slot] (slots), k-major so a warp's loads coalesce
    int *vlist;
    int *vcount;
    float4 *x0;          // float position at the last rebuild (displacement test)
    long long lstride;
    int vcap;            // entries per cell
    unsigned long long *nbhash;
    int *vcand;
    // CIC grids
    double *grid;
    // frames / descriptors
    tm_desc *desc;
    tm_frame *frame;
    int ncol;
    long long nslots_total;
    int want_diag;       // fill nbcount/nbhash/vcand
    // diagnostics: the neighbour lists of sampled cells.  diag_row[off + caller
    // index] is the cell's row in diag_nb (-1: not sampled); diag_cnt[row]
    // counts its neighbours within h this step (zeroed at the step's start).
    int *diag_row;
    int *diag_cnt;
    int *diag_nb;        // caller indices, diag_lcap per row, in no particular order
    int diag_lcap;
};

// slot i holds a live cell of colony d (unsigned: slots below the colony's
// range are not live either)
__device__ __forceinline__ bool tm_live(long long i, const tm_desc &d)
{
    return (unsigned long long)(i - d.off) < (unsigned long long)d.n;
}

// Queue cell i for the octree walk, or set its v = 0 when it needs none.
// Cells with neighbours within h fill the walk list from the front
// (work[2]), isolated cells -- whose walks visit every candidate -- from the
// back (work[3]), so warps of the walk hold walks of similar length.
__device__ __forceinline__ void tm_queue_walk(const tm_arrays &a, int c, long long i, bool isolated, bool walk)
{
    if (!walk) a.v[i] = 0.0;
    const unsigned am = __activemask();
    const unsigned mf = __ballot_sync(am, walk && !isolated), mb = __ballot_sync(am, walk && isolated);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    if ((mf | mb) && lane == __ffs(mf | mb) - 1) {
        atomicAdd(&a.frame[c].walks, (unsigned long long)__popc(mf | mb));
        if (mb) atomicAdd(&a.frame[c].walks_isolated, (unsigned long long)__popc(mb));
    }
    if (mf) {
        const int leader = __ffs(mf) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.work[2], __popc(mf));
        base = __shfl_sync(am, base, leader);
        if (walk && !isolated) a.walk_list[base + __popc(mf & below)] = (int)i;
    }
    if (mb) {
        const int leader = __ffs(mb) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.work[3], __popc(mb));
        base = __shfl_sync(am, base, leader);
        if (walk && isolated) a.walk_list[a.nslots_total - 1 - (base + __popc(mb & below))] = (int)i;
    }
}

// The same for kernels where several lanes share a cell: every lane of the
// warp calls it, the cell's owner lane carries it, and the warp makes one
// append per queue.
__device__ __forceinline__ void tm_queue_walk_owned(const tm_arrays &a, int c, long long i, bool owner,
                                                    bool isolated, bool walk)
{
    if (owner && !walk) a.v[i] = 0.0;
    const unsigned am = __activemask();
    const bool wf = owner && walk && !isolated, wb = owner && walk && isolated;
    const unsigned mf = __ballot_sync(am, wf), mb = __ballot_sync(am, wb);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    if ((mf | mb) && lane == __ffs(mf | mb) - 1) {
        atomicAdd(&a.frame[c].walks, (unsigned long long)__popc(mf | mb));
        if (mb) atomicAdd(&a.frame[c].walks_isolated, (unsigned long long)__popc(mb));
    }
    if (mf) {
        const int leader = __ffs(mf) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.work[2], __popc(mf));
        base = __shfl_sync(am, base, leader);
        if (wf) a.walk_list[base + __popc(mf & below)] = (int)i;
    }
    if (mb) {
        const int leader = __ffs(mb) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.work[3], __popc(mb));
        base = __shfl_sync(am, base, leader);
        if (wb) a.walk_list[a.nslots_total - 1 - (base + __popc(mb & below))] = (int)i;
    }
}

// First slot of the q-th group of worklist wl (q below its length) and the
// group's colony: the colony whose prefix entry is the last one <= q.
__device__ __forceinline__ long long tm_wl_slot(const tm_arrays &a, const uint32_t *wl, uint32_t q, int &c)
{
    int lo = 0, hi = a.ncol;              // wl[lo] <= q < wl[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (wl[mid] <= q) lo = mid;
        else hi = mid;
    }
    c = lo;
    return a.desc[lo].off + 32ll * (long long)(q - wl[lo]);
}

// launch shapes chosen per session (tm_tuning)
struct tm_shapes {
    int pair_lshift;    // candidate ranges from Morton nodes this many levels above the bins (0 or 1)
    int list_variant;   // list kernel block size / register budget, 1..4
    int walk_block;     // octree walk threads per block (64, 128 or 256)
};
