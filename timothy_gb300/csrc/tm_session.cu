// Device-resident sessions: colonies packed in HBM, one launch sequence per
// step for all of them, downloads in caller order.  Implements the tm_* API
// of include/timothy_gb300.h.
#include "tm_kernels.cuh"
#include "timothy_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

static thread_local std::string g_err;

static int tm_fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return tm_fail(TM_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// the same message slot for the other translation units
int tm_report(int code, const char *msg)
{
    g_err = msg;
    return code;
}

extern "C" const char *tm_last_error(void) { return g_err.c_str(); }
extern "C" const char *tm_version(void) { return "timothy_gb300 0.1 sm_103a"; }

extern "C" int tm_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

// ---------------------------------------------------------------------------
// first-fit range allocator

struct range_alloc {
    long long cap = 0, hwm = 0;
    std::vector<std::pair<long long, long long>> freel;   // (start, len), sorted by start
    void init(long long c)
    {
        cap = c;
        hwm = 0;
        freel.clear();
        if (c > 0) freel.push_back({0, c});
    }
    bool alloc(long long len, long long &start)
    {
        for (size_t k = 0; k < freel.size(); k++) {
            if (freel[k].second >= len) {
                start = freel[k].first;
                freel[k].first += len;
                freel[k].second -= len;
                if (freel[k].second == 0) freel.erase(freel.begin() + (long)k);
                hwm = std::max(hwm, start + len);
                return true;
            }
        }
        return false;
    }
    void release(long long start, long long len)
    {
        if (len <= 0) return;
        auto it = std::lower_bound(freel.begin(), freel.end(), std::make_pair(start, 0ll));
        it = freel.insert(it, {start, len});
        size_t k = (size_t)(it - freel.begin());
        if (k + 1 < freel.size() && freel[k].first + freel[k].second == freel[k + 1].first) {
            freel[k].second += freel[k + 1].second;
            freel.erase(freel.begin() + (long)k + 1);
        }
        if (k > 0 && freel[k - 1].first + freel[k - 1].second == freel[k].first) {
            freel[k - 1].second += freel[k].second;
            freel.erase(freel.begin() + (long)k);
        }
        // lower the high-water mark when the tail is free
        if (!freel.empty() && freel.back().first + freel.back().second == cap) hwm = std::min(hwm, freel.back().first);
    }
    long long free_total() const
    {
        long long s = 0;
        for (auto &f : freel) s += f.second;
        return s;
    }
    long long largest() const
    {
        long long m = 0;
        for (auto &f : freel) m = std::max(m, f.second);
        return m;
    }
};

struct colony_host {
    bool used = false;
    int n = 0, nslots = 0, lcap = 1;
    long long off = 0, binoff = 0, nbin = 0, gridoff = -1, ngrid = 0;
    int gsize[3] = {0, 0, 0};
    tm_colony_options opt{};
    int active = 1;
};

// An asynchronous download sends each coordinate in pieces (up to IO_CHUNKS,
// one per 2^20 cells: small colonies go in one, their copies being cheaper
// than the calls that queue them) and an asynchronous upload of the same
// cells sends each piece back as soon as it is on the host, so a host loop
// that feeds back the positions it received keeps both directions of the
// link busy at once.
#define IO_CHUNKS 8

static int io_pieces(long long n)
{
    const long long p = n >> 20;
    return p < 1 ? 1 : (p > IO_CHUNKS ? IO_CHUNKS : (int)p);
}

static long long io_chunk_lo(long long n, int j) { return n * j / io_pieces(n); }

struct tm_session {
    int device = 0;
    cudaStream_t stream = nullptr;
    tm_session_config cfg{};
    tm_consts K{};
    tm_consts *dK = nullptr;
    tm_arrays A{};
    range_alloc slots, bins, grids;
    std::vector<colony_host> cols;
    tm_desc *h_desc = nullptr;
    tm_frame *h_frame = nullptr;
    uint32_t *scan_tmp = nullptr;
    uint32_t *scan_tmp_slots = nullptr;   // scan scratch for slot-sized scans (compaction)
    unsigned long long *d_octsize = nullptr;
    int *d_flag = nullptr;   // set by the upload kernels on a cell type outside the table
    void *d_scratch = nullptr;
    void *d_scratch2 = nullptr;              // second download buffer (copies overlap the next gather)
    cudaStream_t copy_stream = nullptr;
    cudaStream_t h2d_stream = nullptr;    // asynchronous uploads
    cudaEvent_t ev_h2d = nullptr;
    // asynchronous I/O: own staging, so copies overlap the steps
    unsigned char *up_stage = nullptr;    // x, y, z, size (8 B), young, ctype, phase (4 B) per slot
    unsigned char *dl_stage = nullptr;    // the downloaded fields, 8 B per slot each, and the inverse permutation
    unsigned char *up_rec = nullptr;      // an upload's cells as 48-byte records (caller order)
    double *dl_grid = nullptr;            // the grid of an asynchronous download (one colony's grid)
    size_t up_bytes = 0, dl_bytes = 0, rec_bytes = 0, dl_grid_bytes = 0;
    cudaEvent_t ev_up_read = nullptr;     // k_upload_pack has read up_stage
    cudaEvent_t ev_dl_gathered = nullptr, ev_dl_copied = nullptr;
    cudaEvent_t ev_dl_pos = nullptr;      // the positions of the last asynchronous download are on the host
    cudaEvent_t ev_dl_chunk[3][IO_CHUNKS] = {};   // each of its x, y, z chunks
    long long dl_pos_n = -1;              // the cell count those positions were split by
    cudaEvent_t ev_dl_part[16] = {};      // one field of an asynchronous download gathered
    bool dl_pending = false, up_pending = false;
    cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    // profiling
    bool prof = false;
    std::vector<cudaEvent_t> evpool;
    size_t evused = 0;
    long long prof_steps = 0;
    // graph of one step
    bool use_graph = false;
    bool graph_valid[2] = {false, false};
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    long long graph_shape[2][7] = {};     // what colony adds and removes can change in a captured step
    int parity = 0;   // always 0: the state stays in place between steps
    long long launches = 0;
    int kernels_per_step = 0;
    int mass_types = 0;   // types the FP64 density-weight array holds
    int dl_next = 0;      // download buffer the next field uses
    double *env_buf = nullptr;   // gather output staging (grows on demand)
    size_t env_bytes = 0;
    // cell cycle: per-type parameters on the device, the draw stream, state arrays
    void *cy_params = nullptr;   // tm_cycle_type[8] + 2 x [8][TM_CYCLE_MAX_FIELDS] floats + double csize[8]
    int *cy_stream = nullptr;
    size_t cy_stream_cap = 0;
    unsigned long long *cy_marked = nullptr;
    tm_rand_cache rand_cache = {};          // where the last device rand() stream ended
    uint32_t *rand_windows = nullptr;        // per-chunk starting windows of that stream
    int64_t rand_windows_cap = 0;
    int *move_buf = nullptr;     // the drop-in's random-move draws
    size_t move_cap = 0;
    tm_tuning tune{1, 1, 128, 0.1f, 64};
    cudaEvent_t tstart = nullptr, tstop = nullptr;
    // diagnostics: sampled neighbour lists (tm_colony_sample_neighbours)
    int diag_col = -1;
    long long diag_ncells = 0;
    // fences (tm_session_fence): a ring of events
    std::vector<cudaEvent_t> fence_ev;
    cudaEvent_t fence_join = nullptr;
    int64_t fence_next = 0;
};

// ---------------------------------------------------------------------------
// helper kernels

__global__ void k_colony_init(tm_arrays a, int c, long long off, int n, int nslots, int has_phase)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nslots) return;
    long long i = off + k;
    if (k == 0) {
        a.frame[c].force_rebuild = 1;   // the slots no longer match the lists
        a.frame[c].list_ok = 0;
    }
    a.col[i] = c;
    if (k < n) {
        a.perm[i] = (int)k;
        if (!has_phase) a.phase[i] = 1;
    }
    a.rem[i] = 0;
    a.density[i] = 0.0;
    a.v[i] = 0.0;
    a.mindist[i] = 0.0;
    a.fx[i] = 0.0;
    a.fy[i] = 0.0;
    a.fz[i] = 0.0;
    a.nbcount[i] = 0;
    a.nbmin[i] = -1;
    if (a.nbhash) a.nbhash[i] = 0;
    if (a.vcand) a.vcand[i] = -1;
}

// Upload into a colony that keeps its cell count.  The new values arrive in
// input order (in the rebuild scratch, or the asynchronous upload's staging)
// and go through perm to the slots the cells occupy now, so the Morton order
// and the neighbour lists stay valid: the step's rebuild test sees the
// displacement from the list positions, and a cell that changed size or type
// (list radius, FP64 density weight) forces a rebuild.  Cell types outside
// the table are flagged and replaced by 0.

// the cells of an upload in caller order, at [base + caller index]
struct upload_src {
    const double *x, *y, *z, *size;
    const float *young;
    const int *ctype, *phase;
    long long base;
};

// One cell of an upload, 16-byte aligned.  The slots hold the cells in Morton
// order and the caller's arrays in caller order, so putting the cells in
// their slots reads them at random: from seven separate arrays that costs
// seven DRAM bursts per cell, from one record one or two.  k_upload_pack
// writes the records from the staged arrays (both sides in caller order,
// coalesced) and k_upload_keep reads one record per slot.
union up_rec {
    struct {
        double x, y, z, size;
        float young;
        int ctype, phase, pad;
    } f;
    int4 v[3];
};

// fields an upload carries besides the positions (the others keep their values)
#define UP_PHASE 1
#define UP_SIZE 2
#define UP_YOUNG 4
#define UP_CTYPE 8
#define UP_ALL (UP_SIZE | UP_YOUNG | UP_CTYPE)

__global__ void k_upload_pack(upload_src u, int n, int fields, int4 *rec)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long src = u.base + k;
    up_rec r;
    r.f.x = u.x[src];
    r.f.y = u.y[src];
    r.f.z = u.z[src];
    r.f.size = (fields & UP_SIZE) ? u.size[src] : 0.0;
    r.f.young = (fields & UP_YOUNG) ? u.young[src] : 0.0f;
    r.f.ctype = (fields & UP_CTYPE) ? u.ctype[src] : 0;
    r.f.phase = (fields & UP_PHASE) ? u.phase[src] : 0;
    r.f.pad = 0;
    int4 *d = rec + src * 3;
    d[0] = r.v[0];
    d[1] = r.v[1];
    d[2] = r.v[2];
}

__global__ void k_upload_keep(tm_arrays a, const tm_consts *K, int c, long long off, int n, int fields,
                              int *bad, const int4 *rec, long long base)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long s = off + k;
    const int4 *p = rec + (base + a.perm[s]) * 3;
    up_rec r;
    r.v[0] = p[0];
    r.v[1] = p[1];
    r.v[2] = p[2];
    const double x = r.f.x, y = r.f.y, z = r.f.z;
    if (fields & UP_CTYPE) {
        int ct = r.f.ctype;
        if (ct < 0 || ct >= K->ntypes) {
            if (bad) atomicExch(bad, 1);
            else atomicOr(&a.frame[c].error, TM_ERR_TYPES);
            ct = 0;
        }
        if (ct != a.ctype[s]) a.frame[c].force_rebuild = 1;
        a.ctype[s] = ct;
    }
    if (fields & UP_SIZE) {
        if (r.f.size != a.size[s]) a.frame[c].force_rebuild = 1;
        a.size[s] = r.f.size;
    }
    a.x[s] = x;
    a.y[s] = y;
    a.z[s] = z;
    if (fields & UP_YOUNG) a.young[s] = r.f.young;
    if (fields & UP_PHASE) a.phase[s] = r.f.phase;
    a.rem[s] = 0;
    if (a.desc[c].verlet && a.x0) {
        float hx, hy, hz, lx, ly, lz;
        tm_split(x, hx, lx);
        tm_split(y, hy, ly);
        tm_split(z, hz, lz);
        const float4 o = a.x0[s];
        const float ex = hx - o.x, ey = hy - o.y, ez = hz - o.z;
        const unsigned bits = __float_as_uint(sqrtf(fmaf(ex, ex, fmaf(ey, ey, ez * ez))));
        const unsigned m = __reduce_max_sync(__activemask(), bits);
        // one word per colony: only warps past its current value post (it only grows)
        if (bits == m && m > __ldcg(&a.frame[c].maxdisp)) atomicMax(&a.frame[c].maxdisp, m);
    }
}

// cell types of a fresh upload (identity order)
__global__ void k_check_types(tm_arrays a, const tm_consts *K, long long off, int n, int *bad)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int ct = a.ctype[off + k];
    if (ct < 0 || ct >= K->ntypes) {
        atomicExch(bad, 1);
        a.ctype[off + k] = 0;
    }
}

__global__ void k_release_slots(int *col, long long off, int nslots, int none)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nslots) col[off + k] = none;
}

template <typename T>
__global__ void k_unsort(const T *src, const int *perm, long long off, int n, T *dst)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[perm[off + k]] = src[off + k];
}

// Download gathers: the inverse of the slot permutation (iperm[perm[off + s]]
// = s), then one pass per field that reads the field at random and writes it
// in caller order (coalesced).  Measured at 16 M cells: 0.17 ms per 8-byte
// field; scattering the writes instead took 0.3 ms, and packing the fields
// into 16-byte-aligned records to gather whole records took 2.2 ms for the
// ten fields against 1.7 ms.
__global__ void k_invert_perm(const int *perm, long long off, int n, int *iperm)
{
    long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    iperm[perm[off + s]] = (int)s;
}

template <typename T>
__global__ void k_unsort_gather(const T *src, const int *iperm, long long off, int n, T *dst)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[k] = src[off + iperm[k]];
}

static unsigned blocks_for(long long n, int bt) { return (unsigned)std::max(1ll, (n + bt - 1) / bt); }

// the arrays as the kernels of one step see them
static tm_arrays view(const tm_session *s, int /*unused*/ = 0)
{
    tm_arrays a = s->A;
    a.nslots_total = s->slots.hwm * 32;
    a.ncol = (int)s->cols.size();
    return a;
}

static cudaEvent_t next_event(tm_session *s)
{
    if (s->evused == s->evpool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        s->evpool.push_back(e);
    }
    return s->evpool[s->evused++];
}

static void mark(tm_session *s)
{
    if (!s->prof) return;
    cudaEvent_t e = next_event(s);
    if (e) cudaEventRecord(e, s->stream);
}

static void colony_mix(const tm_session *s, bool &any_cic, bool &any64, bool &any32)
{
    any_cic = any64 = any32 = false;
    for (auto &c : s->cols) {
        if (!c.used || !c.active) continue;
        if (c.gridoff >= 0) any_cic = true;
        if (c.opt.precision == TM_PREC_FP64) any64 = true;
        else any32 = true;
    }
}

// Build phase (octbuild): frames, lattice codes, counting sort into Morton
// order.  Colonies that rebuild their neighbour lists this step also move
// their state into Morton order (gather into scratch, copy back).
static int enqueue_build(tm_session *s, int p, int &nk)
{
    cudaStream_t st = s->stream;
    tm_arrays a = view(s, p);
    const long long nsl = a.nslots_total;
    const long long nbin = s->bins.hwm;
    const int ncol = a.ncol;
    CK(cudaMemsetAsync(a.bin_count, 0, (size_t)(nbin + 1) * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(a.bigbins, 0, sizeof(int), st));
    CK(cudaMemsetAsync(a.fix_count, 0, 6 * sizeof(int), st));   // fix count and the five work counters
    if (a.diag_cnt) CK(cudaMemsetAsync(a.diag_cnt, 0, (size_t)s->diag_ncells * sizeof(int), st));
    k_step_init<<<blocks_for(ncol, 128), 128, 0, st>>>(a);
    CK(tm_launch_bbox(a, s->K.ntypes, st));
    k_frame<<<blocks_for(ncol, 128), 128, 0, st>>>(a, s->dK);
    k_codes<<<blocks_for(nsl, 256), 256, 0, st>>>(a);
    CK(cudaGetLastError());
    CK(tm_scan_exclusive(a.bin_count, a.bin_start, nbin + 1, s->scan_tmp, st));
    k_binbase<<<blocks_for(ncol, 128), 128, 0, st>>>(a);
    k_scatter<<<blocks_for(nsl, 256), 256, 0, st>>>(a);
    k_place<<<blocks_for(nsl, 256), 256, 0, st>>>(a, s->dK);
    k_binsort_big<<<64, 256, 0, st>>>(a, s->dK);
    k_worklist<<<1, 1024, 0, st>>>(a, 0);
    k_copyback<<<tm_stream_grid(256, 8), 256, 0, st>>>(a);
    CK(cudaGetLastError());
    nk += 13;   // step_init, bbox, frame, codes, 3 scan passes, binbase, scatter, place, big-bin sort, worklist, copyback
    return TM_OK;
}

// CIC deposit of the current positions (patches_cells2envinfo)
static int enqueue_cic(tm_session *s, int &nk)
{
    bool any_cic, any64, any32;
    colony_mix(s, any_cic, any64, any32);
    if (!any_cic) return TM_OK;
    tm_arrays b = view(s, s->parity);
    CK(cudaMemsetAsync(b.grid, 0, (size_t)s->grids.hwm * sizeof(double), s->stream));
    CK(tm_launch_cic(b, s->dK, s->stream));
    nk++;
    return TM_OK;
}

static tm_shapes shapes_of(const tm_session *s)
{
    tm_shapes sh;
    sh.pair_lshift = s->tune.pair_lshift;
    sh.list_variant = s->tune.list_variant;
    sh.walk_block = s->tune.walk_block;
    return sh;
}

// pair kernel(s) and octree walk on the current (sorted) buffers
static int enqueue_compute(tm_session *s, int &nk, bool with_marks)
{
    bool any_cic, any64, any32;
    colony_mix(s, any_cic, any64, any32);
    tm_arrays b = view(s, s->parity);
    const tm_shapes sh = shapes_of(s);
    const bool lists = b.vcap > 0;
    // search and list-build passes, then the list passes, then the searches of
    // colonies whose lists overflowed and the FP64 density fix-up
    if (any64) CK(tm_launch_search(b, s->dK, 0, sh, 0, s->stream));
    if (any32) CK(tm_launch_search(b, s->dK, 1, sh, 0, s->stream));
    nk += (any64 ? 1 : 0) + (any32 ? 1 : 0);
    if (lists) {
        CK(tm_launch_listbuild(b, s->dK, s->stream));
        nk++;
    }
    if (with_marks) mark(s);
    if (lists) {
        if (any64) CK(tm_launch_list(b, s->dK, 0, sh, s->stream));
        if (any32) CK(tm_launch_list(b, s->dK, 1, sh, s->stream));
        nk += (any64 ? 1 : 0) + (any32 ? 1 : 0);
    }
    if (with_marks) mark(s);
    if (lists) {
        if (any64) CK(tm_launch_search(b, s->dK, 0, sh, 1, s->stream));
        if (any32) CK(tm_launch_search(b, s->dK, 1, sh, 1, s->stream));
        nk += (any64 ? 1 : 0) + (any32 ? 1 : 0);
    }
    if (any32) {
        CK(tm_launch_fix(b, s->dK, s->stream));
        nk++;
    }
    if (with_marks) mark(s);
    CK(tm_launch_octree(b, s->dK, s->tune.walk_block, s->stream));
    nk += 3;   // worklist, mark, walk
    return TM_OK;
}

static int enqueue_update(tm_session *s, int &nk)
{
    tm_arrays b = view(s, s->parity);
    CK(tm_launch_update(b, s->dK, s->stream));
    nk++;
    return TM_OK;
}

// one full step; the parity flips inside (after the build phase)
static int enqueue_step(tm_session *s)
{
    if (s->slots.hwm == 0 || s->cols.empty()) return TM_OK;
    int nk = 0, rc;
    mark(s);
    if ((rc = enqueue_build(s, s->parity, nk))) return rc;
    mark(s);
    if ((rc = enqueue_cic(s, nk))) return rc;
    mark(s);
    if ((rc = enqueue_compute(s, nk, true))) return rc;
    mark(s);
    if ((rc = enqueue_update(s, nk))) return rc;
    mark(s);
    s->kernels_per_step = nk;
    return TM_OK;
}

// The launch parameters of a step that adding or removing a colony can
// change: the slot, bin and grid high-water marks, the colony count and which
// paths the colonies take.  Those two operations keep the captured step when
// these are unchanged (descriptors and frames live in device memory, so a
// colony placed in freed ranges runs in the same launches); every other
// change of the session drops the captured steps.
static void graph_shape_of(const tm_session *s, long long out[7])
{
    bool any_cic = false, any64 = false, any32 = false;
    for (auto &c : s->cols) {
        if (!c.used || !c.active) continue;
        if (c.gridoff >= 0) any_cic = true;
        if (c.opt.precision == TM_PREC_FP64) any64 = true;
        else any32 = true;
    }
    out[0] = s->slots.hwm;
    out[1] = s->bins.hwm;
    out[2] = s->grids.hwm;
    out[3] = (long long)s->cols.size();
    out[4] = any_cic;
    out[5] = any64;
    out[6] = any32;
}

static void drop_graphs(tm_session *s)
{
    for (int k = 0; k < 2; k++) {
        if (s->gexec[k]) cudaGraphExecDestroy(s->gexec[k]);
        s->gexec[k] = nullptr;
        s->graph_valid[k] = false;
    }
}

// A colony's descriptor and frame reach the device as kernel arguments, so the
// values are those of the call even when the host changes its copy before the
// stream gets there (a colony removed and its entry reused without a wait).
__global__ void k_set_desc(tm_desc *dst, tm_desc v) { *dst = v; }
__global__ void k_set_frame(tm_frame *dst, tm_frame v) { *dst = v; }

static int push_desc(tm_session *s, int c)
{
    k_set_desc<<<1, 1, 0, s->stream>>>(&s->A.desc[c], s->h_desc[c]);
    CK(cudaGetLastError());
    return TM_OK;
}

// ---------------------------------------------------------------------------
// session lifetime

template <typename T>
static int dalloc(T **p, long long count)
{
    if (count <= 0) count = 1;
    CK(cudaMalloc((void **)p, (size_t)count * sizeof(T)));
    return TM_OK;
}

// the largest double d2 with sqrt(d2) <= h: the square root is correctly
// rounded and monotone, so sqrt(d2) <= h exactly when d2 <= this bound
static double cutoff_sq(double h)
{
    double x = h * h;
    while (x > 0.0 && std::sqrt(x) > h) x = std::nextafter(x, 0.0);
    for (;;) {
        const double y = std::nextafter(x, HUGE_VAL);
        if (!(std::sqrt(y) <= h)) break;
        x = y;
    }
    return x;
}

static double host_type_const(int dim, int which, double h, double h2, double h3, double h4)
{
    // the reference's own expressions (inline.h:45-46, 71-72)
    if (which == 0) return dim == 2 ? 40 / (7 * M_PI * h2) : 8 / (M_PI * h3);
    return dim == 2 ? (40 * 8) / (7 * M_PI * h3) : 48 / (M_PI * h4);
}

extern "C" int tm_session_destroy(tm_session *s);

// Every device buffer of a session: allocates them (alloc) or only adds up
// their bytes (*bytes), so admission by free memory uses the same list.
static int session_buffers(tm_session *s, long long S, long long B, long long G, int C, bool alloc,
                           long long *bytes)
{
    tm_arrays &a = s->A;
    const tm_session_config *cfg = &s->cfg;
    int rc = TM_OK;
    long long total = 0;
    auto AL = [&](auto &p, long long cnt) {
        using T = typename std::remove_reference<decltype(*p)>::type;
        total += std::max(cnt, 1ll) * (long long)sizeof(T);
        if (alloc && rc == TM_OK) rc = dalloc(&p, cnt);
    };
    AL(a.x, S); AL(a.y, S); AL(a.z, S); AL(a.size, S); AL(a.young, S); AL(a.ctype, S); AL(a.phase, S);
    AL(a.perm, S); AL(a.rem, S);
    AL(a.x2, S); AL(a.y2, S); AL(a.z2, S); AL(a.size2, S); AL(a.young2, S); AL(a.ctype2, S); AL(a.phase2, S);
    AL(a.perm2, S); AL(a.rem2, S);
    AL(a.col, S); AL(a.code, S); AL(a.codes, S); AL(a.bin, S); AL(a.grp, S); AL(a.tmp, S); AL(a.rank, S); AL(a.hi, S);
    AL(a.lo, S);
    AL(a.mass, S * s->K.ntypes);
    AL(a.bin_count, B + 1); AL(a.bin_start, B + 1); AL(a.bigbins, 2 * (S / 33) + 4);
    AL(a.fix_count, 8); AL(a.fix_list, S); AL(a.walk_list, S); AL(a.wl, 2 * (C + 1));
    AL(a.density, S); AL(a.v, S); AL(a.mindist, S); AL(a.fx, S); AL(a.fy, S); AL(a.fz, S); AL(a.nbcount, S);
    AL(a.nbmin, S);
    AL(a.grid, G); AL(a.desc, C + 1); AL(a.frame, C + 1);   // entry C: never active (freed slots)
    AL(s->scan_tmp, tm_scan_tmp_words(B + 1)); AL(s->d_octsize, C); AL(s->dK, 1); AL(s->d_flag, 1);
    AL(s->scan_tmp_slots, tm_scan_tmp_words(S + 1));
    {
        double *scratch = nullptr;        // S + 1 doubles: also two (S + 1)-word scans
        AL(scratch, S + 1);
        s->d_scratch = scratch;
        double *scratch2 = nullptr;
        AL(scratch2, S + 1);
        s->d_scratch2 = scratch2;
    }
    if (cfg->diagnostics) {
        AL(a.nbhash, S);
        AL(a.vcand, S);
    }
    if (cfg->list_capacity > 0) {
        AL(a.vlist, S * (long long)cfg->list_capacity);
        AL(a.vcount, S);
        AL(a.x0, S);
    }
    if (bytes) *bytes = total;
    return rc;
}

static void session_extents(const tm_session_config *cfg, long long &S, long long &B, long long &G, int &C)
{
    S = ((cfg->max_slots + 31) / 32) * 32;
    B = cfg->max_bin_entries > 0 ? cfg->max_bin_entries
                                 : std::max<long long>(1 << 12, 2 * S) + (1ll << (3 * TM_LMAX)) + 2;
    G = cfg->max_grid_entries > 0 ? cfg->max_grid_entries : 257ll * 257 * 257;
    C = cfg->max_colonies;
}

extern "C" int64_t tm_session_bytes(const tm_session_config *cfg, int ntypes)
{
    if (!cfg || cfg->max_slots <= 0 || cfg->max_colonies <= 0 || ntypes < 1 || ntypes > TM_MAX_TYPES) return -1;
    tm_session probe;
    probe.cfg = *cfg;
    probe.K.ntypes = ntypes;
    long long S, B, G, bytes = 0;
    int C;
    session_extents(cfg, S, B, G, C);
    session_buffers(&probe, S, B, G, C, false, &bytes);
    return (int64_t)bytes;
}

extern "C" int tm_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes)
{
    if (!free_bytes || !total_bytes) return tm_fail(TM_EINVAL, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return tm_fail(TM_ENODEV, "no CUDA device");
    if (device < 0 || device >= ndev) return tm_fail(TM_EINVAL, "device %d out of range", device);
    CK(cudaSetDevice(device));
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    *free_bytes = (int64_t)f;
    *total_bytes = (int64_t)t;
    return TM_OK;
}

extern "C" int tm_session_create(tm_session **out, const tm_session_config *cfg, const tm_celltypes *types)
{
    if (!out || !cfg || !types) return tm_fail(TM_EINVAL, "null argument");
    *out = nullptr;
    if (cfg->dimension != 2 && cfg->dimension != 3) return tm_fail(TM_EINVAL, "dimension must be 2 or 3");
    if (types->ntypes < 1 || types->ntypes > TM_MAX_TYPES) return tm_fail(TM_EINVAL, "ntypes must be 1..%d", TM_MAX_TYPES);
    if (cfg->max_slots <= 0 || cfg->max_colonies <= 0) return tm_fail(TM_EINVAL, "max_slots and max_colonies must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return tm_fail(TM_ENODEV, "no CUDA device");
    if (cfg->device < 0 || cfg->device >= ndev) return tm_fail(TM_EINVAL, "device %d out of range", cfg->device);
    CK(cudaSetDevice(cfg->device));

    tm_session *s = new tm_session();
    s->device = cfg->device;
    s->cfg = *cfg;
    tm_consts &K = s->K;
    K.ntypes = types->ntypes;
    K.dim = cfg->dimension;
    for (int t = 0; t < K.ntypes; t++) {
        tm_type &T = K.t[t];
        T.h = types->h[t];
        T.h2 = types->h2[t];
        T.h3 = types->h3[t];
        T.h4 = types->h4[t];
        T.csize = types->size[t];
        T.sc = cfg->dimension == 2 ? T.h2 : T.h3;
        T.cW = host_type_const(cfg->dimension, 0, T.h, T.h2, T.h3, T.h4);
        T.cG = host_type_const(cfg->dimension, 1, T.h, T.h2, T.h3, T.h4);
        T.e = T.h + 0.01;
        T.h_fx = std::fabs(T.h) < 8192.0 ? (long long)std::ldexp(T.h, 47) : 0;
        T.randommove = types->randommove ? types->randommove[t] : 0.0f;
        T.hf = (float)T.h;
        T.h2f = (float)(T.h * T.h);
        T.inv_hf = (float)(1.0 / T.h);
        T.cWf = (float)T.cW;
        T.cGf = (float)T.cG;
        T.kmassf = (float)(T.sc / T.csize);
        T.inv_h = 1.0 / T.h;
        T.h2cut = cutoff_sq(T.h);
        T.kmass = T.sc / T.csize;
        T.thr_lo = (float)(T.h * (1.0 - 1e-5) * T.h * (1.0 - 1e-5));
        T.thr_hi = (float)(T.h * (1.0 + 1e-5) * T.h * (1.0 + 1e-5));
        if (!(T.h > 0.0) || !(T.csize > 0.0)) {
            delete s;
            return tm_fail(TM_EINVAL, "type %d: h and size must be positive", t);
        }
    }

    long long S, B, G;
    int C;
    session_extents(cfg, S, B, G, C);
    s->slots.init(S / 32);
    s->bins.init(B);
    s->grids.init(G);
    s->cols.reserve((size_t)C);

    int rc = TM_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return tm_fail(TM_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    tm_arrays &a = s->A;
    rc = session_buffers(s, S, B, G, C, true, nullptr);
    s->mass_types = K.ntypes;
    if (rc == TM_OK) a.work = a.fix_count + 1;
    a.lstride = S;
    a.wl_stride = C + 1;
    a.vcap = cfg->list_capacity > 0 ? cfg->list_capacity : 0;
    if (rc == TM_OK) {
        if (cudaMallocHost((void **)&s->h_desc, sizeof(tm_desc) * (size_t)C) != cudaSuccess ||
            cudaMallocHost((void **)&s->h_frame, sizeof(tm_frame) * (size_t)C) != cudaSuccess)
            rc = tm_fail(TM_ENOMEM, "pinned host allocation failed");
    }
    if (rc != TM_OK) {
        std::string msg = g_err;
        tm_session_destroy(s);
        g_err = msg;
        return rc == TM_ECUDA ? TM_ENOMEM : rc;
    }
    a.want_diag = cfg->diagnostics ? 1 : 0;
    a.nbin_total = B;
    memset(s->h_desc, 0, sizeof(tm_desc) * (size_t)C);
    memset(s->h_frame, 0, sizeof(tm_frame) * (size_t)C);
    e = cudaMemcpy(s->dK, &s->K, sizeof(tm_consts), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(a.desc, 0, sizeof(tm_desc) * (size_t)(C + 1));
    if (e == cudaSuccess) e = cudaMemset(a.frame, 0, sizeof(tm_frame) * (size_t)(C + 1));
    // the memsets run on the legacy stream, which the session's stream does not wait for
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        tm_session_destroy(s);
        return tm_fail(TM_ECUDA, "session init: %s", cudaGetErrorString(e));
    }
    *out = s;
    return TM_OK;
}

extern "C" int tm_session_destroy(tm_session *s)
{
    if (!s) return TM_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    drop_graphs(s);
    tm_arrays &a = s->A;
    void *ptrs[] = {a.x, a.y, a.z, a.size, a.young, a.ctype, a.phase, a.perm, a.rem, a.x2, a.y2, a.z2, a.size2,
                    a.young2, a.ctype2, a.phase2, a.perm2, a.rem2, a.col, a.code, a.codes, a.bin, a.grp, a.tmp, a.rank, a.hi, a.lo, a.vlist, a.vcount, a.x0,
                    a.mass, a.bin_count, a.bin_start, a.bigbins, a.fix_count, a.fix_list, a.walk_list, a.wl, a.density, a.v, a.mindist, a.fx,
                    a.fy, a.fz, a.nbcount, a.nbmin, a.nbhash, a.vcand, a.grid, a.desc, a.frame, s->scan_tmp, s->scan_tmp_slots, s->d_octsize,
                    s->dK, s->d_scratch, s->d_scratch2, s->d_flag, a.diag_row, a.diag_cnt, a.diag_nb};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto ev : s->evpool) cudaEventDestroy(ev);
    for (auto ev : s->fence_ev)
        if (ev) cudaEventDestroy(ev);
    if (s->fence_join) cudaEventDestroy(s->fence_join);
    if (s->tstart) cudaEventDestroy(s->tstart);
    if (s->tstop) cudaEventDestroy(s->tstop);
    if (s->h_desc) cudaFreeHost(s->h_desc);
    if (s->h_frame) cudaFreeHost(s->h_frame);
    for (int k = 0; k < 2; k++) {
        if (s->ev_ready[k]) cudaEventDestroy(s->ev_ready[k]);
        if (s->ev_copied[k]) cudaEventDestroy(s->ev_copied[k]);
    }
    if (s->env_buf) cudaFree(s->env_buf);
    {
        void *cy[] = {s->A.cy_pt, s->A.cy_g1, s->A.cy_s, s->A.cy_g2, s->A.cy_m, s->A.cy_age, s->cy_params,
                      s->cy_stream, s->cy_marked, s->move_buf, s->rand_windows};
        for (void *p : cy)
            if (p) cudaFree(p);
    }
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->h2d_stream) cudaStreamDestroy(s->h2d_stream);
    if (s->ev_h2d) cudaEventDestroy(s->ev_h2d);
    for (cudaEvent_t e : {s->ev_up_read, s->ev_dl_gathered, s->ev_dl_copied, s->ev_dl_pos})
        if (e) cudaEventDestroy(e);
    for (auto &axis : s->ev_dl_chunk)
        for (cudaEvent_t e : axis)
            if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : s->ev_dl_part)
        if (e) cudaEventDestroy(e);
    if (s->up_stage) cudaFree(s->up_stage);
    if (s->dl_stage) cudaFree(s->dl_stage);
    if (s->dl_grid) cudaFree(s->dl_grid);
    if (s->up_rec) cudaFree(s->up_rec);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return TM_OK;
}

extern "C" void *tm_session_stream(tm_session *s) { return s ? (void *)s->stream : nullptr; }

// ---------------------------------------------------------------------------
// colonies

static int grid_geometry(int dim, float gfh, int gsize[3], double lower[3])
{
    // computegridsize at one rank, grid.c:37-77 (float arithmetic as written there)
    if (!(gfh > 0.0f)) return TM_EINVAL;
    float gx = (float)(1024.0 - (-1024.0) + 1), gz = dim == 3 ? gx : 0.0f;
    long long sx = (long long)((gx + 1) / gfh);
    long long sz = dim == 3 ? (long long)((gz + 1) / gfh) : 0;
    sx += 1 - sx % 1;
    if (dim == 3) sz += 1 - sz % 1;
    else sz = 1;
    gsize[0] = (int)sx;
    gsize[1] = (int)sx;
    gsize[2] = (int)sz;
    lower[0] = -1024.0;
    lower[1] = -1024.0;
    lower[2] = dim == 3 ? -1024.0 : 0.0;
    return TM_OK;
}

// keep: the colony keeps its cell count, so the cells go to their current
// slots (k_upload_keep); otherwise slot k takes input cell k and the lists are
// rebuilt.  Returns TM_EINVAL if a cell type lies outside the table.
static int download_streams(tm_session *s);

// the record buffer of uploads into kept slots (48 B per slot, allocated on first use)
static int upload_records(tm_session *s, int4 **rec)
{
    const size_t need = ((size_t)s->slots.hwm * 32 + 32) * sizeof(up_rec);
    if (s->rec_bytes < need) {
        CK(cudaStreamSynchronize(s->stream));
        if (s->up_rec) CK(cudaFree(s->up_rec));
        s->up_rec = nullptr;
        s->rec_bytes = 0;
        CK(cudaMalloc((void **)&s->up_rec, need));
        s->rec_bytes = need;
    }
    *rec = (int4 *)s->up_rec;
    return TM_OK;
}

// wait = false (a new colony only, its types checked on the host): the copies
// and kernels are queued and the call returns without waiting for them
static int copy_cells_in(tm_session *s, const colony_host &c, const tm_colony_input *in, bool keep,
                         bool wait = true)
{
    const tm_arrays a = view(s, s->parity);
    const long long o = c.off;
    const size_t n = (size_t)in->n;
    const int cid = (int)(&c - s->cols.data());
    cudaStream_t st = s->stream;
    CK(cudaMemsetAsync(s->d_flag, 0, sizeof(int), st));
    double *X = keep ? a.x2 : a.x, *Y = keep ? a.y2 : a.y, *Z = keep ? a.z2 : a.z, *SZ = keep ? a.size2 : a.size;
    float *YG = keep ? a.young2 : a.young;
    int *CT = keep ? a.ctype2 : a.ctype, *PH = keep ? a.phase2 : a.phase;
    if (n) {
        // two streams, so two copies are in flight at a time
        int rc = download_streams(s);
        if (rc) return rc;
        cudaStream_t st2 = s->copy_stream;
        CK(cudaEventRecord(s->ev_ready[0], st));
        CK(cudaStreamWaitEvent(st2, s->ev_ready[0], 0));
        CK(cudaMemcpyAsync(X + o, in->x, n * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(Y + o, in->y, n * 8, cudaMemcpyHostToDevice, st2));
        CK(cudaMemcpyAsync(Z + o, in->z, n * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(SZ + o, in->size, n * 8, cudaMemcpyHostToDevice, st2));
        CK(cudaMemcpyAsync(YG + o, in->young, n * 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(CT + o, in->ctype, n * 4, cudaMemcpyHostToDevice, st2));
        if (in->phase) CK(cudaMemcpyAsync(PH + o, in->phase, n * 4, cudaMemcpyHostToDevice, st));
        CK(cudaEventRecord(s->ev_copied[0], st2));
        CK(cudaStreamWaitEvent(st, s->ev_copied[0], 0));
    }
    if (keep) {
        const upload_src u = {a.x2, a.y2, a.z2, a.size2, a.young2, a.ctype2, a.phase2, o};
        int4 *rec = nullptr;
        int rc = upload_records(s, &rec);
        if (rc) return rc;
        k_upload_pack<<<blocks_for((long long)n, 256), 256, 0, st>>>(u, (int)n, UP_ALL | (in->phase ? UP_PHASE : 0),
                                                                    rec);
        k_upload_keep<<<blocks_for((long long)n, 256), 256, 0, st>>>(a, s->dK, cid, o, (int)n,
                                                                    UP_ALL | (in->phase ? UP_PHASE : 0),
                                                                    s->d_flag, rec, o);
    } else {
        k_check_types<<<blocks_for((long long)n, 256), 256, 0, st>>>(a, s->dK, o, (int)n, s->d_flag);
        k_colony_init<<<blocks_for(c.nslots, 256), 256, 0, st>>>(a, cid, o, (int)n, c.nslots, in->phase ? 1 : 0);
    }
    CK(cudaGetLastError());
    if (!wait && !keep) return TM_OK;
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    // synchronous: the caller may free its buffers on return
    CK(cudaStreamSynchronize(st));
    if (bad) return tm_fail(TM_EDEVICE, "a cell type lies outside 0..%d", s->K.ntypes - 1);
    return TM_OK;
}

// scan_types: check the cell types on the host before anything is placed
// (colony creation); uploads check them on the device
static int check_input(const tm_session *s, const tm_colony_input *in, bool scan_types = true)
{
    if (!in || in->n < 0) return tm_fail(TM_EINVAL, "bad colony input");
    if (in->n > 0 && (!in->x || !in->y || !in->z || !in->size || !in->young || !in->ctype))
        return tm_fail(TM_EINVAL, "colony input arrays missing");
    if (in->n > 0x7fffffffll) return tm_fail(TM_EINVAL, "colony too large");
    if (scan_types)
        for (long long k = 0; k < in->n; k++)
        if (in->ctype[k] < 0 || in->ctype[k] >= s->K.ntypes)
            return tm_fail(TM_EINVAL, "cell %lld has cell type %d outside 0..%d", k, in->ctype[k], s->K.ntypes - 1);
    return TM_OK;
}

static int auto_lcap(const tm_session *s, const tm_colony_input *in)
{
    if (in->n <= 1) return 1;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    const double *p[3] = {in->x, in->y, in->z};
    for (long long k = 0; k < in->n; k++)
        for (int d = 0; d < 3; d++) {
            mn[d] = std::min(mn[d], p[d][k]);
            mx[d] = std::max(mx[d], p[d][k]);
        }
    double hmax = 0.0;
    for (int t = 0; t < s->K.ntypes; t++) hmax = std::max(hmax, s->K.t[t].h);
    double ext = std::max(mx[0] - mn[0], std::max(mx[1] - mn[1], mx[2] - mn[2])) + 2 * (hmax + 0.01);
    // the bin table holds 8^L entries: bins of at least h/2 at the current
    // extent (a colony that grows later uses coarser bins, see k_frame)
    int L = (int)std::floor(std::log2(2.0 * ext / hmax));
    return std::max(1, std::min(TM_LMAX, L));
}

static int colony_add(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id, bool wait);

extern "C" int tm_colony_add(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id)
{
    return colony_add(s, in, opt, id, true);
}

extern "C" int tm_colony_add_async(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id)
{
    return colony_add(s, in, opt, id, false);
}

static int colony_add(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id, bool wait)
{
    if (!s || !opt || !id || !in) return tm_fail(TM_EINVAL, "null argument");
    // room first: a request that cannot fit is turned away before any pass
    // over its cells (admission control tries many)
    {
        const long long want = std::max<long long>(std::max<long long>(in->n, opt->reserve), 1);
        if ((want + 31) / 32 > s->slots.largest())
            return tm_fail(TM_ENOMEM, "no room for %lld slots", (long long)want);
    }
    int rc = check_input(s, in);
    if (rc) return rc;
    if (opt->precision != TM_PREC_FP64 && opt->precision != TM_PREC_FP32C) return tm_fail(TM_EINVAL, "bad precision");
    if (opt->update_mode < 0 || opt->update_mode > 2) return tm_fail(TM_EINVAL, "bad update mode");
    CK(cudaSetDevice(s->device));
    int c = -1;
    for (size_t k = 0; k < s->cols.size(); k++)
        if (!s->cols[k].used) { c = (int)k; break; }
    if (c < 0) {
        if ((int)s->cols.size() >= s->cfg.max_colonies) return tm_fail(TM_ENOMEM, "no free colony entry");
        s->cols.push_back(colony_host());
        c = (int)s->cols.size() - 1;
    }
    colony_host ch;
    ch.n = (int)in->n;
    const long long want = std::max<long long>(std::max<long long>(in->n, opt->reserve), 1);
    if (want > 0x7fffffe0ll) return tm_fail(TM_EINVAL, "colony too large");
    ch.nslots = (int)(((want + 31) / 32) * 32);
    ch.opt = *opt;
    ch.lcap = opt->lcap > 0 ? std::min(opt->lcap, TM_LMAX) : auto_lcap(s, in);
    ch.nbin = (1ll << (3 * ch.lcap)) + 2;
    long long soff;
    if (!s->slots.alloc(ch.nslots / 32, soff)) return tm_fail(TM_ENOMEM, "no room for %d slots", ch.nslots);
    ch.off = soff * 32;
    if (!s->bins.alloc(ch.nbin, ch.binoff)) {
        s->slots.release(soff, ch.nslots / 32);
        return tm_fail(TM_ENOMEM, "no room for %lld bin entries", ch.nbin);
    }
    double glower[3] = {0, 0, 0};
    if (opt->cic) {
        if (grid_geometry(s->K.dim, opt->gfh, ch.gsize, glower)) {
            s->slots.release(soff, ch.nslots / 32);
            s->bins.release(ch.binoff, ch.nbin);
            return tm_fail(TM_EINVAL, "bad grid resolution");
        }
        ch.ngrid = (long long)ch.gsize[0] * ch.gsize[1] * ch.gsize[2];
        if (!s->grids.alloc(ch.ngrid, ch.gridoff)) {
            s->slots.release(soff, ch.nslots / 32);
            s->bins.release(ch.binoff, ch.nbin);
            return tm_fail(TM_ENOMEM, "no room for a %lld-node grid", ch.ngrid);
        }
    }
    ch.used = true;
    ch.active = 1;
    s->cols[c] = ch;
    tm_desc &d = s->h_desc[c];
    memset(&d, 0, sizeof d);
    d.off = ch.off;
    d.binoff = ch.binoff;
    d.gridoff = opt->cic ? ch.gridoff : -1;
    d.n = ch.n;
    d.nslots = ch.nslots;
    d.Lcap = ch.lcap;
    d.precision = opt->precision;
    d.update_mode = opt->update_mode;
    d.active = 1;
    d.dt = opt->dt;
    d.verlet = (opt->verlet && s->A.vcap > 0) ? 1 : 0;
    {
        double hmax = 0.0;
        for (int t = 0; t < s->K.ntypes; t++) hmax = std::max(hmax, s->K.t[t].h);
        d.skin = opt->skin > 0.0f ? opt->skin : (float)(s->tune.skin_over_h * hmax);
    }
    d.rmax = opt->rmax > 0 ? opt->rmax : s->tune.rmax;
    for (int k = 0; k < 3; k++) {
        d.glower[k] = glower[k];
        d.gsize[k] = ch.gsize[k];
    }
    d.gres = opt->gfh;
    tm_frame &f = s->h_frame[c];
    memset(&f, 0, sizeof f);
    f.force_rebuild = 1;
    f.scale = 1.0;
    f.L = 1;
    f.nbins = 8;
    f.binscale = 2.0f;
    k_set_frame<<<1, 1, 0, s->stream>>>(&s->A.frame[c], f);
    CK(cudaGetLastError());
    rc = push_desc(s, c);
    if (rc == TM_OK) rc = copy_cells_in(s, s->cols[c], in, false, wait);
    if (rc != TM_OK) {
        const std::string msg = g_err;
        tm_colony_remove(s, c);
        g_err = msg;
        return rc;
    }
    *id = c;   // the captured step stays unless its launch shape changed (graph_shape_of)
    return TM_OK;
}

static int lookup(tm_session *s, int id)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    if (id < 0 || id >= (int)s->cols.size() || !s->cols[id].used) return tm_fail(TM_ENOENT, "no colony %d", id);
    return TM_OK;
}

static void drop_sample(tm_session *s);

extern "C" int tm_colony_remove(tm_session *s, int id)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    CK(cudaSetDevice(s->device));
    if (s->diag_col == id) drop_sample(s);
    colony_host &c = s->cols[id];
    s->h_desc[id].active = 0;
    s->h_desc[id].n = 0;
    rc = push_desc(s, id);
    if (rc) return rc;
    // freed slots point at the never-active entry, so no later colony that
    // reuses this entry sees them as its own.  Nothing waits: work queued
    // before (steps, the gathers of an asynchronous download) still sees the
    // colony, and a colony placed in the freed ranges later is written by
    // work queued after these kernels on the same stream.
    k_release_slots<<<blocks_for(c.nslots, 256), 256, 0, s->stream>>>(s->A.col, c.off, c.nslots,
                                                                       s->cfg.max_colonies);
    CK(cudaGetLastError());
    s->slots.release(c.off / 32, c.nslots / 32);
    s->bins.release(c.binoff, c.nbin);
    if (c.gridoff >= 0) s->grids.release(c.gridoff, c.ngrid);
    c = colony_host();
    while (!s->cols.empty() && !s->cols.back().used) s->cols.pop_back();
    return TM_OK;   // the captured step stays unless its launch shape changed (graph_shape_of)
}

extern "C" int tm_colony_upload(tm_session *s, int id, const tm_colony_input *in)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    rc = check_input(s, in, false);
    if (rc) return rc;
    colony_host &c = s->cols[id];
    if (in->n > c.nslots) return tm_fail(TM_EINVAL, "colony %d holds at most %d cells", id, c.nslots);
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const bool keep = in->n == c.n && c.n > 0;
    if (!keep) {
        c.n = (int)in->n;
        s->h_desc[id].n = c.n;
        rc = push_desc(s, id);
        if (rc) return rc;
        drop_graphs(s);
    }
    rc = copy_cells_in(s, c, in, keep);
    if (rc == TM_EDEVICE) {
        // a bad cell type: the colony is left empty
        c.n = 0;
        s->h_desc[id].n = 0;
        push_desc(s, id);
        drop_graphs(s);
    }
    return rc;
}

static int async_io_init(tm_session *s)
{
    if (s->h2d_stream) return TM_OK;
    int rc = download_streams(s);
    if (rc) return rc;
    CK(cudaStreamCreateWithFlags(&s->h2d_stream, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&s->ev_h2d, &s->ev_up_read, &s->ev_dl_gathered, &s->ev_dl_copied, &s->ev_dl_pos})
        CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (auto &axis : s->ev_dl_chunk)
        for (cudaEvent_t &e : axis) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t &e : s->ev_dl_part) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return TM_OK;
}

// Upload of the same cells (same n, same order) into the upload staging
// (44 B per slot, allocated on first use): the copies wait only until the
// previous asynchronous upload's kernel has read the staging, so they overlap
// the step before; the kernel that puts the cells into their slots follows on
// the session stream.
extern "C" int tm_colony_upload_async(tm_session *s, int id, const tm_colony_input *in)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!in || in->n < 0 || (in->n > 0 && (!in->x || !in->y || !in->z)))
        return tm_fail(TM_EINVAL, "bad colony input");
    colony_host &c = s->cols[id];
    const int fields = (in->size ? UP_SIZE : 0) | (in->young ? UP_YOUNG : 0) | (in->ctype ? UP_CTYPE : 0) |
                       (in->phase ? UP_PHASE : 0);
    if (in->n != c.n || c.n == 0) {
        if ((fields & UP_ALL) != UP_ALL)
            return tm_fail(TM_EINVAL, "an upload that changes the cell count carries every field");
        return tm_colony_upload(s, id, in);
    }
    CK(cudaSetDevice(s->device));
    if ((rc = async_io_init(s))) return rc;
    const size_t S = (size_t)s->slots.hwm * 32 + 32, need = S * 44;
    if (s->up_bytes < need) {
        CK(cudaStreamSynchronize(s->h2d_stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->up_stage) CK(cudaFree(s->up_stage));
        s->up_stage = nullptr;
        s->up_bytes = 0;
        CK(cudaMalloc((void **)&s->up_stage, need));
        s->up_bytes = need;
        s->up_pending = false;
    }
    double *X = (double *)s->up_stage, *Y = X + S, *Z = Y + S, *SZ = Z + S;
    float *YG = (float *)(SZ + S);
    int *CT = (int *)(YG + S), *PH = CT + S;
    const long long o = c.off;
    const size_t n = (size_t)in->n;
    cudaStream_t h = s->h2d_stream;
    if (s->up_pending) CK(cudaStreamWaitEvent(h, s->ev_up_read, 0));
    // each piece of each coordinate of the asynchronous download queued
    // before this upload reaches the host before the same piece is read here,
    // so a loop may pass the positions it received to this upload: a piece
    // travels up while the next ones still come down (pieces of a download of
    // another cell count: the whole coordinate first)
    double *dst3[3] = {X + o, Y + o, Z + o};
    const double *src3[3] = {in->x, in->y, in->z};
    const bool same_split = s->dl_pos_n == (long long)n;
    const int pieces = io_pieces((long long)n);
    for (int k = 0; k < 3; k++) {
        for (int j = 0; j < pieces; j++) {
            const long long lo = io_chunk_lo((long long)n, j), hi = io_chunk_lo((long long)n, j + 1);
            if (s->dl_pending) CK(cudaStreamWaitEvent(h, s->ev_dl_chunk[k][same_split ? j : IO_CHUNKS - 1], 0));
            if (hi > lo)
                CK(cudaMemcpyAsync(dst3[k] + lo, src3[k] + lo, (size_t)(hi - lo) * 8, cudaMemcpyHostToDevice, h));
        }
    }
    if (s->dl_pending) CK(cudaStreamWaitEvent(h, s->ev_dl_pos, 0));
    if (in->size) CK(cudaMemcpyAsync(SZ + o, in->size, n * 8, cudaMemcpyHostToDevice, h));
    if (in->young) CK(cudaMemcpyAsync(YG + o, in->young, n * 4, cudaMemcpyHostToDevice, h));
    if (in->ctype) CK(cudaMemcpyAsync(CT + o, in->ctype, n * 4, cudaMemcpyHostToDevice, h));
    if (in->phase) CK(cudaMemcpyAsync(PH + o, in->phase, n * 4, cudaMemcpyHostToDevice, h));
    CK(cudaEventRecord(s->ev_h2d, h));
    CK(cudaStreamWaitEvent(s->stream, s->ev_h2d, 0));
    const tm_arrays a = view(s, s->parity);
    const upload_src u = {X, Y, Z, SZ, YG, CT, PH, o};
    int4 *rec = nullptr;
    if ((rc = upload_records(s, &rec))) return rc;
    k_upload_pack<<<blocks_for((long long)n, 256), 256, 0, s->stream>>>(u, (int)n, fields, rec);
    CK(cudaGetLastError());
    CK(cudaEventRecord(s->ev_up_read, s->stream));   // the staging is free for the next upload's copies
    k_upload_keep<<<blocks_for((long long)n, 256), 256, 0, s->stream>>>(a, s->dK, id, o, (int)n, fields,
                                                                      nullptr, rec, o);
    CK(cudaGetLastError());
    s->up_pending = true;
    return TM_OK;
}

extern "C" int tm_colony_set_active(tm_session *s, int id, int active)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    s->cols[id].active = active ? 1 : 0;
    s->h_desc[id].active = active ? 1 : 0;
    rc = push_desc(s, id);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    drop_graphs(s);
    return TM_OK;
}

// ---------------------------------------------------------------------------
// tuning

__global__ void k_force_rebuild(tm_frame *frame, int ncol)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncol) frame[c].force_rebuild = 1;
}

extern "C" int tm_session_get_tuning(tm_session *s, tm_tuning *t)
{
    if (!s || !t) return tm_fail(TM_EINVAL, "null argument");
    *t = s->tune;
    return TM_OK;
}

extern "C" int tm_session_list_rate(tm_session *s, double *rate, int64_t *rebuilds)
{
    if (!s || !rate || !rebuilds) return tm_fail(TM_EINVAL, "null argument");
    CK(cudaSetDevice(s->device));
    const size_t nc = s->cols.size();
    if (nc) {
        CK(cudaMemcpyAsync(s->h_frame, s->A.frame, nc * sizeof(tm_frame), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    double num = 0.0, den = 0.0;
    long long total = 0;
    for (size_t c = 0; c < nc; c++) {
        const colony_host &ch = s->cols[c];
        if (!ch.used) continue;
        const tm_frame &f = s->h_frame[c];
        const tm_desc &d = s->h_desc[c];
        total += (long long)f.rebuilds;
        if (!ch.active || !d.verlet || ch.n < 2) continue;
        float md;
        memcpy(&md, &f.maxdisp, sizeof md);
        const double grow = 2.0 * (double)md / ((double)f.age + 1.0) / (double)d.skin;
        num += (double)ch.n * std::max(1.0 / (double)d.rmax, std::min(1.0, grow));
        den += (double)ch.n;
    }
    *rate = den > 0.0 ? num / den : 0.0;
    *rebuilds = total;
    return TM_OK;
}

extern "C" int tm_session_set_tuning(tm_session *s, const tm_tuning *t)
{
    if (!s || !t) return tm_fail(TM_EINVAL, "null argument");
    if (t->pair_lshift < 0 || t->pair_lshift > 1) return tm_fail(TM_EINVAL, "pair_lshift must be 0 or 1");
    if (t->list_variant < 1 || t->list_variant > 4) return tm_fail(TM_EINVAL, "list_variant must be 1..4");
    if (t->walk_block != 64 && t->walk_block != 128 && t->walk_block != 256)
        return tm_fail(TM_EINVAL, "walk_block must be 64, 128 or 256");
    if (!(t->skin_over_h > 0.0f && t->skin_over_h <= 1.0f)) return tm_fail(TM_EINVAL, "skin_over_h outside (0, 1]");
    if (t->rmax < 1) return tm_fail(TM_EINVAL, "rmax must be positive");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const bool lists_change = t->skin_over_h != s->tune.skin_over_h || t->rmax != s->tune.rmax;
    s->tune = *t;
    if (lists_change) {
        double hmax = 0.0;
        for (int k = 0; k < s->K.ntypes; k++) hmax = std::max(hmax, s->K.t[k].h);
        for (size_t c = 0; c < s->cols.size(); c++) {
            if (!s->cols[c].used) continue;
            s->h_desc[c].skin = (float)(t->skin_over_h * hmax);
            s->h_desc[c].rmax = t->rmax;
            int rc = push_desc(s, (int)c);
            if (rc) return rc;
        }
        if (!s->cols.empty()) {
            k_force_rebuild<<<blocks_for((long long)s->cols.size(), 128), 128, 0, s->stream>>>(s->A.frame,
                                                                                            (int)s->cols.size());
            CK(cudaGetLastError());
        }
        CK(cudaStreamSynchronize(s->stream));
    }
    drop_graphs(s);
    return TM_OK;
}

// ---------------------------------------------------------------------------
// stepping

static int run_step_graph(tm_session *s)
{
    int p = s->parity;
    long long shape[7];
    graph_shape_of(s, shape);
    if (s->graph_valid[p] && memcmp(shape, s->graph_shape[p], sizeof shape) != 0) drop_graphs(s);
    if (!s->graph_valid[p]) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(s);
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        if (rc) {
            if (e == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return tm_fail(TM_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&s->gexec[p], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return tm_fail(TM_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
        s->graph_valid[p] = true;
        memcpy(s->graph_shape[p], shape, sizeof shape);
    }
    CK(cudaGraphLaunch(s->gexec[p], s->stream));
    return TM_OK;
}

extern "C" int tm_session_step(tm_session *s, int nsteps)
{
    if (!s || nsteps < 0) return tm_fail(TM_EINVAL, "bad arguments");
    CK(cudaSetDevice(s->device));
    for (int k = 0; k < nsteps; k++) {
        int rc = (s->use_graph && !s->prof) ? run_step_graph(s) : enqueue_step(s);
        if (rc) return rc;
        s->launches += s->kernels_per_step;
        if (s->prof) s->prof_steps++;
    }
    return TM_OK;
}

extern "C" int tm_session_sync(tm_session *s)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    if (s->copy_stream) CK(cudaStreamSynchronize(s->copy_stream));
    if (s->h2d_stream) CK(cudaStreamSynchronize(s->h2d_stream));
    const int ncol = (int)s->cols.size();
    if (ncol == 0) return TM_OK;
    CK(cudaMemcpy(s->h_frame, s->A.frame, sizeof(tm_frame) * (size_t)ncol, cudaMemcpyDeviceToHost));
    for (int c = 0; c < ncol; c++) {
        if (!s->cols[c].used) continue;
        uint32_t e = s->h_frame[c].error;
        if (e)
            return tm_fail(TM_EDEVICE, "colony %d: device error 0x%x (%s%s%s%s)", c, e,
                           (e & TM_ERR_BIGBIN) ? "more than 2048 cells in one bin; " : "",
                           (e & TM_ERR_STACK) ? "octree walk too deep; " : "",
                           (e & TM_ERR_CODES) ? "coincident lattice codes; " : "",
                           (e & TM_ERR_TYPES) ? "cell type outside the table in an upload; " : "");
    }
    return TM_OK;
}

extern "C" int tm_session_use_graph(tm_session *s, int on)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    s->use_graph = on != 0;
    if (!on) drop_graphs(s);
    return TM_OK;
}

extern "C" int tm_session_set_diagnostics(tm_session *s, int on)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    if (on && !s->A.nbhash) {
        const long long S = ((s->cfg.max_slots + 31) / 32) * 32;
        if (dalloc(&s->A.nbhash, S) != TM_OK || dalloc(&s->A.vcand, S) != TM_OK)
            return tm_fail(TM_ENOMEM, "diagnostics arrays");
        CK(cudaMemsetAsync(s->A.nbhash, 0, (size_t)S * sizeof(unsigned long long), s->stream));
        CK(cudaMemsetAsync(s->A.vcand, 0xff, (size_t)S * sizeof(int), s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    s->A.want_diag = on ? 1 : 0;
    s->cfg.diagnostics = on ? 1 : 0;
    drop_graphs(s);
    return TM_OK;
}

static void drop_sample(tm_session *s)
{
    for (int **p : {&s->A.diag_row, &s->A.diag_cnt, &s->A.diag_nb})
        if (*p) {
            cudaFree(*p);
            *p = nullptr;
        }
    s->A.diag_lcap = 0;
    s->diag_col = -1;
    s->diag_ncells = 0;
}

extern "C" int tm_colony_sample_neighbours(tm_session *s, int id, const int64_t *cells, int64_t ncells, int lcap)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (ncells < 0 || (ncells > 0 && (!cells || lcap <= 0))) return tm_fail(TM_EINVAL, "bad sample");
    if (ncells > 0 && !s->A.want_diag) return tm_fail(TM_EINVAL, "sampled neighbour lists need diagnostics on");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    drop_sample(s);
    drop_graphs(s);
    if (ncells == 0) return TM_OK;
    const colony_host &c = s->cols[id];
    std::vector<int> rows((size_t)c.n, -1);
    for (int64_t k = 0; k < ncells; k++) {
        if (cells[k] < 0 || cells[k] >= c.n) return tm_fail(TM_EINVAL, "sampled cell %lld outside the colony",
                                                            (long long)cells[k]);
        rows[(size_t)cells[k]] = (int)k;
    }
    const long long S = ((s->cfg.max_slots + 31) / 32) * 32;
    if (dalloc(&s->A.diag_row, S) != TM_OK || dalloc(&s->A.diag_cnt, ncells) != TM_OK ||
        dalloc(&s->A.diag_nb, ncells * (long long)lcap) != TM_OK) {
        drop_sample(s);
        return tm_fail(TM_ENOMEM, "sampled neighbour lists");
    }
    CK(cudaMemset(s->A.diag_row, 0xff, (size_t)S * sizeof(int)));
    if (c.n > 0) CK(cudaMemcpy(s->A.diag_row + c.off, rows.data(), (size_t)c.n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(s->A.diag_cnt, 0, (size_t)ncells * sizeof(int)));
    s->A.diag_lcap = lcap;
    s->diag_col = id;
    s->diag_ncells = ncells;
    return TM_OK;
}

extern "C" int tm_colony_read_neighbours(tm_session *s, int id, int32_t *counts, int32_t *lists)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (s->diag_col != id || !counts) return tm_fail(TM_EINVAL, "no neighbour sample on this colony");
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(counts, s->A.diag_cnt, (size_t)s->diag_ncells * sizeof(int), cudaMemcpyDeviceToHost));
    if (lists)
        CK(cudaMemcpy(lists, s->A.diag_nb, (size_t)s->diag_ncells * (size_t)s->A.diag_lcap * sizeof(int),
                      cudaMemcpyDeviceToHost));
    return TM_OK;
}

#define TM_FENCES 64

extern "C" int tm_session_fence(tm_session *s, int64_t *fence)
{
    if (!s || !fence) return tm_fail(TM_EINVAL, "null argument");
    CK(cudaSetDevice(s->device));
    if (s->fence_ev.empty()) {
        s->fence_ev.resize(TM_FENCES, nullptr);
        for (auto &e : s->fence_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&s->fence_join, cudaEventDisableTiming));
    }
    cudaEvent_t e = s->fence_ev[(size_t)(s->fence_next % TM_FENCES)];
    if (s->copy_stream) {
        // the work queued so far on the session stream and on the copy stream
        CK(cudaEventRecord(s->fence_join, s->stream));
        CK(cudaStreamWaitEvent(s->copy_stream, s->fence_join, 0));
        CK(cudaEventRecord(e, s->copy_stream));
    } else {
        CK(cudaEventRecord(e, s->stream));
    }
    *fence = s->fence_next++;
    return TM_OK;
}

extern "C" int tm_session_wait(tm_session *s, int64_t fence)
{
    if (!s || fence < 0 || fence >= s->fence_next) return tm_fail(TM_EINVAL, "no such fence");
    CK(cudaSetDevice(s->device));
    // a fence older than the ring is covered by the newer record in its place
    CK(cudaEventSynchronize(s->fence_ev[(size_t)(fence % TM_FENCES)]));
    return TM_OK;
}

extern "C" int tm_session_profile(tm_session *s, int on)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaStreamSynchronize(s->stream));
    s->prof = on != 0;
    s->evused = 0;
    s->prof_steps = 0;
    return TM_OK;
}

extern "C" int tm_session_profile_read(tm_session *s, double *ms, int nphase, int64_t *steps)
{
    if (!s || !ms) return tm_fail(TM_EINVAL, "null argument");
    CK(cudaStreamSynchronize(s->stream));
    const int per = 8;   // marks per step
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    long long nst = (long long)(s->evused / per);
    for (long long k = 0; k < nst; k++) {
        for (int ph = 0; ph < 7; ph++) {
            float t = 0.0f;
            CK(cudaEventElapsedTime(&t, s->evpool[k * per + ph], s->evpool[k * per + ph + 1]));
            acc[ph] += t;
        }
    }
    // recording order: build, cic, search, list, fallback + fix, octree, update;
    // reported: build, search, list, fix, octree, update, cic
    const double order[7] = {acc[0], acc[2], acc[3], acc[4], acc[5], acc[6], acc[1]};
    for (int k = 0; k < nphase && k < 7; k++) ms[k] = nst ? order[k] / (double)nst : 0.0;
    if (steps) *steps = nst;
    return TM_OK;
}

extern "C" int tm_session_capacity(tm_session *s, int64_t *free_slots, int64_t *free_bins, int *free_colonies)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    if (free_slots) *free_slots = s->slots.free_total() * 32;
    if (free_bins) *free_bins = s->bins.free_total();
    if (free_colonies) {
        int used = 0;
        for (auto &c : s->cols) used += c.used ? 1 : 0;
        *free_colonies = s->cfg.max_colonies - used;
    }
    return TM_OK;
}

// ---------------------------------------------------------------------------
// downloads

template <typename T>
static int unsort_to_host(tm_session *s, const T *src, const colony_host &c, T *host)
{
    if (!host || c.n == 0) return TM_OK;
    // two device buffers: field k is gathered on the session stream into buffer
    // k % 2 while field k - 1 is copied to the host on the copy stream
    const int b = s->dl_next;
    s->dl_next ^= 1;
    const tm_arrays a = view(s, s->parity);
    T *tmp = (T *)(b ? s->d_scratch2 : s->d_scratch);
    CK(cudaStreamWaitEvent(s->stream, s->ev_copied[b], 0));     // buffer b is free again
    k_unsort<T><<<blocks_for(c.n, 256), 256, 0, s->stream>>>(src, a.perm, c.off, c.n, tmp);
    CK(cudaGetLastError());
    CK(cudaEventRecord(s->ev_ready[b], s->stream));
    CK(cudaStreamWaitEvent(s->copy_stream, s->ev_ready[b], 0));
    CK(cudaMemcpyAsync(host, tmp, sizeof(T) * (size_t)c.n, cudaMemcpyDeviceToHost, s->copy_stream));
    CK(cudaEventRecord(s->ev_copied[b], s->copy_stream));
    return TM_OK;
}

static int download_streams(tm_session *s)
{
    if (s->copy_stream) return TM_OK;
    CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) {
        CK(cudaEventCreateWithFlags(&s->ev_ready[k], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&s->ev_copied[k], cudaEventDisableTiming));
        CK(cudaEventRecord(s->ev_copied[k], s->copy_stream));
    }
    return TM_OK;
}

static int download_queue(tm_session *s, int id, const tm_colony_output *out, bool wait);

extern "C" int tm_colony_download(tm_session *s, int id, const tm_colony_output *out)
{
    return download_queue(s, id, out, true);
}

extern "C" int tm_colony_download_async(tm_session *s, int id, const tm_colony_output *out)
{
    return download_queue(s, id, out, false);
}

// Asynchronous download: each requested field is gathered into its own part
// of the download staging (8 B per slot per field, allocated on first use,
// the inverse permutation in the last part) on the session stream, then
// copied to the host on the copy stream, so the copies overlap the steps that
// follow; the next asynchronous download waits for these copies before it
// touches the staging.
#define DL_MAX_FIELDS 13

static int download_async_queue(tm_session *s, int id, const tm_colony_output *out)
{
    int rc = async_io_init(s);
    if (rc) return rc;
    const colony_host &c = s->cols[id];
    const tm_arrays a = view(s, s->parity);
    const size_t S = (size_t)s->slots.hwm * 32 + 32, need = S * 8 * (DL_MAX_FIELDS + 1);
    if (s->dl_bytes < need) {
        CK(cudaStreamSynchronize(s->copy_stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->dl_stage) CK(cudaFree(s->dl_stage));
        s->dl_stage = nullptr;
        s->dl_bytes = 0;
        CK(cudaMalloc((void **)&s->dl_stage, need));
        s->dl_bytes = need;
        s->dl_pending = false;
    }
    if (s->dl_pending) CK(cudaStreamWaitEvent(s->stream, s->ev_dl_copied, 0));
    struct want { const void *src; void *host; int size; };
    const want all[DL_MAX_FIELDS] = {
        {a.x, out->x, 8}, {a.y, out->y, 8}, {a.z, out->z, 8}, {a.density, out->density, 8}, {a.v, out->v, 8},
        {a.mindist, out->mindist, 8}, {a.fx, out->fx, 8}, {a.fy, out->fy, 8}, {a.fz, out->fz, 8},
        {a.rem, out->removecell, 1}, {a.nbcount, out->nbcount, 4},
        {a.nbhash, a.nbhash ? (void *)out->nbhash : nullptr, 8}, {a.vcand, a.vcand ? (void *)out->vcand : nullptr, 4}};
    std::vector<std::pair<void *, std::pair<const void *, size_t>>> copies;
    // the last of the positions asked for: a following asynchronous upload
    // waits for it to reach the host
    const void *last_pos = out->z ? (const void *)a.z : out->y ? (const void *)a.y : out->x ? (const void *)a.x
                                                                                              : nullptr;
    const void *pos3[3] = {a.x, a.y, a.z};
    bool axis_sent[3] = {out->x && c.n > 0, out->y && c.n > 0, out->z && c.n > 0};
    if (c.n > 0) {
        int *iperm = (int *)(s->dl_stage + (size_t)DL_MAX_FIELDS * S * 8);
        bool inverted = false;
        int part = 0;
        for (const want &w : all) {
            if (!w.host) continue;
            if (!inverted) {
                k_invert_perm<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.perm, c.off, c.n, iperm);
                inverted = true;
            }
            unsigned char *dst = s->dl_stage + (size_t)part++ * S * 8;
            const unsigned g = blocks_for(c.n, 256);
            if (w.size == 8)
                k_unsort_gather<unsigned long long><<<g, 256, 0, s->stream>>>(
                    (const unsigned long long *)w.src, iperm, c.off, c.n, (unsigned long long *)dst);
            else if (w.size == 4)
                k_unsort_gather<unsigned><<<g, 256, 0, s->stream>>>((const unsigned *)w.src, iperm, c.off, c.n,
                                                                   (unsigned *)dst);
            else
                k_unsort_gather<unsigned char><<<g, 256, 0, s->stream>>>((const unsigned char *)w.src, iperm, c.off,
                                                                        c.n, dst);
            // each field travels as soon as it is gathered, the positions first
            CK(cudaGetLastError());
            CK(cudaEventRecord(s->ev_dl_part[part - 1], s->stream));
            CK(cudaStreamWaitEvent(s->copy_stream, s->ev_dl_part[part - 1], 0));
            int axis = -1;
            for (int k = 0; k < 3; k++)
                if (w.src == pos3[k]) axis = k;
            if (axis < 0) {
                CK(cudaMemcpyAsync(w.host, dst, (size_t)w.size * (size_t)c.n, cudaMemcpyDeviceToHost,
                                   s->copy_stream));
            } else {
                // a coordinate in pieces, each announced to a following upload
                // (the last event marks the whole coordinate, for an upload of
                // another cell count)
                const int pieces = io_pieces(c.n);
                for (int j = 0; j < pieces; j++) {
                    const long long lo = io_chunk_lo(c.n, j), hi = io_chunk_lo(c.n, j + 1);
                    if (hi > lo)
                        CK(cudaMemcpyAsync((double *)w.host + lo, (const double *)dst + lo, (size_t)(hi - lo) * 8,
                                           cudaMemcpyDeviceToHost, s->copy_stream));
                    CK(cudaEventRecord(s->ev_dl_chunk[axis][j], s->copy_stream));
                }
                if (pieces < IO_CHUNKS) CK(cudaEventRecord(s->ev_dl_chunk[axis][IO_CHUNKS - 1], s->copy_stream));
            }
            copies.push_back({w.host, {(const void *)dst, (size_t)w.size * (size_t)c.n}});
            if (w.src == last_pos) CK(cudaEventRecord(s->ev_dl_pos, s->copy_stream));
        }
    }
    // the grid goes through staging of its own too: the next step clears and
    // deposits the session grid while this copy may still be running
    const bool want_grid = out->grid && c.gridoff >= 0 && c.ngrid > 0;
    if (want_grid) {
        const size_t gb = sizeof(double) * (size_t)c.ngrid;
        if (s->dl_grid_bytes < gb) {
            CK(cudaStreamSynchronize(s->copy_stream));
            if (s->dl_grid) CK(cudaFree(s->dl_grid));
            s->dl_grid = nullptr;
            s->dl_grid_bytes = 0;
            CK(cudaMalloc((void **)&s->dl_grid, gb));
            s->dl_grid_bytes = gb;
        }
        CK(cudaMemcpyAsync(s->dl_grid, a.grid + c.gridoff, gb, cudaMemcpyDeviceToDevice, s->stream));
    }
    CK(cudaEventRecord(s->ev_dl_gathered, s->stream));
    CK(cudaStreamWaitEvent(s->copy_stream, s->ev_dl_gathered, 0));
    const int npos = (out->x ? 1 : 0) + (out->y ? 1 : 0) + (out->z ? 1 : 0);
    if (npos == 0 || copies.empty()) CK(cudaEventRecord(s->ev_dl_pos, s->copy_stream));
    for (int k = 0; k < 3; k++)
        if (!axis_sent[k]) {
            for (int j = 0; j < io_pieces(c.n); j++) CK(cudaEventRecord(s->ev_dl_chunk[k][j], s->copy_stream));
            CK(cudaEventRecord(s->ev_dl_chunk[k][IO_CHUNKS - 1], s->copy_stream));
        }
    s->dl_pos_n = c.n;
    if (want_grid)
        CK(cudaMemcpyAsync(out->grid, s->dl_grid, sizeof(double) * (size_t)c.ngrid, cudaMemcpyDeviceToHost,
                           s->copy_stream));
    CK(cudaEventRecord(s->ev_dl_copied, s->copy_stream));
    s->dl_pending = true;
    return TM_OK;
}

static int download_queue(tm_session *s, int id, const tm_colony_output *out, bool wait)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!out) return tm_fail(TM_EINVAL, "null output");
    if (!wait) {
        CK(cudaSetDevice(s->device));
        return download_async_queue(s, id, out);
    }
    CK(cudaSetDevice(s->device));
    if ((rc = download_streams(s))) return rc;
    const colony_host &c = s->cols[id];
    const tm_arrays a = view(s, s->parity);
    if ((rc = unsort_to_host(s, (const double *)a.x, c, out->x))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.y, c, out->y))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.z, c, out->z))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.density, c, out->density))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.v, c, out->v))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.mindist, c, out->mindist))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.fx, c, out->fx))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.fy, c, out->fy))) return rc;
    if ((rc = unsort_to_host(s, (const double *)a.fz, c, out->fz))) return rc;
    if ((rc = unsort_to_host(s, (const unsigned char *)a.rem, c, out->removecell))) return rc;
    if ((rc = unsort_to_host(s, (const int32_t *)a.nbcount, c, out->nbcount))) return rc;
    if (a.nbhash && (rc = unsort_to_host(s, (const unsigned long long *)a.nbhash, c,
                                         (unsigned long long *)out->nbhash)))
        return rc;
    if (a.vcand && (rc = unsort_to_host(s, (const int32_t *)a.vcand, c, out->vcand))) return rc;
    if (out->grid && c.gridoff >= 0) {
        CK(cudaEventRecord(s->ev_ready[0], s->stream));
        CK(cudaStreamWaitEvent(s->copy_stream, s->ev_ready[0], 0));
        CK(cudaMemcpyAsync(out->grid, a.grid + c.gridoff, sizeof(double) * (size_t)c.ngrid, cudaMemcpyDeviceToHost,
                           s->copy_stream));
        CK(cudaEventRecord(s->ev_copied[0], s->copy_stream));
    }
    if (wait) {
        // the caller may read its buffers on return
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaStreamSynchronize(s->copy_stream));
    }
    return TM_OK;
}

extern "C" int tm_colony_stats(tm_session *s, int id, tm_colony_info *st)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!st) return tm_fail(TM_EINVAL, "null output");
    CK(cudaSetDevice(s->device));
    const colony_host &c = s->cols[id];
    const tm_arrays a = view(s, s->parity);
    CK(cudaMemsetAsync(s->d_octsize + id, 0, sizeof(unsigned long long), s->stream));
    k_octsize<<<blocks_for(a.nslots_total, 256), 256, 0, s->stream>>>(a, s->d_octsize);
    CK(cudaGetLastError());
    unsigned long long octs = 0;
    CK(cudaMemcpyAsync(&octs, s->d_octsize + id, sizeof octs, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&s->h_frame[id], &a.frame[id], sizeof(tm_frame), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const tm_frame &f = s->h_frame[id];
    memset(st, 0, sizeof *st);
    for (int k = 0; k < 3; k++) st->aff_shift[k] = f.shift[k];
    st->aff_scale = f.scale;
    st->octsize = c.n >= 2 ? (int64_t)(1 + octs) : (int64_t)c.n;
    st->removecount = (int64_t)f.removecount;
    for (int k = 0; k < 3; k++) {
        st->patch_lower[k] = f.patch_lo[k];
        st->patch_upper[k] = f.patch_hi[k];
        st->grid_size[k] = c.gsize[k];
    }
    if (s->K.dim == 2) {
        st->patch_lower[2] = 0;
        st->patch_upper[2] = 0;
    }
    st->device_errors = f.error;
    st->bin_level = f.L;
    st->n = c.n;
    st->list_rebuilds = (int64_t)f.rebuilds;
    st->codes_slow = (int64_t)f.codes_slow;
    st->density_fp64_cells = (int64_t)f.fix64;
    st->walked_cells = (int64_t)f.walks;
    st->walked_isolated_cells = (int64_t)f.walks_isolated;
    memcpy(&st->list_maxdisp, &f.maxdisp, sizeof(float));   // stored as the float's bits
    st->list_skin = s->h_desc[id].skin;
    st->list_age = f.age;
    return TM_OK;
}

extern "C" int tm_session_timer(tm_session *s, int op, double *ms)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaSetDevice(s->device));
    if (!s->tstart) CK(cudaEventCreate(&s->tstart));
    if (!s->tstop) CK(cudaEventCreate(&s->tstop));
    if (op == 0) {
        CK(cudaEventRecord(s->tstart, s->stream));
        return TM_OK;
    }
    CK(cudaEventRecord(s->tstop, s->stream));
    CK(cudaEventSynchronize(s->tstop));
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, s->tstart, s->tstop));
    if (ms) *ms = t;
    return TM_OK;
}

extern "C" int64_t tm_session_launches(tm_session *s) { return s ? (int64_t)s->launches : 0; }

extern "C" int tm_host_register(void *ptr, int64_t bytes)
{
    if (!ptr || bytes <= 0) return tm_fail(TM_EINVAL, "bad host range");
    CK(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
    return TM_OK;
}

extern "C" int tm_host_unregister(void *ptr)
{
    if (!ptr) return tm_fail(TM_EINVAL, "null pointer");
    CK(cudaHostUnregister(ptr));
    return TM_OK;
}

// ---------------------------------------------------------------------------
// internal entry points for the reference-signature drop-ins

#include "tm_dropin_api.h"

struct tm_stage {
    void *ptr = nullptr;
    long long bytes = 0;
};
static tm_stage g_stage;   // one staging buffer per process (the drop-ins use one session)

extern "C" int tmi_reserve_stage(tm_session *s, int64_t bytes)
{
    if (bytes <= g_stage.bytes) return TM_OK;
    CK(cudaSetDevice(s->device));
    if (g_stage.ptr) CK(cudaFree(g_stage.ptr));
    g_stage.ptr = nullptr;
    g_stage.bytes = 0;
    CK(cudaMalloc(&g_stage.ptr, (size_t)bytes));
    g_stage.bytes = bytes;
    return TM_OK;
}

__global__ void k_unpack_aos(const unsigned char *aos, tmi_aos_layout lay, long long n, tm_arrays a, long long off)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned char *c = aos + k * lay.stride;
    const long long i = off + k;
    a.x[i] = *(const double *)(c + lay.x);
    a.y[i] = *(const double *)(c + lay.y);
    a.z[i] = *(const double *)(c + lay.z);
    a.size[i] = *(const double *)(c + lay.size);
    a.young[i] = *(const float *)(c + lay.young);
    a.ctype[i] = *(const int *)(c + lay.ctype);
    a.phase[i] = lay.phase >= 0 ? *(const int *)(c + lay.phase) : 1;
    a.perm[i] = (int)k;
}

__global__ void k_max_ctype(const int *ctype, long long off, long long n, int *out)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int v = k < n ? ctype[off + k] : -1;
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v >= 0) atomicMax(out, v);
}

__global__ void k_unsort3(const double *s0, const double *s1, const double *s2, const int *perm, long long off,
                          long long n, double *dst)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long c = perm[off + k];
    dst[3 * c] = s0[off + k];
    dst[3 * c + 1] = s1[off + k];
    dst[3 * c + 2] = s2[off + k];
}

__global__ void k_sort3(const double *src, const int *perm, long long off, long long n, double *d0, double *d1,
                        double *d2)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long c = perm[off + k];
    d0[off + k] = src[3 * c];
    d1[off + k] = src[3 * c + 1];
    d2[off + k] = src[3 * c + 2];
}

__global__ void k_sort_u8(const unsigned char *src, const int *perm, long long off, long long n, unsigned char *dst)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[off + k] = src[perm[off + k]];
}

__global__ void k_read_box(const double *grid, int gy, int gz, long long lx, long long ly, long long lz,
                           long long sx, long long sy, long long sz, double *dst)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= sx * sy * sz) return;
    const long long i = k / (sy * sz), j = (k / sz) % sy, l = k % sz;
    dst[k] = grid[((lx + i) * gy + (ly + j)) * gz + (lz + l)];
}

extern "C" int tmi_set_types(tm_session *s, const tm_celltypes *types)
{
    if (!s || !types || types->ntypes < 1 || types->ntypes > TM_MAX_TYPES) return tm_fail(TM_EINVAL, "bad types");
    if (types->ntypes > s->mass_types) {
        // the per-type density weights need one slot array per type
        CK(cudaStreamSynchronize(s->stream));
        double *m = nullptr;
        CK(cudaMalloc((void **)&m, sizeof(double) * (size_t)(s->slots.cap * 32) * (size_t)types->ntypes));
        CK(cudaFree(s->A.mass));
        s->A.mass = m;
        s->mass_types = types->ntypes;
        drop_graphs(s);
    }
    tm_consts &K = s->K;
    K.ntypes = types->ntypes;
    for (int t = 0; t < K.ntypes; t++) {
        tm_type &T = K.t[t];
        T.h = types->h[t];
        T.h2 = types->h2[t];
        T.h3 = types->h3[t];
        T.h4 = types->h4[t];
        T.csize = types->size[t];
        T.sc = K.dim == 2 ? T.h2 : T.h3;
        T.cW = host_type_const(K.dim, 0, T.h, T.h2, T.h3, T.h4);
        T.cG = host_type_const(K.dim, 1, T.h, T.h2, T.h3, T.h4);
        T.e = T.h + 0.01;
        T.h_fx = std::fabs(T.h) < 8192.0 ? (long long)std::ldexp(T.h, 47) : 0;
        T.randommove = types->randommove ? types->randommove[t] : 0.0f;
        T.hf = (float)T.h;
        T.h2f = (float)(T.h * T.h);
        T.inv_hf = (float)(1.0 / T.h);
        T.cWf = (float)T.cW;
        T.cGf = (float)T.cG;
        T.kmassf = (float)(T.sc / T.csize);
        T.inv_h = 1.0 / T.h;
        T.h2cut = cutoff_sq(T.h);
        T.kmass = T.sc / T.csize;
        T.thr_lo = (float)(T.h * (1.0 - 1e-5) * T.h * (1.0 - 1e-5));
        T.thr_hi = (float)(T.h * (1.0 + 1e-5) * T.h * (1.0 + 1e-5));
    }
    CK(cudaMemcpyAsync(s->dK, &s->K, sizeof(tm_consts), cudaMemcpyHostToDevice, s->stream));
    return TM_OK;
}

extern "C" int tmi_set_dimension(tm_session *s, int dim)
{
    if (!s || (dim != 2 && dim != 3)) return tm_fail(TM_EINVAL, "bad dimension");
    if (s->K.dim == dim) return TM_OK;
    s->K.dim = dim;
    CK(cudaMemcpyAsync(s->dK, &s->K, sizeof(tm_consts), cudaMemcpyHostToDevice, s->stream));
    return TM_OK;
}

extern "C" int tmi_upload_aos(tm_session *s, int cid, const void *cells, int64_t n, const tmi_aos_layout *lay)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    colony_host &c = s->cols[cid];
    if (n > c.nslots) return tm_fail(TM_EINVAL, "colony %d holds at most %d cells", cid, c.nslots);
    CK(cudaSetDevice(s->device));
    if ((rc = tmi_reserve_stage(s, std::max<int64_t>(n * lay->stride, 8)))) return rc;
    if (n > 0)
        CK(cudaMemcpyAsync(g_stage.ptr, cells, (size_t)(n * lay->stride), cudaMemcpyHostToDevice, s->stream));
    const tm_arrays a = view(s, s->parity);
    if (n > 0)
        k_unpack_aos<<<blocks_for(n, 256), 256, 0, s->stream>>>((const unsigned char *)g_stage.ptr, *lay, n, a, c.off);
    // outputs and marks as after an upload
    c.n = (int)n;
    s->h_desc[cid].n = c.n;
    if ((rc = push_desc(s, cid))) return rc;
    k_colony_init<<<blocks_for(c.nslots, 256), 256, 0, s->stream>>>(a, cid, c.off, (int)n, c.nslots, 1);
    CK(cudaGetLastError());
    drop_graphs(s);
    return TM_OK;
}

// caller-order AoS cells (device staging) -> upload records (caller order)
__global__ void k_aos_to_rec(const unsigned char *aos, tmi_aos_layout lay, long long n, int4 *rec, long long base)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned char *c = aos + k * lay.stride;
    up_rec r;
    r.f.x = *(const double *)(c + lay.x);
    r.f.y = *(const double *)(c + lay.y);
    r.f.z = *(const double *)(c + lay.z);
    r.f.size = *(const double *)(c + lay.size);
    r.f.young = *(const float *)(c + lay.young);
    r.f.ctype = *(const int *)(c + lay.ctype);
    r.f.phase = lay.phase >= 0 ? *(const int *)(c + lay.phase) : 1;
    r.f.pad = 0;
    int4 *d = rec + (base + k) * 3;
    d[0] = r.v[0];
    d[1] = r.v[1];
    d[2] = r.v[2];
}

// The same cells in the same caller order as the colony holds: they keep
// their slots (tm_colony_upload's rule), so neighbour lists stay valid unless
// a cell moved too far or changed size or type.
extern "C" int tmi_upload_aos_keep(tm_session *s, int cid, const void *cells, int64_t n, const tmi_aos_layout *lay)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    colony_host &c = s->cols[cid];
    if (n != c.n || n == 0) return tmi_upload_aos(s, cid, cells, n, lay);
    CK(cudaSetDevice(s->device));
    if ((rc = tmi_reserve_stage(s, std::max<int64_t>(n * lay->stride, 8)))) return rc;
    CK(cudaMemcpyAsync(g_stage.ptr, cells, (size_t)(n * lay->stride), cudaMemcpyHostToDevice, s->stream));
    int4 *rec = nullptr;
    if ((rc = upload_records(s, &rec))) return rc;
    const tm_arrays a = view(s, s->parity);
    k_aos_to_rec<<<blocks_for(n, 256), 256, 0, s->stream>>>((const unsigned char *)g_stage.ptr, *lay, n, rec, c.off);
    k_upload_keep<<<blocks_for(n, 256), 256, 0, s->stream>>>(a, s->dK, cid, c.off, (int)n,
                                                            UP_ALL | (lay->phase >= 0 ? UP_PHASE : 0),
                                                            nullptr, rec, c.off);
    CK(cudaGetLastError());
    return TM_OK;
}

extern "C" int tmi_max_ctype(tm_session *s, int cid, int *maxtype)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    const tm_arrays a = view(s, s->parity);
    int *d = (int *)s->d_scratch;
    CK(cudaMemsetAsync(d, 0, sizeof(int), s->stream));
    if (c.n > 0) k_max_ctype<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.ctype, c.off, c.n, d);
    CK(cudaMemcpyAsync(maxtype, d, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

extern "C" int tmi_phase(tm_session *s, int which)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaSetDevice(s->device));
    int nk = 0, rc = TM_OK;
    switch (which) {
    case 0: rc = enqueue_build(s, s->parity, nk); break;
    case 1: rc = enqueue_compute(s, nk, false); break;
    case 2: rc = enqueue_update(s, nk); break;
    case 3: rc = enqueue_cic(s, nk); break;
    default: return tm_fail(TM_EINVAL, "bad phase");
    }
    s->launches += nk;
    return rc;
}

// Three doubles of every caller record written by the device straight into
// page-locked host records (rec: the records' device address, off: the first
// of the three doubles in a record): a thread per record, in caller order, so
// a warp writes 32 consecutive records; the values are gathered from their
// slots through the inverse permutation.  A strided DMA copy of 24 of every
// 112 bytes ran at about a tenth of the link's rate.
__global__ void k_write_aos3(const double *s0, const double *s1, const double *s2, const int *iperm, long long soff,
                             long long n, unsigned char *rec, long long stride, long long off)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long s = soff + iperm[k];
    double *d = (double *)(rec + k * stride + off);
    d[0] = s0[s];
    d[1] = s1[s];
    d[2] = s2[s];
}

extern "C" int tmi_download_aos3(tm_session *s, int cid, void *cells, int64_t stride, int64_t off, int which,
                                 int pinned)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.n == 0) return TM_OK;
    const tm_arrays a = view(s, s->parity);
    double *tmp = (double *)g_stage.ptr;
    if ((rc = tmi_reserve_stage(s, (int64_t)c.n * 24))) return rc;
    tmp = (double *)g_stage.ptr;
    // records the device can write (page-locked, 8-byte aligned fields): the
    // kernel writes them; otherwise a gather and a strided copy
    void *drec = nullptr;
    if (pinned && ((uintptr_t)cells | (uintptr_t)stride | (uintptr_t)off) % 8 == 0) {
        CK(cudaHostGetDevicePointer(&drec, cells, 0));
        int *iperm = (int *)tmp;
        k_invert_perm<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.perm, c.off, c.n, iperm);
        const double *f0 = which == 0 ? a.v : a.x, *f1 = which == 0 ? a.density : a.y,
                     *f2 = which == 0 ? a.mindist : a.z;
        k_write_aos3<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(f0, f1, f2, iperm, c.off, c.n,
                                                                  (unsigned char *)drec, stride, off);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s->stream));
        return TM_OK;
    }
    if (which == 0) k_unsort3<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.v, a.density, a.mindist, a.perm, c.off, c.n, tmp);
    else k_unsort3<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.x, a.y, a.z, a.perm, c.off, c.n, tmp);
    CK(cudaGetLastError());
    CK(cudaMemcpy2DAsync((char *)cells + off, (size_t)stride, tmp, 24, 24, (size_t)c.n, cudaMemcpyDeviceToHost,
                         s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

extern "C" int tmi_download_forces(tm_session *s, int cid, double *f3)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.n == 0) return TM_OK;
    const tm_arrays a = view(s, s->parity);
    if ((rc = tmi_reserve_stage(s, (int64_t)c.n * 24))) return rc;
    double *tmp = (double *)g_stage.ptr;
    k_unsort3<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.fx, a.fy, a.fz, a.perm, c.off, c.n, tmp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(f3, tmp, (size_t)c.n * 24, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

extern "C" int tmi_upload_forces(tm_session *s, int cid, const double *f3)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.n == 0) return TM_OK;
    const tm_arrays a = view(s, s->parity);
    if ((rc = tmi_reserve_stage(s, (int64_t)c.n * 24))) return rc;
    double *tmp = (double *)g_stage.ptr;
    CK(cudaMemcpyAsync(tmp, f3, (size_t)c.n * 24, cudaMemcpyHostToDevice, s->stream));
    k_sort3<<<blocks_for(c.n, 256), 256, 0, s->stream>>>(tmp, a.perm, c.off, c.n, a.fx, a.fy, a.fz);
    CK(cudaGetLastError());
    return TM_OK;
}

extern "C" int tmi_upload_removecell(tm_session *s, int cid, const unsigned char *rem)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.n == 0) return TM_OK;
    const tm_arrays a = view(s, s->parity);
    if ((rc = tmi_reserve_stage(s, (int64_t)c.n))) return rc;
    CK(cudaMemcpyAsync(g_stage.ptr, rem, (size_t)c.n, cudaMemcpyHostToDevice, s->stream));
    k_sort_u8<<<blocks_for(c.n, 256), 256, 0, s->stream>>>((const unsigned char *)g_stage.ptr, a.perm, c.off, c.n,
                                                           a.rem);
    CK(cudaGetLastError());
    // the update adds to removecount: count this step's marks only
    CK(cudaMemsetAsync(&s->A.frame[cid].removecount, 0, sizeof(unsigned long long), s->stream));
    return TM_OK;
}

extern "C" int tmi_download_removecell(tm_session *s, int cid, unsigned char *rem, int64_t *newly_marked)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    const tm_arrays a = view(s, s->parity);
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, &s->A.frame[cid].removecount, sizeof cnt, cudaMemcpyDeviceToHost, s->stream));
    if (c.n > 0) {
        if ((rc = tmi_reserve_stage(s, (int64_t)c.n))) return rc;
        k_unsort<unsigned char><<<blocks_for(c.n, 256), 256, 0, s->stream>>>(a.rem, a.perm, c.off, c.n,
                                                                             (unsigned char *)g_stage.ptr);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(rem, g_stage.ptr, (size_t)c.n, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    if (newly_marked) *newly_marked = (int64_t)cnt;
    return TM_OK;
}

extern "C" int tmi_set_update(tm_session *s, int cid, int mode, double dt)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    s->cols[cid].opt.update_mode = mode;
    s->cols[cid].opt.dt = dt;
    s->h_desc[cid].update_mode = mode;
    s->h_desc[cid].dt = dt;
    return push_desc(s, cid);
}

extern "C" int tmi_set_cic(tm_session *s, int cid, const double lower[3], float res, const int64_t gsize[3])
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    colony_host &c = s->cols[cid];
    const long long ng = gsize[0] * gsize[1] * gsize[2];
    if (ng <= 0) return tm_fail(TM_EINVAL, "empty grid");
    if (c.gridoff < 0 || c.ngrid != ng) {
        if (c.gridoff >= 0) s->grids.release(c.gridoff, c.ngrid);
        c.gridoff = -1;
        if (!s->grids.alloc(ng, c.gridoff)) return tm_fail(TM_ENOMEM, "no room for a %lld-node grid", ng);
        c.ngrid = ng;
    }
    for (int k = 0; k < 3; k++) c.gsize[k] = (int)gsize[k];
    c.opt.cic = 1;
    c.opt.gfh = res;
    tm_desc &d = s->h_desc[cid];
    d.gridoff = c.gridoff;
    d.gres = res;
    for (int k = 0; k < 3; k++) {
        d.glower[k] = lower[k];
        d.gsize[k] = (int)gsize[k];
    }
    drop_graphs(s);
    return push_desc(s, cid);
}

extern "C" int tmi_patch_box(tm_session *s, int cid, int64_t lo[3], int64_t hi[3])
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    CK(cudaMemcpyAsync(&s->h_frame[cid], &s->A.frame[cid], sizeof(tm_frame), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < 3; k++) {
        lo[k] = s->h_frame[cid].patch_lo[k];
        hi[k] = s->h_frame[cid].patch_hi[k];
    }
    if (s->K.dim == 2) {
        lo[2] = 0;
        hi[2] = 0;
    }
    return TM_OK;
}

extern "C" int tmi_read_patch(tm_session *s, int cid, const int64_t lo[3], const int64_t hi[3], double *dst)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.gridoff < 0) return tm_fail(TM_EINVAL, "colony %d has no grid", cid);
    long long sz[3];
    for (int k = 0; k < 3; k++) {
        sz[k] = hi[k] - lo[k] + 1;
        if (lo[k] < 0 || sz[k] <= 0 || hi[k] >= c.gsize[k]) return tm_fail(TM_EINVAL, "patch outside the grid");
    }
    const long long tot = sz[0] * sz[1] * sz[2];
    if ((rc = tmi_reserve_stage(s, tot * 8))) return rc;
    k_read_box<<<blocks_for(tot, 256), 256, 0, s->stream>>>(s->A.grid + c.gridoff, c.gsize[1], c.gsize[2], lo[0],
                                                            lo[1], lo[2], sz[0], sz[1], sz[2],
                                                            (double *)g_stage.ptr);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst, g_stage.ptr, (size_t)tot * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

// ---------------------------------------------------------------------------
// grid -> cell gather and field gradient (tm_field.cu) for session colonies
// and the drop-ins

static int env_reserve(tm_session *s, size_t bytes)
{
    if (bytes <= s->env_bytes) return TM_OK;
    if (s->env_buf) CK(cudaFree(s->env_buf));
    s->env_buf = nullptr;
    s->env_bytes = 0;
    CK(cudaMalloc((void **)&s->env_buf, bytes));
    s->env_bytes = bytes;
    return TM_OK;
}

extern "C" int tm_colony_env2cells(tm_session *s, int id, const double lower[3], float resolution,
                                   const int64_t gsize[3], int nfields, const double *data, const double *gradient,
                                   double *cellenv)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!lower || !gsize || !data || !gradient || !cellenv || nfields < 1 || !(resolution > 0.0f))
        return tm_fail(TM_EINVAL, "bad gather arguments");
    if (gsize[0] < 1 || gsize[1] < 1 || gsize[2] < 1 || (s->K.dim == 2 && gsize[2] != 1))
        return tm_fail(TM_EINVAL, "bad grid size");
    const colony_host &c = s->cols[id];
    if (c.n == 0) return TM_OK;
    CK(cudaSetDevice(s->device));
    const size_t bytes = (size_t)nfields * (size_t)c.n * 4 * sizeof(double);
    if ((rc = env_reserve(s, bytes))) return rc;
    const int64_t hi[3] = {gsize[0] - 1, gsize[1] - 1, s->K.dim == 3 ? gsize[2] - 1 : 0};
    const int64_t lo[3] = {0, 0, 0};
    const tm_envgeom g = tm_make_envgeom(lower, resolution, hi, lo, gsize, nfields);
    CK(tm_launch_env2cells_colony(g, view(s, s->parity), c.off, c.n, data, gradient, s->env_buf, s->stream));
    CK(cudaMemcpyAsync(cellenv, s->env_buf, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

// drop-in patches_applyenv2cells: the host patch (fields, then gradients, the
// reference's buffer layout) is staged on the device and gathered for the
// colony's cells; cellenv[f] receives n cellenvdata_t of field f
extern "C" int tmi_env2cells_patch(tm_session *s, int cid, const double *patch, int nfields, const int64_t box_lo[3],
                                   const int64_t box_size[3], const double lower[3], float resolution,
                                   const int64_t grid_hi[3], double **cellenv)
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    const colony_host &c = s->cols[cid];
    if (c.n == 0 || nfields < 1) return TM_OK;
    CK(cudaSetDevice(s->device));
    const int64_t vol = box_size[0] * box_size[1] * box_size[2];
    const size_t pbytes = (size_t)(4 * (int64_t)nfields * vol) * sizeof(double);
    const size_t obytes = (size_t)nfields * (size_t)c.n * 4 * sizeof(double);
    if ((rc = tmi_reserve_stage(s, (int64_t)pbytes))) return rc;
    if ((rc = env_reserve(s, obytes))) return rc;
    CK(cudaMemcpyAsync(g_stage.ptr, patch, pbytes, cudaMemcpyHostToDevice, s->stream));
    const double *dd = (const double *)g_stage.ptr;
    const tm_envgeom g = tm_make_envgeom(lower, resolution, grid_hi, box_lo, box_size, nfields);
    CK(tm_launch_env2cells_colony(g, view(s, s->parity), c.off, c.n, dd, dd + (size_t)nfields * (size_t)vol,
                                  s->env_buf, s->stream));
    for (int f = 0; f < nfields; f++)
        CK(cudaMemcpyAsync(cellenv[f], s->env_buf + (size_t)f * (size_t)c.n * 4, (size_t)c.n * 4 * sizeof(double),
                           cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

// drop-in fieldgradient: one field, host data in, host gradient out
extern "C" int tmi_field_gradient_host(tm_session *s, const double *data, const int64_t gsize[3], float resolution,
                                       double *gradient)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    CK(cudaSetDevice(s->device));
    const int64_t G = gsize[0] * gsize[1] * gsize[2];
    if (G <= 0) return TM_OK;
    int rc = tmi_reserve_stage(s, 4 * G * (int64_t)sizeof(double));
    if (rc) return rc;
    double *dd = (double *)g_stage.ptr;
    CK(cudaMemcpyAsync(dd, data, (size_t)G * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    const tm_envgeom g = tm_make_envgeom(nullptr, resolution, nullptr, nullptr, gsize, 1);
    CK(tm_launch_field_gradient(g, gsize, dd, dd + G, s->stream));
    CK(cudaMemcpyAsync(gradient, dd + G, (size_t)(3 * G) * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

// ---------------------------------------------------------------------------
// VTK file of a colony (writevtk, io.c:372-516, at one rank)

extern "C" int tm_colony_write_vtk(tm_session *s, int id, const char *path, int rank)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!path) return tm_fail(TM_EINVAL, "null path");
    const colony_host &c = s->cols[id];
    const long long n = c.n;
    // the text of io.c:397-497, in the same order; n stands for globalcount.n
    char num[64];
    std::string img;
    tm_vtk_layout L;
    img += "# vtk DataFile Version 2.0\nTimothy output\nBINARY\nDATASET UNSTRUCTURED_GRID";
    snprintf(num, sizeof num, "\nPOINTS %lld float\n", n);
    img += num;
    L.points = (long long)img.size();
    img.append((size_t)(12 * n), '\0');
    snprintf(num, sizeof num, "\nCELL_TYPES %lld\n", n);
    img += num;
    L.celltypes = (long long)img.size();
    img.append((size_t)(4 * n), '\0');
    snprintf(num, sizeof num, "\nPOINT_DATA %lld", n);
    img += num;
    img += "\nSCALARS rank integer 1\nLOOKUP_TABLE default\n";
    L.ranks = (long long)img.size();
    img.append((size_t)(4 * n), '\0');
    img += "\nSCALARS type integer 1\nLOOKUP_TABLE default\n";
    L.types = (long long)img.size();
    img.append((size_t)(4 * n), '\0');
    img += "\nSCALARS density float 1\nLOOKUP_TABLE default\n";
    L.density = (long long)img.size();
    img.append((size_t)(4 * n), '\0');
    img += "\nVECTORS force float\n";
    L.forces = (long long)img.size();
    img.append((size_t)(12 * n), '\0');
    if (n > 0) {
        CK(cudaSetDevice(s->device));
        if ((rc = env_reserve(s, img.size()))) return rc;
        unsigned char *dimg = (unsigned char *)s->env_buf;
        CK(cudaMemcpyAsync(dimg, img.data(), img.size(), cudaMemcpyHostToDevice, s->stream));
        CK(tm_launch_vtk_pack(view(s, s->parity), c.off, n, rank, L, dimg, s->stream));
        CK(cudaMemcpyAsync(&img[0], dimg, img.size(), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    FILE *f = fopen(path, "wb");
    if (!f) return tm_fail(TM_EINVAL, "cannot open %s for writing", path);
    const size_t w = fwrite(img.data(), 1, img.size(), f);
    const int cl = fclose(f);
    if (w != img.size() || cl != 0) return tm_fail(TM_EINVAL, "writing %s failed", path);
    return TM_OK;
}

// ---------------------------------------------------------------------------
// death compaction and appends (cellsdeath, cells.c:290-336, and the
// appends of mitosis, cells.c:124-205, for resident colonies)

// keep flags in caller order and in slot order
__global__ void k_keep_flags(tm_arrays a, long long off, int n, uint32_t *keep_caller, uint32_t *keep_slot)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
    if (k == n) {                              // one past the end: the scans' totals
        keep_caller[n] = 0;
        keep_slot[n] = 0;
        return;
    }
    const uint32_t keep = a.rem[off + k] ? 0u : 1u;
    keep_caller[a.perm[off + k]] = keep;
    keep_slot[k] = keep;
}

// survivors move to their compacted slot (scratch copies), with their new
// caller index; every per-cell field moves with the cell
__global__ void k_compact_gather(tm_arrays a, long long off, int n, const uint32_t *new_caller,
                                 const uint32_t *new_slot, double *ob)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long s = off + k;
    if (a.rem[s]) return;
    const long long d = off + new_slot[k];
    a.x2[d] = a.x[s];
    a.y2[d] = a.y[s];
    a.z2[d] = a.z[s];
    a.size2[d] = a.size[s];
    a.young2[d] = a.young[s];
    a.ctype2[d] = a.ctype[s];
    a.phase2[d] = a.phase[s];
    a.perm2[d] = (int)new_caller[a.perm[s]];
    a.rem2[d] = 0;
    // outputs, 7 values per cell, into ob (slot-indexed from off)
    const long long o = (long long)new_slot[k] * 7;
    ob[o + 0] = a.density[s];
    ob[o + 1] = a.v[s];
    ob[o + 2] = a.mindist[s];
    ob[o + 3] = a.fx[s];
    ob[o + 4] = a.fy[s];
    ob[o + 5] = a.fz[s];
    ob[o + 6] = (double)a.nbcount[s];
}

__global__ void k_compact_scatter(tm_arrays a, long long off, int m, const double *ob)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const long long s = off + k;
    a.x[s] = a.x2[s];
    a.y[s] = a.y2[s];
    a.z[s] = a.z2[s];
    a.size[s] = a.size2[s];
    a.young[s] = a.young2[s];
    a.ctype[s] = a.ctype2[s];
    a.phase[s] = a.phase2[s];
    a.perm[s] = a.perm2[s];
    a.rem[s] = 0;
    const double *o = ob + k * 7;
    a.density[s] = o[0];
    a.v[s] = o[1];
    a.mindist[s] = o[2];
    a.fx[s] = o[3];
    a.fy[s] = o[4];
    a.fz[s] = o[5];
    a.nbcount[s] = (int)o[6];
}

// cell-cycle state (caller-indexed) of the survivors, 6 words each, via scratch
__global__ void k_compact_cycle_gather(tm_arrays a, long long off, int n, const uint32_t *keep_caller,
                                       const uint32_t *new_caller, double *scratch)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || !keep_caller[c]) return;
    float *w = (float *)scratch + (long long)new_caller[c] * 6;
    const long long i = off + c;
    w[0] = a.cy_pt[i];
    w[1] = a.cy_g1[i];
    w[2] = a.cy_s[i];
    w[3] = a.cy_g2[i];
    w[4] = a.cy_m[i];
    w[5] = __int_as_float(a.cy_age[i]);
}

__global__ void k_compact_cycle_scatter(tm_arrays a, long long off, int m, const double *scratch)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    const float *w = (const float *)scratch + c * 6;
    const long long i = off + c;
    a.cy_pt[i] = w[0];
    a.cy_g1[i] = w[1];
    a.cy_s[i] = w[2];
    a.cy_g2[i] = w[3];
    a.cy_m[i] = w[4];
    a.cy_age[i] = __float_as_int(w[5]);
}

__global__ void k_append_cols(int *col, long long first, int m, int c)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) col[first + k] = c;
}

__global__ void k_force_rebuild_one(tm_frame *frame, int c)
{
    frame[c].force_rebuild = 1;   // slots changed: the lists are rebuilt at the next step
    frame[c].list_ok = 0;
}

extern "C" int tm_colony_compact(tm_session *s, int id, int64_t *removed)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    colony_host &c = s->cols[id];
    if (removed) *removed = 0;
    // cells.c:294: with a single cell in the simulation nothing is removed
    if (c.n <= 1) return TM_OK;
    CK(cudaSetDevice(s->device));
    const tm_arrays a = view(s, s->parity);
    const int n = c.n;
    uint32_t *keep_caller = (uint32_t *)s->d_scratch;          // n + 1 words
    uint32_t *new_caller = keep_caller + (n + 1);               // n + 1 words (d_scratch holds 2 S words)
    uint32_t *keep_slot = (uint32_t *)s->d_scratch2;
    uint32_t *new_slot = keep_slot + (n + 1);
    if ((rc = env_reserve(s, (size_t)n * 7 * sizeof(double)))) return rc;
    cudaStream_t st = s->stream;
    k_keep_flags<<<blocks_for(n + 1, 256), 256, 0, st>>>(a, c.off, n, keep_caller, keep_slot);
    CK(cudaGetLastError());
    CK(tm_scan_exclusive(keep_caller, new_caller, n + 1, s->scan_tmp_slots, st));
    CK(tm_scan_exclusive(keep_slot, new_slot, n + 1, s->scan_tmp_slots, st));
    uint32_t survivors = 0;
    CK(cudaMemcpyAsync(&survivors, new_slot + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((int)survivors == n) return TM_OK;
    k_compact_gather<<<blocks_for(n, 256), 256, 0, st>>>(a, c.off, n, new_caller, new_slot, s->env_buf);
    k_compact_scatter<<<blocks_for(survivors, 256), 256, 0, st>>>(a, c.off, (int)survivors, s->env_buf);
    k_force_rebuild_one<<<1, 1, 0, st>>>(a.frame, id);
    CK(cudaGetLastError());
    if (a.cy_pt) {
        // cell-cycle state follows the caller indices (after the outputs: env_buf is reused)
        k_compact_cycle_gather<<<blocks_for(n, 256), 256, 0, st>>>(a, c.off, n, keep_caller, new_caller, s->env_buf);
        k_compact_cycle_scatter<<<blocks_for(survivors, 256), 256, 0, st>>>(a, c.off, (int)survivors,
                                                                          s->env_buf);
        CK(cudaGetLastError());
    }
    c.n = (int)survivors;
    s->h_desc[id].n = c.n;
    if ((rc = push_desc(s, id))) return rc;
    CK(cudaStreamSynchronize(st));
    drop_graphs(s);
    if (removed) *removed = n - (int)survivors;
    return TM_OK;
}

__global__ void k_append_init(tm_arrays a, long long off, int n0, int m, int has_phase, const tm_consts *K, int *bad)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const long long s = off + n0 + k;
    a.perm[s] = n0 + (int)k;
    a.rem[s] = 0;
    if (!has_phase) a.phase[s] = 1;
    const int ct = a.ctype[s];
    if (ct < 0 || ct >= K->ntypes) {
        atomicExch(bad, 1);
        a.ctype[s] = 0;
    }
    a.density[s] = 0.0;
    a.v[s] = 0.0;
    a.mindist[s] = 0.0;
    a.fx[s] = 0.0;
    a.fy[s] = 0.0;
    a.fz[s] = 0.0;
    a.nbcount[s] = 0;
    a.nbmin[s] = -1;
}

extern "C" int tm_colony_append(tm_session *s, int id, const tm_colony_input *in)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    rc = check_input(s, in, false);
    if (rc) return rc;
    colony_host &c = s->cols[id];
    const long long m = in->n;
    if (m == 0) return TM_OK;
    if (c.n + m > c.nslots)
        return tm_fail(TM_ENOMEM, "colony %d holds %d slots; %d cells plus %lld appended do not fit", id, c.nslots,
                       c.n, m);
    CK(cudaSetDevice(s->device));
    const tm_arrays a = view(s, s->parity);
    cudaStream_t st = s->stream;
    const long long o = c.off + c.n;
    const size_t n = (size_t)m;
    CK(cudaMemsetAsync(s->d_flag, 0, sizeof(int), st));
    CK(cudaMemcpyAsync(a.x + o, in->x, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a.y + o, in->y, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a.z + o, in->z, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a.size + o, in->size, n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a.young + o, in->young, n * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(a.ctype + o, in->ctype, n * 4, cudaMemcpyHostToDevice, st));
    if (in->phase) CK(cudaMemcpyAsync(a.phase + o, in->phase, n * 4, cudaMemcpyHostToDevice, st));
    k_append_init<<<blocks_for(m, 256), 256, 0, st>>>(a, c.off, c.n, (int)m, in->phase ? 1 : 0, s->dK, s->d_flag);
    if (a.cy_pt) {
        const long long o2 = c.off + c.n;
        CK(cudaMemsetAsync(a.cy_pt + o2, 0, n * 4, st));
        CK(cudaMemsetAsync(a.cy_g1 + o2, 0, n * 4, st));
        CK(cudaMemsetAsync(a.cy_s + o2, 0, n * 4, st));
        CK(cudaMemsetAsync(a.cy_g2 + o2, 0, n * 4, st));
        CK(cudaMemsetAsync(a.cy_m + o2, 0, n * 4, st));
        CK(cudaMemsetAsync(a.cy_age + o2, 0, n * 4, st));
    }
    k_force_rebuild_one<<<1, 1, 0, st>>>(a.frame, id);
    CK(cudaGetLastError());
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c.n += (int)m;
    s->h_desc[id].n = c.n;
    if ((rc = push_desc(s, id))) return rc;
    CK(cudaStreamSynchronize(st));
    drop_graphs(s);
    if (bad) return tm_fail(TM_EDEVICE, "an appended cell type lies outside 0..%d (set to 0)", s->K.ntypes - 1);
    return TM_OK;
}

// ---------------------------------------------------------------------------
// cell cycle (tm_cycle.cu)

#define TM_CYCLE_MAX_FIELDS 16

static int cycle_alloc(tm_session *s)
{
    if (s->A.cy_pt) return TM_OK;
    const long long S = ((s->cfg.max_slots + 31) / 32) * 32;
    tm_arrays &a = s->A;
    int rc = TM_OK;
    if (rc == TM_OK) rc = dalloc(&a.cy_pt, S);
    if (rc == TM_OK) rc = dalloc(&a.cy_g1, S);
    if (rc == TM_OK) rc = dalloc(&a.cy_s, S);
    if (rc == TM_OK) rc = dalloc(&a.cy_g2, S);
    if (rc == TM_OK) rc = dalloc(&a.cy_m, S);
    if (rc == TM_OK) rc = dalloc(&a.cy_age, S);
    const size_t pbytes = sizeof(tm_cycle_type) * TM_MAX_TYPES + 2 * sizeof(float) * TM_MAX_TYPES * TM_CYCLE_MAX_FIELDS +
                          sizeof(double) * TM_MAX_TYPES;
    if (rc == TM_OK) rc = dalloc((unsigned char **)&s->cy_params, (long long)pbytes);
    if (rc == TM_OK) rc = dalloc(&s->cy_marked, 1);
    if (rc == TM_OK) {
        // on the session stream: it does not wait for the legacy default stream
        CK(cudaMemsetAsync(a.cy_pt, 0, S * 4, s->stream));
        CK(cudaMemsetAsync(a.cy_g1, 0, S * 4, s->stream));
        CK(cudaMemsetAsync(a.cy_s, 0, S * 4, s->stream));
        CK(cudaMemsetAsync(a.cy_g2, 0, S * 4, s->stream));
        CK(cudaMemsetAsync(a.cy_m, 0, S * 4, s->stream));
        CK(cudaMemsetAsync(a.cy_age, 0, S * 4, s->stream));
    }
    drop_graphs(s);
    return rc;
}

extern "C" int tm_colony_set_cycle(tm_session *s, int id, const float *phasetime, const float *g1,
                                   const float *sphase, const float *g2, const float *m, const int *age)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!phasetime || !g1 || !sphase || !g2 || !m || !age) return tm_fail(TM_EINVAL, "null cycle array");
    CK(cudaSetDevice(s->device));
    if ((rc = cycle_alloc(s))) return rc;
    const colony_host &c = s->cols[id];
    const size_t b = (size_t)c.n * 4;
    const tm_arrays &a = s->A;
    if (b) {
        CK(cudaMemcpyAsync(a.cy_pt + c.off, phasetime, b, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(a.cy_g1 + c.off, g1, b, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(a.cy_s + c.off, sphase, b, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(a.cy_g2 + c.off, g2, b, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(a.cy_m + c.off, m, b, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(a.cy_age + c.off, age, b, cudaMemcpyHostToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return TM_OK;
}

extern "C" int tm_colony_get_cycle(tm_session *s, int id, float *phasetime, float *g1, float *sphase, float *g2,
                                   float *m, int *age, int *phase, double *size, float *young)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    CK(cudaSetDevice(s->device));
    const colony_host &c = s->cols[id];
    const size_t b = (size_t)c.n * 4;
    const tm_arrays &a = s->A;
    CK(cudaStreamSynchronize(s->stream));
    if (b && a.cy_pt) {
        float *fl[5] = {phasetime, g1, sphase, g2, m};
        const float *src[5] = {a.cy_pt, a.cy_g1, a.cy_s, a.cy_g2, a.cy_m};
        for (int k = 0; k < 5; k++)
            if (fl[k]) CK(cudaMemcpyAsync(fl[k], src[k] + c.off, b, cudaMemcpyDeviceToHost, s->stream));
        if (age) CK(cudaMemcpyAsync(age, a.cy_age + c.off, b, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if ((rc = download_streams(s))) return rc;
    if (phase && (rc = unsort_to_host(s, (const int32_t *)a.phase, c, (int32_t *)phase))) return rc;
    if (size && (rc = unsort_to_host(s, (const double *)a.size, c, size))) return rc;
    if (young && (rc = unsort_to_host(s, (const float *)a.young, c, young))) return rc;
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaStreamSynchronize(s->copy_stream));
    return TM_OK;
}

extern "C" int tm_colony_cellcycle(tm_session *s, int id, const tm_cycle_params *p, int64_t *divided, int64_t *marked)
{
    int rc = lookup(s, id);
    if (rc) return rc;
    if (!p || !p->types) return tm_fail(TM_EINVAL, "null cycle parameters");
    if (p->nfields < 0 || p->nfields > TM_CYCLE_MAX_FIELDS) return tm_fail(TM_EINVAL, "nfields must be 0..%d",
                                                                         TM_CYCLE_MAX_FIELDS);
    if (p->nfields > 0 && (!p->cellenv || !p->criticallevel1 || !p->criticallevel2))
        return tm_fail(TM_EINVAL, "fields need cellenv and critical levels");
    colony_host &c = s->cols[id];
    if (divided) *divided = 0;
    if (marked) *marked = 0;
    const long long n = c.n;
    if (n == 0) return TM_OK;
    CK(cudaSetDevice(s->device));
    if ((rc = cycle_alloc(s))) return rc;
    const int nt = s->K.ntypes, nf = p->nfields;
    // parameters to the device
    std::vector<unsigned char> hp(sizeof(tm_cycle_type) * TM_MAX_TYPES + 2 * sizeof(float) * TM_MAX_TYPES *
                                  TM_CYCLE_MAX_FIELDS + sizeof(double) * TM_MAX_TYPES, 0);
    tm_cycle_type *ht = (tm_cycle_type *)hp.data();
    float *hc1 = (float *)(ht + TM_MAX_TYPES), *hc2 = hc1 + TM_MAX_TYPES * TM_CYCLE_MAX_FIELDS;
    double *hcs = (double *)(hc2 + TM_MAX_TYPES * TM_CYCLE_MAX_FIELDS);
    for (int t = 0; t < nt; t++) {
        ht[t] = p->types[t];
        hcs[t] = s->K.t[t].csize;
        for (int f = 0; f < nf; f++) {
            hc1[t * nf + f] = p->criticallevel1[t * nf + f];
            hc2[t * nf + f] = p->criticallevel2[t * nf + f];
        }
    }
    cudaStream_t st = s->stream;
    CK(cudaMemcpyAsync(s->cy_params, hp.data(), hp.size(), cudaMemcpyHostToDevice, st));
    tm_cycle_dev P;
    P.types = (const tm_cycle_type *)s->cy_params;
    P.cl1 = (const float *)(P.types + TM_MAX_TYPES);
    P.cl2 = P.cl1 + TM_MAX_TYPES * TM_CYCLE_MAX_FIELDS;
    P.csize = (const double *)(P.cl2 + TM_MAX_TYPES * TM_CYCLE_MAX_FIELDS);
    P.cellenv = p->cellenv;
    P.off = c.off;
    P.nfields = nf;
    P.simulationstart = p->simulationstart;
    P.sps = p->secondsperstep;
    P.shrink = std::pow(2.0, -(1.0 / 3.0));
    const tm_arrays a = view(s, s->parity);
    // pass 1: draws and divisions per cell, in the caller's order; their scans
    uint32_t *draws = (uint32_t *)s->d_scratch, *draw_off = draws + (n + 1);
    uint32_t *divs = (uint32_t *)s->d_scratch2, *div_off = divs + (n + 1);
    CK(tm_launch_cycle_count(P, a, c.off, n, s->K.dim, draws, divs, st));
    CK(tm_scan_exclusive(draws, draw_off, n + 1, s->scan_tmp_slots, st));
    CK(tm_scan_exclusive(divs, div_off, n + 1, s->scan_tmp_slots, st));
    uint32_t tot[2] = {0, 0};
    CK(cudaMemcpyAsync(&tot[0], draw_off + n, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tot[1], div_off + n, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (n + (long long)tot[1] > c.nslots)
        return tm_fail(TM_ENOMEM, "colony %d: %lld cells and %u daughters exceed its %d slots", id, n, tot[1],
                       c.nslots);
    // the random values, in the reference's order
    const size_t nd = tot[0] > 0 ? tot[0] : 1;
    if (s->cy_stream_cap < nd) {
        if (s->cy_stream) CK(cudaFree(s->cy_stream));
        s->cy_stream = nullptr;
        s->cy_stream_cap = 0;
        if ((rc = dalloc(&s->cy_stream, (long long)nd))) return rc;
        s->cy_stream_cap = nd;
    }
    std::vector<int> hs;
    if (p->rand_seeded && p->rand_offset) {
        // the C library's stream after srand(rand_seed), generated on the device
        const int64_t chunks = ((int64_t)tot[0] + TM_RAND_CHUNK - 1) / TM_RAND_CHUNK + 1;
        if (s->rand_windows_cap < chunks) {
            if (s->rand_windows) CK(cudaFree(s->rand_windows));
            s->rand_windows = nullptr;
            s->rand_windows_cap = 0;
            if ((rc = dalloc(&s->rand_windows, chunks * 31))) return rc;
            s->rand_windows_cap = chunks;
        }
        if (tm_libc_rand_device(p->rand_seed, *p->rand_offset, (int64_t)tot[0], s->cy_stream, &s->rand_cache,
                                s->rand_windows, s->rand_windows_cap, st) != 0)
            return tm_fail(TM_ECUDA, "device rand() stream failed");
        *p->rand_offset += (int64_t)tot[0];
    } else {
        hs.resize(nd);
        for (uint32_t k = 0; k < tot[0]; k++) hs[k] = p->draw ? p->draw(p->draw_ctx) : rand();
        CK(cudaMemcpyAsync(s->cy_stream, hs.data(), hs.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemsetAsync(s->cy_marked, 0, sizeof(unsigned long long), st));
    // pass 2: the transitions
    // the per-cell division counts are spent: their array takes the list of dividing cells
    CK(tm_launch_cycle_apply(P, a, c.off, n, s->K.dim, draw_off, div_off, s->cy_stream, s->cy_marked, divs,
                             (long long)tot[1], st));
    unsigned long long mk = 0;
    CK(cudaMemcpyAsync(&mk, s->cy_marked, sizeof mk, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (tot[1] > 0) {
        // daughters joined the colony: their slots need the colony's entry, the lists a rebuild
        k_append_cols<<<blocks_for(tot[1], 256), 256, 0, st>>>(s->A.col, c.off + n, (int)tot[1], id);
        k_force_rebuild_one<<<1, 1, 0, st>>>(a.frame, id);
        CK(cudaGetLastError());
        c.n += (int)tot[1];
        s->h_desc[id].n = c.n;
        if ((rc = push_desc(s, id))) return rc;
        CK(cudaStreamSynchronize(st));
        drop_graphs(s);
    }
    if (divided) *divided = tot[1];
    if (marked) *marked = (int64_t)mk;
    return TM_OK;
}

// ---------------------------------------------------------------------------
// drop-in helpers for cellsupdate (cells.c:525-543): the random move's draws,
// the cell cycle and the death compaction on the host's celldata_t records

extern "C" int tmi_set_move_draws(tm_session *s, const int *draws, int64_t count)
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    if (!draws || count <= 0) {
        if (s->A.move_draws) drop_graphs(s);
        s->A.move_draws = nullptr;
        return TM_OK;
    }
    CK(cudaSetDevice(s->device));
    if (s->move_cap < (size_t)count) {
        if (s->move_buf) CK(cudaFree(s->move_buf));
        s->move_buf = nullptr;
        s->move_cap = 0;
        int rc = dalloc(&s->move_buf, count);
        if (rc) return rc;
        s->move_cap = (size_t)count;
    }
    CK(cudaMemcpyAsync(s->move_buf, draws, (size_t)count * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    s->A.move_draws = s->move_buf;
    drop_graphs(s);
    return TM_OK;
}

// The random move's draws generated on the device: count values of the C
// library's stream from the window w (31 words, oldest first); end receives
// the window after them.
extern "C" int tmi_set_move_draws_window(tm_session *s, const uint32_t w[31], int64_t count, uint32_t end[31])
{
    if (!s || !w || !end || count <= 0) return tm_fail(TM_EINVAL, "bad arguments");
    CK(cudaSetDevice(s->device));
    if (s->move_cap < (size_t)count) {
        if (s->move_buf) CK(cudaFree(s->move_buf));
        s->move_buf = nullptr;
        s->move_cap = 0;
        int rc = dalloc(&s->move_buf, count);
        if (rc) return rc;
        s->move_cap = (size_t)count;
    }
    const int64_t chunks = (count + TM_RAND_CHUNK - 1) / TM_RAND_CHUNK + 1;
    if (s->rand_windows_cap < chunks) {
        if (s->rand_windows) CK(cudaFree(s->rand_windows));
        s->rand_windows = nullptr;
        s->rand_windows_cap = 0;
        int rc = dalloc(&s->rand_windows, chunks * 31);
        if (rc) return rc;
        s->rand_windows_cap = chunks;
    }
    if (tm_libc_rand_from_window(w, count, s->move_buf, end, s->rand_windows, s->rand_windows_cap, s->stream) != 0)
        return tm_fail(TM_ECUDA, "device rand() stream failed");
    s->A.move_draws = s->move_buf;
    drop_graphs(s);
    return TM_OK;
}

// celldata_t byte offsets (global.h:100-120, 112-byte records)
#define CD_PHASE 4
#define CD_AGE 8
#define CD_DEATH 12
#define CD_PT 16
#define CD_G1 20
#define CD_S 24
#define CD_G2 28
#define CD_M 32
#define CD_YOUNG 36
#define CD_GID 40
#define CD_X 48
#define CD_Y 56
#define CD_Z 64
#define CD_SIZE 72
#define CD_V 80
#define CD_DENSITY 88
#define CD_CTYPE 104
#define CD_BYTES 112

template <typename T>
__device__ __forceinline__ T &cd_field(unsigned char *rec, int off)
{
    return *(T *)(rec + off);
}

// records (caller order, identity slots after an upload) -> the cycle's inputs
__global__ void k_cycle_from_aos(const unsigned char *aos, long long n, tm_arrays a, long long off)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned char *r = (unsigned char *)aos + k * CD_BYTES;
    const long long i = off + k;
    a.density[i] = cd_field<double>(r, CD_DENSITY);
    a.cy_pt[i] = cd_field<float>(r, CD_PT);
    a.cy_g1[i] = cd_field<float>(r, CD_G1);
    a.cy_s[i] = cd_field<float>(r, CD_S);
    a.cy_g2[i] = cd_field<float>(r, CD_G2);
    a.cy_m[i] = cd_field<float>(r, CD_M);
    a.cy_age[i] = cd_field<int>(r, CD_AGE);
}

// the cycle's results into the records (cells keep every other field;
// daughters get the fields mitosis sets, cells.c:156-205).  cnt[0..5] gets
// the change of the phase counters (a cell leaving a phase takes one off it,
// the phase it enters gets one), cnt[8 + t] the daughters of type t.
__global__ void k_cycle_to_aos(unsigned char *aos, long long n, long long total, tm_arrays a, long long off,
                               unsigned long long *cnt)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total) return;
    const long long s = off + k;                  // identity order: slot = caller index
    unsigned char *r = aos + k * CD_BYTES;
    const int ph = a.phase[s];
    if (k >= n) {
        cd_field<int>(r, CD_GID) = (int)k;        // rank * maxlocalcells + index at one rank
        cd_field<double>(r, CD_V) = 0.0;
        cd_field<int>(r, CD_DEATH) = 0;
        cd_field<double>(r, CD_DENSITY) = a.density[s];
        cd_field<int>(r, CD_CTYPE) = a.ctype[s];
        atomicAdd(&cnt[8 + a.ctype[s]], 1ull);
    } else {
        const int old = cd_field<int>(r, CD_PHASE);
        if (old != ph) {
            if (old >= 0 && old < 6) atomicAdd(&cnt[old], ~0ull);    // -1
            if (ph >= 0 && ph < 6) atomicAdd(&cnt[ph], 1ull);
        }
    }
    cd_field<int>(r, CD_PHASE) = ph;
    cd_field<int>(r, CD_AGE) = a.cy_age[s];
    cd_field<float>(r, CD_PT) = a.cy_pt[s];
    cd_field<float>(r, CD_G1) = a.cy_g1[s];
    cd_field<float>(r, CD_S) = a.cy_s[s];
    cd_field<float>(r, CD_G2) = a.cy_g2[s];
    cd_field<float>(r, CD_M) = a.cy_m[s];
    cd_field<float>(r, CD_YOUNG) = a.young[s];
    cd_field<double>(r, CD_X) = a.x[s];
    cd_field<double>(r, CD_Y) = a.y[s];
    cd_field<double>(r, CD_Z) = a.z[s];
    cd_field<double>(r, CD_SIZE) = a.size[s];
}

__global__ void k_rem_out(const tm_arrays a, long long off, long long n, unsigned char *out)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = a.rem[off + k];
}

static int64_t round256(int64_t b) { return (b + 255) & ~(int64_t)255; }

// updatecellcycles on the host's records: cells[0, n) in, cells[0, *nout)
// out (the caller's array holds cap records); removecell (n entries) in and
// out.  The cell types' cycle parameters and levels are in p, the fields'
// values in cellenv[f][c] (host, cellenvdata_t layout).
extern "C" int tmi_cycle_aos(tm_session *s, int cid, void *cells, int64_t n, int64_t cap, const tm_cycle_params *p,
                             double *const *cellenv, unsigned char *removecell, int64_t *marked, int64_t *nout,
                             int64_t counts[8 + TM_MAX_TYPES])
{
    int rc = lookup(s, cid);
    if (rc) return rc;
    *nout = n;
    *marked = 0;
    for (int k = 0; k < 8 + TM_MAX_TYPES; k++) counts[k] = 0;
    if (n == 0) return TM_OK;
    CK(cudaSetDevice(s->device));
    if ((rc = cycle_alloc(s))) return rc;
    colony_host &c = s->cols[cid];
    if (cap > c.nslots) cap = c.nslots;
    const tm_arrays a = view(s, s->parity);
    // the marks first: their upload passes through the staging buffer the records use next
    if ((rc = tmi_upload_removecell(s, cid, removecell))) return rc;
    // the records' cycle inputs (the positions, sizes, types and phases came with tmi_upload_aos)
    const int64_t cnt_at = round256(cap * CD_BYTES + cap);
    if ((rc = tmi_reserve_stage(s, cnt_at + 8 * (8 + TM_MAX_TYPES)))) return rc;
    unsigned char *st = (unsigned char *)g_stage.ptr, *rem_dev = st + cap * CD_BYTES;
    unsigned long long *cnt = (unsigned long long *)(st + cnt_at);
    CK(cudaMemsetAsync(cnt, 0, 8 * (8 + TM_MAX_TYPES), s->stream));
    CK(cudaMemcpyAsync(st, cells, (size_t)(n * CD_BYTES), cudaMemcpyHostToDevice, s->stream));
    k_cycle_from_aos<<<blocks_for(n, 256), 256, 0, s->stream>>>(st, n, a, c.off);
    CK(cudaGetLastError());
    tm_cycle_params q = *p;
    if (p->nfields > 0) {
        if ((rc = env_reserve(s, (size_t)p->nfields * (size_t)n * 4 * sizeof(double)))) return rc;
        for (int f = 0; f < p->nfields; f++)
            CK(cudaMemcpyAsync(s->env_buf + (size_t)f * (size_t)n * 4, cellenv[f], (size_t)n * 4 * sizeof(double),
                               cudaMemcpyHostToDevice, s->stream));
        q.cellenv = s->env_buf;
    }
    int64_t div = 0;
    if ((rc = tm_colony_cellcycle(s, cid, &q, &div, marked))) return rc;
    const long long total = n + div;
    if (total > cap) return tm_fail(TM_ENOMEM, "too many local cells after mitosis");
    const tm_arrays b = view(s, s->parity);
    // the daughters' records keep the bytes mitosis does not set (lifetime, mindist)
    if (div > 0)
        CK(cudaMemcpyAsync(st + n * CD_BYTES, (const unsigned char *)cells + n * CD_BYTES, (size_t)(div * CD_BYTES),
                           cudaMemcpyHostToDevice, s->stream));
    k_cycle_to_aos<<<blocks_for(total, 256), 256, 0, s->stream>>>(st, n, total, b, c.off, cnt);
    k_rem_out<<<blocks_for(n, 256), 256, 0, s->stream>>>(b, c.off, n, rem_dev);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cells, st, (size_t)(total * CD_BYTES), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(removecell, rem_dev, (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(counts, cnt, 8 * (8 + TM_MAX_TYPES), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *nout = total;
    return TM_OK;
}

__global__ void k_keep_records(const unsigned char *rem, const unsigned char *aos, long long oldlnc, long long n,
                               uint32_t *keep, unsigned long long *removed)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > n) return;
    if (k == n || k >= oldlnc) {
        keep[k] = k == n ? 0u : 1u;
        return;
    }
    keep[k] = rem[k] ? 0u : 1u;
    if (rem[k]) {
        // the counters a removed cell leaves (cells.c:308-333): its phase's, if 0..4, and its type's
        const unsigned char *r = aos + k * CD_BYTES;
        const int t = *(const int *)(r + CD_CTYPE), ph = *(const int *)(r + CD_PHASE);
        if (t >= 0 && t < TM_MAX_TYPES) atomicAdd(&removed[t * 8 + (ph >= 0 && ph < 5 ? ph : 7)], 1ull);
    }
}

__global__ void k_move_records(const unsigned char *src, const uint32_t *keep, const uint32_t *dst_idx, long long n,
                               unsigned char *dst)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || !keep[k]) return;
    const uint4 *s4 = (const uint4 *)(src + k * CD_BYTES);
    uint4 *d4 = (uint4 *)(dst + (long long)dst_idx[k] * CD_BYTES);
    for (int w = 0; w < CD_BYTES / 16; w++) d4[w] = s4[w];
}

// cellsdeath (cells.c:290-336) on the host's records: the unmarked cells
// before oldlnc, then every cell from oldlnc on, in order; *nout = count;
// removed[t * 8 + p] = removed cells of type t in phase p (p = 7: phase 5)
extern "C" int tmi_compact_aos(tm_session *s, void *cells, int64_t n, int64_t oldlnc, const unsigned char *removecell,
                               int64_t *nout, int64_t removed[8 * TM_MAX_TYPES])
{
    if (!s) return tm_fail(TM_EINVAL, "null session");
    *nout = n;
    for (int k = 0; k < 8 * TM_MAX_TYPES; k++) removed[k] = 0;
    if (n == 0) return TM_OK;
    if (oldlnc > n) oldlnc = n;
    if (n + 1 > s->cfg.max_slots + 1) return tm_fail(TM_EINVAL, "more records than the session's slots");
    CK(cudaSetDevice(s->device));
    const int64_t rb = n * CD_BYTES, cnt_at = round256(2 * rb + oldlnc);
    int rc = tmi_reserve_stage(s, cnt_at + 8 * 8 * TM_MAX_TYPES);
    if (rc) return rc;
    unsigned char *src = (unsigned char *)g_stage.ptr, *dst = src + rb, *rem = dst + rb;
    unsigned long long *cnt = (unsigned long long *)(src + cnt_at);
    uint32_t *keep = (uint32_t *)s->d_scratch, *idx = keep + (n + 1);
    CK(cudaMemsetAsync(cnt, 0, 8 * 8 * TM_MAX_TYPES, s->stream));
    CK(cudaMemcpyAsync(src, cells, (size_t)rb, cudaMemcpyHostToDevice, s->stream));
    if (oldlnc > 0) CK(cudaMemcpyAsync(rem, removecell, (size_t)oldlnc, cudaMemcpyHostToDevice, s->stream));
    k_keep_records<<<blocks_for(n + 1, 256), 256, 0, s->stream>>>(rem, src, oldlnc, n, keep, cnt);
    CK(cudaGetLastError());
    CK(tm_scan_exclusive(keep, idx, n + 1, s->scan_tmp_slots, s->stream));
    uint32_t m = 0;
    CK(cudaMemcpyAsync(&m, idx + n, 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(removed, cnt, 8 * 8 * TM_MAX_TYPES, cudaMemcpyDeviceToHost, s->stream));
    k_move_records<<<blocks_for(n, 256), 256, 0, s->stream>>>(src, keep, idx, n, dst);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    if (m > 0) CK(cudaMemcpyAsync(cells, dst, (size_t)m * CD_BYTES, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *nout = m;
    return TM_OK;
}
