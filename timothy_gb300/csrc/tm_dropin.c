/* Reference-signature drop-ins (include/timothy_refabi.h) on top of one
 * device-resident colony.
 *
 * Flow of one reference step (main.c:67-79, step.c:41-100):
 *   octbuild            cells (host AoS) -> device, Morton sort = implicit octree
 *   patches_alloc       CIC deposit on the device + patch bounding box
 *   patches_cells2envinfo  patch field 0 <- deposit
 *   computepotential    pair kernel + octree walk; density/v/mindist -> host AoS
 *   computegradient     forces (from the same fused pass) -> host
 *   updatepositions     host forces -> device, x += F, positions + marks -> host
 *   patches_applyenv2cells  received patch -> device, gather of every field and
 *                       its gradient for the cells -> host cellenvdata
 *   fieldgradient       each field -> device, gradient -> host
 * The drop-ins assume, as the reference step loop guarantees, that the cells'
 * positions are not changed by the host between octbuild and updatepositions.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "timothy_refabi.h"
#include "tm_dropin_api.h"

double3dv_t affShift;
double affScale;

/* the host program's error exit (utils.c:103-109) when it has one */
extern void terminate(systeminfo_t systeminfo, char *msg, char *file, int line) __attribute__((weak));

static tm_session *g_sess;
static int g_cid = -1;
static int64_t g_cap;
static int g_dim;
static void *g_pinned;
static size_t g_pinned_bytes;
static systeminfo_t g_si;
/* tm_dropin_set_precision: the pair maths of the drop-in colony and whether
 * it keeps neighbour lists between steps */
static int g_prec = TM_PREC_FP64;
static int g_lists;
/* the device colony holds the caller's cells in the caller's order (set by a
 * step, cleared when the cell set changes), so the next octbuild may keep
 * slots and lists */
static int g_same_cells;
static int64_t g_last_n = -1;

static void die(const char *what, int rc, int line)
{
    char msg[640];
    snprintf(msg, sizeof msg, "timothy_gb300 %s failed (%d): %s", what, rc, tm_last_error());
    if (terminate) terminate(g_si, msg, (char *)__FILE__, line);
    fprintf(stderr, "error: %s (%s, line %d)\n", msg, __FILE__, line);
    abort();
}

#define TRY(what, call)                                  \
    do {                                                 \
        int rc_ = (call);                                \
        if (rc_ != TM_OK) die(what, rc_, __LINE__);      \
    } while (0)

static void pin_cells(celldata_t *cells, int64_t n)
{
    size_t bytes = (size_t)n * sizeof(celldata_t);
    if ((void *)cells == g_pinned && bytes <= g_pinned_bytes) return;
    if (g_pinned) tm_host_unregister(g_pinned);
    g_pinned = NULL;
    g_pinned_bytes = 0;
    if (tm_host_register(cells, (int64_t)bytes) == TM_OK) {
        g_pinned = cells;
        g_pinned_bytes = bytes;
    }
}

/* the caller's first localcount.n records lie in the page-locked range */
static int records_pinned(const cellsinfo_t *ci)
{
    return g_pinned && (void *)ci->cells == g_pinned &&
           (size_t)ci->localcount.n * sizeof(celldata_t) <= g_pinned_bytes;
}

/* session with room for n cells and the colony's options */
static void ensure_session(int64_t n, int dim)
{
    if (g_sess && n <= g_cap && dim == g_dim) return;
    if (g_sess) {
        tm_session_destroy(g_sess);
        g_sess = NULL;
    }
    int64_t cap = g_cap > n ? g_cap : n;
    if (cap < 1024) cap = 1024;
    if (n > g_cap) cap = n + n / 4;
    double one = 1.5, sz = 1.0;
    tm_celltypes t = {1, &one, &one, &one, &one, &sz, NULL};
    tm_session_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.dimension = dim;
    cfg.device = 0;
    cfg.max_slots = cap + 64;
    cfg.max_colonies = 1;
    cfg.list_capacity = g_lists ? 384 : 0;
    TRY("session create", tm_session_create(&g_sess, &cfg, &t));
    g_same_cells = 0;
    g_cap = cap;
    g_dim = dim;
    tm_colony_options opt;
    memset(&opt, 0, sizeof opt);
    opt.precision = g_prec;
    opt.verlet = g_lists;
    opt.update_mode = TM_UPDATE_REFERENCE;
    opt.dt = 1.0;
    opt.gfh = 8.0f;
    opt.lcap = 8;
    opt.reserve = cap;
    tm_colony_input in;
    memset(&in, 0, sizeof in);
    TRY("colony add", tm_colony_add(g_sess, &in, &opt, &g_cid));
}

static void push_types(const cellsinfo_t *ci, const celltype_t *celltype)
{
    int maxtype = 0;
    TRY("cell types", tmi_max_ctype(g_sess, g_cid, &maxtype));
    int nt = maxtype + 1;
    if (nt > 8) die("more than 8 cell types", TM_EINVAL, __LINE__);
    double h[8], h2[8], h3[8], h4[8], sz[8];
    float rm[8];
    for (int t = 0; t < nt; t++) {
        h[t] = celltype[t].h;
        h2[t] = celltype[t].h2;
        h3[t] = celltype[t].h3;
        h4[t] = celltype[t].h4;
        sz[t] = celltype[t].size;
        rm[t] = celltype[t].randommove;
    }
    tm_celltypes tt = {nt, h, h2, h3, h4, sz, rm};
    TRY("dimension", tmi_set_dimension(g_sess, ci->dimension));
    TRY("cell types", tmi_set_types(g_sess, &tt));
}

static const tmi_aos_layout *cell_layout(void)
{
    static const tmi_aos_layout lay = {(int64_t)sizeof(celldata_t), offsetof(celldata_t, x), offsetof(celldata_t, y),
                                       offsetof(celldata_t, z), offsetof(celldata_t, size),
                                       offsetof(celldata_t, young), offsetof(celldata_t, ctype),
                                       offsetof(celldata_t, phase)};
    return &lay;
}

void octbuild(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype)
{
    g_si = systeminfo;
    int64_t n = (int64_t)cellsinfo->localcount.n;
    if (n == 0) return;                                /* octree.c:152-153 */
    ensure_session(n, cellsinfo->dimension);
    pin_cells(cellsinfo->cells, n);
    if (g_lists && g_same_cells && n == g_last_n)
        TRY("upload", tmi_upload_aos_keep(g_sess, g_cid, cellsinfo->cells, n, cell_layout()));
    else
        TRY("upload", tmi_upload_aos(g_sess, g_cid, cellsinfo->cells, n, cell_layout()));
    g_last_n = n;
    g_same_cells = 1;
    push_types(cellsinfo, celltype);
    TRY("build", tmi_phase(g_sess, 0));
    tm_colony_info info;
    TRY("stats", tm_colony_stats(g_sess, g_cid, &info));
    if (info.device_errors) die("octree build", TM_EDEVICE, __LINE__);
    affShift.x = info.aff_shift[0];
    affShift.y = info.aff_shift[1];
    affShift.z = info.aff_shift[2];
    affScale = info.aff_scale;
    cellsinfo->octree = NULL;                         /* the tree lives on the device */
    cellsinfo->octsize = info.octsize;
    cellsinfo->octmaxsize = n * 64;                   /* octree.c:193 */
}

void octfree(cellsinfo_t *cellsinfo)
{
    (void)cellsinfo;                                  /* device memory is reused next step */
}

void computepotential(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                      cellcommdata_t cellcommdata)
{
    (void)celltype;
    (void)cellcommdata;
    g_si = systeminfo;
    if (cellsinfo->localcount.n <= 1) return;         /* potential.c:89 */
    TRY("pair kernel", tmi_phase(g_sess, 1));
    TRY("sync", tm_session_sync(g_sess));
    TRY("download", tmi_download_aos3(g_sess, g_cid, cellsinfo->cells, (int64_t)sizeof(celldata_t),
                                      offsetof(celldata_t, v), 0, records_pinned(cellsinfo)));
}

static void no_remote(systeminfo_t systeminfo, cellcommdata_t cellcommdata)
{
    if (cellcommdata.numimp <= 0) return;
    g_si = systeminfo;
    die("halo cells: the GB300 path runs one MPI rank", TM_EINVAL, __LINE__);
}

void computeremotepotential(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                            cellcommdata_t cellcommdata)
{
    (void)cellsinfo;
    (void)celltype;
    no_remote(systeminfo, cellcommdata);
}

void computegradient(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                     cellcommdata_t cellcommdata)
{
    (void)celltype;
    (void)cellcommdata;
    g_si = systeminfo;
    if (cellsinfo->localcount.n <= 1) return;         /* potential.c:212 */
    TRY("forces", tmi_download_forces(g_sess, g_cid, (double *)cellsinfo->forces));
}

void computeremotegradient(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                           cellcommdata_t cellcommdata)
{
    (void)cellsinfo;
    (void)celltype;
    no_remote(systeminfo, cellcommdata);
}

/* The random move's rand() values without n calls of rand() on the host.
 *
 * updatepositions takes dim values per cell from the host program's rand()
 * whatever the cell types' randommove (cells.c:353-356), so the generator
 * must advance by that many values; at 16 M cells the calls alone take about
 * a second.  The C library's rand() (glibc) is its random() generator: 31
 * words r and a rear index, each call adding the word 28 places back
 * (mod 31) to the oldest one and returning the sum >> 1 (the published
 * additive generator, x_k = x_{k-31} + x_{k-3} mod 2^32).  initstate() hands
 * back the caller's state array with the rear index stored in its first word
 * (5 * rear + 3 for this generator type) and setstate() puts it back
 * unchanged, so the window of the caller's generator can be read.  The
 * window is trusted only when it predicts the next rand() exactly: one real
 * call is made and compared (any other generator, or a rand() of its own,
 * fails the check and the values come from rand() calls as before).  The
 * values are then generated on the device from the window, and the window
 * after them is written back into the caller's state array, which leaves the
 * generator where nd calls of rand() would have left it.  The host program
 * calls the drop-ins from one thread, as the reference does. */
static char g_rand_scratch[128] __attribute__((aligned(8)));

/* the caller's generator window, oldest word first; prev = its state array */
static int libc_rand_window(uint32_t w[31], int32_t **prev_out)
{
    char *prev = initstate(1u, g_rand_scratch, sizeof g_rand_scratch);
    if (!prev) return -1;
    int32_t *p = (int32_t *)(void *)prev;
    const int32_t head = p[0];
    const int type = head % 5, rear = head / 5;
    if (type != 3 || rear < 0 || rear >= 31) {
        setstate(prev);
        return -1;
    }
    const int front = (rear + 3) % 31;
    for (int i = 0; i < 31; i++) w[i] = (uint32_t)p[1 + (front + i) % 31];
    setstate(prev);
    *prev_out = p;
    return 0;
}

/* make w (oldest first) the caller's generator window */
static void libc_rand_set_window(int32_t *prev, const uint32_t w[31])
{
    char *cur = initstate(1u, g_rand_scratch, sizeof g_rand_scratch);   /* saves the caller's position */
    int32_t *p = (int32_t *)(void *)cur;
    if (p != prev) {                                     /* not the array read before: leave it alone */
        setstate(cur);
        return;
    }
    p[0] = 5 * 28 + 3;                                   /* rear 28, front 0: the oldest word at index 0 */
    for (int i = 0; i < 31; i++) p[1 + i] = (int32_t)w[i];
    setstate(cur);
}

/* nd draws of the caller's rand() for the random move, on the device when
 * the generator is the C library's; 0 when done, -1 when the caller must
 * call rand() for draws[1..nd) (draws[0] is taken here in both cases) */
static int move_draws_device(int64_t nd, int *draws)
{
    uint32_t w[31], end[31];
    int32_t *prev = NULL;
    const int have = libc_rand_window(w, &prev) == 0;
    draws[0] = rand();
    if (!have || draws[0] != (int)((w[0] + w[28]) >> 1)) return -1;
    TRY("random move", tmi_set_move_draws_window(g_sess, w, nd, end));
    libc_rand_set_window(prev, end);
    return 0;
}

void updatepositions(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo, unsigned char *removecell,
                     int64_t *removecount)
{
    (void)celltype;
    int64_t n = (int64_t)cellsinfo->localcount.n;
    if (n == 0 || !g_sess) return;
    TRY("dimension", tmi_set_dimension(g_sess, settings.dimension));
    TRY("forces", tmi_upload_forces(g_sess, g_cid, (const double *)cellsinfo->forces));
    TRY("marks", tmi_upload_removecell(g_sess, g_cid, removecell));
    /* the random move takes dim rand() values per cell in cell order whatever
     * the cell types' randommove (cells.c:353-356): drawn here, so that the
     * caller's generator stays where the reference leaves it */
    const int64_t nd = n * (settings.dimension == 3 ? 3 : 2);
    int first = 0;
    int *draws = NULL;
    if (move_draws_device(nd, &first) != 0) {
        draws = (int *)malloc((size_t)nd * sizeof(int));
        if (!draws) die("random move draws", -2, __LINE__);
        draws[0] = first;
        for (int64_t k = 1; k < nd; k++) draws[k] = rand();
        TRY("random move", tmi_set_move_draws(g_sess, draws, nd));
    }
    TRY("update", tmi_phase(g_sess, 2));
    TRY("sync", tm_session_sync(g_sess));
    free(draws);
    TRY("random move", tmi_set_move_draws(g_sess, NULL, 0));
    TRY("positions", tmi_download_aos3(g_sess, g_cid, cellsinfo->cells, (int64_t)sizeof(celldata_t),
                                       offsetof(celldata_t, x), 1, records_pinned(cellsinfo)));
    int64_t marked = 0;
    TRY("marks", tmi_download_removecell(g_sess, g_cid, removecell, &marked));
    *removecount += marked;
}

static uint64_t *phase_counter(cellcount_t *c, int phase)
{
    switch (phase) {
    case 0: return &c->g0phase;
    case 1: return &c->g1phase;
    case 2: return &c->sphase;
    case 3: return &c->g2phase;
    case 4: return &c->mphase;
    default: return &c->necroticphase;
    }
}

/* One cell-cycle step of every local cell (cells.c:370-523) with mitosis
 * (cells.c:124-205), on the device.  The records go up as they are, the cycle
 * draws the caller's rand() values in the reference's order and the records,
 * daughters appended, come back with removecell and the counters.  The colony
 * count stands in for globalcount.n (the two agree at one rank). */
int updatecellcycles(systeminfo_t systeminfo, settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo,
                     cellenvdata_t **cellenvdata, unsigned char *removecell, int64_t *removecount)
{
    g_si = systeminfo;
    const int64_t n = (int64_t)cellsinfo->localcount.n;
    if (n == 0) return 0;
    /* records the caller's array holds: settings.maxlocalcells (mitosis,
     * cells.c:130-131, stops beyond it); one division per cell at most */
    int64_t room = settings.maxlocalcells > n ? settings.maxlocalcells : n;
    if (room > 2 * n) room = 2 * n;
    ensure_session(room, settings.dimension);
    pin_cells(cellsinfo->cells, room);
    TRY("upload", tmi_upload_aos(g_sess, g_cid, cellsinfo->cells, n, cell_layout()));
    g_same_cells = 0;   /* a fresh upload: the next octbuild uploads afresh too */
    push_types(cellsinfo, celltype);
    int maxtype = 0;
    TRY("cell types", tmi_max_ctype(g_sess, g_cid, &maxtype));
    const int nt = maxtype + 1, nf = settings.numberoffields;
    if (nf > 16) die("more than 16 fields", TM_EINVAL, __LINE__);
    tm_cycle_type ct[8];
    float cl1[8 * 16], cl2[8 * 16];
    for (int t = 0; t < nt; t++) {
        ct[t].g1 = celltype[t].g1;
        ct[t].s = celltype[t].s;
        ct[t].g2 = celltype[t].g2;
        ct[t].m = celltype[t].m;
        ct[t].v = celltype[t].v;
        ct[t].rd = celltype[t].rd;
        ct[t].criticaldensity = celltype[t].criticaldensity;
        for (int f = 0; f < nf; f++) {
            cl1[t * nf + f] = celltype[t].criticallevel1[f];
            cl2[t * nf + f] = celltype[t].criticallevel2[f];
        }
    }
    tm_cycle_params p;
    memset(&p, 0, sizeof p);
    p.types = ct;
    p.nfields = nf;
    p.criticallevel1 = cl1;
    p.criticallevel2 = cl2;
    p.simulationstart = settings.simulationstart;
    p.secondsperstep = settings.secondsperstep;
    double *env[16];
    for (int f = 0; f < nf; f++) env[f] = (double *)cellenvdata[f];
    int64_t marked = 0, nout = n, counts[16];
    TRY("cell cycle", tmi_cycle_aos(g_sess, g_cid, cellsinfo->cells, n, room, &p, env, removecell, &marked, &nout,
                                    counts));
    *removecount += marked;
    for (int ph = 0; ph < 6; ph++) *phase_counter(&cellsinfo->localcount, ph) += (uint64_t)counts[ph];
    for (int t = 0; t < nt; t++) {
        cellsinfo->localtypecount[t].n += (uint64_t)counts[8 + t];
        cellsinfo->localtypecount[t].g1phase += (uint64_t)counts[8 + t];
    }
    cellsinfo->localcount.n += (uint64_t)(nout - n);
    cellsinfo->localcount.g1phase += (uint64_t)(nout - n);
    return 0;
}

/* Removal of the marked cells (cells.c:290-336): the records are compacted
 * on the device in the reference's order and the counters of the removed
 * cells' phases and types are taken down. */
void cellsdeath(int oldlnc, cellsinfo_t *cellsinfo, unsigned char *removecell, int64_t removecount)
{
    if (cellsinfo->globalcount.n == 1) return;
    const int64_t n = (int64_t)cellsinfo->localcount.n;
    if (n == 0 || removecount == 0) {
        cellsinfo->localcount.n -= (uint64_t)removecount;
        return;
    }
    ensure_session(n, cellsinfo->dimension);
    g_same_cells = 0;
    int64_t nout = n, removed[64];
    TRY("cell removal", tmi_compact_aos(g_sess, cellsinfo->cells, n, oldlnc, removecell, &nout, removed));
    for (int t = 0; t < 8; t++)
        for (int ph = 0; ph < 8; ph++) {
            const int64_t r = removed[t * 8 + ph];
            if (!r) continue;
            if (ph < 5) {
                *phase_counter(&cellsinfo->localcount, ph) -= (uint64_t)r;
                *phase_counter(&cellsinfo->localtypecount[t], ph) -= (uint64_t)r;
            }
            cellsinfo->localtypecount[t].n -= (uint64_t)r;
        }
    cellsinfo->localcount.n -= (uint64_t)removecount;
}

/* grid of this rank (grid.c:80-136): lower corner, resolution, index box */
static void grid_setup(systeminfo_t si, const grid_t *grid, int dim)
{
    if (si.size != 1) die("CIC patches: the GB300 path runs one MPI rank", TM_EINVAL, __LINE__);
    double lower[3] = {grid->lowercorner.x, grid->lowercorner.y, grid->lowercorner.z};
    int64_t gs[3] = {grid->localsize.x, grid->localsize.y, dim == 3 ? grid->localsize.z : 1};
    TRY("grid", tmi_set_cic(g_sess, g_cid, lower, grid->resolution, gs));
}

void patches_alloc(systeminfo_t systeminfo, settings_t settings, patches_t *patches, cellsinfo_t *cellsinfo,
                   grid_t *grid)
{
    g_si = systeminfo;
    int p, size = systeminfo.size;
    patches->data = (double **)calloc((size_t)size, sizeof(double *));
    patches->intersect = (int *)calloc((size_t)size, sizeof(int));
    patches->lowercorner = (int643dv_t *)calloc((size_t)size, sizeof(int643dv_t));
    patches->uppercorner = (int643dv_t *)calloc((size_t)size, sizeof(int643dv_t));
    patches->lowercornerR = (int643dv_t *)calloc((size_t)size, sizeof(int643dv_t));
    patches->uppercornerR = (int643dv_t *)calloc((size_t)size, sizeof(int643dv_t));
    patches->size = (int643dv_t *)calloc((size_t)size, sizeof(int643dv_t));
    for (p = 0; p < size; p++) {                      /* patches.c:61-78 */
        patches->lowercorner[p].x = 2147483647;
        patches->lowercorner[p].y = 2147483647;
        patches->lowercorner[p].z = cellsinfo->dimension == 3 ? 2147483647 : 0;
        patches->uppercorner[p].x = -2147483647 - 1;
        patches->uppercorner[p].y = -2147483647 - 1;
        patches->uppercorner[p].z = cellsinfo->dimension == 3 ? -2147483647 - 1 : 0;
    }
    if (cellsinfo->localcount.n == 0 || !g_sess) return;
    grid_setup(systeminfo, grid, cellsinfo->dimension);
    TRY("CIC", tmi_phase(g_sess, 3));
    int64_t lo[3], hi[3];
    TRY("patch box", tmi_patch_box(g_sess, g_cid, lo, hi));
    if (hi[0] < lo[0]) return;                        /* no node touched */
    patches->intersect[0] = 1;
    patches->lowercorner[0].x = lo[0];
    patches->lowercorner[0].y = lo[1];
    patches->lowercorner[0].z = lo[2];
    patches->uppercorner[0].x = hi[0];
    patches->uppercorner[0].y = hi[1];
    patches->uppercorner[0].z = hi[2];
    patches->size[0].x = hi[0] - lo[0] + 1;           /* patches.c:134-145 */
    patches->size[0].y = hi[1] - lo[1] + 1;
    patches->size[0].z = cellsinfo->dimension == 3 ? hi[2] - lo[2] + 1 : 1;
    patches->data[0] = (double *)calloc((size_t)(patches->size[0].x * patches->size[0].y * patches->size[0].z *
                                                 settings.numberoffields),
                                        sizeof(double));
}

void patches_cells2envinfo(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                           cellsinfo_t *cellsinfo, grid_t *grid)
{
    (void)grid;
    g_si = systeminfo;
    if (!patches->intersect || !patches->intersect[0] || !g_sess || cellsinfo->localcount.n == 0) return;
    const int64_t vol = patches->size[0].x * patches->size[0].y * patches->size[0].z;
    memset(patches->data[0], 0, (size_t)(vol * settings.numberoffields) * sizeof(double));
    int64_t lo[3] = {patches->lowercorner[0].x, patches->lowercorner[0].y, patches->lowercorner[0].z};
    int64_t hi[3] = {patches->uppercorner[0].x, patches->uppercorner[0].y, patches->uppercorner[0].z};
    if (settings.numberoffields > 0) TRY("patch", tmi_read_patch(g_sess, g_cid, lo, hi, patches->data[0]));
}

void patches_applyenv2cells(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                            cellsinfo_t *cellsinfo, grid_t *grid, cellenvdata_t ***cellenvdata)
{
    g_si = systeminfo;
    const int nf = settings.numberoffields;
    const int64_t n = (int64_t)cellsinfo->localcount.n;
    int f, p;
    /* zeroed per-field arrays, patches.c:522-534 */
    *cellenvdata = (cellenvdata_t **)calloc((size_t)(nf > 0 ? nf : 1), sizeof(cellenvdata_t *));
    if (!*cellenvdata) die("cellenvdata allocation", TM_ENOMEM, __LINE__);
    for (f = 0; f < nf; f++) {
        (*cellenvdata)[f] = (cellenvdata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(cellenvdata_t));
        if (!(*cellenvdata)[f]) die("cellenvdata allocation", TM_ENOMEM, __LINE__);
    }
    if (systeminfo.size != 1) die("grid-to-cell gather: the GB300 path runs one MPI rank", TM_EINVAL, __LINE__);
    const int64_t vol = patches->size ? patches->size[0].x * patches->size[0].y * patches->size[0].z : 0;
    if (n > 0 && nf > 0 && g_sess && vol > 0 && patches->buff && patches->buff[0]) {
        const int64_t lo[3] = {patches->lowercorner[0].x, patches->lowercorner[0].y, patches->lowercorner[0].z};
        const int64_t sz[3] = {patches->size[0].x, patches->size[0].y, patches->size[0].z};
        const double lower[3] = {grid->lowercorner.x, grid->lowercorner.y, grid->lowercorner.z};
        const int64_t hi[3] = {grid->upperidx[0].x, grid->upperidx[0].y, grid->upperidx[0].z};
        double **dst = (double **)malloc(sizeof(double *) * (size_t)nf);
        if (!dst) die("cellenvdata allocation", TM_ENOMEM, __LINE__);
        for (f = 0; f < nf; f++) dst[f] = (double *)(*cellenvdata)[f];
        TRY("grid-to-cell gather",
            tmi_env2cells_patch(g_sess, g_cid, patches->buff[0], nf, lo, sz, lower, grid->resolution, hi, dst));
        free(dst);
    }
    /* the received patches are released here (patches.c:590-592) */
    if (patches->buff) {
        for (p = 0; p < systeminfo.size; p++) free(patches->buff[p]);
        free(patches->buff);
        patches->buff = NULL;
    }
}

void fieldgradient(systeminfo_t systeminfo, settings_t settings, environment_t **environment, grid_t *grid)
{
    g_si = systeminfo;
    if (settings.numberoffields == 0) return;
    if (systeminfo.size != 1) die("field gradient: the GB300 path runs one MPI rank", TM_EINVAL, __LINE__);
    if (!g_sess) ensure_session(1, settings.dimension);
    const int64_t gs[3] = {grid->localsize.x, grid->localsize.y, grid->localsize.z};
    for (int f = 0; f < settings.numberoffields; f++)
        TRY("field gradient", tmi_field_gradient_host(g_sess, (*environment)[f].data, gs, grid->resolution,
                                                      (*environment)[f].gradient));
}

/* ------------------------------------------------------------------------
 * Fields: environment.c without Hypre.  The reference assembles the implicit
 * step in environment_initsystem / environment_initboundary and solves it
 * with Hypre's PCG + BoomerAMG in environment_solve; here the step runs on
 * the GPU (tm_diffusion).  As in the reference, environment_compute starts
 * every field from its initialconditionmean and leaves environment[f].data
 * as it was (the loop meant to copy the solution back is empty,
 * environment.c:495-507); tm_dropin_env_solution reads the solution, and
 * tm_dropin_set_env_writeback(1) copies it into data after each step. */
static tm_diffusion *g_diff;
static int64_t g_diff_gs[3];
static int g_env_writeback;

/* environment.c:33-55 without the solver's own arrays */
void environment_allocate(systeminfo_t systeminfo, settings_t settings, grid_t grid, environment_t **environment,
                          void *solverdata, void *solversettings)
{
    (void)solverdata;
    (void)solversettings;
    if (settings.numberoffields == 0) return;
    const size_t G = (size_t)(grid.localsize.x * grid.localsize.y * grid.localsize.z);
    for (int i = 0; i < settings.numberoffields; i++)
        if (!((*environment)[i].data = (double *)calloc(G, sizeof(double))))
            die("environment->data allocation", TM_ENOMEM, __LINE__);
    for (int i = 0; i < settings.numberoffields; i++)
        if (!((*environment)[i].production = (double *)calloc(G, sizeof(double))))
            die("environment->production allocation", TM_ENOMEM, __LINE__);
    for (int i = 0; i < settings.numberoffields; i++)
        if (!((*environment)[i].gradient = (double *)calloc(G * 3, sizeof(double))))
            die("environment->gradient allocation", TM_ENOMEM, __LINE__);
    (void)systeminfo;
}

/* environment.c:56-72: mean + rand() / RAND_MAX * variance per node.  The
 * loop order and the conversion of each value are the reference's on
 * purpose: the host program's rand() stream is consumed here, so a seeded
 * run must take the same values in the same order, node for node, for its
 * fields and for every later draw (cell cycle, random move) to match. */
void environment_init(systeminfo_t systeminfo, settings_t settings, grid_t grid, environment_t **environment)
{
    (void)systeminfo;
    if (settings.numberoffields == 0) return;
    const int64_t yz = grid.localsize.y * grid.localsize.z;
    for (int f = 0; f < settings.numberoffields; f++)
        for (int64_t i = 0; i < grid.localsize.x; i++)
            for (int64_t j = 0; j < grid.localsize.y; j++)
                for (int64_t k = 0; k < grid.localsize.z; k++)
                    (*environment)[f].data[yz * i + grid.localsize.z * j + k] =
                        (*environment)[f].initialconditionmean +
                        ((double)(rand()) / RAND_MAX) * (*environment)[f].initialconditionvariance;
}

/* environment.c:131-233: the step's parameters are derived again by
 * environment_compute; nothing to assemble */
void environment_initsystem(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                            void *solverdata, void *solversettings)
{
    (void)systeminfo;
    (void)settings;
    (void)grid;
    (void)environment;
    (void)solverdata;
    (void)solversettings;
}

void environment_compute(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                         void *solverdata, void *solversettings)
{
    (void)solverdata;
    (void)solversettings;
    g_si = systeminfo;
    const int nf = settings.numberoffields;
    if (nf == 0) return;
    if (systeminfo.size != 1) die("diffusion: the GB300 path runs one MPI rank", TM_EINVAL, __LINE__);
    if (nf > 64) die("diffusion: more than 64 fields", TM_EINVAL, __LINE__);
    const int64_t gs[3] = {grid->localsize.x, grid->localsize.y, grid->localsize.z};
    if (!g_diff || gs[0] != g_diff_gs[0] || gs[1] != g_diff_gs[1] || gs[2] != g_diff_gs[2]) {
        if (g_diff) tm_diffusion_destroy(g_diff);
        g_diff = NULL;
        TRY("diffusion solver", tm_diffusion_create(&g_diff, gs, 0));
        memcpy(g_diff_gs, gs, sizeof gs);
    }
    double mean[64], dc[64], bc[64], lam[64];
    for (int f = 0; f < nf; f++) {
        mean[f] = (*environment)[f].initialconditionmean;
        dc[f] = (*environment)[f].diffusioncoefficient;
        bc[f] = (*environment)[f].boundarycondition;
        lam[f] = (*environment)[f].lambdadelay;
    }
    tm_diffusion_stats st;
    TRY("diffusion step", tmi_env_compute(g_diff, nf, mean, dc, bc, lam, grid->resolution, settings.secondsperstep,
                                          settings.gfdt, settings.step, &st));
    if (g_env_writeback)
        for (int f = 0; f < nf; f++) TRY("diffusion result", tmi_env_solution(g_diff, f, (*environment)[f].data));
}

int tm_dropin_env_solution(int field, double *out)
{
    if (!g_diff) return TM_EINVAL;
    return tmi_env_solution(g_diff, field, out);
}

void tm_dropin_set_env_writeback(int on) { g_env_writeback = on ? 1 : 0; }

void tm_dropin_set_precision(int precision, int neighbour_lists)
{
    const int prec = precision == TM_PREC_FP32C ? TM_PREC_FP32C : TM_PREC_FP64;
    const int lists = neighbour_lists ? 1 : 0;
    if (prec == g_prec && lists == g_lists) return;
    g_prec = prec;
    g_lists = lists;
    /* the next octbuild makes a session with these options */
    if (g_sess) tm_session_destroy(g_sess);
    g_sess = NULL;
    g_cid = -1;
    g_cap = 0;
    g_same_cells = 0;
}

int64_t tm_dropin_pinned_bytes(void) { return (int64_t)g_pinned_bytes; }

void tm_dropin_shutdown(void)
{
    if (g_diff) tm_diffusion_destroy(g_diff);
    g_diff = NULL;
    if (g_pinned) tm_host_unregister(g_pinned);
    g_pinned = NULL;
    g_pinned_bytes = 0;
    if (g_sess) tm_session_destroy(g_sess);
    g_sess = NULL;
    g_cid = -1;
    g_cap = 0;
    g_same_cells = 0;
}
