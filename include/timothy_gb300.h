/* timothy_gb300 -- GB300-native cell-mechanics hot path of Timothy.
 *
 * Two C interfaces, both exported by libtimothy_gb300.so:
 *
 *  1. The device-resident session API (tm_*): colonies live in HBM across
 *     steps; one call advances every active colony.  This is what batching,
 *     serving and the benchmarks use.
 *
 *  2. The reference-signature drop-ins (octbuild, computepotential, ...):
 *     declared in timothy_refabi.h with the exact signatures of the reference
 *     functions they replace, so the reference step loop links against them
 *     unchanged.
 *
 * Errors: every tm_* function returns TM_OK (0) or a negative TM_E* code;
 * tm_last_error() describes the most recent failure of the calling thread.
 * No function falls back to a CPU implementation: without a usable CUDA
 * device the session cannot be created.
 */
#ifndef TIMOTHY_GB300_H
#define TIMOTHY_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TM_OK 0
#define TM_EINVAL (-1)    /* bad argument */
#define TM_ENOMEM (-2)    /* device or host allocation failed, or no room */
#define TM_ECUDA (-3)     /* CUDA runtime error */
#define TM_EDEVICE (-4)   /* a kernel flagged an input it cannot handle */
#define TM_ENODEV (-5)    /* no CUDA device */
#define TM_ENOENT (-6)    /* unknown colony id */

/* device-side error bits reported by tm_colony_stats / TM_EDEVICE */
#define TM_DEVERR_BIGBIN 1u   /* > 2048 cells in one Morton bin */
#define TM_DEVERR_STACK 2u    /* octree walk deeper than its stack */
#define TM_DEVERR_CODES 4u    /* two cells share a lattice code (coincident cells) */
#define TM_DEVERR_TYPES 8u    /* an asynchronous upload carried a cell type outside the table (read as 0) */

#define TM_PREC_FP64 0        /* plain FP64, the reference's arithmetic */
#define TM_PREC_FP32C 1       /* FP32 pair maths, Kahan sums, FP64 cutoff band + FP64 positions */

#define TM_UPDATE_REFERENCE 0 /* x += F (+ random move), cells.c:342-365 */
#define TM_UPDATE_DT 1        /* x += dt * F */
#define TM_UPDATE_NONE 2

typedef struct tm_session tm_session;

/* Per-type constants (the celltype_t fields the path reads, global.h:315-335).
 * h2/h3/h4 are used as given, never derived from h. */
typedef struct {
    int ntypes;               /* 1..8 */
    const double *h, *h2, *h3, *h4, *size;
    const float *randommove;  /* may be NULL: no random move */
} tm_celltypes;

typedef struct {
    int dimension;            /* 2 or 3 */
    int device;               /* CUDA device ordinal */
    int64_t max_slots;        /* total cells over all colonies (padded to 32 per colony) */
    int max_colonies;
    int64_t max_bin_entries;  /* 0: derived from max_slots */
    int64_t max_grid_entries; /* 0: one 257^3 grid */
    int diagnostics;          /* fill neighbour counts/fingerprints and v candidates */
    int list_capacity;        /* neighbour-list entries per cell (multiple of 4); 0: none */
} tm_session_config;

/* One colony's cells in caller order (host memory). */
typedef struct {
    int64_t n;
    const double *x, *y, *z, *size;
    const float *young;
    const int *ctype;
    const int *phase;         /* may be NULL (all 1) */
} tm_colony_input;

typedef struct {
    int precision;            /* TM_PREC_* */
    int update_mode;          /* TM_UPDATE_* */
    double dt;                /* TM_UPDATE_DT only */
    int cic;                  /* deposit onto a grid each step */
    float gfh;                /* grid resolution (settings.gfh) */
    int lcap;                 /* deepest bin level, 0: from the colony's extent */
    int64_t reserve;          /* slots to reserve (>= n) so later uploads can grow */
    int verlet;               /* 1: keep neighbour lists within h + skin between rebuilds */
    float skin;               /* list margin (0: the session's skin_over_h * largest h) */
    int rmax;                 /* rebuild the lists at least every rmax steps (0: the session's rmax) */
} tm_colony_options;

/* Outputs in caller order (host memory); any pointer may be NULL. */
typedef struct {
    double *x, *y, *z;
    double *density, *v, *mindist;
    double *fx, *fy, *fz;
    unsigned char *removecell;
    int32_t *nbcount;         /* diagnostics: neighbours within h */
    uint64_t *nbhash;         /* diagnostics: sum of mix64(j+1) over them */
    int32_t *vcand;           /* diagnostics: caller index of v's candidate or -1 */
    double *grid;             /* CIC grid, x-major with z fastest */
} tm_colony_output;

typedef struct {
    double aff_shift[3], aff_scale;   /* affShift / affScale of the last step */
    int64_t octsize;                  /* node count of the reference octree */
    int64_t removecount;              /* cells newly marked for removal */
    int64_t patch_lower[3], patch_upper[3];   /* CIC patch corners (patches.c:61-132) */
    int64_t grid_size[3];
    uint32_t device_errors;           /* TM_DEVERR_* */
    int bin_level;
    int64_t n;
    int64_t list_rebuilds;            /* steps that rebuilt the neighbour lists */
    int64_t codes_slow;               /* lattice codes of the last step decided in FP64 */
    float list_maxdisp;               /* largest cell displacement since the lists were built */
    float list_skin;                  /* the colony's list skin */
    int32_t list_age;                 /* steps since the lists were built */
    int64_t density_fp64_cells;       /* FP32 path: cells of the last step whose density was redone in FP64 */
    int64_t walked_cells;             /* cells of the last step whose v (or mindist) took the octree walk */
    int64_t walked_isolated_cells;    /* those of them without a neighbour within h (mindist from the walk) */
} tm_colony_info;

const char *tm_last_error(void);
const char *tm_version(void);
int tm_device_count(void);
/* Measured FP32 FMA rate of `device` in TFLOP/s (eight independent FMA chains
 * per thread on every SM, best of two timed launches): the compute
 * denominator of the list pass's roofline. */
int tm_measure_fp32_peak(int device, double *tflops);
/* Self-check of the arithmetic the kernels form themselves: on n
 * pseudo-random inputs each, mismatches[0] counts quotients a / b formed from
 * RN(1/b) by an FMA correction that differ from the correctly rounded
 * division, mismatches[1] integer double -> float roundings that differ from
 * the hardware conversion, mismatches[2] integer float -> double conversions
 * that do.  All three must be 0. */
int tm_check_numerics(int device, int64_t n, uint64_t seed, int64_t *mismatches);

int tm_session_create(tm_session **out, const tm_session_config *cfg, const tm_celltypes *types);
int tm_session_destroy(tm_session *s);
/* cudaStream_t the session launches on */
void *tm_session_stream(tm_session *s);

/* Device bytes a session with this configuration allocates (-1 on a bad
 * configuration); with tm_device_memory, what admission by free HBM uses. */
int64_t tm_session_bytes(const tm_session_config *cfg, int ntypes);
/* Free and total bytes of a device (cudaMemGetInfo). */
int tm_device_memory(int device, int64_t *free_bytes, int64_t *total_bytes);

/* Launch shapes and neighbour-list parameters of a session, as an autotuner
 * sets them.  Defaults: {1, 1, 128, 0.1, 64}. */
typedef struct tm_tuning {
    int pair_lshift;     /* search candidates from Morton nodes 0 or 1 level above the bins */
    int list_variant;    /* list kernel block/registers: 1 = 256 threads, 64 registers; 2 = 128/64;
                            3 = 256/80; 4 = 512/64 */
    int walk_block;      /* octree walk threads per block: 64, 128 or 256 */
    float skin_over_h;   /* list skin as a fraction of the largest h, in (0, 1] */
    int rmax;            /* rebuild the lists at least every rmax steps */
} tm_tuning;
int tm_session_get_tuning(tm_session *s, tm_tuning *t);
/* Set all fields (validated; TM_EINVAL leaves the tuning unchanged).  A new
 * skin_over_h or rmax applies to every colony (overriding its options) and
 * to colonies added later whose options leave skin / rmax at 0; their lists
 * are rebuilt at the next step. */
int tm_session_set_tuning(tm_session *s, const tm_tuning *t);

/* Expected fraction of cells whose neighbour lists are rebuilt per step,
 * extrapolating each colony's displacement since its last rebuild linearly
 * (at least 1/rmax), weighted by cells; and the rebuilds so far over all
 * colonies.  Meaningful after a step. */
int tm_session_list_rate(tm_session *s, double *rate, int64_t *rebuilds);

/* Add a colony; its id is written to *id.  Uploads the cells. */
int tm_colony_add(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id);
/* The same without waiting: the cells' copies and the colony's set-up are
 * queued on the session stream behind the work already there (a step in
 * flight keeps running), and the call returns.  Cell types are checked on
 * the host first.  From page-locked memory the copies read in's arrays when
 * they run, so the caller leaves them unchanged until a later
 * tm_session_sync or a waited fence; other host memory is read during the
 * call. */
int tm_colony_add_async(tm_session *s, const tm_colony_input *in, const tm_colony_options *opt, int *id);
/* Removes a colony without waiting: work queued before it still sees the
 * colony, and its slots, bins and grid are free for colonies added after. */
int tm_colony_remove(tm_session *s, int id);
/* Remove the colony's cells marked for removal (outside the box after an
 * update), as cellsdeath does at one rank (cells.c:290-336): the survivors
 * keep their order, and their caller indices close up (cell k of the caller's
 * order becomes k minus the removed cells before it).  Nothing is removed
 * from a colony of one cell (cells.c:294).  *removed receives the count. */
int tm_colony_compact(tm_session *s, int id, int64_t *removed);
/* Append cells after the colony's current ones (caller indices n, n+1, ...),
 * as mitosis appends daughters (cells.c:156-205); the colony must have slots
 * for them (tm_colony_options.reserve).  Lists are rebuilt at the next step. */
int tm_colony_append(tm_session *s, int id, const tm_colony_input *in);
/* Cell-cycle parameters of one cell type (celltype_t, global.h:315-335). */
typedef struct tm_cycle_type {
    float g1, s, g2, m;       /* phase lengths (hours) */
    float v;                  /* relative spread of the lengths drawn at division */
    float rd;                 /* death probability at G1->S and G2->M */
    float criticaldensity;    /* growth stops above it */
} tm_cycle_type;

/* One cell-cycle step (updatecellcycles, cells.c:370-523, with mitosis,
 * cells.c:124-205) for a colony.  draw supplies the random values in the
 * order the reference calls rand() (NULL: the C library's rand()); to follow
 * a reference run exactly, the generator first skips the values the
 * reference's updatepositions takes (2 or 3 per cell, cells.c:353-355). */
typedef struct tm_cycle_params {
    const tm_cycle_type *types;   /* one per cell type */
    int nfields;
    const float *criticallevel1;  /* [type][field] */
    const float *criticallevel2;
    const double *cellenv;        /* device, nfields x n x 4 as tm_colony_env2cells writes; NULL if nfields == 0 */
    int simulationstart;
    float secondsperstep;
    int (*draw)(void *ctx);
    void *draw_ctx;
    /* rand_seeded = 1: the values come from the C library's rand() stream
     * after srand(rand_seed), starting after *rand_offset earlier values,
     * generated on the device (the same values rand() would return, without
     * calling it); *rand_offset advances by the values taken.  draw is then
     * unused. */
    int rand_seeded;
    uint32_t rand_seed;
    int64_t *rand_offset;
} tm_cycle_params;

/* Cell-cycle state of a colony's cells in the caller's order (n entries):
 * phase time and lengths (hours), age; get also returns phase, size and young. */
int tm_colony_set_cycle(tm_session *s, int id, const float *phasetime, const float *g1, const float *sphase,
                        const float *g2, const float *m, const int *age);
int tm_colony_get_cycle(tm_session *s, int id, float *phasetime, float *g1, float *sphase, float *g2, float *m,
                        int *age, int *phase, double *size, float *young);
/* Runs the step; dividing cells append their daughter (caller indices n, n+1,
 * ... in the order of their parents; the colony needs reserved slots), dying
 * cells are marked for removal (tm_colony_compact removes them).  *divided
 * and *marked receive the counts. */
int tm_colony_cellcycle(tm_session *s, int id, const tm_cycle_params *p, int64_t *divided, int64_t *marked);

/* Asynchronous host I/O for pipelined loops (upload of step k + 1 while the
 * results of step k travel back).  tm_colony_upload_async takes the same
 * cells in the same order as the colony holds (same n; other uploads go
 * through tm_colony_upload); a cell type outside the table is read as 0 and
 * reported as TM_DEVERR_TYPES by the next tm_session_sync.  Both return once
 * the work is queued: the caller leaves in's arrays unchanged, and reads
 * out's arrays only, after tm_session_sync.  With the same n, the upload's
 * size, young, ctype and phase may be NULL: those attributes keep their
 * values (an upload of positions only).  An asynchronous download sends each
 * of x, y, z in up to eight pieces (one per 2^20 cells), and an asynchronous
 * upload reads each piece of
 * each coordinate only after the same piece of the asynchronous download
 * queued before it has reached the host (the whole coordinate when the two
 * cell counts differ), and its other arrays after all three, so a host loop
 * may pass one step's downloaded positions to the next step's upload without
 * waiting; a piece travels up while the next ones still come down, and the
 * other fields of that download keep travelling while the upload runs.  They
 * stage through device buffers of their own, 44 and 112 bytes per slot and,
 * for a downloaded grid, one copy of the colony's grid, allocated on first
 * use (not counted by tm_session_bytes). */
int tm_colony_upload_async(tm_session *s, int id, const tm_colony_input *in);
int tm_colony_download_async(tm_session *s, int id, const tm_colony_output *out);
/* Replace the cells of an existing colony (at most the slots it holds).  With
 * the same n the cells are taken as the same cells in the same order as the
 * colony's input: they keep their slots, and neighbour lists stay valid unless
 * a cell moved too far, changed size or changed type.  Such uploads (and
 * tm_colony_upload_async) reorder the cells through a record buffer of 48
 * bytes per slot, allocated on first use (not counted by tm_session_bytes).
 * Cell types are checked on the device; one outside the table returns
 * TM_EDEVICE and leaves the colony empty. */
int tm_colony_upload(tm_session *s, int id, const tm_colony_input *in);
int tm_colony_set_active(tm_session *s, int id, int active);
int tm_colony_download(tm_session *s, int id, const tm_colony_output *out);
int tm_colony_stats(tm_session *s, int id, tm_colony_info *st);

/* A fence after the work queued so far (session stream and the copy stream
 * of asynchronous downloads): tm_session_wait blocks until it is done.  A
 * host loop that waits for the fence of step k - 1 after queuing step k stays
 * one step ahead of the device, so the device never waits for the host. */
int tm_session_fence(tm_session *s, int64_t *fence);
int tm_session_wait(tm_session *s, int64_t fence);

/* Enqueue nsteps steps of every active colony on the session stream.
 * Returns without waiting; tm_session_sync waits and reports device errors. */
int tm_session_step(tm_session *s, int nsteps);
int tm_session_sync(tm_session *s);

/* Capture one step into a CUDA graph and replay it from then on (0: off). */
int tm_session_use_graph(tm_session *s, int on);

/* Diagnostics for the following steps (the session configuration's
 * `diagnostics`, switched at run time): neighbour-set fingerprints (nbhash),
 * v's candidate (vcand) and the octree walk of every cell.  Its arrays are
 * allocated on first use and not counted by tm_session_bytes. */
int tm_session_set_diagnostics(tm_session *s, int on);
/* With diagnostics on, every following step records the neighbours within h
 * of the sampled cells (caller indices cells[0..ncells) of colony id) as the
 * pair kernels decide them: up to lcap caller indices per cell.  ncells = 0
 * ends the sampling. */
int tm_colony_sample_neighbours(tm_session *s, int id, const int64_t *cells, int64_t ncells, int lcap);
/* The sampled lists of the last step: counts[k] neighbours within h of
 * cells[k] (more than lcap: only lcap were kept), their caller indices at
 * lists[k * lcap + q], q < min(counts[k], lcap), in no particular order. */
int tm_colony_read_neighbours(tm_session *s, int id, int32_t *counts, int32_t *lists);

/* Per-phase timing with CUDA events on the session stream: phase 0 build,
 * 1 search / list-build passes, 2 list passes, 3 overflow searches and the
 * FP64 density fix-up, 4 octree walk, 5 update, 6 CIC.  ms[k] = mean per
 * step since profiling was switched on (k < nphase <= 7). */
int tm_session_profile(tm_session *s, int on);
int tm_session_profile_read(tm_session *s, double *ms, int nphase, int64_t *steps);

/* Device timer on the session stream: op 0 records the start event; op 1
 * records the stop event, waits for it and writes the elapsed milliseconds. */
int tm_session_timer(tm_session *s, int op, double *ms);

/* Number of kernels the session has launched (graph replays included). */
int64_t tm_session_launches(tm_session *s);

/* Page-lock caller memory so host<->device copies run at full speed
 * (cudaHostRegister); tm_host_unregister undoes it. */
int tm_host_register(void *ptr, int64_t bytes);
int tm_host_unregister(void *ptr);

/* Grid -> cell gather: patches_applyenv2cells (patches.c:512-593) at one
 * rank, on device arrays.  data holds nfields fields of the grid (gsize[0] x
 * gsize[1] x gsize[2] nodes, x-major, z fastest; gsize[2] = 1 in 2-D),
 * gradient three values per node and field (fieldgradient.c layout);
 * cellenv receives, per field f and cell c, cellenvdata_t {value, gx, gy, gz}
 * at cellenv[(f*n + c)*4].  Corners outside the grid are skipped as in the
 * reference; results match its FP64 roundings bit for bit. */
int tm_env2cells(const double *x, const double *y, const double *z, int64_t n, int dimension,
                 const double lower[3], float resolution, const int64_t gsize[3], int nfields,
                 const double *data, const double *gradient, double *cellenv, void *stream);
/* Field gradient: fieldgradient_compute (fieldgradient.c:149-225) at one rank
 * on device arrays: central differences (u[i+1] - u[i-1]) / resolution inside,
 * one-sided differences on the faces, 0 along an axis of one node. */
int tm_field_gradient(const double *data, const int64_t gsize[3], float resolution, int nfields,
                      double *gradient, void *stream);
/* Implicit diffusion step: environment_compute (environment.c:131-523) at one
 * rank on device fields (nfields x gsize[0] x gsize[1] x gsize[2], x-major, z
 * fastest, as environment_t.data).  Per field: z = dc * gfdt / (res * res)
 * (res * res in float), the operator (1 + 6 z + lambda gfdt) u_i - z * (the
 * in-grid neighbours), and as many solves per step as environment_initsystem
 * picks from secondsperstep / gfdt (environment.c:144-164), each of
 * A u = u + z bc (once per grid face the node lies on) + source, starting
 * from data, which receives the result.  source: device, same layout, or
 * NULL.  Each solve reaches a relative FP64 residual |b - A u| / |b| <= tol
 * (the reference asks its Hypre PCG for 1e-12) by iterative refinement: FP64
 * residuals, FP32 corrections by preconditioned conjugate gradients (a
 * geometric multigrid V-cycle preconditions stiff operators). */
typedef struct tm_diffusion tm_diffusion;
typedef struct tm_diffusion_stats {
    int solves_per_field;          /* numberofiters */
    int iterations;                /* FP32 CG iterations over all solves */
    int max_iterations;            /* of one solve */
    int refinements;               /* FP64 residual corrections over all solves */
    int multigrid_fields;          /* fields solved with the multigrid preconditioner */
    int levels;                    /* multigrid levels of the grid */
    double max_relative_residual;  /* largest final |b - A u| / |b| */
} tm_diffusion_stats;
/* A solver for grids of gsize nodes (its work vectors and multigrid levels
 * are allocated once). */
int tm_diffusion_create(tm_diffusion **d, const int64_t gsize[3], int device);
int tm_diffusion_destroy(tm_diffusion *d);
int tm_diffusion_levels(const tm_diffusion *d);
/* One step on data (host parameters dc, bc, lambda: nfields each).  Runs on
 * stream; the host waits for each CG iteration's residual norm. */
int tm_diffusion_step(tm_diffusion *d, double *data, float resolution, int nfields, const double *dc,
                      const double *bc, const double *lambda, float secondsperstep, float gfdt, const double *source,
                      double tol, tm_diffusion_stats *stats, void *stream);
/* The same with a solver made and released for the call. */
int tm_field_diffuse(double *data, const int64_t gsize[3], float resolution, int nfields, const double *dc,
                     const double *bc, const double *lambda, float secondsperstep, float gfdt, const double *source,
                     double tol, tm_diffusion_stats *stats, void *stream);
/* The gather for the cells of a session colony, written to host memory in
 * the caller's cell order (cellenv as above, n = the colony's cells); data
 * and gradient are device arrays of the grid described by lower, resolution
 * and gsize. */
int tm_colony_env2cells(tm_session *s, int id, const double lower[3], float resolution, const int64_t gsize[3],
                        int nfields, const double *data, const double *gradient, double *cellenv);

/* writevtk (io.c:372-516) at one rank for a session colony: writes the
 * reference's legacy binary VTK file (big-endian float positions, cell type,
 * rank, cell type index, the density constant 1.0, float forces of the last
 * step) to path, cells in the caller's order; the file image is assembled on
 * the device. */
int tm_colony_write_vtk(tm_session *s, int id, const char *path, int rank);

/* No counterpart in the reference.  CIC deposit of n cells onto field 0 of a
 * grid, the work of patches_alloc + patches_cells2envinfo at one rank, for
 * callers that cannot allocate device memory: code running while a CUDA
 * graph is captured, host programs with a fixed device-memory budget, or
 * real-time loops where an allocation may block.  Every input and output is
 * the caller's device memory: x, y, z (double), phase (int) in caller order;
 * grid (double, gsize[0]*gsize[1]*gsize[2], x-major with z fastest), zeroed
 * and then deposited; corners (int64[6]: lower x,y,z then upper x,y,z of the
 * touched nodes).  The call is asynchronous on `stream` (a cudaStream_t, 0
 * for the default stream) and allocates nothing: its scratch is a fixed
 * 3 MiB array in device memory, held by every GPU that loads the library
 * until the process exits, which limits n to 16,777,216 cells (larger n
 * returns TM_EINVAL).  The first call on a device, and the first call after
 * its context was created anew (after cudaDeviceReset, or in another
 * context), looks up that array's address; make it before any stream
 * capture.  Only this call's own launch failures are reported (TM_ECUDA);
 * an error left by earlier work stays for its owner to read.  All calls share the array,
 * so calls that overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller. */
int tm_cic_deposit_noalloc(const double *x, const double *y, const double *z, const int *phase, int64_t n,
                           int dimension, const double lower[3], float resolution, const int64_t gsize[3],
                           double *grid, int64_t *corners, void *stream);

/* Slots and memory still free (admission control). */
int tm_session_capacity(tm_session *s, int64_t *free_slots, int64_t *free_bins, int *free_colonies);

#ifdef __cplusplus
}
#endif
#endif
