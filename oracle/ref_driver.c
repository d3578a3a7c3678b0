/* Test-infrastructure driver around the reference's own hot-path functions.
 *
 * Compiled only into oracle/_ref/libtimothy_ref*.so, together with the
 * unmodified reference sources (octree.c, potential.c, cells.c, patches.c,
 * grid.c, utils.c, fieldgradient.c, io.c) and the single-rank MPI shim.  It replays the hot part of
 * the reference step loop (main.c:67-79, step.c:41-100) on structure-of-arrays
 * inputs and copies the outputs back, so tests and the CPU baseline can call
 * the reference through ctypes.  Nothing in the product links against it.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <omp.h>
#include <sys/time.h>
#include <unistd.h>

#include "global.h"
#include "potential.h"
#include "patches.h"
#include "grid.h"
#include "fieldgradient.h"
#include "io.h"
#include "cells.h"
#include "utils.h"

/* defined in octree.c with external linkage (octree.h:24-27) */
extern double3dv_t affShift;
extern double affScale;
void octbuild(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype);
void octfree(cellsinfo_t *cellsinfo);
/* cells.c:342 and patches.c:156 have no prototype in the reference headers */
void updatepositions(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo,
                     unsigned char *removecell, int64_t *removecount);
void patches_cells2envinfo(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                           cellsinfo_t *cellsinfo, grid_t *grid);
void patches_commcells2envinit(systeminfo_t systeminfo, settings_t settings, patches_t *patches);
int patches_commcells2envwait(systeminfo_t systeminfo, patches_t *patches);
int patches_applycells2env(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                           grid_t *grid, environment_t **environment);

static double wall(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

/* Size of the reference structs, for the ABI checks in the tests. */
int64_t ref_sizeof(int which)
{
    switch (which) {
    case 0: return sizeof(celldata_t);
    case 1: return sizeof(cellsinfo_t);
    case 2: return sizeof(celltype_t);
    case 3: return sizeof(systeminfo_t);
    case 4: return sizeof(settings_t);
    case 5: return sizeof(cellcommdata_t);
    case 6: return sizeof(grid_t);
    case 7: return sizeof(patches_t);
    case 8: return sizeof(octnode_t);
    case 9: return sizeof(environment_t);
    case 10: return sizeof(cellenvdata_t);
    default: return -1;
    }
}

/*
 * Run `nsteps` steps of the reference hot path.
 *
 * update_mode 0: the reference's updatepositions (x += F, cells.c:342-365);
 * update_mode 1: the harness restatement x += dt*F with the same removal rule;
 * update_mode 2: no position update.
 * The density/v/mindist/force outputs are those of the last step, computed
 * before its position update; x/y/z return the positions after all steps.
 * With do_cic the CIC deposit of the last step (field 0 of
 * environment[0].production, grid.c:37-136 geometry at one rank) is copied to
 * grid_out (x-major, z fastest) when grid_cap is large enough.
 * timing[0..4] accumulate seconds for octbuild, computepotential,
 * computegradient, position update and CIC.
 */
int ref_run(int64_t n, int dim, int ntypes,
            const double *th, const double *th2, const double *th3, const double *th4,
            const double *tsize, const float *trandommove,
            double *x, double *y, double *z, const double *size, const float *young,
            const int *ctype, const int *phase,
            int nsteps, int update_mode, double dt,
            double *density, double *v, double *mindist,
            double *fx, double *fy, double *fz,
            unsigned char *removecell, int64_t *removecount,
            int64_t *octsize, double *aff,
            int do_cic, float gfh, double *grid_out, int64_t grid_cap, int64_t *grid_dims,
            double *timing)
{
    systeminfo_t si;
    settings_t st;
    cellsinfo_t ci;
    celltype_t *ct;
    cellcommdata_t cc;
    grid_t grid;
    environment_t *env = NULL;
    int64_t i;
    int s, t;

    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&ci, 0, sizeof(ci));
    memset(&cc, 0, sizeof(cc));
    memset(&grid, 0, sizeof(grid));
    si.rank = 0;
    si.size = 1;
    si.nthreads = omp_get_max_threads();
    si.dim[0] = si.dim[1] = si.dim[2] = 1;
    si.coords = (int **)malloc(sizeof(int *));
    si.coords[0] = (int *)calloc(3, sizeof(int));

    st.dimension = dim;
    st.numberofcelltypes = ntypes;
    st.numberoffields = do_cic ? 1 : 0;
    st.gfh = gfh;
    st.maxlocalcells = n > 0 ? n : 1;

    ct = (celltype_t *)calloc((size_t)ntypes, sizeof(celltype_t));
    for (t = 0; t < ntypes; t++) {
        ct[t].h = th[t];
        ct[t].h2 = th2[t];
        ct[t].h3 = th3[t];
        ct[t].h4 = th4[t];
        ct[t].size = tsize[t];
        ct[t].randommove = trandommove ? trandommove[t] : 0.0f;
    }

    ci.dimension = dim;
    ci.localcount.n = (uint64_t)n;
    ci.cells = (celldata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(celldata_t));
    ci.forces = (double3dv_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(double3dv_t));
    for (i = 0; i < n; i++) {
        ci.cells[i].x = x[i];
        ci.cells[i].y = y[i];
        ci.cells[i].z = z[i];
        ci.cells[i].size = size[i];
        ci.cells[i].young = young[i];
        ci.cells[i].ctype = ctype[i];
        ci.cells[i].phase = phase ? phase[i] : 1;
        ci.cells[i].gid = (int)i;
    }
    for (i = 0; i < n; i++) removecell[i] = 0;
    *removecount = 0;

    if (do_cic) {
        allocategrid(si, st, &grid);
        env = (environment_t *)calloc(1, sizeof(environment_t));
        env[0].production = (double *)calloc((size_t)(grid.localsize.x * grid.localsize.y * grid.localsize.z),
                                             sizeof(double));
        grid_dims[0] = grid.localsize.x;
        grid_dims[1] = grid.localsize.y;
        grid_dims[2] = grid.localsize.z;
    }

    for (s = 0; s < nsteps; s++) {
        patches_t patches;
        double t0 = wall();
        octbuild(si, &ci, ct);
        double t1 = wall();
        if (do_cic) {
            patches_alloc(si, st, &patches, &ci, &grid);
            patches_cells2envinit(si, st, &patches, &ci, &grid);
        }
        double t2 = wall();
        computepotential(si, &ci, ct, cc);
        double t3 = wall();
        if (do_cic) {
            patches_cells2envwait(si, st, &patches, &grid, &env);
            patches_free(&patches);
        }
        double t4 = wall();
        computegradient(si, &ci, ct, cc);
        double t5 = wall();
        if (update_mode == 0) {
            updatepositions(st, ct, &ci, removecell, removecount);
        } else if (update_mode == 1) {
            for (i = 0; i < n; i++) {
                celldata_t *c = &ci.cells[i];
                c->x += dt * ci.forces[i].x;
                c->y += dt * ci.forces[i].y;
                if (dim == 3) c->z += dt * ci.forces[i].z;
                if ((c->x - c->size <= -BOXSIZEX / 2.0 || c->x + c->size >= BOXSIZEX / 2.0 ||
                     c->y - c->size <= -BOXSIZEY / 2.0 || c->y + c->size >= BOXSIZEY / 2.0 ||
                     (dim == 3 && (c->z - c->size <= -BOXSIZEZ / 2.0 || c->z + c->size >= BOXSIZEZ / 2.0))) &&
                    removecell[i] == 0) {
                    removecell[i] = 1;
                    (*removecount)++;
                }
            }
        }
        double t6 = wall();
        if (octsize) *octsize = ci.octsize;
        octfree(&ci);
        if (timing) {
            timing[0] += t1 - t0;
            timing[1] += t3 - t2;
            timing[2] += t5 - t4;
            timing[3] += t6 - t5;
            timing[4] += (t2 - t1) + (t4 - t3);
        }
    }

    for (i = 0; i < n; i++) {
        x[i] = ci.cells[i].x;
        y[i] = ci.cells[i].y;
        z[i] = ci.cells[i].z;
        if (density) density[i] = ci.cells[i].density;
        if (v) v[i] = ci.cells[i].v;
        if (mindist) mindist[i] = ci.cells[i].mindist;
        if (fx) fx[i] = ci.forces[i].x;
        if (fy) fy[i] = ci.forces[i].y;
        if (fz) fz[i] = ci.forces[i].z;
    }
    if (aff) {
        aff[0] = affShift.x;
        aff[1] = affShift.y;
        aff[2] = affShift.z;
        aff[3] = affScale;
    }
    if (do_cic) {
        int64_t g = grid.localsize.x * grid.localsize.y * grid.localsize.z;
        if (grid_out && grid_cap >= g) memcpy(grid_out, env[0].production, (size_t)g * sizeof(double));
        free(env[0].production);
        free(env);
        free(grid.loweridx);
        free(grid.upperidx);
        free(grid.lowleftnear);
        free(grid.uprightfar);
    }
    free(ci.cells);
    free(ci.forces);
    free(ct);
    free(si.coords[0]);
    free(si.coords);
    return 0;
}

/* Grid-to-cell gather (step.c:84-86: patches_env2cellsinit and
 * patches_env2cellswait, patches.c:380-416, 512-593, 643-657) at one rank:
 * the patch geometry comes from patches_alloc and the cell-to-grid exchange
 * that precedes it in the step (step.c:46-47, 58-59).  data holds nfields
 * fields of the grid (x-major, z fastest), gradient 3 values per node and
 * field; cellenv receives cellenvdata_t[f][c] = {value, gx, gy, gz}.  Returns
 * the number of grid nodes per field, or -1 when cap_nodes is too small. */
int64_t ref_env2cells(int64_t n, int dim, const double *x, const double *y, const double *z, const int *phase,
                      float gfh, int nfields, const double *data, const double *gradient, int64_t cap_nodes,
                      double *cellenv)
{
    systeminfo_t si;
    settings_t st;
    cellsinfo_t ci;
    grid_t grid;
    patches_t patches;
    cellenvdata_t **ce = NULL;
    environment_t *env;
    int64_t i, g;
    int f;

    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&ci, 0, sizeof(ci));
    memset(&grid, 0, sizeof(grid));
    si.rank = 0;
    si.size = 1;
    si.nthreads = omp_get_max_threads();
    si.dim[0] = si.dim[1] = si.dim[2] = 1;
    si.coords = (int **)malloc(sizeof(int *));
    si.coords[0] = (int *)calloc(3, sizeof(int));
    st.dimension = dim;
    st.numberoffields = nfields;
    st.gfh = gfh;
    st.maxlocalcells = n > 0 ? n : 1;
    st.step = 1;

    allocategrid(si, st, &grid);
    g = grid.localsize.x * grid.localsize.y * grid.localsize.z;
    if (g > cap_nodes) return -1;

    ci.dimension = dim;
    ci.localcount.n = (uint64_t)n;
    ci.cells = (celldata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(celldata_t));
    for (i = 0; i < n; i++) {
        ci.cells[i].x = x[i];
        ci.cells[i].y = y[i];
        ci.cells[i].z = z[i];
        ci.cells[i].phase = phase ? phase[i] : 1;
    }
    env = (environment_t *)calloc((size_t)nfields, sizeof(environment_t));
    for (f = 0; f < nfields; f++) {
        env[f].data = (double *)data + (size_t)f * (size_t)g;
        env[f].gradient = (double *)gradient + (size_t)f * 3 * (size_t)g;
        env[f].production = (double *)calloc((size_t)g, sizeof(double));
    }

    patches_alloc(si, st, &patches, &ci, &grid);
    patches_cells2envinit(si, st, &patches, &ci, &grid);
    patches_cells2envwait(si, st, &patches, &grid, &env);
    patches_env2cellsinit(si, st, &patches, &grid, &env);
    patches_env2cellswait(si, st, &patches, &ci, &grid, &ce);
    patches_free(&patches);

    for (f = 0; f < nfields; f++) {
        for (i = 0; i < n; i++) {
            double *o = cellenv + ((size_t)f * (size_t)n + (size_t)i) * 4;
            o[0] = ce[f][i].value;
            o[1] = ce[f][i].gx;
            o[2] = ce[f][i].gy;
            o[3] = ce[f][i].gz;
        }
        free(ce[f]);
        free(env[f].production);
    }
    free(ce);
    free(env);
    free(ci.cells);
    free(grid.loweridx);
    free(grid.upperidx);
    free(grid.lowleftnear);
    free(grid.uprightfar);
    free(si.coords[0]);
    free(si.coords);
    return g;
}

/* Field gradient of fieldgradient.c:149-225 (through fieldgradient(),
 * fieldgradient.c:253-272) at one rank on the grid of the given resolution;
 * data holds nfields fields, gradient receives 3 values per node and field.
 * Returns the nodes per field (dims[3] filled), or -1 when cap_nodes is too
 * small. */
int64_t ref_fieldgradient(int dim, float gfh, int nfields, const double *data, int64_t cap_nodes, double *gradient,
                          int64_t *dims)
{
    systeminfo_t si;
    settings_t st;
    grid_t grid;
    environment_t *env;
    int64_t g;
    int f;

    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&grid, 0, sizeof(grid));
    si.rank = 0;
    si.size = 1;
    si.dim[0] = si.dim[1] = si.dim[2] = 1;
    si.coords = (int **)malloc(sizeof(int *));
    si.coords[0] = (int *)calloc(3, sizeof(int));
    st.dimension = dim;
    st.numberoffields = nfields;
    st.gfh = gfh;
    allocategrid(si, st, &grid);
    g = grid.localsize.x * grid.localsize.y * grid.localsize.z;
    dims[0] = grid.localsize.x;
    dims[1] = grid.localsize.y;
    dims[2] = grid.localsize.z;
    if (g > cap_nodes) return -1;
    env = (environment_t *)calloc((size_t)nfields, sizeof(environment_t));
    for (f = 0; f < nfields; f++) {
        env[f].data = (double *)data + (size_t)f * (size_t)g;
        env[f].gradient = gradient + (size_t)f * 3 * (size_t)g;
    }
    fieldgradient(si, st, &env, &grid);
    free(env);
    free(grid.loweridx);
    free(grid.upperidx);
    free(grid.lowleftnear);
    free(grid.uprightfar);
    free(si.coords[0]);
    free(si.coords);
    return g;
}

/* writevtk (io.c:372-516) at one rank for cells in caller order: writes
 * <dir>/vtk/step<step>.vtk (the reference's file name, relative to the
 * working directory, so the driver runs it from dir).  Returns 0 or -1. */
int ref_write_vtk(const char *dir, int step, int64_t n, const double *x, const double *y, const double *z,
                  const int *ctype, const double *fx, const double *fy, const double *fz)
{
    systeminfo_t si;
    settings_t st;
    cellsinfo_t ci;
    char cwd[4096];
    int64_t i;
    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&ci, 0, sizeof(ci));
    si.rank = 0;
    si.size = 1;
    si.endian = 1;      /* little-endian host: the file is big-endian (checkendiannes) */
    st.step = step;
    ci.localcount.n = (uint64_t)n;
    ci.globalcount.n = (uint64_t)n;
    ci.cellsperproc = (uint64_t *)calloc(1, sizeof(uint64_t));
    ci.cellsperproc[0] = (uint64_t)n;
    ci.cells = (celldata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(celldata_t));
    ci.forces = (double3dv_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(double3dv_t));
    for (i = 0; i < n; i++) {
        ci.cells[i].x = x[i];
        ci.cells[i].y = y[i];
        ci.cells[i].z = z[i];
        ci.cells[i].ctype = ctype[i];
        ci.forces[i].x = fx[i];
        ci.forces[i].y = fy[i];
        ci.forces[i].z = fz[i];
    }
    if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return -1;
    writevtk(si, st, ci);
    int rc = chdir(cwd);
    free(ci.cells);
    free(ci.forces);
    free(ci.cellsperproc);
    return rc == 0 ? 0 : -1;
}

/* cellsdeath (cells.c:290-336) on cells tagged by their index: returns the
 * new cell count and writes the surviving tags in their new order.  oldlnc
 * is the count before the step's appends; n the count with them. */
int64_t ref_cellsdeath(int64_t n, int64_t oldlnc, const unsigned char *removecell, int64_t removecount,
                       int64_t globalcount, int64_t *order)
{
    cellsinfo_t ci;
    int64_t i;
    memset(&ci, 0, sizeof(ci));
    ci.localcount.n = (uint64_t)n;
    ci.globalcount.n = (uint64_t)globalcount;
    ci.localtypecount = (cellcount_t *)calloc(1, sizeof(cellcount_t));
    ci.cells = (celldata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(celldata_t));
    for (i = 0; i < n; i++) {
        ci.cells[i].gid = (ZOLTAN_ID_TYPE)i;
        ci.cells[i].phase = 1;
    }
    cellsdeath((int)oldlnc, &ci, (unsigned char *)removecell, removecount);
    for (i = 0; i < (int64_t)ci.localcount.n; i++) order[i] = (int64_t)ci.cells[i].gid;
    int64_t m = (int64_t)ci.localcount.n;
    free(ci.cells);
    free(ci.localtypecount);
    return m;
}

/* updatecellcycles (cells.c:370-523), with mitosis (cells.c:124-205), on
 * structure-of-arrays cells, after srand(seed).  The arrays hold room for
 * cap cells: daughters are appended at [n, *nout).  mitosis reads
 * cellsinfo->velocity (cells.c:134) only to overwrite the value, so a zeroed
 * array stands in for the one the reference never allocates. */
int updatecellcycles(systeminfo_t systeminfo, settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo,
                     cellenvdata_t **cellenvdata, unsigned char *removecell, int64_t *removecount);

int ref_cellcycle(int64_t n, int dim, int ntypes, const float *tg1, const float *ts, const float *tg2,
                  const float *tm, const float *tv, const float *trd, const float *tcd, const double *tsize,
                  int nfields, const float *cl1, const float *cl2, int simulationstart, float sps, unsigned seed,
                  const double *envvalue, int *phase, float *phasetime, float *g1, float *s, float *g2, float *m,
                  int *age, double *size, float *young, double *x, double *y, double *z, double *density, int *ctype,
                  unsigned char *removecell, int64_t *removecount, int64_t cap, int64_t *nout)
{
    systeminfo_t si;
    settings_t st;
    cellsinfo_t ci;
    celltype_t *ct = (celltype_t *)calloc((size_t)ntypes, sizeof(celltype_t));
    cellenvdata_t **ce = (cellenvdata_t **)calloc((size_t)(nfields > 0 ? nfields : 1), sizeof(cellenvdata_t *));
    int64_t i;
    int t, f;
    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&ci, 0, sizeof(ci));
    si.rank = 0;
    si.size = 1;
    st.dimension = dim;
    st.numberoffields = nfields;
    st.numberofcelltypes = ntypes;
    st.simulationstart = simulationstart;
    st.secondsperstep = sps;
    st.maxlocalcells = cap;
    for (t = 0; t < ntypes; t++) {
        ct[t].g1 = tg1[t];
        ct[t].s = ts[t];
        ct[t].g2 = tg2[t];
        ct[t].m = tm[t];
        ct[t].v = tv[t];
        ct[t].rd = trd[t];
        ct[t].criticaldensity = tcd[t];
        ct[t].size = tsize[t];
        ct[t].criticallevel1 = (float *)cl1 + (size_t)t * (size_t)nfields;
        ct[t].criticallevel2 = (float *)cl2 + (size_t)t * (size_t)nfields;
    }
    for (f = 0; f < nfields; f++) {
        ce[f] = (cellenvdata_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(cellenvdata_t));
        for (i = 0; i < n; i++) ce[f][i].value = envvalue[(size_t)f * (size_t)n + (size_t)i];
    }
    ci.dimension = dim;
    ci.localcount.n = (uint64_t)n;
    ci.globalcount.n = (uint64_t)n;
    ci.localtypecount = (cellcount_t *)calloc((size_t)ntypes, sizeof(cellcount_t));
    ci.cells = (celldata_t *)calloc((size_t)cap, sizeof(celldata_t));
    ci.velocity = (double3dv_t *)calloc((size_t)cap, sizeof(double3dv_t));
    for (i = 0; i < n; i++) {
        celldata_t *c = &ci.cells[i];
        c->phase = phase[i];
        c->phasetime = phasetime[i];
        c->g1 = g1[i];
        c->s = s[i];
        c->g2 = g2[i];
        c->m = m[i];
        c->age = age[i];
        c->size = size[i];
        c->young = young[i];
        c->x = x[i];
        c->y = y[i];
        c->z = z[i];
        c->density = density[i];
        c->ctype = ctype[i];
        c->gid = (ZOLTAN_ID_TYPE)i;
    }
    srand(seed);
    updatecellcycles(si, st, ct, &ci, ce, removecell, removecount);
    *nout = (int64_t)ci.localcount.n;
    for (i = 0; i < *nout; i++) {
        const celldata_t *c = &ci.cells[i];
        phase[i] = c->phase;
        phasetime[i] = c->phasetime;
        g1[i] = c->g1;
        s[i] = c->s;
        g2[i] = c->g2;
        m[i] = c->m;
        age[i] = c->age;
        size[i] = c->size;
        young[i] = c->young;
        x[i] = c->x;
        y[i] = c->y;
        z[i] = c->z;
        density[i] = c->density;
        ctype[i] = c->ctype;
    }
    for (f = 0; f < nfields; f++) free(ce[f]);
    free(ce);
    free(ci.cells);
    free(ci.velocity);
    free(ci.localtypecount);
    free(ct);
    return 0;
}

/* The reference step loop with the whole cell update (main.c:67-79,
 * step.c:41-100 without fields; cells.c:525-543 cellsupdate: random move,
 * cell cycle with mitosis, removal, global counts) for nsteps steps after
 * srand(seed), on the caller's celldata_t records (cap of them, *n in use).
 * counts holds localcount's 7 values then localtypecount's 7 per type, in
 * and out.  The velocity array mitosis reads only to overwrite the value is
 * zeroed. */
void cellsupdate(systeminfo_t systeminfo, settings_t settings, celltype_t *celltype, cellenvdata_t **cellenvdata,
                 cellsinfo_t *cellsinfo);

int ref_cellsupdate_run(void *cells, int64_t *n, int64_t cap, int dim, int ntypes, const double *th,
                        const double *th2, const double *th3, const double *th4, const double *tsize,
                        const float *trandommove, const float *tg1, const float *ts, const float *tg2,
                        const float *tm, const float *tv, const float *trd, const float *tcd, int simulationstart,
                        float sps, unsigned seed, int nsteps, uint64_t *counts)
{
    systeminfo_t si;
    settings_t st;
    cellsinfo_t ci;
    cellcommdata_t cc;
    celltype_t *ct = (celltype_t *)calloc((size_t)ntypes, sizeof(celltype_t));
    int t, s;
    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&ci, 0, sizeof(ci));
    memset(&cc, 0, sizeof(cc));
    si.rank = 0;
    si.size = 1;
    si.nthreads = omp_get_max_threads();
    si.dim[0] = si.dim[1] = si.dim[2] = 1;
    st.dimension = dim;
    st.numberofcelltypes = ntypes;
    st.numberoffields = 0;
    st.simulationstart = simulationstart;
    st.secondsperstep = sps;
    st.maxlocalcells = cap;
    st.maxcells = cap;
    for (t = 0; t < ntypes; t++) {
        ct[t].h = th[t];
        ct[t].h2 = th2[t];
        ct[t].h3 = th3[t];
        ct[t].h4 = th4[t];
        ct[t].size = tsize[t];
        ct[t].randommove = trandommove[t];
        ct[t].g1 = tg1[t];
        ct[t].s = ts[t];
        ct[t].g2 = tg2[t];
        ct[t].m = tm[t];
        ct[t].v = tv[t];
        ct[t].rd = trd[t];
        ct[t].criticaldensity = tcd[t];
    }
    ci.dimension = dim;
    ci.cells = (celldata_t *)cells;
    ci.forces = (double3dv_t *)calloc((size_t)cap, sizeof(double3dv_t));
    ci.velocity = (double3dv_t *)calloc((size_t)cap, sizeof(double3dv_t));
    ci.localtypecount = (cellcount_t *)calloc((size_t)ntypes, sizeof(cellcount_t));
    ci.cellsperproc = (uint64_t *)calloc(1, sizeof(uint64_t));
    uint64_t *lc = &ci.localcount.n;
    for (t = 0; t < 7; t++) lc[t] = counts[t];
    for (t = 0; t < ntypes; t++) {
        uint64_t *tc = &ci.localtypecount[t].n;
        for (s = 0; s < 7; s++) tc[s] = counts[7 + 7 * t + s];
    }
    updateglobalcounts(&ci);
    srand(seed);
    for (s = 0; s < nsteps; s++) {
        if (ci.localcount.n == 0) break;
        octbuild(si, &ci, ct);
        computepotential(si, &ci, ct, cc);
        computegradient(si, &ci, ct, cc);
        cellsupdate(si, st, ct, NULL, &ci);
        octfree(&ci);
    }
    *n = (int64_t)ci.localcount.n;
    for (t = 0; t < 7; t++) counts[t] = lc[t];
    for (t = 0; t < ntypes; t++) {
        uint64_t *tc = &ci.localtypecount[t].n;
        for (s = 0; s < 7; s++) counts[7 + 7 * t + s] = tc[s];
    }
    free(ci.forces);
    free(ci.velocity);
    free(ci.localtypecount);
    free(ci.cellsperproc);
    free(ct);
    return 0;
}
