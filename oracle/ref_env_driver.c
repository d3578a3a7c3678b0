/* Test-infrastructure driver around the reference's environment.c (the
 * implicit diffusion step, environment.c:131-523), compiled unmodified with
 * -DHYPRE against the Hypre stand-in in oracle/shim_hypre, at one rank.
 * It sets up the grid with the reference's allocategrid (grid.c:80-136), runs
 * environment_allocate, environment_initsystem and ncalls x
 * environment_compute, and reads back what the reference assembled: the
 * 7 stencil coefficients per node, the right-hand side of the last solve and
 * the solution the stand-in's solver found for it (box order: x fastest).
 * Nothing in the product links against it. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "global.h"
#include "grid.h"

void environment_allocate(systeminfo_t systeminfo, settings_t settings, grid_t grid, environment_t **environment,
                          solverdata_t *solverdata, solversettings_t *solversettings);
void environment_initsystem(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                            solverdata_t *solverdata, solversettings_t *solversettings);
void environment_compute(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                         solverdata_t *solverdata, solversettings_t *solversettings);
int hs_read_matrix(int var, double *out, int *size);
int hs_read_vector(int which, int var, double *out);
void hs_info(double *tol, int *maxiter, int *nsolves, int *last_iters);
void hs_reset(void);

/* gsize (out): the local grid; info (out): numberofiters, stand-in maxiter,
 * solves, last solve's CG iterations; z (out, nfields); tol (out).  coef,
 * b, x: nfields x G x 7, nfields x G, nfields x G.  Returns G or -1 when cap
 * (nodes) is too small. */
int64_t ref_environment(int dim, float gfh, float sps, float gfdt, int step, int nfields, const double *dc,
                        const double *bc, const double *mean, const double *lambda, int ncalls, int64_t cap,
                        int64_t *gsize, int *info, double *z, double *tol, double *coef, double *b, double *x)
{
    systeminfo_t si;
    settings_t st;
    grid_t grid;
    solverdata_t sd;
    solversettings_t ss;
    environment_t *env;
    int f, c;
    memset(&si, 0, sizeof(si));
    memset(&st, 0, sizeof(st));
    memset(&grid, 0, sizeof(grid));
    memset(&sd, 0, sizeof(sd));
    memset(&ss, 0, sizeof(ss));
    si.rank = 0;
    si.size = 1;
    si.dim[0] = si.dim[1] = si.dim[2] = 1;
    si.coords = (int **)malloc(sizeof(int *));
    si.coords[0] = (int *)calloc(3, sizeof(int));
    st.dimension = dim;
    st.gfh = gfh;
    st.gfdt = gfdt;
    st.secondsperstep = sps;
    st.numberoffields = nfields;
    st.step = step;
    allocategrid(si, st, &grid);
    const int64_t G = grid.localsize.x * grid.localsize.y * grid.localsize.z;
    gsize[0] = grid.localsize.x;
    gsize[1] = grid.localsize.y;
    gsize[2] = grid.localsize.z;
    if (G > cap) return -1;
    env = (environment_t *)calloc((size_t)nfields, sizeof(environment_t));
    for (f = 0; f < nfields; f++) {
        env[f].diffusioncoefficient = dc[f];
        env[f].boundarycondition = bc[f];
        env[f].initialconditionmean = mean[f];
        env[f].initialconditionvariance = 0.0;
        env[f].lambdadelay = lambda[f];
    }
    hs_reset();
    environment_allocate(si, st, grid, &env, &sd, &ss);
    environment_initsystem(si, st, &grid, &env, &sd, &ss);
    for (c = 0; c < ncalls; c++) environment_compute(si, st, &grid, &env, &sd, &ss);
    int size = 0, nsolves = 0, iters = 0, maxiter = 0;
    for (f = 0; f < nfields; f++) {
        hs_read_matrix(f, coef + (size_t)f * (size_t)G * 7, &size);
        hs_read_vector(0, f, b + (size_t)f * (size_t)G);
        hs_read_vector(1, f, x + (size_t)f * (size_t)G);
        z[f] = ss.z[f];
    }
    hs_info(tol, &maxiter, &nsolves, &iters);
    info[0] = ss.numberofiters;
    info[1] = maxiter;
    info[2] = nsolves;
    info[3] = iters;
    for (f = 0; f < nfields; f++) {
        free(env[f].data);
        free(env[f].production);
        free(env[f].gradient);
    }
    free(env);
    free(grid.loweridx);
    free(grid.upperidx);
    free(grid.lowleftnear);
    free(grid.uprightfar);
    free(si.coords[0]);
    free(si.coords);
    return G;
}
