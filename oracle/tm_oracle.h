/* CPU oracle for the Timothy cell-mechanics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (pointer octree built by insertion, per-cell depth-first walk,
 * FP64 pair maths in the reference's operation order, x += F update, CIC
 * deposit).  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it, and only as the checker or the timed CPU baseline; the GPU product
 * never calls it.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own functions
 * (compiled unmodified from its sources by oracle/Makefile into oracle/_ref),
 * and tests/test_oracle_golden.py checks this restatement against them.
 */
#ifndef TM_ORACLE_H
#define TM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Runs nsteps steps of the hot path on structure-of-arrays cells.
 *
 * Arguments mirror ref_run() in oracle/ref_driver.c so that tests can call
 * the reference and the restatement interchangeably:
 *   th..tsize, trandommove  per-type h, h2, h3, h4, size, randommove (the
 *                           celltype_t fields, global.h:315-335)
 *   update_mode             0 reference updatepositions (cells.c:342-365),
 *                           1 x += dt*F with the same removal rule, 2 none
 *   density..fz             outputs of the last step (before its update)
 *   octsize, aff            node count of the last octree, affShift/affScale
 *   do_cic, gfh, grid_out   CIC deposit of the last step into the one-rank
 *                           grid (grid.c:37-136), x-major with z fastest
 *   timing[5]               seconds spent in build, potential, gradient,
 *                           update, CIC (accumulated)
 *   nthreads                OpenMP threads (<= 0: runtime default)
 * Returns 0, or a negative code: -1 bad arguments, -2 two cells share a
 * lattice code down to the last two levels (the reference's insertion is
 * undefined there, octree.c:101-107), -3 out of memory.
 */
int tmo_run(int64_t n, int dim, int ntypes,
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
            double *timing, int nthreads);

/* One octree build plus one walk per cell, returning per-cell diagnostics:
 * nbcount/nbhash  size and order-free fingerprint (sum of tm_mix64(j+1)) of
 *                 the set {j != p : candidate, dist(p,j) <= h_p}
 * vcand           the candidate whose potential the reference assigns to v
 *                 (the last one visited, potential.c:118-125), or -1
 * ncand           number of candidates visited (leaves intersecting the box)
 * If nb_offsets/nb_list are non-NULL the neighbour lists are written in
 * visiting order (CSR; nb_list must hold nb_offsets[n] entries, which a
 * first call with nb_list == NULL returns). */
int tmo_neighbours(int64_t n, int dim, int ntypes, const double *th,
                   const double *x, const double *y, const double *z, const int *ctype,
                   int32_t *nbcount, uint64_t *nbhash, int64_t *vcand, int32_t *ncand,
                   int64_t *nb_offsets, int64_t *nb_list, int nthreads);

/* Grid -> cell gather at one rank (patches_applyenv2cells): data holds
 * nfields fields of the one-rank grid of resolution gfh (x-major, z
 * fastest), gradient 3 values per node and field; cellenv[(f*n + c)*4 + k]
 * receives cellenvdata_t {value, gx, gy, gz}.  Returns 0 or -1. */
int tmo_env2cells(int64_t n, int dim, const double *x, const double *y, const double *z, float gfh, int nfields,
                  const double *data, const double *gradient, double *cellenv);

/* Field gradient (fieldgradient_compute at one rank) of nfields fields on
 * the one-rank grid of resolution gfh; dims receives the grid size. */
int tmo_fieldgradient(int dim, float gfh, int nfields, const double *data, double *gradient, int64_t *dims);

/* updatecellcycles with mitosis on caller-ordered arrays (room for cap
 * cells), the rand() values taken from draws[]; see tm_oracle.c. */
int tmo_cellcycle(int64_t n, int dim, const float *tg1, const float *ts, const float *tg2, const float *tm,
                  const float *tv, const float *trd, const float *tcd, const double *tsize, int nfields,
                  const float *cl1, const float *cl2, int simulationstart, float sps, const double *envvalue,
                  const int *draws, int64_t ndraws_cap, int *phase, float *phasetime, float *g1, float *s, float *g2,
                  float *m, int *age, double *size, float *young, double *x, double *y, double *z, double *density,
                  int *ctype, unsigned char *removecell, int64_t *removecount, int64_t cap, int64_t *nout,
                  int64_t *ndraws);

/* writevtk at one rank: the legacy binary VTK file of the cells (caller
 * order) with their forces.  Returns 0 or a negative code. */
int tmo_write_vtk(const char *path, int64_t n, const double *x, const double *y, const double *z, const int *ctype,
                  const double *fx, const double *fy, const double *fz, int rank);

/* The fingerprint mixer shared with the GPU diagnostics (SplitMix64 final mix). */
uint64_t tm_mix64(uint64_t z);

/* The implicit diffusion step of environment_compute at one rank
 * (environment.c:131-523).  See tm_oracle.c. */
int tmo_diffusion_iters(float secondsperstep, float gfdt);
double tmo_diffusion_z(double dc, float gfdt, float resolution);
int tmo_diffuse(int64_t nx, int64_t ny, int64_t nz, float resolution, float secondsperstep, float gfdt, int step,
                int nfields, const double *dc, const double *bc, const double *mean, const double *lambda,
                const double *u0, const double *source, double tol, double *u, double *b_last, int *iters_out,
                int *cg_iters);

#ifdef __cplusplus
}
#endif
#endif
