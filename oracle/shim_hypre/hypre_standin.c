/* Test infrastructure: the stand-in behind hypre_standin.h.  One part, one box;
 * per variable a dense array of stencil coefficients (box order, x fastest,
 * stencil entries innermost) and dense vectors.  The PCG "solve" is plain
 * conjugate gradients run to a relative residual of 1e-15 (or until the
 * residual stops falling), i.e. the solution the reference's Krylov solver
 * approximates to its tolerance; tolerance and iteration cap are recorded,
 * not used. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "hypre_standin.h"

#define HS_MAXV 16

struct hs_grid { int lo[3], hi[3], n[3], nvars; };
struct hs_stencil { int size, off[32][3]; };
struct hs_graph { struct hs_grid *g; struct hs_stencil *st[HS_MAXV]; };
struct hs_matrix { struct hs_graph *gr; double *c[HS_MAXV]; };
struct hs_vector { struct hs_grid *g; double *v[HS_MAXV]; };
struct hs_solver { double tol; int maxiter; };

static struct hs_matrix *g_A;
static struct hs_vector *g_b, *g_x;
static double g_tol;
static int g_maxiter, g_nsolves, g_last_iters;

static long long npts(const struct hs_grid *g) { return (long long)g->n[0] * g->n[1] * g->n[2]; }

static long long node(const struct hs_grid *g, int i, int j, int k)
{
    return (long long)(i - g->lo[0]) + (long long)g->n[0] * ((j - g->lo[1]) + (long long)g->n[1] * (k - g->lo[2]));
}

HYPRE_Int HYPRE_SStructGridCreate(MPI_Comm comm, HYPRE_Int ndim, HYPRE_Int nparts, HYPRE_SStructGrid *grid)
{
    (void)comm; (void)ndim; (void)nparts;
    *grid = (struct hs_grid *)calloc(1, sizeof(struct hs_grid));
    return 0;
}

HYPRE_Int HYPRE_SStructGridSetExtents(HYPRE_SStructGrid grid, HYPRE_Int part, HYPRE_Int *ilower, HYPRE_Int *iupper)
{
    (void)part;
    for (int d = 0; d < 3; d++) {
        grid->lo[d] = ilower[d];
        grid->hi[d] = iupper[d];
        grid->n[d] = iupper[d] - ilower[d] + 1;
    }
    return 0;
}

HYPRE_Int HYPRE_SStructGridSetVariables(HYPRE_SStructGrid grid, HYPRE_Int part, HYPRE_Int nvars,
                                        HYPRE_SStructVariable *vartypes)
{
    (void)part; (void)vartypes;
    grid->nvars = nvars;
    return 0;
}

HYPRE_Int HYPRE_SStructGridAssemble(HYPRE_SStructGrid grid) { (void)grid; return 0; }

HYPRE_Int HYPRE_SStructStencilCreate(HYPRE_Int ndim, HYPRE_Int size, HYPRE_SStructStencil *stencil)
{
    (void)ndim;
    *stencil = (struct hs_stencil *)calloc(1, sizeof(struct hs_stencil));
    (*stencil)->size = size;
    return 0;
}

HYPRE_Int HYPRE_SStructStencilSetEntry(HYPRE_SStructStencil stencil, HYPRE_Int entry, HYPRE_Int *offset,
                                       HYPRE_Int var)
{
    (void)var;
    for (int d = 0; d < 3; d++) stencil->off[entry][d] = offset[d];
    return 0;
}

HYPRE_Int HYPRE_SStructGraphCreate(MPI_Comm comm, HYPRE_SStructGrid grid, HYPRE_SStructGraph *graph)
{
    (void)comm;
    *graph = (struct hs_graph *)calloc(1, sizeof(struct hs_graph));
    (*graph)->g = grid;
    return 0;
}

HYPRE_Int HYPRE_SStructGraphSetObjectType(HYPRE_SStructGraph graph, HYPRE_Int type) { (void)graph; (void)type; return 0; }

HYPRE_Int HYPRE_SStructGraphSetStencil(HYPRE_SStructGraph graph, HYPRE_Int part, HYPRE_Int var,
                                       HYPRE_SStructStencil stencil)
{
    (void)part;
    graph->st[var] = stencil;
    return 0;
}

HYPRE_Int HYPRE_SStructGraphAssemble(HYPRE_SStructGraph graph) { (void)graph; return 0; }

HYPRE_Int HYPRE_SStructMatrixCreate(MPI_Comm comm, HYPRE_SStructGraph graph, HYPRE_SStructMatrix *matrix)
{
    (void)comm;
    struct hs_matrix *m = (struct hs_matrix *)calloc(1, sizeof(struct hs_matrix));
    m->gr = graph;
    for (int v = 0; v < graph->g->nvars; v++)
        m->c[v] = (double *)calloc((size_t)(npts(graph->g) * graph->st[v]->size), sizeof(double));
    *matrix = m;
    g_A = m;
    return 0;
}

HYPRE_Int HYPRE_SStructMatrixSetObjectType(HYPRE_SStructMatrix matrix, HYPRE_Int type) { (void)matrix; (void)type; return 0; }
HYPRE_Int HYPRE_SStructMatrixInitialize(HYPRE_SStructMatrix matrix) { (void)matrix; return 0; }

static void matrix_box(HYPRE_SStructMatrix m, HYPRE_Int *lo, HYPRE_Int *hi, int var, int ne, const HYPRE_Int *ent,
                       const double *val, int add)
{
    const struct hs_grid *g = m->gr->g;
    const int size = m->gr->st[var]->size;
    long long q = 0;
    for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++, q++) {
                double *c = m->c[var] + node(g, i, j, k) * size;
                for (int e = 0; e < ne; e++) {
                    if (add) c[ent[e]] += val[q * ne + e];
                    else c[ent[e]] = val[q * ne + e];
                }
            }
}

HYPRE_Int HYPRE_SStructMatrixSetBoxValues(HYPRE_SStructMatrix matrix, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Int nentries, HYPRE_Int *entries,
                                          HYPRE_Complex *values)
{
    (void)part;
    matrix_box(matrix, ilower, iupper, var, nentries, entries, values, 0);
    return 0;
}

HYPRE_Int HYPRE_SStructMatrixAddToBoxValues(HYPRE_SStructMatrix matrix, HYPRE_Int part, HYPRE_Int *ilower,
                                            HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Int nentries,
                                            HYPRE_Int *entries, HYPRE_Complex *values)
{
    (void)part;
    matrix_box(matrix, ilower, iupper, var, nentries, entries, values, 1);
    return 0;
}

HYPRE_Int HYPRE_SStructMatrixAssemble(HYPRE_SStructMatrix matrix) { (void)matrix; return 0; }

HYPRE_Int HYPRE_SStructMatrixGetObject(HYPRE_SStructMatrix matrix, void **object)
{
    *object = matrix;
    return 0;
}

HYPRE_Int HYPRE_SStructVectorCreate(MPI_Comm comm, HYPRE_SStructGrid grid, HYPRE_SStructVector *vector)
{
    (void)comm;
    struct hs_vector *v = (struct hs_vector *)calloc(1, sizeof(struct hs_vector));
    v->g = grid;
    for (int q = 0; q < grid->nvars; q++) v->v[q] = (double *)calloc((size_t)npts(grid), sizeof(double));
    *vector = v;
    /* environment_initboundary creates b, then x */
    if (!g_b || g_x) {
        g_b = v;
        g_x = NULL;
    } else {
        g_x = v;
    }
    return 0;
}

HYPRE_Int HYPRE_SStructVectorSetObjectType(HYPRE_SStructVector vector, HYPRE_Int type) { (void)vector; (void)type; return 0; }
HYPRE_Int HYPRE_SStructVectorInitialize(HYPRE_SStructVector vector) { (void)vector; return 0; }

static void vector_box(HYPRE_SStructVector v, HYPRE_Int *lo, HYPRE_Int *hi, int var, double *val, int mode)
{
    long long q = 0;
    for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++, q++) {
                double *p = v->v[var] + node(v->g, i, j, k);
                if (mode == 0) *p = val[q];
                else if (mode == 1) *p += val[q];
                else val[q] = *p;
            }
}

HYPRE_Int HYPRE_SStructVectorSetBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values)
{
    (void)part;
    vector_box(vector, ilower, iupper, var, values, 0);
    return 0;
}

HYPRE_Int HYPRE_SStructVectorAddToBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                            HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values)
{
    (void)part;
    vector_box(vector, ilower, iupper, var, values, 1);
    return 0;
}

HYPRE_Int HYPRE_SStructVectorGetBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values)
{
    (void)part;
    vector_box(vector, ilower, iupper, var, values, 2);
    return 0;
}

HYPRE_Int HYPRE_SStructVectorAssemble(HYPRE_SStructVector vector) { (void)vector; return 0; }
HYPRE_Int HYPRE_SStructVectorGather(HYPRE_SStructVector vector) { (void)vector; return 0; }

HYPRE_Int HYPRE_SStructVectorGetObject(HYPRE_SStructVector vector, void **object)
{
    *object = vector;
    return 0;
}

HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm comm, HYPRE_Solver *solver)
{
    (void)comm;
    *solver = (struct hs_solver *)calloc(1, sizeof(struct hs_solver));
    return 0;
}

HYPRE_Int HYPRE_ParCSRPCGSetTol(HYPRE_Solver solver, HYPRE_Real tol)
{
    solver->tol = tol;
    g_tol = tol;
    return 0;
}

HYPRE_Int HYPRE_ParCSRPCGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level) { (void)solver; (void)level; return 0; }

HYPRE_Int HYPRE_ParCSRPCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter)
{
    solver->maxiter = max_iter;
    g_maxiter = max_iter;
    return 0;
}

HYPRE_Int HYPRE_ParCSRPCGSetPrecond(HYPRE_Solver solver, HYPRE_PtrToParSolverFcn precond,
                                    HYPRE_PtrToParSolverFcn precond_setup, HYPRE_Solver precond_solver)
{
    (void)solver; (void)precond; (void)precond_setup; (void)precond_solver;
    return 0;
}

HYPRE_Int HYPRE_ParCSRPCGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
    (void)solver; (void)A; (void)b; (void)x;
    return 0;
}

/* y = A u for variable var (neighbours outside the box contribute nothing) */
static void matvec(const struct hs_matrix *A, int var, const double *u, double *y)
{
    const struct hs_grid *g = A->gr->g;
    const struct hs_stencil *st = A->gr->st[var];
    for (int k = g->lo[2]; k <= g->hi[2]; k++)
        for (int j = g->lo[1]; j <= g->hi[1]; j++)
            for (int i = g->lo[0]; i <= g->hi[0]; i++) {
                const long long p = node(g, i, j, k);
                const double *c = A->c[var] + p * st->size;
                double s = 0.0;
                for (int e = 0; e < st->size; e++) {
                    const int a = i + st->off[e][0], b = j + st->off[e][1], d = k + st->off[e][2];
                    if (a < g->lo[0] || a > g->hi[0] || b < g->lo[1] || b > g->hi[1] || d < g->lo[2] || d > g->hi[2])
                        continue;
                    s += c[e] * u[node(g, a, b, d)];
                }
                y[p] = s;
            }
}

static double dot(const double *a, const double *b, long long n)
{
    double s = 0.0;
    for (long long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

HYPRE_Int HYPRE_ParCSRPCGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
    (void)solver;
    const long long n = npts(A->gr->g);
    double *r = (double *)malloc((size_t)n * sizeof(double)), *p = (double *)malloc((size_t)n * sizeof(double));
    double *q = (double *)malloc((size_t)n * sizeof(double));
    g_nsolves++;
    for (int var = 0; var < A->gr->g->nvars; var++) {
        double *u = x->v[var];
        const double *f = b->v[var];
        matvec(A, var, u, q);
        for (long long i = 0; i < n; i++) r[i] = f[i] - q[i];
        memcpy(p, r, (size_t)n * sizeof(double));
        const double bb = dot(f, f, n);
        double rr = dot(r, r, n), best = rr;
        int it = 0, stall = 0;
        while (rr > 1e-30 * bb && it < 100000 && stall < 50) {
            matvec(A, var, p, q);
            const double alpha = rr / dot(p, q, n);
            for (long long i = 0; i < n; i++) {
                u[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            const double rr1 = dot(r, r, n);
            for (long long i = 0; i < n; i++) p[i] = r[i] + (rr1 / rr) * p[i];
            rr = rr1;
            if (rr < best) {
                best = rr;
                stall = 0;
            } else {
                stall++;
            }
            it++;
        }
        g_last_iters = it;
    }
    free(r);
    free(p);
    free(q);
    return 0;
}

HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *solver)
{
    *solver = (struct hs_solver *)calloc(1, sizeof(struct hs_solver));
    return 0;
}

HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter) { (void)solver; (void)max_iter; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver solver, HYPRE_Real tol) { (void)solver; (void)tol; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level) { (void)solver; (void)level; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver solver, HYPRE_Int type) { (void)solver; (void)type; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver solver, HYPRE_Int type) { (void)solver; (void)type; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetNumSweeps(HYPRE_Solver solver, HYPRE_Int sweeps) { (void)solver; (void)sweeps; return 0; }
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
    (void)solver; (void)A; (void)b; (void)x;
    return 0;
}
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x)
{
    (void)solver; (void)A; (void)b; (void)x;
    return 0;
}

/* readers for the driver: the last assembled matrix (size coefficients per
 * node), right-hand side and solution of variable var, box order */
int hs_read_matrix(int var, double *out, int *size)
{
    if (!g_A) return -1;
    *size = g_A->gr->st[var]->size;
    memcpy(out, g_A->c[var], (size_t)(npts(g_A->gr->g) * *size) * sizeof(double));
    return 0;
}

int hs_read_vector(int which, int var, double *out)
{
    const struct hs_vector *v = which ? g_x : g_b;
    if (!v) return -1;
    memcpy(out, v->v[var], (size_t)npts(v->g) * sizeof(double));
    return 0;
}

void hs_info(double *tol, int *maxiter, int *nsolves, int *last_iters)
{
    *tol = g_tol;
    *maxiter = g_maxiter;
    *nsolves = g_nsolves;
    *last_iters = g_last_iters;
}

void hs_reset(void)
{
    g_A = NULL;
    g_b = g_x = NULL;
    g_nsolves = 0;
}
