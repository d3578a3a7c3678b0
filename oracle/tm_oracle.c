/* CPU oracle for the Timothy cell-mechanics hot path -- TEST INFRASTRUCTURE.
 *
 * A restatement, in plain C with OpenMP, of the reference algorithm:
 *   - octree build by sequential insertion    octree.c:40-207
 *   - query box / region location / walk      octree.c:246-316, inline.h:26-32,
 *                                             potential.c:87-138, 209-259
 *   - pair density + potential                potential.c:39-78, inline.h:40-51
 *   - pair force (SPH kernel gradient)        inline.h:59-83, potential.c:193-202
 *   - position update + removal marks         cells.c:41-58, 342-365
 *   - grid -> cell gather, field gradient     patches.c:512-593, fieldgradient.c:149-225
 *   - VTK writer                              io.c:372-516
 *   - cell cycle and mitosis                  cells.c:124-205, 370-523
 *   - CIC deposit at one rank                 grid.c:37-136, patches.c:47-234,
 *                                             patches.c:321-367
 * Expressions keep the reference's evaluation order (C left-to-right
 * associativity, no contraction: build with -ffp-contract=off) so that the
 * outputs match the reference bit for bit.  See tm_oracle.h for the API.
 */
#include "tm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TMO_ROOT_LEVEL 29            /* global.h:65-66 */
#define TMO_LATTICE 536870912.0f     /* powf(2,29), global.h:67 */
#define TMO_BOX_HALF 1024.0          /* BOXSIZE{X,Y,Z}/2.0, global.h:59-61 */

uint64_t tm_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static double tmo_wall(void)
{
    struct timeval tv;
    gettimeofday(&tv, NULL);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

/* ------------------------------------------------------------------------ */
/* octree                                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t lo[3];   /* node origin in lattice codes (xcode, ycode, zcode) */
    uint32_t hi[3];   /* exclusive limits (xlimit, ylimit, zlimit)          */
    int32_t kid[8];   /* child node index or -1                             */
    int32_t item;     /* >= 0 the one cell held, -1 empty, -2 inner node    */
} tmo_node;

typedef struct {
    tmo_node *node;
    int64_t count, cap;
    uint32_t *code;   /* 3 lattice codes per cell */
    double shift[3], scale;
} tmo_tree;

typedef struct {
    int dim;
    const double *th, *th2, *th3, *th4, *tsize;
    const double *x, *y, *z, *size;
    const float *young;
    const int *ctype;
} tmo_cells;

/* child index from one bit level of three codes: x + 2y + 4z (octree.c:101-107);
 * defined for level >= 2, the only levels a valid tree reaches */
static inline int tmo_digit(const uint32_t c[3], unsigned level)
{
    return (int)(((c[0] >> level) & 1u) | (((c[1] >> level) & 1u) << 1) | (((c[2] >> level) & 1u) << 2));
}

static int64_t tmo_newnode(tmo_tree *t, int64_t parent, int digit)
{
    if (t->count == t->cap) {
        int64_t ncap = t->cap ? 2 * t->cap : 1024;
        tmo_node *nn = (tmo_node *)realloc(t->node, (size_t)ncap * sizeof(tmo_node));
        if (!nn) return -1;
        t->node = nn;
        t->cap = ncap;
    }
    int64_t id = t->count++;
    tmo_node *d = &t->node[id];
    if (parent < 0) {                         /* octemptynode, octree.c:48-54 */
        for (int k = 0; k < 3; k++) {
            d->lo[k] = 0;
            d->hi[k] = 1u << TMO_ROOT_LEVEL;
        }
    } else {                                  /* octree.c:56-63 */
        const tmo_node *p = &t->node[parent];
        uint32_t half = (p->hi[0] - p->lo[0]) / 2;
        for (int k = 0; k < 3; k++) {
            d->lo[k] = p->lo[k] | (((uint32_t)(digit >> k) & 1u) * half);
            d->hi[k] = d->lo[k] + half;
        }
    }
    for (int k = 0; k < 8; k++) d->kid[k] = -1;
    d->item = -1;
    return id;
}

/* octinsertcell, octree.c:84-140 */
static int tmo_insert(tmo_tree *t, int64_t c)
{
    int64_t at = 0;
    unsigned level = TMO_ROOT_LEVEL - 1;
    for (;;) {
        tmo_node *nd = &t->node[at];
        if (nd->item == -1) {
            nd->item = (int32_t)c;
            return 0;
        }
        if (level < 2) return -2;             /* codes equal down to the last two bits */
        if (nd->item == -2) {
            int dg = tmo_digit(&t->code[3 * c], level);
            level--;
            int64_t ch = nd->kid[dg];
            if (ch == -1) {
                ch = tmo_newnode(t, at, dg);
                if (ch < 0) return -3;
                t->node[at].kid[dg] = (int32_t)ch;
            }
            at = ch;
        } else {                              /* occupied leaf: push its cell down one level */
            int64_t oc = nd->item;
            int dg = tmo_digit(&t->code[3 * oc], level);
            int64_t ch = tmo_newnode(t, at, dg);
            if (ch < 0) return -3;
            t->node[at].kid[dg] = (int32_t)ch;
            t->node[ch].item = (int32_t)oc;
            t->node[at].item = -2;
        }
    }
}

/* octbuild, octree.c:145-207 */
static int tmo_build(tmo_tree *t, int64_t n, const tmo_cells *cs)
{
    const double eps = 0.01;
    double bmin[3] = {DBL_MAX, DBL_MAX, DBL_MAX};
    double bmax[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    t->count = 0;
    if (n == 0) return 0;
    for (int64_t i = 0; i < n; i++) {
        double p[3] = {cs->x[i], cs->y[i], cs->z[i]};
        double e = cs->th[cs->ctype[i]] + eps;
        for (int k = 0; k < 3; k++) {
            bmin[k] = (p[k] - e < bmin[k] ? p[k] - e : bmin[k]);
            bmax[k] = (p[k] + e > bmax[k] ? p[k] + e : bmax[k]);
        }
    }
    t->scale = bmax[0] - bmin[0];
    t->scale = (t->scale > bmax[1] - bmin[1] ? t->scale : bmax[1] - bmin[1]);
    t->scale = (t->scale > bmax[2] - bmin[2] ? t->scale : bmax[2] - bmin[2]);
    for (int k = 0; k < 3; k++) t->shift[k] = bmin[k];

    free(t->code);
    t->code = (uint32_t *)malloc((size_t)n * 3 * sizeof(uint32_t));
    if (!t->code) return -3;
    for (int64_t i = 0; i < n; i++) {
        double p[3] = {cs->x[i], cs->y[i], cs->z[i]};
        for (int k = 0; k < 3; k++)
            t->code[3 * i + k] = (uint32_t)(((p[k] - t->shift[k]) / t->scale) * TMO_LATTICE);
    }
    if (tmo_newnode(t, -1, 0) < 0) return -3;
    for (int64_t i = 0; i < n; i++) {
        int rc = tmo_insert(t, i);
        if (rc) return rc;
    }
    return 0;
}

/* octcomputebox, octree.c:246-266 */
static void tmo_box(const tmo_tree *t, const tmo_cells *cs, int64_t p, uint32_t bmin[3], uint32_t bmax[3])
{
    double h = cs->th[cs->ctype[p]];
    double c[3] = {cs->x[p], cs->y[p], cs->z[p]};
    for (int k = 0; k < 3; k++) {
        double lo = (c[k] - h - t->shift[k]) / t->scale;
        double hi = (c[k] + h - t->shift[k]) / t->scale;
        bmin[k] = (uint32_t)(lo * TMO_LATTICE);
        bmax[k] = (uint32_t)(hi * TMO_LATTICE);
    }
}

/* octlocateregion + octtraversetolevel, octree.c:271-316 */
static int64_t tmo_locate(const tmo_tree *t, const uint32_t bmin[3], const uint32_t bmax[3])
{
    uint32_t dx = bmin[0] ^ bmax[0], dy = bmin[1] ^ bmax[1], dz = bmin[2] ^ bmax[2];
    unsigned l1 = TMO_ROOT_LEVEL, l2 = TMO_ROOT_LEVEL, lm = TMO_ROOT_LEVEL;
    while (!(dx & (1u << l1)) && l1) l1--;
    while (!(dy & (1u << l2)) && (l2 > l1)) l2--;
    while (!(dz & (1u << lm)) && (lm > l2)) lm--;
    lm++;
    unsigned level = TMO_ROOT_LEVEL - 1;
    unsigned steps = level - lm + 1;
    int64_t at = 0, parent = 0;
    while (steps--) {
        int dg = tmo_digit(bmin, level);
        level--;
        parent = at;
        at = t->node[at].kid[dg];
        if (at < 0) break;
        if (t->node[at].item != -2) break;   /* a leaf */
    }
    return at < 0 ? parent : at;
}

/* octnodeintersection, inline.h:26-32: half-open in the node, strict at the box top */
static inline int tmo_hits(const tmo_node *nd, const uint32_t bmin[3], const uint32_t bmax[3])
{
    for (int k = 0; k < 3; k++)
        if (bmax[k] <= nd->lo[k] || bmin[k] >= nd->hi[k]) return 0;
    return 1;
}

/* The walk of potential.c:108-133 / 227-255: the children of the located node
 * that intersect the box go on a LIFO stack; popping a leaf yields a candidate
 * cell, popping an inner node pushes its intersecting children 0..7.
 * visit(ctx, j) is called for every candidate j != p in visiting order. */
typedef void (*tmo_visit_fn)(void *ctx, int64_t j);

static int tmo_walk(const tmo_tree *t, const tmo_cells *cs, int64_t p,
                    int32_t **stack, int64_t *stack_cap, tmo_visit_fn visit, void *ctx)
{
    uint32_t bmin[3], bmax[3];
    tmo_box(t, cs, p, bmin, bmax);
    int64_t start = tmo_locate(t, bmin, bmax);
    int64_t top = 0;
#define TMO_PUSH(id)                                                                       \
    do {                                                                                   \
        if (top == *stack_cap) {                                                           \
            int64_t nc = *stack_cap ? 2 * *stack_cap : 64;                                 \
            int32_t *ns = (int32_t *)realloc(*stack, (size_t)nc * sizeof(int32_t));        \
            if (!ns) return -3;                                                            \
            *stack = ns;                                                                   \
            *stack_cap = nc;                                                               \
        }                                                                                  \
        (*stack)[top++] = (id);                                                            \
    } while (0)
    for (int s = 0; s < 8; s++) {
        int32_t id = t->node[start].kid[s];
        if (id != -1 && tmo_hits(&t->node[id], bmin, bmax)) TMO_PUSH(id);
    }
    while (top > 0) {
        int32_t id = (*stack)[--top];
        const tmo_node *nd = &t->node[id];
        if (nd->item >= 0) {
            if (nd->item != p) visit(ctx, nd->item);
        } else {
            for (int s = 0; s < 8; s++) {
                int32_t k = nd->kid[s];
                if (k != -1 && tmo_hits(&t->node[k], bmin, bmax)) TMO_PUSH(k);
            }
        }
    }
#undef TMO_PUSH
    return 0;
}

/* ------------------------------------------------------------------------ */
/* pair maths                                                                 */
/* ------------------------------------------------------------------------ */

/* sphkernel, inline.h:40-51 -- note the float return type */
static inline float tmo_kernel(int dim, double dist, double h, double h2, double h3)
{
    double u, c = 1.0;
    if (dist < 0.0) return 0.0;
    u = dist / h;
    if (dim == 2) c = 40 / (7 * M_PI * h2);
    if (dim == 3) c = 8 / (M_PI * h3);
    if (u >= 0.0 && u <= 0.5) return c * (1 - 6 * u * u + 6 * u * u * u);
    if (u > 0.5 && u <= 1.0) return c * (2 * (1 - u) * (1 - u) * (1 - u));
    return 0.0;
}

typedef struct {
    const tmo_cells *cs;
    int64_t p;
    double density, v, mindist;
    double f[3];
} tmo_acc;

/* potential(), potential.c:39-78; v takes the value of the last call */
static void tmo_visit_potential(void *vctx, int64_t j)
{
    tmo_acc *a = (tmo_acc *)vctx;
    const tmo_cells *cs = a->cs;
    int64_t p = a->p;
    int tp = cs->ctype[p];
    double h = cs->th[tp], h2 = cs->th2[tp], h3 = cs->th3[tp], csize = cs->tsize[tp];
    double poisson = 0.33;
    double dx = cs->x[p] - cs->x[j], dy = cs->y[p] - cs->y[j], dz = cs->z[p] - cs->z[j];
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    a->mindist = (dist < a->mindist ? dist : a->mindist);
    if (dist <= h) {
        double sc = (cs->dim == 2 ? h2 : h3);
        double s1 = cs->size[p], s2 = cs->size[j];
        a->density += sc * (s2 / csize) * tmo_kernel(cs->dim, dist, h, h2, h3);
        double xc = s1 + s2 - dist;
        if (xc <= 0.0) {
            a->v = 0.0;
            return;
        }
        double D = 0.75 * ((1.0 - poisson * poisson) / cs->young[p] + (1.0 - poisson * poisson / cs->young[j]));
        double r01 = (s1 * s1 - s2 * s2 + dist * dist) / (2 * dist);
        double r02 = dist - r01;
        double area = M_PI * ((s1 * s1 * (s1 - r01) - (s1 * s1 * s1 - r01 * r01 * r01) / 3) +
                              (s2 * s2 * (s2 - r02) - (s2 * s2 * s2 - r02 * r02 * r02) / 3));
        /* pow(xc, 5/2) has an integer exponent of 2 */
        a->v = (2.0 * (xc * xc) / (5.0 * D)) * sqrt((s1 * s2) / (s1 + s2)) + area * 0.1;
    } else {
        a->v = 0.0;
    }
}

/* sphgradient, inline.h:59-83, accumulated as in potential.c:241-247 */
static void tmo_visit_gradient(void *vctx, int64_t j)
{
    tmo_acc *a = (tmo_acc *)vctx;
    const tmo_cells *cs = a->cs;
    int64_t p = a->p;
    int tp = cs->ctype[p];
    double h = cs->th[tp], h3 = cs->th3[tp], h4 = cs->th4[tp];
    double u, c = 1.0, w = 1.0;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    double dx = cs->x[p] - cs->x[j], dy = cs->y[p] - cs->y[j], dz = cs->z[p] - cs->z[j];
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    if (dist >= 0.0 && dist <= h) {
        u = dist / h;
        if (cs->dim == 2) c = (40 * 8) / (7 * M_PI * h3);
        if (cs->dim == 3) c = 48 / (M_PI * h4);
        if (u >= 0.0 && u <= 0.5) w = -2.0 * u + 3.0 * u * u;
        if (u > 0.5 && u <= 1.0) w = -(1.0 - u) * (1.0 - u);
        if (u > 1.0) w = 0.0;
        fx = w * c * (cs->x[j] - cs->x[p]) / dist;
        fy = w * c * (cs->y[j] - cs->y[p]) / dist;
        if (cs->dim == 3) fz = w * c * (cs->z[j] - cs->z[p]) / dist;
    }
    a->f[0] += fx;
    a->f[1] += fy;
    a->f[2] += fz;
}

/* ------------------------------------------------------------------------ */
/* CIC deposit at one rank                                                    */
/* ------------------------------------------------------------------------ */

typedef struct {
    double lower[3];
    float res;
    int64_t size[3];   /* localsize == globalsize at one rank */
} tmo_grid;

/* computegridsize, grid.c:37-77, with dim[] = {1,1,1} */
static void tmo_grid_geometry(int dim, float gfh, tmo_grid *g)
{
    float gx, gy, gz;
    double upper[3];
    g->res = gfh;
    g->lower[0] = -2048 / 2.0;
    g->lower[1] = -2048 / 2.0;
    g->lower[2] = (dim == 3 ? -2048 / 2.0 : 0.0);
    upper[0] = 2048 / 2.0;
    upper[1] = 2048 / 2.0;
    upper[2] = (dim == 3 ? 2048 / 2.0 : 0.0);
    gx = upper[0] - g->lower[0] + 1;
    gy = upper[1] - g->lower[1] + 1;
    gz = (dim == 3 ? upper[2] - g->lower[2] + 1 : 0.0f);
    g->size[0] = (int64_t)((gx + 1) / g->res);
    g->size[1] = (int64_t)((gy + 1) / g->res);
    g->size[2] = (dim == 3 ? (int64_t)((gz + 1) / g->res) : 0);
    /* padding to a multiple of the process grid always adds dim - size % dim */
    g->size[0] += 1 - g->size[0] % 1;
    g->size[1] += 1 - g->size[1] % 1;
    if (dim == 3) g->size[2] += 1 - g->size[2] % 1;
    else g->size[2] = 1;
}

/* patches_alloc + patches_cells2envinfo + patches_applycells2env at one rank
 * (patches.c:47-234, 321-367): the patch is the bounding box of touched grid
 * nodes; its field 0 receives 0.75 (G0) or 1.0 (G1..M) times the trilinear
 * weights, necrotic cells (phase 5) add nothing; the patch is then added into
 * the zeroed grid. */
static int tmo_cic(int64_t n, int dim, const tmo_grid *g, const double *x, const double *y, const double *z,
                   const int *phase, double *grid)
{
    int64_t up[3] = {g->size[0] - 1, g->size[1] - 1, (dim == 3 ? g->size[2] - 1 : 0)};
    int64_t plo[3] = {INT32_MAX, INT32_MAX, (dim == 3 ? INT32_MAX : 0)};
    int64_t phi[3] = {INT32_MIN, INT32_MIN, (dim == 3 ? INT32_MIN : 0)};
    int any = 0;
    for (int64_t c = 0; c < n; c++) {
        int64_t ci[3];
        ci[0] = (int64_t)((x[c] - g->lower[0]) / g->res);
        ci[1] = (int64_t)((y[c] - g->lower[1]) / g->res);
        ci[2] = (int64_t)((z[c] - g->lower[2]) / g->res);
        for (int ax = 0; ax < 2; ax++)
            for (int ay = 0; ay < 2; ay++)
                for (int az = 0; az < 2; az++) {
                    int64_t a[3] = {ci[0] + ax, ci[1] + ay, ci[2] + az};
                    if (a[0] >= 0 && a[1] >= 0 && a[2] >= 0 && a[0] <= up[0] && a[1] <= up[1] && a[2] <= up[2]) {
                        plo[0] = (plo[0] > a[0] ? a[0] : plo[0]);
                        plo[1] = (plo[1] > a[1] ? a[1] : plo[1]);
                        if (dim == 3) plo[2] = (plo[2] > a[2] ? a[2] : plo[2]);
                        phi[0] = (phi[0] < a[0] ? a[0] : phi[0]);
                        phi[1] = (phi[1] < a[1] ? a[1] : phi[1]);
                        if (dim == 3) phi[2] = (phi[2] < a[2] ? a[2] : phi[2]);
                        any = 1;
                    }
                }
    }
    int64_t gtot = g->size[0] * g->size[1] * g->size[2];
    memset(grid, 0, (size_t)gtot * sizeof(double));
    if (!any) return 0;
    int64_t ps[3] = {phi[0] - plo[0] + 1, phi[1] - plo[1] + 1, (dim == 3 ? phi[2] - plo[2] + 1 : 1)};
    double *patch = (double *)calloc((size_t)(ps[0] * ps[1] * ps[2]), sizeof(double));
    if (!patch) return -3;
    for (int64_t c = 0; c < n; c++) {
        int64_t ci[3];
        double pos[3] = {x[c], y[c], z[c]};
        for (int k = 0; k < 3; k++) ci[k] = (int64_t)((pos[k] - g->lower[k]) / g->res);
        for (int ax = 0; ax < 2; ax++)
            for (int ay = 0; ay < 2; ay++)
                for (int az = 0; az < 2; az++) {
                    int64_t a[3] = {ci[0] + ax, ci[1] + ay, ci[2] + az};
                    if (!(a[0] >= 0 && a[1] >= 0 && a[2] >= 0 && a[0] <= up[0] && a[1] <= up[1] && a[2] <= up[2]))
                        continue;
                    int64_t ix = a[0] - plo[0], iy = a[1] - plo[1], iz = a[2] - plo[2];
                    double d[3], t[3];
                    for (int k = 0; k < 3; k++) {
                        /* grid->lowercorner + cellIdx * resolution: int64 * float is a float product */
                        double cic = g->lower[k] + (float)ci[k] * g->res;
                        d[k] = (pos[k] - cic) / g->res;
                        t[k] = 1.0 - d[k];
                    }
                    if (phase[c] == 5) continue;
                    double wph = (phase[c] == 0 ? 0.75 : 1.0);
                    double w = wph * (ax * d[0] + (1 - ax) * t[0]) * (ay * d[1] + (1 - ay) * t[1]) *
                               (az * d[2] + (1 - az) * t[2]);
                    patch[ps[1] * ps[2] * ix + ps[2] * iy + iz] += w;
                }
    }
    for (int64_t i = plo[0]; i <= phi[0]; i++)
        for (int64_t j = plo[1]; j <= phi[1]; j++)
            for (int64_t k = plo[2]; k <= phi[2]; k++) {
                int64_t gi = g->size[2] * g->size[1] * i + g->size[2] * j + k;
                grid[gi] += patch[ps[2] * ps[1] * (i - plo[0]) + ps[2] * (j - plo[1]) + (k - plo[2])];
            }
    free(patch);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* grid -> cell gather and field gradient at one rank                         */
/* ------------------------------------------------------------------------ */

/* patches_applyenv2cells, patches.c:512-593, at one rank: the patch holds
 * every grid node a local cell touches, so each cell gathers its in-grid
 * corners directly from the grid, in the corner order ax, ay, az and with the
 * product buff * wx * wy * wz of the reference; field values first, then the
 * three gradient components of the same corners. */
int tmo_env2cells(int64_t n, int dim, const double *x, const double *y, const double *z, float gfh, int nfields,
                  const double *data, const double *gradient, double *cellenv)
{
    tmo_grid g;
    if (n < 0 || nfields < 0 || (dim != 2 && dim != 3) || !(gfh > 0.0f)) return -1;
    tmo_grid_geometry(dim, gfh, &g);
    const int64_t up[3] = {g.size[0] - 1, g.size[1] - 1, (dim == 3 ? g.size[2] - 1 : 0)};
    const int64_t G = g.size[0] * g.size[1] * g.size[2];
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; c++) {
        const double pos[3] = {x[c], y[c], z[c]};
        int64_t ci[3];
        double d[3], t[3];
        for (int k = 0; k < 3; k++) {
            ci[k] = (int64_t)((pos[k] - g.lower[k]) / g.res);
            /* grid->lowercorner + cellIdx * resolution: int64 * float is a float product */
            const double cic = g.lower[k] + (float)ci[k] * g.res;
            d[k] = (pos[k] - cic) / g.res;
            t[k] = 1.0 - d[k];
        }
        for (int f = 0; f < nfields; f++) {
            double *o = cellenv + ((size_t)f * (size_t)n + (size_t)c) * 4;
            o[0] = o[1] = o[2] = o[3] = 0.0;
        }
        for (int ax = 0; ax < 2; ax++)
            for (int ay = 0; ay < 2; ay++)
                for (int az = 0; az < 2; az++) {
                    const int64_t a[3] = {ci[0] + ax, ci[1] + ay, ci[2] + az};
                    if (!(a[0] >= 0 && a[1] >= 0 && a[2] >= 0 && a[0] <= up[0] && a[1] <= up[1] && a[2] <= up[2]))
                        continue;
                    const int64_t node = g.size[1] * g.size[2] * a[0] + g.size[2] * a[1] + a[2];
                    const double wx = ax * d[0] + (1 - ax) * t[0];
                    const double wy = ay * d[1] + (1 - ay) * t[1];
                    const double wz = az * d[2] + (1 - az) * t[2];
                    for (int f = 0; f < nfields; f++) {
                        double *o = cellenv + ((size_t)f * (size_t)n + (size_t)c) * 4;
                        o[0] += data[(size_t)f * G + node] * wx * wy * wz;
                    }
                    for (int f = 0; f < nfields; f++) {
                        double *o = cellenv + ((size_t)f * (size_t)n + (size_t)c) * 4;
                        const double *gr = gradient + ((size_t)f * G + node) * 3;
                        o[1] += gr[0] * wx * wy * wz;
                        o[2] += gr[1] * wx * wy * wz;
                        o[3] += gr[2] * wx * wy * wz;
                    }
                }
    }
    return 0;
}

/* fieldgradient_compute, fieldgradient.c:149-225, with no neighbouring rank:
 * inside, (data[i+1] - data[i-1]) / resolution (no factor 1/2); on each face
 * the one-sided (data[1] - data[0]) / resolution and
 * (data[n-1] - data[n-2]) / resolution.  An axis of one node (the z axis of a
 * 2-D grid) gets 0: there the reference reads the neighbouring row and, at
 * the first node, one element before the array. */
int tmo_fieldgradient(int dim, float gfh, int nfields, const double *data, double *gradient, int64_t *dims)
{
    tmo_grid g;
    if (nfields < 0 || (dim != 2 && dim != 3) || !(gfh > 0.0f)) return -1;
    tmo_grid_geometry(dim, gfh, &g);
    const int64_t nx = g.size[0], ny = g.size[1], nz = g.size[2], G = nx * ny * nz;
    const double res = (double)g.res;
    dims[0] = nx;
    dims[1] = ny;
    dims[2] = nz;
    for (int f = 0; f < nfields; f++) {
        const double *u = data + (size_t)f * G;
        double *gr = gradient + (size_t)f * 3 * G;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < nx; i++)
            for (int64_t j = 0; j < ny; j++)
                for (int64_t k = 0; k < nz; k++) {
                    const int64_t o = ny * nz * i + nz * j + k;
                    const int64_t n3[3] = {nx, ny, nz}, ix[3] = {i, j, k}, st[3] = {ny * nz, nz, 1};
                    for (int c = 0; c < 3; c++) {
                        double v;
                        if (n3[c] < 2) v = 0.0;
                        else if (ix[c] == 0) v = (u[o + st[c]] - u[o]) / res;
                        else if (ix[c] == n3[c] - 1) v = (u[o] - u[o - st[c]]) / res;
                        else v = (u[o + st[c]] - u[o - st[c]]) / res;
                        gr[3 * o + c] = v;
                    }
                }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* cell cycle                                                                 */
/* ------------------------------------------------------------------------ */

#define TMO_RAND_MAX 2147483647

/* (float)rand()/RAND_MAX with the draw r, as the reference forms it */
static float tmo_frand(int r) { return (float)r / TMO_RAND_MAX; }

/* updatecellcycles, cells.c:370-523, with mitosis, cells.c:124-205: the
 * random draws are taken from draws[] in the order the reference calls
 * rand() (death at G1->S and G2->M; at mitosis three (two in 2-D) shift
 * components, the parent's g1, g2, s, m, the daughter's young and the
 * daughter's g1, g2, s, m).  mitosis's read of the unallocated velocity
 * (cells.c:134) is left out: its value is overwritten before use.  Daughters
 * are appended after the n cells (caller arrays hold cap entries); *nout is
 * the new count, *ndraws the draws used.  Returns 0, or -1 when cap is too
 * small. */
int tmo_cellcycle(int64_t n, int dim, const float *tg1, const float *ts, const float *tg2, const float *tm,
                  const float *tv, const float *trd, const float *tcd, const double *tsize, int nfields,
                  const float *cl1, const float *cl2, int simulationstart, float sps, const double *envvalue,
                  const int *draws, int64_t ndraws_cap, int *phase, float *phasetime, float *g1, float *s, float *g2,
                  float *m, int *age, double *size, float *young, double *x, double *y, double *z, double *density,
                  int *ctype, unsigned char *removecell, int64_t *removecount, int64_t cap, int64_t *nout,
                  int64_t *ndraws)
{
    int64_t nn = n, k = 0;
    const double shrink = pow(2.0, -(1.0 / 3.0));
#define DRAW() (k < ndraws_cap ? draws[k++] : (k++, 0))
    for (int64_t c = 0; c < n; c++) {
        const int t = ctype[c];
        const double eps = tcd[t], csize = tsize[t], rd = trd[t];
        if (removecell[c]) continue;
        int low1 = 0, low2 = 0;
        for (int f = 0; f < nfields; f++) {
            const double val = envvalue[(size_t)f * (size_t)n + (size_t)c];
            if (val < cl1[t * nfields + f]) { low1 = 1; break; }
            if (val < cl2[t * nfields + f]) { low2 = 1; break; }
        }
        if (!simulationstart) continue;
        if (phase[c] != 0 && density[c] <= eps) phasetime[c] += sps / 3600.0;
        switch (phase[c]) {
        case 0:
            if (low2) { phase[c] = 5; phasetime[c] = 0; break; }
            if (density[c] <= eps || n == 1 || !low1) phase[c] = 1;
            break;
        case 1:
            if (density[c] > eps || low1) {
                if (low2) { phase[c] = 5; phasetime[c] = 0; }
                else phase[c] = 0;
                break;
            }
            if (size[c] < csize) size[c] += (csize - shrink * csize) * (sps) / (3600.0 * g1[c]);
            if (size[c] > csize) size[c] = csize;
            if (phasetime[c] >= g1[c]) {
                phase[c] = 2;
                phasetime[c] = 0;
                if (tmo_frand(DRAW()) < rd && removecell[c] == 0) { removecell[c] = 1; (*removecount)++; }
            }
            break;
        case 2:
            if (low2) { phase[c] = 5; phasetime[c] = 0; break; }
            if (phasetime[c] >= s[c]) { phase[c] = 3; phasetime[c] = 0; }
            break;
        case 3:
            if (low2) { phase[c] = 5; phasetime[c] = 0; break; }
            if (phasetime[c] >= g2[c]) {
                phase[c] = 4;
                phasetime[c] = 0;
                if (tmo_frand(DRAW()) < rd && removecell[c] == 0) { removecell[c] = 1; (*removecount)++; }
            }
            break;
        case 4:
            if (low2) { phase[c] = 5; phasetime[c] = 0; }
            else if (phasetime[c] >= m[c]) {
                if (nn + 1 > cap) return -1;
                double sh[3];
                sh[0] = ((double)DRAW() / TMO_RAND_MAX) * 2.0 - 1.0;
                sh[1] = ((double)DRAW() / TMO_RAND_MAX) * 2.0 - 1.0;
                sh[2] = dim == 3 ? ((double)DRAW() / TMO_RAND_MAX) * 2.0 - 1.0 : 0.0;
                double sc = sqrt(sh[0] * sh[0] + sh[1] * sh[1] + sh[2] * sh[2]);
                sc = size[c] / (2 * sc);
                for (int q = 0; q < 3; q++) sh[q] = sc * sh[q];
                const int64_t d = nn;
                x[d] = x[c] + sh[0];
                y[d] = y[c] + sh[1];
                z[d] = z[c] + sh[2];
                size[d] = shrink * size[c];
                ctype[d] = ctype[c];
                age[d] = age[c] + 1;
                x[c] -= sh[0];
                y[c] -= sh[1];
                z[c] -= sh[2];
                size[c] = size[d];
                age[c] += 1;
                g1[c] = tg1[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * tv[t]);
                g2[c] = tg2[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * tv[t]);
                s[c] = ts[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * tv[t]);
                m[c] = tm[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * tv[t]);
                density[d] = density[c];
                young[d] = 2100.0 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * 100.0;
                phase[d] = 1;
                phasetime[d] = 0.0f;
                removecell[d] = 0;
                /* the daughter's own v is 0 (cells.c:184), so its draws do not change its lengths */
                g1[d] = tg1[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * 0.0);
                g2[d] = tg2[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * 0.0);
                s[d] = ts[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * 0.0);
                m[d] = tm[t] * (1 + ((tmo_frand(DRAW())) * 2.0 - 1.0) * 0.0);
                nn++;
                phase[c] = 1;
                phasetime[c] = 0;
            }
            break;
        }
    }
#undef DRAW
    *nout = nn;
    *ndraws = k;
    return k > ndraws_cap ? -2 : 0;
}

/* ------------------------------------------------------------------------ */
/* VTK writer at one rank                                                     */
/* ------------------------------------------------------------------------ */

static void put_be32(unsigned char *p, uint32_t v)
{
    p[0] = (unsigned char)(v >> 24);
    p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8);
    p[3] = (unsigned char)v;
}

static int put_floats_be(FILE *f, const float *v, int64_t count)
{
    for (int64_t i = 0; i < count; i++) {
        unsigned char b[4];
        uint32_t u;
        memcpy(&u, &v[i], 4);
        put_be32(b, u);
        if (fwrite(b, 1, 4, f) != 4) return -1;
    }
    return 0;
}

/* count big-endian ints: v[i], or `value` for every one when v is NULL */
static int put_ints_be(FILE *f, int value, const int *v, int64_t count)
{
    for (int64_t i = 0; i < count; i++) {
        unsigned char b[4];
        put_be32(b, (uint32_t)(v ? v[i] : value));
        if (fwrite(b, 1, 4, f) != 4) return -1;
    }
    return 0;
}

/* writevtk, io.c:372-516, at one rank: legacy binary VTK with big-endian
 * float positions, cell type 1 for every cell, the rank, the cell type, a
 * density of 1.0 (the reference writes the constant) and float forces. */
int tmo_write_vtk(const char *path, int64_t n, const double *x, const double *y, const double *z, const int *ctype,
                  const double *fx, const double *fy, const double *fz, int rank)
{
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    char head[512];
    int rc = 0;
    float *v = (float *)calloc((size_t)(n > 0 ? n : 1) * 3, sizeof(float));
    if (!v) {
        fclose(f);
        return -3;
    }
    rc |= fputs("# vtk DataFile Version 2.0\nTimothy output\nBINARY\nDATASET UNSTRUCTURED_GRID", f) < 0;
    snprintf(head, sizeof head, "\nPOINTS %lld float\n", (long long)n);
    rc |= fputs(head, f) < 0;
    for (int64_t i = 0; i < n; i++) {
        v[3 * i] = (float)x[i];
        v[3 * i + 1] = (float)y[i];
        v[3 * i + 2] = (float)z[i];
    }
    rc |= put_floats_be(f, v, 3 * n);
    snprintf(head, sizeof head, "\nCELL_TYPES %lld\n", (long long)n);
    rc |= fputs(head, f) < 0;
    rc |= put_ints_be(f, 1, NULL, n);
    snprintf(head, sizeof head, "\nPOINT_DATA %lld", (long long)n);
    rc |= fputs(head, f) < 0;
    rc |= fputs("\nSCALARS rank integer 1\nLOOKUP_TABLE default\n", f) < 0;
    rc |= put_ints_be(f, rank, NULL, n);
    rc |= fputs("\nSCALARS type integer 1\nLOOKUP_TABLE default\n", f) < 0;
    rc |= put_ints_be(f, 0, ctype, n);
    rc |= fputs("\nSCALARS density float 1\nLOOKUP_TABLE default\n", f) < 0;
    for (int64_t i = 0; i < n; i++) v[i] = 1.0f;
    rc |= put_floats_be(f, v, n);
    rc |= fputs("\nVECTORS force float\n", f) < 0;
    for (int64_t i = 0; i < n; i++) {
        v[3 * i] = (float)fx[i];
        v[3 * i + 1] = (float)fy[i];
        v[3 * i + 2] = (float)fz[i];
    }
    rc |= put_floats_be(f, v, 3 * n);
    free(v);
    rc |= fclose(f) != 0;
    return rc ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* drivers                                                                    */
/* ------------------------------------------------------------------------ */

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
            double *timing, int nthreads)
{
    if (n < 0 || (dim != 2 && dim != 3) || ntypes < 1) return -1;
    tmo_cells cs = {dim, th, th2, th3, th4, tsize, x, y, z, size, young, ctype};
    tmo_tree tree;
    memset(&tree, 0, sizeof(tree));
    int rc = 0;
    double *dens = (double *)calloc((size_t)(n ? n : 1), sizeof(double));
    double *vv = (double *)calloc((size_t)(n ? n : 1), sizeof(double));
    double *md = (double *)calloc((size_t)(n ? n : 1), sizeof(double));
    double *ff = (double *)calloc((size_t)(n ? n : 1) * 3, sizeof(double));
    tmo_grid g;
    double *grid = NULL;
    memset(&g, 0, sizeof(g));
    if (!dens || !vv || !md || !ff) rc = -3;
    if (do_cic && !rc) {
        tmo_grid_geometry(dim, gfh, &g);
        grid_dims[0] = g.size[0];
        grid_dims[1] = g.size[1];
        grid_dims[2] = g.size[2];
        grid = (double *)malloc((size_t)(g.size[0] * g.size[1] * g.size[2]) * sizeof(double));
        if (!grid) rc = -3;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int64_t i = 0; i < n; i++) removecell[i] = 0;
    *removecount = 0;

    for (int s = 0; s < nsteps && !rc; s++) {
        double t0 = tmo_wall();
        rc = tmo_build(&tree, n, &cs);
        if (rc) break;
        double t1 = tmo_wall();
        if (do_cic) {
            rc = tmo_cic(n, dim, &g, x, y, z, phase, grid);
            if (rc) break;
        }
        double t2 = tmo_wall();
        /* computepotential, potential.c:87-138 (nothing is written for n <= 1) */
        if (n > 1) {
            int err = 0;
#pragma omp parallel
            {
                int32_t *stack = NULL;
                int64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
                for (int64_t p = 0; p < n; p++) {
                    tmo_acc a;
                    a.cs = &cs;
                    a.p = p;
                    a.density = 0.0;
                    a.v = 0.0;
                    a.mindist = DBL_MAX;
                    if (tmo_walk(&tree, &cs, p, &stack, &cap, tmo_visit_potential, &a)) err = 1;
                    dens[p] = a.density;
                    vv[p] = a.v;
                    md[p] = a.mindist;
                }
                free(stack);
            }
            if (err) { rc = -3; break; }
        }
        double t3 = tmo_wall();
        /* computegradient, potential.c:209-259 */
        if (n > 1) {
            int err = 0;
#pragma omp parallel
            {
                int32_t *stack = NULL;
                int64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
                for (int64_t p = 0; p < n; p++) {
                    tmo_acc a;
                    a.cs = &cs;
                    a.p = p;
                    a.f[0] = a.f[1] = a.f[2] = 0.0;
                    if (tmo_walk(&tree, &cs, p, &stack, &cap, tmo_visit_gradient, &a)) err = 1;
                    ff[3 * p] = a.f[0];
                    ff[3 * p + 1] = a.f[1];
                    ff[3 * p + 2] = a.f[2];
                }
                free(stack);
            }
            if (err) { rc = -3; break; }
        }
        double t4 = tmo_wall();
        if (octsize) *octsize = tree.count;
        /* updatepositions, cells.c:342-365 (forces of a 0/1-cell step stay 0) */
        if (update_mode == 0 || update_mode == 1) {
            for (int64_t c = 0; c < n; c++) {
                double *px = &x[c], *py = &y[c], *pz = &z[c];
                if (update_mode == 0) {
                    float rm = trandommove ? trandommove[ctype[c]] : 0.0f;
                    *px += ff[3 * c];
                    *py += ff[3 * c + 1];
                    if (dim == 3) *pz += ff[3 * c + 2];
                    *px += rm * (((float)rand() / RAND_MAX) * 2.0 - 1.0);
                    *py += rm * (((float)rand() / RAND_MAX) * 2.0 - 1.0);
                    if (dim == 3) *pz += rm * (((float)rand() / RAND_MAX) * 2.0 - 1.0);
                } else {
                    *px += dt * ff[3 * c];
                    *py += dt * ff[3 * c + 1];
                    if (dim == 3) *pz += dt * ff[3 * c + 2];
                }
                double r = size[c];
                int out = (*px - r <= -TMO_BOX_HALF || *px + r >= TMO_BOX_HALF) ||
                          (*py - r <= -TMO_BOX_HALF || *py + r >= TMO_BOX_HALF) ||
                          (dim == 3 && (*pz - r <= -TMO_BOX_HALF || *pz + r >= TMO_BOX_HALF));
                if (out && removecell[c] == 0) {
                    removecell[c] = 1;
                    (*removecount)++;
                }
            }
        }
        double t5 = tmo_wall();
        if (timing) {
            timing[0] += t1 - t0;
            timing[1] += t3 - t2;
            timing[2] += t4 - t3;
            timing[3] += t5 - t4;
            timing[4] += t2 - t1;
        }
    }
    if (!rc) {
        for (int64_t i = 0; i < n; i++) {
            if (density) density[i] = dens[i];
            if (v) v[i] = vv[i];
            if (mindist) mindist[i] = md[i];
            if (fx) fx[i] = ff[3 * i];
            if (fy) fy[i] = ff[3 * i + 1];
            if (fz) fz[i] = ff[3 * i + 2];
        }
        if (aff) {
            aff[0] = tree.shift[0];
            aff[1] = tree.shift[1];
            aff[2] = tree.shift[2];
            aff[3] = tree.scale;
        }
        if (do_cic && grid_out) {
            int64_t gt = g.size[0] * g.size[1] * g.size[2];
            if (grid_cap >= gt) memcpy(grid_out, grid, (size_t)gt * sizeof(double));
        }
    }
    free(grid);
    free(tree.node);
    free(tree.code);
    free(dens);
    free(vv);
    free(md);
    free(ff);
    return rc;
}

typedef struct {
    const tmo_cells *cs;
    int64_t p;
    int32_t count, ncand;
    uint64_t hash;
    int64_t last;
    int64_t *list;       /* optional */
} tmo_nbacc;

static void tmo_visit_nb(void *vctx, int64_t j)
{
    tmo_nbacc *a = (tmo_nbacc *)vctx;
    const tmo_cells *cs = a->cs;
    int64_t p = a->p;
    double h = cs->th[cs->ctype[p]];
    double dx = cs->x[p] - cs->x[j], dy = cs->y[p] - cs->y[j], dz = cs->z[p] - cs->z[j];
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    a->ncand++;
    a->last = j;
    if (dist <= h) {
        if (a->list) a->list[a->count] = j;
        a->count++;
        a->hash += tm_mix64((uint64_t)j + 1);
    }
}

int tmo_neighbours(int64_t n, int dim, int ntypes, const double *th,
                   const double *x, const double *y, const double *z, const int *ctype,
                   int32_t *nbcount, uint64_t *nbhash, int64_t *vcand, int32_t *ncand,
                   int64_t *nb_offsets, int64_t *nb_list, int nthreads)
{
    if (n < 0 || (dim != 2 && dim != 3) || ntypes < 1) return -1;
    tmo_cells cs;
    memset(&cs, 0, sizeof(cs));
    cs.dim = dim;
    cs.th = th;
    cs.x = x;
    cs.y = y;
    cs.z = z;
    cs.ctype = ctype;
    tmo_tree tree;
    memset(&tree, 0, sizeof(tree));
    int rc = tmo_build(&tree, n, &cs);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (!rc && n > 1) {
        int err = 0;
#pragma omp parallel
        {
            int32_t *stack = NULL;
            int64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
            for (int64_t p = 0; p < n; p++) {
                tmo_nbacc a;
                a.cs = &cs;
                a.p = p;
                a.count = 0;
                a.ncand = 0;
                a.hash = 0;
                a.last = -1;
                a.list = (nb_list && nb_offsets) ? nb_list + nb_offsets[p] : NULL;
                if (tmo_walk(&tree, &cs, p, &stack, &cap, tmo_visit_nb, &a)) err = 1;
                if (nbcount) nbcount[p] = a.count;
                if (nbhash) nbhash[p] = a.hash;
                if (vcand) vcand[p] = a.last;
                if (ncand) ncand[p] = a.ncand;
            }
            free(stack);
        }
        if (err) rc = -3;
        if (!rc && nb_offsets && !nb_list && nbcount) {
            nb_offsets[0] = 0;
            for (int64_t p = 0; p < n; p++) nb_offsets[p + 1] = nb_offsets[p] + nbcount[p];
        }
    } else if (!rc) {
        for (int64_t p = 0; p < n; p++) {
            if (nbcount) nbcount[p] = 0;
            if (nbhash) nbhash[p] = 0;
            if (vcand) vcand[p] = -1;
            if (ncand) ncand[p] = 0;
        }
        if (nb_offsets) for (int64_t p = 0; p <= n; p++) nb_offsets[p] = 0;
    }
    free(tree.node);
    free(tree.code);
    return rc;
}

/* ------------------------------------------------------------------------
 * Implicit diffusion step (environment.c:131-523) at one rank.
 *
 * environment_initsystem (environment.c:144-164) picks the number of solves
 * per step from secondsperstep / gfdt in float arithmetic, then sets every
 * field's dt to gfdt (environment.c:221) and z = dc * dt / (res * res), the
 * product res * res in float (environment.c:222).  The operator is the
 * 7-point stencil with 1 + 6 z + lambda dt on the diagonal and -z for each
 * neighbour (environment.c:227-230); the Dirichlet faces (environment.c:
 * 332-375) move z * bc to the right-hand side once per grid face the node
 * lies on (x-, x+, y-, y+, z-, z+ in turn; both z faces on a one-layer grid)
 * and leave the couplings to nodes outside the grid, which no solve uses.
 * environment_compute starts from u = initialconditionmean (a new solution
 * vector each call, environment.c:298-316) and, numberofiters times, solves
 * A u = u + faces + pc (environment.c:438-488), pc being 100 at node
 * (5, 5, 5) from step 1 on (environment_pcfunction, environment.c:251-266).
 * The solve here is conjugate gradients to a relative residual of tol (the
 * reference's Hypre PCG with a BoomerAMG preconditioner stops at 1e-12 or 50
 * iterations, environment.c:404-422).  u0 (x-major, z fastest, nfields
 * fields) replaces the mean as the start when given; source replaces pc.
 * Outputs u and the last right-hand side b_last in the same layout. */
int tmo_diffusion_iters(float secondsperstep, float gfdt)
{
    if ((secondsperstep / gfdt) > 1) {
        const int intdiv = (int)(secondsperstep / gfdt) + 1;
        const float a1 = secondsperstep / intdiv;
        const float a2 = secondsperstep / (intdiv - 1);
        return (gfdt - a1) < (a2 - gfdt) ? intdiv : intdiv - 1;
    }
    return 1;
}

double tmo_diffusion_z(double dc, float gfdt, float resolution)
{
    const double dt = gfdt;
    const float r2 = resolution * resolution;
    return dc * dt / r2;
}

static void diff_apply(int64_t nx, int64_t ny, int64_t nz, double diag, double off, const double *u, double *y)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nx; i++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
                const int64_t p = (i * ny + j) * nz + k;
                double s = diag * u[p];
                if (i > 0) s += off * u[p - ny * nz];
                if (i < nx - 1) s += off * u[p + ny * nz];
                if (j > 0) s += off * u[p - nz];
                if (j < ny - 1) s += off * u[p + nz];
                if (k > 0) s += off * u[p - 1];
                if (k < nz - 1) s += off * u[p + 1];
                y[p] = s;
            }
}

static double diff_dot(const double *a, const double *b, int64_t n)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

int tmo_diffuse(int64_t nx, int64_t ny, int64_t nz, float resolution, float secondsperstep, float gfdt, int step,
                int nfields, const double *dc, const double *bc, const double *mean, const double *lambda,
                const double *u0, const double *source, double tol, double *u, double *b_last, int *iters_out,
                int *cg_iters)
{
    const int64_t G = nx * ny * nz;
    const int iters = tmo_diffusion_iters(secondsperstep, gfdt);
    double *r = (double *)malloc((size_t)G * sizeof(double)), *p = (double *)malloc((size_t)G * sizeof(double));
    double *q = (double *)malloc((size_t)G * sizeof(double));
    if (!r || !p || !q) return -1;
    *iters_out = iters;
    int cg_total = 0;
    for (int f = 0; f < nfields; f++) {
        const double z = tmo_diffusion_z(dc[f], gfdt, resolution);
        const double dt = gfdt;
        const double diag = 1 + 6.0 * z + lambda[f] * dt, off = -z, zb = z * bc[f];
        double *uf = u + (size_t)f * (size_t)G, *bf = b_last + (size_t)f * (size_t)G;
        for (int64_t i = 0; i < G; i++) uf[i] = u0 ? u0[(size_t)f * (size_t)G + i] : mean[f];
        for (int it = 0; it < iters; it++) {
            /* right-hand side in the reference's order of additions */
            for (int64_t i = 0; i < nx; i++)
                for (int64_t j = 0; j < ny; j++)
                    for (int64_t k = 0; k < nz; k++) {
                        const int64_t o = (i * ny + j) * nz + k;
                        double v = uf[o];
                        if (i == 0) v += zb;
                        if (i == nx - 1) v += zb;
                        if (j == 0) v += zb;
                        if (j == ny - 1) v += zb;
                        if (k == 0) v += zb;
                        if (k == nz - 1) v += zb;
                        if (source) v += source[(size_t)f * (size_t)G + o];
                        else v += (step != 0 && i == 5 && j == 5 && k == 5) ? 100.0 : 0.0;
                        bf[o] = v;
                    }
            /* conjugate gradients from the current u */
            diff_apply(nx, ny, nz, diag, off, uf, q);
            for (int64_t i = 0; i < G; i++) r[i] = bf[i] - q[i];
            memcpy(p, r, (size_t)G * sizeof(double));
            const double bb = diff_dot(bf, bf, G);
            double rr = diff_dot(r, r, G), best = rr;
            int n = 0, stall = 0;
            while (rr > tol * tol * bb && n < 100000 && stall < 50) {
                diff_apply(nx, ny, nz, diag, off, p, q);
                const double alpha = rr / diff_dot(p, q, G);
                for (int64_t i = 0; i < G; i++) {
                    uf[i] += alpha * p[i];
                    r[i] -= alpha * q[i];
                }
                const double rr1 = diff_dot(r, r, G);
                for (int64_t i = 0; i < G; i++) p[i] = r[i] + (rr1 / rr) * p[i];
                rr = rr1;
                if (rr < best) {
                    best = rr;
                    stall = 0;
                } else {
                    stall++;
                }
                n++;
            }
            cg_total += n;
        }
    }
    if (cg_iters) *cg_iters = cg_total;
    free(r);
    free(p);
    free(q);
    return 0;
}
