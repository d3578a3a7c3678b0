/* Reference-signature drop-ins for Timothy's cell-mechanics hot path.
 *
 * The functions below have exactly the signatures of the reference functions
 * they replace, so the reference step loop (main.c:67-79, step.c:41-100)
 * links against libtimothy_gb300.so unchanged once octree.c and potential.c
 * are dropped from its build and the replaced functions of cells.c,
 * patches.c and fieldgradient.c are weakened.  Each runs on the GPU
 * through the device-resident session of include/timothy_gb300.h; errors
 * end in terminate() as in the reference (utils.c:103-109).
 *
 * The structs restate the layout of the reference's global.h:90-352 field
 * by field: the ABI of a by-value struct argument is its layout, so these
 * declarations must stay identical to the reference's.  A program that
 * already includes the reference's global.h defines TM_USE_REFERENCE_GLOBAL_H
 * before including this header and gets only the prototypes.
 *
 * MPI_Comm / MPI_Request: taken from <mpi.h> when it has been included
 * (build the drop-in layer with the host program's mpicc); otherwise the
 * single-rank stand-ins below (int handles, as in MPICH).
 */
#ifndef TIMOTHY_REFABI_H
#define TIMOTHY_REFABI_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef TM_USE_REFERENCE_GLOBAL_H

#if defined(MPI_VERSION)
typedef MPI_Comm tm_mpi_comm;
typedef MPI_Request tm_mpi_request;
#else
typedef int tm_mpi_comm;
typedef int tm_mpi_request;
#endif

typedef struct cellcount_t {            /* global.h:90-98 */
    uint64_t n;
    uint64_t g0phase;
    uint64_t g1phase;
    uint64_t sphase;
    uint64_t g2phase;
    uint64_t mphase;
    uint64_t necroticphase;
} cellcount_t;

typedef struct celldata_t {             /* global.h:100-120, 112 bytes */
    int lifetime;
    int phase;                          /* 0=G0 1=G1 2=S 3=G2 4=M 5=necrotic */
    int age;
    int death;
    float phasetime;
    float g1;
    float s;
    float g2;
    float m;
    float young;
    int gid;                            /* ZOLTAN_ID_TYPE */
    double x;
    double y;
    double z;
    double size;
    double v;
    double density;
    double mindist;
    int ctype;
} celldata_t;

typedef struct double3dv_t {            /* global.h:129-133 */
    double x;
    double y;
    double z;
} double3dv_t;

typedef struct int643dv_t {             /* global.h:141-145 */
    int64_t x;
    int64_t y;
    int64_t z;
} int643dv_t;

typedef struct octnode_t {              /* global.h:153-164 */
    unsigned int xcode;
    unsigned int ycode;
    unsigned int zcode;
    unsigned int xlimit;
    unsigned int ylimit;
    unsigned int zlimit;
    unsigned int level;
    int64_t father;
    int64_t child[8];
    int data;
} octnode_t;

typedef struct cellsinfo_t {            /* global.h:166-179 */
    cellcount_t localcount;
    cellcount_t globalcount;
    cellcount_t *localtypecount;
    cellcount_t *globaltypecount;
    uint64_t *cellsperproc;
    celldata_t *cells;
    double3dv_t *forces;
    octnode_t *octree;
    int64_t octsize;
    int64_t octmaxsize;
    int dimension;
    double3dv_t *velocity;
} cellsinfo_t;

typedef struct grid_t {                 /* global.h:182-190 */
    int643dv_t globalsize;
    double3dv_t lowercorner, uppercorner;
    int643dv_t localsize;
    float resolution;
    int643dv_t *loweridx, *upperidx;
    double3dv_t *lowleftnear, *uprightfar;
} grid_t;

typedef struct explist_t {              /* global.h:212-215 */
    int64_t cell;
    int proc;
} explist_t;

typedef struct cellindata_t {           /* global.h:247-254 */
    double x;
    double y;
    double z;
    double size;
    double young;
    int ctype;
} cellindata_t;

typedef struct celloutdata_t {          /* global.h:256-259 */
    double v;
    double density;
} celloutdata_t;

typedef struct cellcommdata_t {         /* global.h:261-276 */
    explist_t *explist;
    int explistmaxsize;
    tm_mpi_request *reqsend;
    tm_mpi_request *reqrecv;
    int64_t *sendoffset;
    int64_t *recvoffset;
    int *recvcount;
    int *sendcount;
    cellindata_t *sendcellindata;
    cellindata_t *recvcellindata;
    celloutdata_t *sendcelloutdata;
    celloutdata_t *recvcelloutdata;
    int numexp;
    int numimp;
} cellcommdata_t;

typedef struct settings_t {             /* global.h:278-298 */
    int64_t maxcells;
    int64_t maxlocalcells;
    int numberofsteps;
    float secondsperstep;
    int numberofcelltypes;
    int numberoffields;
    int dimension;
    int restart;
    char rstfilename[128];
    char outdir[128];
    int visoutstep;
    int statoutstep;
    int rstoutstep;
    float maxspeed;
    float gfdt;
    float gfh;
    int simulationstart;
    unsigned int rseed;
    int step;
} settings_t;

typedef struct systeminfo_t {           /* global.h:300-312 */
    int rank;
    int size;
    int nthreads;
    int dim[3];
    int noderank;
    int nodesize;
    int memperproc;
    tm_mpi_comm MPI_CART_COMM;
    int **coords;
    int endian;
} systeminfo_t;

typedef struct celltype_t {             /* global.h:315-335 */
    char name[128];
    float g1;
    float s;
    float g2;
    float m;
    float v;
    float rd;
    double size;
    double h;
    double h2;
    double h3;
    double h4;
    char inputfile[128];
    float criticaldensity;
    float *production;
    float *consumption;
    float *criticallevel1;
    float *criticallevel2;
    float randommove;
} celltype_t;

typedef struct patches_t {              /* global.h:337-352 */
    double **data;
    int *intersect;
    int *receiver;
    int *sender;
    double **recvdata;
    tm_mpi_request *reqsend;
    tm_mpi_request *reqrecv;
    int643dv_t *lowercorner;
    int643dv_t *uppercorner;
    int643dv_t *lowercornerR;
    int643dv_t *uppercornerR;
    int643dv_t *size;
    double **commbuff;
    double **buff;
} patches_t;

typedef struct cellenvdata_t {          /* global.h:122-127 */
    double value;
    double gx;
    double gy;
    double gz;
} cellenvdata_t;

typedef struct environment_t {          /* global.h:354-364 */
    char name[128];
    double diffusioncoefficient;
    double boundarycondition;
    double initialconditionmean;
    double initialconditionvariance;
    double lambdadelay;
    double *data;
    double *gradient;
    double *production;
} environment_t;

#endif /* TM_USE_REFERENCE_GLOBAL_H */

/* affine map of the last octbuild (octree.h:24-25) */
extern double3dv_t affShift;
extern double affScale;

/* octree.c:145 -- uploads the cells and sorts them into Morton order on the
 * device (the implicit octree); sets affShift/affScale and octsize. */
void octbuild(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype);
/* octree.c:321 */
void octfree(cellsinfo_t *cellsinfo);
/* potential.c:87 -- density, v and mindist of every local cell */
void computepotential(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                      cellcommdata_t cellcommdata);
/* potential.c:144 -- halo cells exist only with several MPI ranks */
void computeremotepotential(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                            cellcommdata_t cellcommdata);
/* potential.c:209 -- forces[] of every local cell */
void computegradient(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                     cellcommdata_t cellcommdata);
/* potential.c:265 */
void computeremotegradient(systeminfo_t systeminfo, cellsinfo_t *cellsinfo, celltype_t *celltype,
                           cellcommdata_t cellcommdata);
/* cells.c:342 -- x += F, removal marks */
void updatepositions(settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo, unsigned char *removecell,
                     int64_t *removecount);
/* patches.c:47 -- bounding box of the grid nodes the cells touch, zeroed patch buffers */
void patches_alloc(systeminfo_t systeminfo, settings_t settings, patches_t *patches, cellsinfo_t *cellsinfo,
                   grid_t *grid);
/* patches.c:156 -- CIC deposit of the cells into field 0 of the patch */
void patches_cells2envinfo(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                           cellsinfo_t *cellsinfo, grid_t *grid);

/* patches.c:512 -- grid -> cell gather of every field and its gradient from
 * the received patch (patches->buff[0]) into freshly allocated
 * (*cellenvdata)[f][c]; frees the patch buffers as the reference does */
void patches_applyenv2cells(systeminfo_t systeminfo, settings_t settings, patches_t *patches,
                            cellsinfo_t *cellsinfo, grid_t *grid, cellenvdata_t ***cellenvdata);
/* fieldgradient.c:256 -- gradient of every field (one rank) */
void fieldgradient(systeminfo_t systeminfo, settings_t settings, environment_t **environment, grid_t *grid);

/* cells.c:370 -- cell cycle with mitosis of every local cell (one rank);
 * cells.c:290 -- removal of the marked cells */
int updatecellcycles(systeminfo_t systeminfo, settings_t settings, celltype_t *celltype, cellsinfo_t *cellsinfo,
                     cellenvdata_t **cellenvdata, unsigned char *removecell, int64_t *removecount);
void cellsdeath(int oldlnc, cellsinfo_t *cellsinfo, unsigned char *removecell, int64_t removecount);
/* environment.c:33, 56, 131, 515 -- the fields without Hypre: allocation,
 * initial values, (nothing to) set up, and the implicit diffusion step on the
 * GPU.  solverdata_t / solversettings_t (global.h:366-392, Hypre handles) are
 * never touched, so they are passed as untyped pointers. */
void environment_allocate(systeminfo_t systeminfo, settings_t settings, grid_t grid, environment_t **environment,
                          void *solverdata, void *solversettings);
void environment_init(systeminfo_t systeminfo, settings_t settings, grid_t grid, environment_t **environment);
void environment_initsystem(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                            void *solverdata, void *solversettings);
void environment_compute(systeminfo_t systeminfo, settings_t settings, grid_t *grid, environment_t **environment,
                         void *solverdata, void *solversettings);
/* the solution of field f after the last environment_compute (G values,
 * environment_t.data layout); TM_OK or a negative code */
int tm_dropin_env_solution(int field, double *out);
/* 1: environment_compute also copies the solution into environment[f].data
 * (the reference leaves data unchanged, environment.c:495-507) */
void tm_dropin_set_env_writeback(int on);
/* No counterpart in the reference.  The arithmetic of the drop-ins' pair
 * maths from the next octbuild on: 0 = TM_PREC_FP64 (the default, the
 * reference's own roundings) or 1 = TM_PREC_FP32C (FP32 pair maths with
 * compensated sums, the cutoff rechecked in FP64 near h, FP64 positions;
 * within 1e-6 of the FP64 results, identical neighbour sets); with
 * neighbour_lists = 1 the colony keeps Verlet lists between steps as long as
 * the host keeps the same cells in the same order (a step loop without cell
 * divisions or removals).  Changing either releases the device session. */
void tm_dropin_set_precision(int precision, int neighbour_lists);
/* Releases the device session the drop-ins keep between calls (no
 * counterpart in the reference; optional at exit). */
void tm_dropin_shutdown(void);
/* No counterpart in the reference.  Bytes of the caller's cell records the
 * drop-ins hold page-locked for their copies (0: the last registration
 * failed and the copies run from pageable memory, at a lower rate). */
int64_t tm_dropin_pinned_bytes(void);

#ifdef __cplusplus
}
#endif
#endif
