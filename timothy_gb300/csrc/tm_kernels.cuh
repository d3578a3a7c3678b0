// Kernel entry points of the hot path (host-callable launchers).
#pragma once
#include "tm_arrays.cuh"

__global__ void k_step_init(tm_arrays a);
cudaError_t tm_launch_bbox(const tm_arrays &a, int ntypes, cudaStream_t st);
__global__ void k_frame(tm_arrays a, const tm_consts *K);
__global__ void k_codes(tm_arrays a);
__global__ void k_binbase(tm_arrays a);
__global__ void k_scatter(tm_arrays a);
__global__ void k_place(tm_arrays a, const tm_consts *K);
__global__ void k_binsort_big(tm_arrays a, const tm_consts *K);
__global__ void k_copyback(tm_arrays a);
__global__ void k_worklist(tm_arrays a, int which);
// blocks of a grid-stride launch: `per_sm` blocks of `block` threads per SM
unsigned tm_stream_grid(int block, int per_sm);
__global__ void k_octsize(tm_arrays a, unsigned long long *out);

cudaError_t tm_scan_exclusive(const uint32_t *in, uint32_t *out, long long n, uint32_t *tmp, cudaStream_t st);
long long tm_scan_tmp_words(long long n);
cudaError_t tm_launch_search(const tm_arrays &a, const tm_consts *K, int prec, const tm_shapes &sh, int fallback,
                             cudaStream_t st);
cudaError_t tm_launch_listbuild(const tm_arrays &a, const tm_consts *K, cudaStream_t st);
cudaError_t tm_launch_list(const tm_arrays &a, const tm_consts *K, int prec, const tm_shapes &sh, cudaStream_t st);
cudaError_t tm_launch_fix(const tm_arrays &a, const tm_consts *K, cudaStream_t st);
cudaError_t tm_launch_octree(const tm_arrays &a, const tm_consts *K, int block, cudaStream_t st);
cudaError_t tm_launch_update(const tm_arrays &a, const tm_consts *K, cudaStream_t st);
cudaError_t tm_launch_cic(const tm_arrays &a, const tm_consts *K, cudaStream_t st);

// geometry of a grid -> cell gather or a field gradient (tm_field.cu): the
// grid's lower corner and resolution, its last node index per axis, and the
// box of nodes the data arrays hold (the whole grid, or a patch)
struct tm_envgeom {
    double lower[3];
    double res, inv;     // inv = 1 / res = 2^inv_exp when res is a power of two (pow2)
    float resf;
    int pow2, inv_exp;
    long long hi[3];
    long long blo[3], bsz[3];
    int nfields;
};
tm_envgeom tm_make_envgeom(const double lower[3], float res, const int64_t grid_hi[3], const int64_t box_lo[3],
                           const int64_t box_size[3], int nfields);
cudaError_t tm_launch_env2cells(const tm_envgeom &g, const double *x, const double *y, const double *z, long long n,
                                const double *data, const double *grad, double *out, cudaStream_t st);
cudaError_t tm_launch_env2cells_colony(const tm_envgeom &g, const tm_arrays &a, long long off, long long n,
                                       const double *data, const double *grad, double *out, cudaStream_t st);
cudaError_t tm_launch_field_gradient(const tm_envgeom &g, const int64_t gsize[3], const double *data, double *grad,
                                     cudaStream_t st);

// byte offsets of the binary sections in a VTK file image (tm_vtk.cu)
struct tm_vtk_layout {
    long long points, celltypes, ranks, types, density, forces;
};
cudaError_t tm_launch_vtk_pack(const tm_arrays &a, long long off, long long n, int rank, const tm_vtk_layout &L,
                               unsigned char *img, cudaStream_t st);

// cell cycle (tm_cycle.cu): per-type parameters and the step's inputs on the device
#include "timothy_gb300.h"
struct tm_cycle_dev {
    const tm_cycle_type *types;    // ntypes
    const float *cl1, *cl2;        // [type][field]
    const double *csize;           // celltype size per type
    const double *cellenv;         // nfields x n x 4, caller order (tm_colony_env2cells layout)
    long long off;                 // colony offset (cell-cycle arrays are indexed off + caller index)
    int nfields, simulationstart;
    float sps;                     // settings.secondsperstep
    double shrink;                 // pow(2, -1/3)
};
cudaError_t tm_launch_cycle_count(const tm_cycle_dev &P, const tm_arrays &a, long long off, long long n, int dim,
                                  uint32_t *draws, uint32_t *divs, cudaStream_t st);
cudaError_t tm_launch_cycle_apply(const tm_cycle_dev &P, const tm_arrays &a, long long off, long long n, int dim,
                                  const uint32_t *draw_off, const uint32_t *div_off, const int *stream,
                                  unsigned long long *marked, uint32_t *divlist, long long ndiv, cudaStream_t st);

// the C library's rand() stream on the device (tm_libcrand.cu)
// values per chunk of the device rand() stream (one thread each); a call of
// count values needs count / TM_RAND_CHUNK + 2 windows of 31 words
#define TM_RAND_CHUNK 992
struct tm_rand_cache {
    int valid;
    uint32_t seed;
    int64_t offset;
    uint32_t window[31];
};
int tm_libc_rand_device(uint32_t seed, int64_t offset, int64_t count, int *out, tm_rand_cache *cache,
                        uint32_t *d_windows, int64_t windows_cap, cudaStream_t st);
int tm_libc_rand_from_window(const uint32_t w[31], int64_t count, int *out, uint32_t end[31], uint32_t *d_windows,
                             int64_t windows_cap, cudaStream_t st);

