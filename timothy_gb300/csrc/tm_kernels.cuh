// Kernel entry points of the hot path (host-callable launchers).
#pragma once
#include "tm_arrays.cuh"

__global__ void k_step_init(tm_arrays a);
__global__ void k_bbox(tm_arrays a, int ntypes);
__global__ void k_frame(tm_arrays a, const tm_consts *K);
__global__ void k_codes(tm_arrays a);
__global__ void k_binbase(tm_arrays a);
__global__ void k_scatter(tm_arrays a);
__global__ void k_binsort_small(tm_arrays a);
__global__ void k_binsort_big(tm_arrays a);
__global__ void k_gather(tm_arrays a, const tm_consts *K);
__global__ void k_copyback(tm_arrays a);
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
