// VTK writer (writevtk, io.c:372-516) for device-resident cells: the legacy
// binary file image is assembled on the device -- big-endian float positions,
// cell type 1, the rank, the cell type, the density constant 1.0 the
// reference writes, big-endian float forces -- in the caller's cell order,
// then copied to the host in one piece and written.
#include "tm_arrays.cuh"
#include "tm_kernels.cuh"

__device__ __forceinline__ void put_be32(unsigned char *p, uint32_t v)
{
    p[0] = (unsigned char)(v >> 24);
    p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8);
    p[3] = (unsigned char)v;
}

__global__ void __launch_bounds__(256) k_vtk_pack(tm_arrays a, long long off, long long n, int rank, tm_vtk_layout L,
                                                  unsigned char *img)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long s = off + k;
        const long long c = a.perm[s];
        const double p[3] = {a.x[s], a.y[s], a.z[s]};
        const double f[3] = {a.fx[s], a.fy[s], a.fz[s]};
        for (int d = 0; d < 3; d++) {
            put_be32(img + L.points + 12 * c + 4 * d, __float_as_uint(__double2float_rn(p[d])));
            put_be32(img + L.forces + 12 * c + 4 * d, __float_as_uint(__double2float_rn(f[d])));
        }
        put_be32(img + L.celltypes + 4 * c, 1u);
        put_be32(img + L.ranks + 4 * c, (uint32_t)rank);
        put_be32(img + L.types + 4 * c, (uint32_t)a.ctype[s]);
        put_be32(img + L.density + 4 * c, __float_as_uint(1.0f));
    }
}

cudaError_t tm_launch_vtk_pack(const tm_arrays &a, long long off, long long n, int rank, const tm_vtk_layout &L,
                               unsigned char *img, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const long long b = (n + 255) / 256;
    k_vtk_pack<<<(unsigned)(b < 152 * 32 ? b : 152 * 32), 256, 0, st>>>(a, off, n, rank, L, img);
    return cudaGetLastError();
}
