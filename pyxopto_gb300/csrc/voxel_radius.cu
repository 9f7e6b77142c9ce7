// Homogeneous-cube radius of every voxel, the table behind FAST-mode free
// flight in the voxelized transport kernels.
//
// radius[v] is the largest k (capped) such that the cube of voxels within
// Chebyshev distance k of v lies inside the grid and holds v's material
// only.  A packet anywhere inside voxel v is then at least k * min(voxel
// size) away from every other material and from the grid's surface, so a
// sampled free path shorter than that can be taken in one move: the
// exponential free path is memoryless, and the reference's walk, which stops
// at every voxel wall and draws a new path length when the next voxel holds
// the same material (xopto/mcvox/kernel/mcvox.template.c:760-1038), samples
// the same interaction points in distribution.
//
// radius[v] is the Chebyshev distance from v to the set B of voxels that lie
// on the grid surface or have one of their 26 neighbours in another
// material (a voxel within distance k - 1 of v that is not in B has all its
// neighbours in its own material, so the cube of radius k around v is
// homogeneous).  It is computed by in-place relaxation,
// r(v) <- min(r(v), 1 + min over the 26 neighbours of r(u)), started from
// 0 on B and the cap elsewhere: every read value is an upper bound of the
// true distance, the values only decrease, and each pass carries the exact
// distances one voxel further, so cap passes give the exact capped result.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xopto_gb300.h"
#include "errors.h"

namespace {

__global__ void radius_init_kernel(const uint8_t *__restrict__ vox, uint8_t *radius, int nx, int ny,
                                   int nz, uint8_t cap) {
    const size_t n = (size_t)nx * ny * nz;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        int x = (int)(i % nx);
        int y = (int)((i / nx) % ny);
        int z = (int)(i / ((size_t)nx * ny));
        uint8_t r = cap;
        if (x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1) {
            r = 0;
        } else {
            const uint8_t m = vox[i];
            for (int dz = -1; dz <= 1 && r; ++dz)
                for (int dy = -1; dy <= 1 && r; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        size_t j = ((size_t)(z + dz) * ny + (y + dy)) * nx + (x + dx);
                        if (vox[j] != m) {
                            r = 0;
                            break;
                        }
                    }
        }
        radius[i] = r;
    }
}

__global__ void radius_relax_kernel(uint8_t *radius, int nx, int ny, int nz) {
    const size_t n = (size_t)nx * ny * nz;
    volatile uint8_t *rv = radius;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        uint8_t r = rv[i];
        /* 0 on B, which includes the grid surface: a voxel with r > 0 has
           all 26 neighbours inside the grid */
        if (r == 0) continue;
        int x = (int)(i % nx);
        int y = (int)((i / nx) % ny);
        int z = (int)(i / ((size_t)nx * ny));
        uint8_t m = r;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    size_t j = ((size_t)(z + dz) * ny + (y + dy)) * nx + (x + dx);
                    uint8_t u = rv[j];
                    m = u < m ? u : m;
                }
        uint8_t c = (uint8_t)(m + 1u);
        if (c < r) rv[i] = c;
    }
}

}  // namespace

extern "C" int mcgb_voxel_radius(const uint8_t *dev_voxels, const int32_t shape[3], uint8_t *dev_radius,
                                 uint32_t max_radius, void *stream) {
    if (!dev_voxels || !dev_radius || !shape)
        return mcgb_internal::set_error(MCGB_E_INVALID, "mcgb_voxel_radius: NULL argument");
    const int nx = shape[0], ny = shape[1], nz = shape[2];
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return mcgb_internal::set_error(MCGB_E_INVALID, "mcgb_voxel_radius: shape must be positive");
    if (max_radius < 1 || max_radius > MCGB_VOXEL_RADIUS_MAX)
        return mcgb_internal::set_error(MCGB_E_INVALID, "mcgb_voxel_radius: max_radius must be in [1, 64]");
    const size_t n = (size_t)nx * ny * nz;
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (blocks > 152u * 64u) blocks = 152u * 64u;
    cudaStream_t s = (cudaStream_t)stream;
    radius_init_kernel<<<blocks, 256, 0, s>>>(dev_voxels, dev_radius, nx, ny, nz, (uint8_t)max_radius);
    for (uint32_t k = 0; k < max_radius; ++k) radius_relax_kernel<<<blocks, 256, 0, s>>>(dev_radius, nx, ny, nz);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mcgb_internal::set_error(MCGB_E_CUDA, cudaGetErrorString(e));
    return MCGB_OK;
}
