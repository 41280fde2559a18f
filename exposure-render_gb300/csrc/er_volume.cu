/*
 * er_volume.cu - per-volume pre-passes of the delta tracker.
 *
 *   k_brick_minmax : min and max voxel of every brick's footprint (the
 *                    brick^3 voxels plus a one-voxel apron on each side,
 *                    which covers every corner a trilinear lookup inside the
 *                    brick can touch, Source/buffer3d.h:222-242).  One warp
 *                    per brick, coalesced reads along x.
 *   k_rmq_level    : level k of a sparse table of running maxima over the
 *                    sigma table (sigma[I] = DensityScale * Opacity(I)).
 *   k_majorant     : majorant[brick] = DensityScale * max sigma[lo..hi].
 *
 * A lookup inside a brick is a truncated trilinear blend of voxels in
 * [lo, hi], so its integer intensity lies in [lo, hi] and its extinction
 * DensityScale * sigma[I] is bounded by the brick's majorant exactly (max of
 * the same floats, one multiply).  The CPU oracle builds the same grid by
 * brute force; the tests compare them bit for bit through the rendered paths.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "er_kernels.h"

__global__ void k_brick_minmax(const uint16_t* __restrict__ vox, int rx, int ry, int rz, int B, int nbx, int nby, int nbz,
                               uint32_t* __restrict__ minmax)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int total = nbx * nby * nbz;
    if (warp >= total) return;
    const int bx = warp % nbx, by = (warp / nbx) % nby, bz = warp / (nbx * nby);
    int x0 = bx * B - 1, x1 = (bx + 1) * B + 1;
    int y0 = by * B - 1, y1 = (by + 1) * B + 1;
    int z0 = bz * B - 1, z1 = (bz + 1) * B + 1;
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0; z0 = z0 < 0 ? 0 : z0;
    x1 = x1 > rx - 1 ? rx - 1 : x1; y1 = y1 > ry - 1 ? ry - 1 : y1; z1 = z1 > rz - 1 ? rz - 1 : z1;
    const int wx = x1 - x0 + 1;
    const int rows = (y1 - y0 + 1) * (z1 - z0 + 1);
    unsigned int lo = 65535u, hi = 0u;
    for (int r = 0; r < rows; r++) {
        const int y = y0 + r % (y1 - y0 + 1);
        const int z = z0 + r / (y1 - y0 + 1);
        const uint16_t* row = vox + ((size_t)z * ry + y) * (size_t)rx + x0;
        for (int x = lane; x < wx; x += 32) {
            const unsigned int v = __ldg(row + x);
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned int a = __shfl_xor_sync(0xffffffffu, lo, o);
        const unsigned int b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if (lane == 0) minmax[warp] = lo | (hi << 16);
}

__global__ void k_rmq_level(const float* __restrict__ prev, float* __restrict__ next, int n, int half)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = prev[i];
    const float b = (i + half < n) ? prev[i + half] : a;
    next[i] = b > a ? b : a;
}

__global__ void k_majorant(const uint32_t* __restrict__ minmax, const float* __restrict__ table, int n, int levels, float ds,
                           float* __restrict__ majorant, int total)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const uint32_t mm = minmax[i];
    int lo = (int)(mm & 0xffffu), hi = (int)(mm >> 16);
    lo = lo > n - 1 ? n - 1 : lo;
    hi = hi > n - 1 ? n - 1 : hi;
    const int len = hi - lo + 1;
    int k = 31 - __clz(len);
    k = k > levels - 1 ? levels - 1 : k;
    const float* lvl = table + (size_t)k * n;
    const float a = lvl[lo];
    const float b = lvl[hi - (1 << k) + 1];
    float m = b > a ? b : a;
    m = m > 0.0f ? m : 0.0f;
    majorant[i] = ds * m;
}

cudaError_t er_launch_majorant(const uint16_t* vox, const int res[3], int B, const int nb[3], const float* sigma, int n,
                               float* rmq, int levels, uint32_t* minmax, float density_scale, float* majorant, cudaStream_t s)
{
    const int total = nb[0] * nb[1] * nb[2];
    k_brick_minmax<<<(total * 32 + 255) / 256, 256, 0, s>>>(vox, res[0], res[1], res[2], B, nb[0], nb[1], nb[2], minmax);
    cudaError_t e = cudaMemcpyAsync(rmq, sigma, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    for (int k = 1; k < levels; k++)
        k_rmq_level<<<(n + 255) / 256, 256, 0, s>>>(rmq + (size_t)(k - 1) * n, rmq + (size_t)k * n, n, 1 << (k - 1));
    k_majorant<<<(total + 255) / 256, 256, 0, s>>>(minmax, rmq, n, levels, density_scale, majorant, total);
    return cudaGetLastError();
}
