/*
 * er_volume.cu - per-volume pre-passes of the delta tracker.
 *
 *   k_brick_minmax : min and max voxel of every brick's footprint: voxels
 *                    b B .. (b + 1) B per axis, every corner a trilinear
 *                    lookup (Source/buffer3d.h:222-242) at local coordinates
 *                    in [b B, (b + 1) B] can blend with a nonzero weight (the
 *                    trackers clamp their lookups to that range,
 *                    er_path.cuh sigma_point_in_brick).  One warp per brick,
 *                    coalesced reads along x.
 *   k_rmq_level    : level k of a sparse table of running maxima over the
 *                    sigma table (sigma[I] = DensityScale * Opacity(I)).
 *   k_majorant     : majorant[brick] = DensityScale * max sigma[lo..hi].
 *
 * A lookup inside a brick is a truncated trilinear blend of voxels in
 * [lo, hi]; float rounding of a blend (1 - t) a + t b can fall just below
 * min(a, b), which the truncation turns into one intensity less, so its
 * integer intensity lies in [lo - 1, hi] and its extinction
 * DensityScale * sigma[I] is bounded by the max over that range exactly
 * (max of the same floats, one multiply).  The CPU oracle builds the same grid by
 * brute force; the tests compare them bit for bit through the rendered paths.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdio>

#include "er_capi.h"
#include "er_kernels.h"

__global__ void k_brick_minmax(const uint16_t* __restrict__ vox, int rx, int ry, int rz, int B, int nbx, int nby, int nbz,
                               uint32_t* __restrict__ minmax)
{
    const int lane = threadIdx.x & 31;
    const long long total = (long long)nbx * nby * nbz;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    /* one warp per brick, grid-stride over the bricks (2^27 at 1^3 bricks of 512^3) */
    for (long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp < total; warp += nwarps) {
    const int bx = (int)(warp % nbx), by = (int)((warp / nbx) % nby), bz = (int)(warp / ((long long)nbx * nby));
    const int x0 = bx * B, y0 = by * B, z0 = bz * B;
    int x1 = (bx + 1) * B, y1 = (by + 1) * B, z1 = (bz + 1) * B;
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
                           float* __restrict__ majorant, long long total)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const uint32_t mm = minmax[i];
    int lo = (int)(mm & 0xffffu) - 1, hi = (int)(mm >> 16);
    lo = lo < 0 ? 0 : (lo > n - 1 ? n - 1 : lo);
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
    const long long total = (long long)nb[0] * nb[1] * nb[2];
    const long long want = (total * 32 + 255) / 256;
    k_brick_minmax<<<(unsigned)(want < 65536 ? want : 65536), 256, 0, s>>>(vox, res[0], res[1], res[2], B, nb[0], nb[1], nb[2],
                                                                           minmax);
    cudaError_t e = cudaMemcpyAsync(rmq, sigma, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    for (int k = 1; k < levels; k++)
        k_rmq_level<<<(n + 255) / 256, 256, 0, s>>>(rmq + (size_t)(k - 1) * n, rmq + (size_t)k * n, n, 1 << (k - 1));
    k_majorant<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(minmax, rmq, n, levels, density_scale, majorant, total);
    return cudaGetLastError();
}

/* Empty-space distances of the majorant grid.  For an empty brick (majorant
   0) dist = min over non-empty bricks q of max_a |b_a - q_a| (Chebyshev
   distance in bricks), capped at ER_SKIP_CAP; computed exactly by three 1D
   passes (x: nearest non-empty along the row; y and z: min over offsets of
   max(offset, previous pass)).  The last pass writes -dist into the empty
   bricks of the majorant grid: a tracker in such a brick knows every brick
   within dist-1 of it is empty too (er_path.cuh dda_jump). */
#define ER_SKIP_CAP 32

__global__ void k_skip_pass(const float* __restrict__ majorant, const uint8_t* __restrict__ in, uint8_t* __restrict__ out,
                            float* __restrict__ majorant_out, int axis, int nbx, int nby, int nbz, long long total)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const int b[3] = { (int)(i % nbx), (int)((i / nbx) % nby), (int)(i / ((long long)nbx * nby)) };
        const int n = axis == 0 ? nbx : (axis == 1 ? nby : nbz);
        const long long step = axis == 0 ? 1 : (axis == 1 ? (long long)nbx : (long long)nbx * nby);
        int best = ER_SKIP_CAP;
        for (int o = -(ER_SKIP_CAP - 1); o <= ER_SKIP_CAP - 1; o++) {
            const int c = b[axis] + o;
            if (c < 0 || c >= n) continue;
            const int ao = o < 0 ? -o : o;
            if (ao >= best) continue;
            const long long j = i + (long long)o * step;
            const int v = axis == 0 ? (majorant[j] > 0.0f ? 0 : ER_SKIP_CAP) : (int)in[j];
            const int d = v > ao ? v : ao;
            best = d < best ? d : best;
        }
        if (axis < 2) out[i] = (uint8_t)best;
        else if (!(majorant_out[i] > 0.0f)) majorant_out[i] = -(float)best;
    }
}

cudaError_t er_launch_empty_skip(float* majorant, const int nb[3], uint8_t* tmp, cudaStream_t s)
{
    const long long total = (long long)nb[0] * nb[1] * nb[2];
    const long long want = (total + 255) / 256;
    const unsigned blocks = (unsigned)(want < 65536 ? want : 65536);
    k_skip_pass<<<blocks, 256, 0, s>>>(majorant, nullptr, tmp, nullptr, 0, nb[0], nb[1], nb[2], total);
    k_skip_pass<<<blocks, 256, 0, s>>>(majorant, tmp, tmp + total, nullptr, 1, nb[0], nb[1], nb[2], total);
    k_skip_pass<<<blocks, 256, 0, s>>>(majorant, tmp + total, nullptr, majorant, 2, nb[0], nb[1], nb[2], total);
    return cudaGetLastError();
}

/* corner quads: for voxel (x, y, z) the intensities at (x, y), (x+1, y),
   (x, y+1), (x+1, y+1) of slice z, packed as two uint16 pairs, so that a
   trilinear lookup reads two 8-byte words instead of eight 2-byte ones;
   stored x fastest or in 8^3 bricks (quad_index, er_device.cuh).  This
   kernel writes the quads of the voxels in the box [lo, lo + n) (a region
   edit changes the quads of the voxels one below it in x and y as well) and
   finds the largest voxel value in the box. */
__global__ void k_box_quads_max(const uint16_t* __restrict__ vox, int rx, int ry, int x0, int y0, int z0, int nx, int ny, int nz,
                                uint2* __restrict__ quad, int qb_nbx, unsigned long long qb_slab, unsigned int* __restrict__ vmax)
{
    const size_t n = (size_t)nx * ny * nz;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    unsigned int m = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int x = x0 + (int)(i % nx), y = y0 + (int)((i / nx) % ny), z = z0 + (int)(i / ((size_t)nx * ny));
        const size_t zb = (size_t)z * rx * ry;
        const int x1 = x + 1 < rx ? x + 1 : rx - 1, y1 = y + 1 < ry ? y + 1 : ry - 1;
        const uint32_t v00 = vox[zb + (size_t)y * rx + x], v10 = vox[zb + (size_t)y * rx + x1];
        const uint32_t v01 = vox[zb + (size_t)y1 * rx + x], v11 = vox[zb + (size_t)y1 * rx + x1];
        if (quad) quad[erd::quad_index(x, y, z, rx, ry, qb_nbx, qb_slab)] = make_uint2(v00 | (v10 << 16), v01 | (v11 << 16));
        m = v00 > m ? v00 : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned int t = __shfl_xor_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(vmax, m);
}

cudaError_t er_launch_box_quads_max(const uint16_t* vox, const int res[3], const int lo[3], const int n[3], uint2* quad, int qb_nbx,
                                    unsigned long long qb_slab, unsigned int* vmax, cudaStream_t s)
{
    const size_t total = (size_t)n[0] * n[1] * n[2];
    if (total == 0) return cudaSuccess;
    size_t blocks = (total + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_box_quads_max<<<(unsigned)blocks, 256, 0, s>>>(vox, res[0], res[1], lo[0], lo[1], lo[2], n[0], n[1], n[2], quad, qb_nbx, qb_slab,
                                                     vmax);
    return cudaGetLastError();
}

/* ====================================================================== */
/* Allocation-free majorant build                                           */
/* ====================================================================== */
/*
 * Some callers cannot call cudaMalloc or cudaFree at the point where they
 * need a majorant grid: an application that rebuilds the grid inside its
 * frame loop (every edit of the opacity transfer function changes it), where
 * cudaMalloc/cudaFree would synchronise the whole device and stall the
 * frame; and hosts whose device memory is owned by their own pool allocator
 * and forbid allocations behind its back.  er_build_majorant_device_noalloc
 * serves them: the caller passes the inputs (voxels, sigma table) and the
 * output grid, and the two scratch buffers of the build (per-brick voxel
 * min/max, range-maximum table over the sigma table) live in the file-scope
 * device arrays below instead of library allocations.
 *
 * Limits: at most ER_NOALLOC_MAX_BRICKS bricks (2^20: a 1024x1024x512 volume
 * with 8^3 bricks) and ER_NOALLOC_MAX_SIGMA sigma entries (the full uint16
 * range).  Together the arrays take 8.25 MiB of device memory on every GPU
 * that loads the library, held until the process exits.
 *
 * Sharing: every call uses the same arrays, which keep the previous call's
 * contents.  Nothing in them has to start at zero: each call writes every
 * min/max entry and every range-table entry it reads before reading it.
 * Calls that overlap on the GPU (for example on two streams at once) race on
 * the arrays and must be serialised by the caller.
 *
 * Set-up: the first call on a device, with that device current, resolves the
 * arrays' device addresses with cudaGetSymbolAddress (the host-side names of
 * __device__ arrays are not device addresses).  Make that first call before
 * any stream capture.  The addresses belong to the device's current context;
 * when that context is replaced (cudaDeviceReset, then new work), the next
 * call sees a new context ID and resolves them again.
 */
#include <cuda.h>
#include <mutex>

#define ER_NOALLOC_MAX_BRICKS (1u << 20)
#define ER_NOALLOC_MAX_SIGMA 65536
#define ER_NOALLOC_MAX_LEVELS 17

static __device__ __align__(256) uint32_t g_noalloc_minmax[ER_NOALLOC_MAX_BRICKS];
static __device__ __align__(256) float g_noalloc_rmq[ER_NOALLOC_MAX_LEVELS * ER_NOALLOC_MAX_SIGMA];

namespace {

struct NoallocScratch {
    uint32_t* minmax;
    float* rmq;
    unsigned long long ctx_id;     /* context the addresses belong to (0: unknown) */
    bool ready;
};

#define ER_NOALLOC_MAX_DEVICES 64
std::mutex g_noalloc_mutex;
NoallocScratch g_noalloc[ER_NOALLOC_MAX_DEVICES];

/* The driver's cuCtxGetCurrent and cuCtxGetId, looked up through the runtime
   (the library does not link libcuda).  A context's ID is unique for the
   life of the process, so a device whose context was destroyed and made
   again (cudaDeviceReset) shows a new ID, and the arrays' addresses, which
   belong to the module loaded into the old context, are resolved again. */
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_ctx_fns_looked_up = false;

/* ID of the current context, 0 when it cannot be read */
unsigned long long current_context_id()
{
    if (!g_ctx_fns_looked_up) {
        g_ctx_fns_looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = (CtxGetCurrentFn)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = (CtxGetIdFn)f;
        cudaGetLastError();
    }
    if (!g_ctx_get_current || !g_ctx_get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_ctx_get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

/* device addresses of the scratch arrays in the current device's context:
   resolved once per context (the first call on a device, and again after
   its context was replaced); every call when the context ID cannot be read */
cudaError_t noalloc_scratch(int device, NoallocScratch* out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocScratch& s = g_noalloc[device];
    const unsigned long long id = current_context_id();
    if (!s.ready || id == 0 || id != s.ctx_id) {
        void* a = nullptr;
        void* b = nullptr;
        s.ready = false;
        cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_minmax);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&b, g_noalloc_rmq);
        if (e != cudaSuccess) return e;
        s.minmax = (uint32_t*)a;
        s.rmq = (float*)b;
        /* the first runtime call above makes the primary context current
           when nothing had: read the ID again */
        s.ctx_id = id ? id : current_context_id();
        s.ready = true;
    }
    *out = s;
    return cudaSuccess;
}

er_status noalloc_fail(er_status st, const char* msg)
{
    er_internal_set_error(msg);
    return st;
}

}  // namespace

extern "C" ER_API er_status er_build_majorant_device_noalloc(const uint16_t* d_voxels, const int32_t resolution[3], int32_t brick,
                                                             const float* d_sigma, int32_t sigma_count, float density_scale,
                                                             float* d_majorant, void* stream)
{
    char msg[256];
    if (!d_voxels || !resolution || !d_sigma || !d_majorant) return noalloc_fail(ER_ERR_INVALID_ARGUMENT, "NULL argument");
    if (brick < 1 || brick > 64) {
        snprintf(msg, sizeof(msg), "brick %d out of range [1, 64]", brick);
        return noalloc_fail(ER_ERR_INVALID_ARGUMENT, msg);
    }
    if (sigma_count < 1 || sigma_count > ER_NOALLOC_MAX_SIGMA) {
        snprintf(msg, sizeof(msg), "sigma_count %d out of range [1, %d]", sigma_count, ER_NOALLOC_MAX_SIGMA);
        return noalloc_fail(ER_ERR_INVALID_ARGUMENT, msg);
    }
    int res[3], nb[3];
    for (int i = 0; i < 3; i++) {
        if (resolution[i] <= 0) return noalloc_fail(ER_ERR_INVALID_ARGUMENT, "resolution must be positive");
        res[i] = resolution[i];
        nb[i] = (res[i] + brick - 1) / brick;
    }
    const unsigned long long total = (unsigned long long)nb[0] * nb[1] * nb[2];
    if (total > ER_NOALLOC_MAX_BRICKS) {
        snprintf(msg, sizeof(msg),
                 "%llu bricks exceed the allocation-free limit of %u (use a larger brick or er_build_majorant_device)", total,
                 ER_NOALLOC_MAX_BRICKS);
        return noalloc_fail(ER_ERR_INVALID_ARGUMENT, msg);
    }
    int levels = 1;
    while ((1 << levels) <= sigma_count) levels++;
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e == cudaSuccess && (device < 0 || device >= ER_NOALLOC_MAX_DEVICES)) return noalloc_fail(ER_ERR_INVALID_ARGUMENT, "device index out of range");
    NoallocScratch s;
    if (e == cudaSuccess) e = noalloc_scratch(device, &s);
    if (e == cudaSuccess)
        e = er_launch_majorant(d_voxels, res, brick, nb, d_sigma, sigma_count, s.rmq, levels, s.minmax, density_scale, d_majorant,
                               (cudaStream_t)stream);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "er_build_majorant_device_noalloc: %s", cudaGetErrorString(e));
        return noalloc_fail(ER_ERR_CUDA, msg);
    }
    return ER_OK;
}
