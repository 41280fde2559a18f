/*
 * er_post.cu - post-processing kernels (compiled with --fmad=false).
 *
 *   k_post_frame  : the three reference kernels that follow the transport
 *                   kernel in RenderEstimate (Source/core.cu:130-135) fused
 *                   into one pass: 3x3 Gaussian of the frame
 *                   (Source/filterframeestimate.cuh:33-64), running estimate
 *                   R += (F - R) / max(N, 1) (Source/estimate.cuh:27-32) and
 *                   tone map to RGBA8 (Source/tonemap.cuh:30-59).  One read of
 *                   the 3x3 neighbourhood (cached), one read and one write of
 *                   the running estimate, one 4-byte write.
 *   k_post_mean   : the same for the spp-batched path: sample mean of a sum
 *                   buffer, Gaussian of the mean, tone map.
 *   k_tonemap     : tone map of a scaled XYZA buffer.
 *   k_bilateral_h/v : separable bilateral filter on RGBA8, the design of
 *                   Source/filterrunningestimate.cuh:35-200 (window end
 *                   exclusive, alpha 255, luminance-difference range weight).
 *   k_gradient_magnitude : per-voxel |grad I| at voxel centres
 *                   (Source/gradientmagnitude.cuh:28-44 design,
 *                   Source/volumes.h:93-114 arithmetic) with a max reduction.
 */
#include "er_kernels.h"
#include "er_path.cuh"

using namespace erd;

ER_D uchar4 tonemap_px(float4 R, float exposure)
{
    float rgb[3];
    rgb[0] = 3.240479f * R.x - 1.537150f * R.y - 0.498535f * R.z;
    rgb[1] = -0.969256f * R.x + 1.875991f * R.y + 0.041556f * R.z;
    rgb[2] = 0.055648f * R.x - 0.204043f * R.y + 1.057311f * R.z;
    unsigned char o[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float c = 1.0f - er_expf(-(rgb[i] / exposure));
        c = smax(0.0f, smin(c, 1.0f));
        o[i] = (unsigned char)(255.0f * c);
    }
    return make_uchar4(o[0], o[1], o[2], (unsigned char)(R.w * 255.0f));
}

/* Gauss2D(1, dx, dy) - Source/filterframeestimate.cuh:28-31 */
ER_D float gauss_w(int dx, int dy) { return er_expf(-((float)(dx * dx + dy * dy) / (2 * 1.0f * 1.0f))); }

template <bool FROM_SUM>
ER_D float4 filtered_pixel(const float4* __restrict__ src, float inv_n_div, int x, int y, int W, int H, int filter)
{
    const size_t c = (size_t)y * W + x;
    if (!filter) {
        float4 v = src[c];
        if (FROM_SUM) v = make_float4(v.x / inv_n_div, v.y / inv_n_div, v.z / inv_n_div, v.w / inv_n_div);
        return v;
    }
    const int x0 = (x - 1) > 0 ? (x - 1) : 0;
    const int x1 = (x + 1) < (W - 1) ? (x + 1) : (W - 1);
    const int y0 = (y - 1) > 0 ? (y - 1) : 0;
    const int y1 = (y + 1) < (H - 1) ? (y + 1) : (H - 1);
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f, tot = 0.0f;
    for (int yy = y0; yy <= y1; yy++) {
        for (int xx = x0; xx <= x1; xx++) {
            const float w = gauss_w(xx - x, yy - y);
            float4 f = src[(size_t)yy * W + xx];
            if (FROM_SUM) f = make_float4(f.x / inv_n_div, f.y / inv_n_div, f.z / inv_n_div, f.w / inv_n_div);
            s0 += f.x * w; s1 += f.y * w; s2 += f.z * w; s3 += f.w * w;
            tot += w;
        }
    }
    float4 ctr = src[c];
    if (FROM_SUM) ctr.w = ctr.w / inv_n_div;
    s3 = ctr.w;
    if (tot > 0.0f) return make_float4(s0 / tot, s1 / tot, s2 / tot, s3 / tot);
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_post_frame(const float4* __restrict__ frame, float4* __restrict__ running, uchar4* __restrict__ rgba, int W,
                             int H, int no_iterations, float exposure, int filter)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t c = (size_t)y * W + x;
    const float4 F = filtered_pixel<false>(frame, 1.0f, x, y, W, H, filter);
    const float div = smax((float)no_iterations, 1.0f);
    const float4 A = running[c];
    const float4 R = make_float4(A.x + (F.x - A.x) / div, A.y + (F.y - A.y) / div, A.z + (F.z - A.z) / div, A.w + (F.w - A.w) / div);
    running[c] = R;
    rgba[c] = tonemap_px(R, exposure);
}

__global__ void k_post_mean(const float4* __restrict__ sum, float n, float4* __restrict__ running, uchar4* __restrict__ rgba, int W,
                            int H, float exposure, int filter)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t c = (size_t)y * W + x;
    const float4 R = filtered_pixel<true>(sum, n, x, y, W, H, filter);
    running[c] = R;
    rgba[c] = tonemap_px(R, exposure);
}

/* k_post_mean for every view of a batch (blockIdx.z = view); an accumulating
   view's sum holds samples [0, first + spp) of its stream */
__global__ void k_post_batch(const WfView* __restrict__ views)
{
    const WfView& V = views[blockIdx.z];
    if (!V.display) return;
    const int W = V.P.film[0], H = V.P.film[1];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const float n = V.accumulate ? (float)(V.first + (uint32_t)V.spp) : (float)V.spp;
    const size_t c = (size_t)y * W + x;
    const float4 R = filtered_pixel<true>(V.sum, n, x, y, W, H, V.filter);
    V.running[c] = R;
    V.rgba[c] = tonemap_px(R, V.exposure);
}

__global__ void k_tonemap(const float4* __restrict__ xyza, float scale, uchar4* __restrict__ rgba, int n, float exposure)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = xyza[i];
    if (scale != 1.0f) v = make_float4(v.x * scale, v.y * scale, v.z * scale, v.w * scale);
    rgba[i] = tonemap_px(v, exposure);
}

/* luminance with the weights of the LUMINANCE macro (Source/color.h:37-51) */
ER_D float lum255(uchar4 c)
{
    float L = 0.0f;
    L += 0.212671f * (float)c.x;
    L += 0.715160f * (float)c.y;
    L += 0.072169f * (float)c.z;
    return L;
}

template <bool HORIZONTAL>
__global__ void k_bilateral(const uchar4* __restrict__ in, uchar4* __restrict__ out, int W, int H, BilateralTables T)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int r = T.radius;
    const int i = HORIZONTAL ? x : y;
    const int lim = HORIZONTAL ? W : H;
    const int r0 = (i - r) > 0 ? (i - r) : 0;
    const int r1 = (i + r) < (lim - 1) ? (i + r) : (lim - 1);
    const uchar4 ctr = in[(size_t)y * W + x];
    const float lc = lum255(ctr);
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, tot = 0.0f;
    for (int k = r0; k < r1; k++) {     /* window end exclusive (Source/filterrunningestimate.cuh:88,157) */
        const uchar4 c = HORIZONTAL ? in[(size_t)y * W + k] : in[(size_t)k * W + x];
        int d = (int)fabsf(lum255(c) - lc);
        d = d > 255 ? 255 : d;
        const float w = T.spatial[r + k - i] * T.range[d];
        tot += w;
        s0 += (float)c.x * w; s1 += (float)c.y * w; s2 += (float)c.z * w;
    }
    uchar4 o;
    if (tot > 0.0f) {
        o.x = (unsigned char)eclamp(s0 / tot, 0.0f, 255.0f);
        o.y = (unsigned char)eclamp(s1 / tot, 0.0f, 255.0f);
        o.z = (unsigned char)eclamp(s2 / tot, 0.0f, 255.0f);
    } else {
        o.x = 0; o.y = 0; o.z = 0;
    }
    o.w = 255;
    out[(size_t)y * W + x] = o;
}

/* per-voxel gradient magnitude at voxel centres + max; the magnitude volume
   (optional) saturates at 65535 */
__global__ void k_gradient_magnitude(const Params P, uint16_t* __restrict__ gm, unsigned int* __restrict__ max_bits)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y * blockDim.y + threadIdx.y;
    const int Z = blockIdx.z * blockDim.z + threadIdx.z;
    float g = 0.0f;
    if (X < P.res[0] && Y < P.res[1] && Z < P.res[2]) {
        const float sx = 2.0f * P.half_size[0], sy = 2.0f * P.half_size[1], sz = 2.0f * P.half_size[2];
        const v3 p = V3(P.minp[0] + sx * (((float)X + 0.5f) * (1.0f / (float)P.res[0])),
                        P.minp[1] + sy * (((float)Y + 0.5f) * (1.0f / (float)P.res[1])),
                        P.minp[2] + sz * (((float)Z + 0.5f) * (1.0f / (float)P.res[2])));
        g = gradient_magnitude(P, p);
        if (gm) {
            const size_t idx = (size_t)Z * P.res[0] * P.res[1] + (size_t)Y * P.res[0] + X;
            gm[idx] = (uint16_t)(g < 65535.0f ? g : 65535.0f);
        }
    }
    /* block max through warp shuffles, one atomic per warp; non-negative
       floats order like their bit patterns */
    unsigned int b = __float_as_uint(g);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned int v = __shfl_xor_sync(0xffffffffu, b, o);
        b = v > b ? v : b;
    }
    if ((threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y) % 32 == 0) atomicMax(max_bits, b);
}

__global__ void k_math_eval(int fn, int n, const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = x[i];
    const float b = y ? y[i] : 0.0f;
    float r = 0.0f;
    switch (fn) {
    case 0: r = er_logf(a); break;
    case 1: r = er_expf(a); break;
    case 2: r = er_sinf(a); break;
    case 3: r = er_cosf(a); break;
    case 4: r = er_tanf(a); break;
    case 5: r = er_powf(a, b); break;
    case 6: r = er_acosf(a); break;
    case 7: r = er_atan2f(a, b); break;
    default: break;
    }
    out[i] = r;
}

/* ---- launchers ---- */

cudaError_t er_launch_math_eval(int fn, int n, const float* x, const float* y, float* out, cudaStream_t s)
{
    k_math_eval<<<(n + 255) / 256, 256, 0, s>>>(fn, n, x, y, out);
    return cudaGetLastError();
}

cudaError_t er_launch_post_frame(const float4* frame, float4* running, uchar4* rgba, int W, int H, int n_iter, float exposure,
                                 int filter, cudaStream_t s)
{
    const dim3 b(16, 8), g((W + 15) / 16, (H + 7) / 8);
    k_post_frame<<<g, b, 0, s>>>(frame, running, rgba, W, H, n_iter, exposure, filter);
    return cudaGetLastError();
}

cudaError_t er_launch_post_mean(const float4* sum, float n, float4* running, uchar4* rgba, int W, int H, float exposure, int filter,
                                cudaStream_t s)
{
    const dim3 b(16, 8), g((W + 15) / 16, (H + 7) / 8);
    k_post_mean<<<g, b, 0, s>>>(sum, n, running, rgba, W, H, exposure, filter);
    return cudaGetLastError();
}

cudaError_t er_launch_post_batch(const WfView* d_views, int n_views, int max_w, int max_h, cudaStream_t s)
{
    const dim3 b(16, 8), g((max_w + 15) / 16, (max_h + 7) / 8, n_views);
    k_post_batch<<<g, b, 0, s>>>(d_views);
    return cudaGetLastError();
}

cudaError_t er_launch_tonemap(const float4* xyza, float scale, uchar4* rgba, int n, float exposure, cudaStream_t s)
{
    k_tonemap<<<(n + 255) / 256, 256, 0, s>>>(xyza, scale, rgba, n, exposure);
    return cudaGetLastError();
}

cudaError_t er_launch_bilateral(const uchar4* in, uchar4* tmp, uchar4* out, int W, int H, const BilateralTables& T,
                                cudaStream_t s)
{
    const dim3 b(16, 8), g((W + 15) / 16, (H + 7) / 8);
    k_bilateral<true><<<g, b, 0, s>>>(in, tmp, W, H, T);
    k_bilateral<false><<<g, b, 0, s>>>(tmp, out, W, H, T);
    return cudaGetLastError();
}

cudaError_t er_launch_gradient_magnitude(const Params& P, uint16_t* gm, unsigned int* max_bits, cudaStream_t s)
{
    const dim3 b(8, 8, 8);
    const dim3 g((P.res[0] + 7) / 8, (P.res[1] + 7) / 8, (P.res[2] + 7) / 8);
    k_gradient_magnitude<<<g, b, 0, s>>>(P, gm, max_bits);
    return cudaGetLastError();
}
