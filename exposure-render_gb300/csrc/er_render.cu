/*
 * er_render.cu - reference-order transport kernels (compiled with --fmad=false).
 *
 *   k_trace_frame : KrnlSingleScattering (Source/singlescattering.cuh:27-32):
 *                   one sample per pixel with the RNG lanes read from and
 *                   written back to per-pixel buffers.
 *   k_trace_sum   : `spp` counter-seeded samples per pixel in one launch,
 *                   summed in registers (one HBM write per pixel).
 *   k_sigma_table : DensityScale * Opacity1D(I) for every integer I.
 *   k_shade_table : the shading transfer functions for every integer I.
 */
#include "er_kernels.h"
#include "er_path.cuh"

using namespace erd;

__global__ void __launch_bounds__(128) k_trace_frame(const Params P, uint32_t* __restrict__ lanes, float4* __restrict__ frame)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = P.film[0], H = P.film[1];
    if (x >= W || y >= H) return;
    const size_t p = (size_t)y * (size_t)W + (size_t)x;
    const size_t n = (size_t)W * (size_t)H;
    Rng rng;
    rng.s0 = lanes[p];
    rng.s1 = lanes[n + p];
    frame[p] = single_scattering(P, x, y, rng);
    lanes[p] = rng.s0;
    lanes[n + p] = rng.s1;
}

__global__ void __launch_bounds__(128) k_trace_sum(const Params P, int spp, uint32_t view, uint32_t first, float4* __restrict__ sum,
                                                   int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = P.film[0], H = P.film[1];
    if (x >= W || y >= H) return;
    const uint32_t pix = (uint32_t)y * (uint32_t)W + (uint32_t)x;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int k = 0; k < spp; k++) {
        Rng rng;
        er_seed_lanes(P.seed, view, pix, first + (uint32_t)k, &rng.s0, &rng.s1);
        const float4 o = single_scattering(P, x, y, rng, view, (int64_t)(first + (uint32_t)k));
        a0 += o.x; a1 += o.y; a2 += o.z; a3 += o.w;
    }
    float4 r = make_float4(a0, a1, a2, a3);
    if (accumulate) {
        const float4 q = sum[pix];
        r = make_float4(q.x + a0, q.y + a1, q.z + a2, q.w + a3);
    }
    sum[pix] = r;
}

__global__ void k_sigma_table(const Plf* __restrict__ opacity, float density_scale, float* __restrict__ table, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    table[i] = density_scale * plf_eval(*opacity, (float)i);
}

/* the shading transfer functions at every integer intensity (shade_tf) */
__global__ void k_shade_table(const Tfs* __restrict__ tfs, float4* __restrict__ tab, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float I = (float)i;
    const c3 Kd = ctf_eval(tfs->diffuse, I), Ks = ctf_eval(tfs->specular, I), Le = ctf_eval(tfs->emission, I);
    const float exponent = 1000000.0f * pow_c(plf_eval(tfs->glossiness, I), 7.0f);
    tab[3 * i] = make_float4(Kd.r, Kd.g, Kd.b, exponent);
    tab[3 * i + 1] = make_float4(Ks.r, Ks.g, Ks.b, plf_eval(tfs->opacity, I));
    tab[3 * i + 2] = make_float4(Le.r, Le.g, Le.b, 0.0f);
}

/* ---- launchers ---- */

/* KrnlComputeAutoFocusDistance (Source/autofocus.cuh:26-62, one thread):
   100 rays through the screen point of film pixel (u, v), each moved by
   0.01 x ConcentricSampleDisk(Get2()), traced by the fixed-step march; the
   mean camera-to-event distance.  The event is not reset between rays (a
   miss after a hit counts the previous hit again); without any hit the
   result is the distance from the camera to the origin. */
__global__ void k_autofocus(const Params P, int u, int v, uint32_t lane0, uint32_t lane1, float* out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    Rng rng;
    rng.s0 = lane0;
    rng.s1 = lane1;
    Event SE;
    SE.type = 0; SE.valid = false; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
    SE.P = V3(0, 0, 0); SE.N = V3(0, 0, 0); SE.Wo = V3(0, 0, 0);
    Ray Rc;
    Rc.O = vload(P.pos); Rc.D = vload(P.N); Rc.MinT = P.clip_near; Rc.MaxT = P.clip_far;
    float Sum = 0.0f, SumWeight = 0.0f;
    for (int i = 0; i < 100; i++) {
        float sp0 = P.screen00 + (P.inv_screen0 * (float)u);
        float sp1 = P.screen10 + (P.inv_screen1 * (float)v);
        const v2 d = concentric_sample_disk(rng.get2());
        sp0 += 0.01f * d.x;
        sp1 += 0.01f * d.y;
        Rc.O = vload(P.pos);
        Rc.D = vnorm(vsub(vadd(vload(P.N), vscale(vload(P.U), sp0)), vscale(vload(P.V), sp1)));
        Rc.MinT = P.clip_near;
        Rc.MaxT = P.clip_far;
        sample_volume<false>(P, Rc, rng, SE);
        if (SE.valid) {
            Sum += vlen(vsub(SE.P, Rc.O));
            SumWeight += 1.0f;
        }
    }
    *out = Sum <= 0.0f ? vlen(vsub(SE.P, Rc.O)) : Sum / SumWeight;
}

cudaError_t er_launch_autofocus(const Params& P, int u, int v, uint32_t lane0, uint32_t lane1, float* out, cudaStream_t s)
{
    k_autofocus<<<1, 32, 0, s>>>(P, u, v, lane0, lane1, out);
    return cudaGetLastError();
}

cudaError_t er_launch_trace_frame(const Params& P, uint32_t* lanes, float4* frame, cudaStream_t s)
{
    const dim3 b(16, 8);
    const dim3 g((P.film[0] + 15) / 16, (P.film[1] + 7) / 8);
    k_trace_frame<<<g, b, 0, s>>>(P, lanes, frame);
    return cudaGetLastError();
}

cudaError_t er_launch_trace_sum(const Params& P, int spp, uint32_t view, uint32_t first, float4* sum, int accumulate,
                                cudaStream_t s)
{
    const dim3 b(16, 8);
    const dim3 g((P.film[0] + 15) / 16, (P.film[1] + 7) / 8);
    k_trace_sum<<<g, b, 0, s>>>(P, spp, view, first, sum, accumulate);
    return cudaGetLastError();
}

cudaError_t er_launch_shade_table(const Tfs* tfs, float4* tab, int n, cudaStream_t s)
{
    k_shade_table<<<(n + 127) / 128, 128, 0, s>>>(tfs, tab, n);
    return cudaGetLastError();
}

cudaError_t er_launch_sigma_table(const Plf* opacity, float density_scale, float* table, int n, cudaStream_t s)
{
    k_sigma_table<<<(n + 255) / 256, 256, 0, s>>>(opacity, density_scale, table, n);
    return cudaGetLastError();
}
