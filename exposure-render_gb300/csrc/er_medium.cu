/*
 * er_medium.cu - the differentiable medium: forward estimator, path-replay
 * adjoint and majorant build (compiled with --fmad=false; extension with no
 * reference counterpart).
 *
 * Medium: sigma(x) = scale * alpha(rho(x)).  rho is the trilinear
 * interpolation of a float density grid with the addressing of the
 * intensity volume (Source/buffer3d.h:222-242, without the unsigned-short
 * truncation); alpha is a uniform cubic B-spline of n opacity values over
 * u = 2 + rho * (n - 5), C2 in rho on [-1/(n-5), 1 + 1/(n-5)] and linear in
 * the values.
 *
 * Estimator (one thread per sample): the camera ray's tentative collisions
 * come from a fixed majorant grid (the delta tracker's DDA); at each, with
 * probability q (a draw independent of the medium) a next-event estimate to
 * one uniformly picked light with a ratio-tracked shadow segment, weighted
 * by sigma/mu and the ratio-tracked throughput T = prod(1 - sigma_j/mu_j) of
 * the earlier collisions.  The RNG draws do not depend on the medium, so for
 * fixed seeds a sample is a smooth function of density and opacity values.
 *
 * Adjoint (path replay): the same draws again; with the sample's forward
 * value Ltot and the prefix L_<=k of contributions,
 *     dL/dsigma_k = T_k A_k / mu_k - (Ltot - L_<=k) / (mu_k - sigma_k)
 * at every primary collision and -(g . c_k) / (mu_i - sigma_i) at every
 * collision i of the shadow segment of contribution c_k.  The forward value
 * comes from the stored samples or, without them, from a first pass of the
 * same thread.  Opacity gradients gather in shared memory per block,
 * density gradients go to global memory with atomic adds.
 *
 * The arithmetic is the CPU oracle's (oracle/er_oracle.c, dm_*), operation
 * for operation: forward samples are bit-identical to it.
 */
#include "er_capi.h"
#include "er_kernels.h"
#include "er_path.cuh"

using namespace erd;

namespace {

#define DM_INV_4PI 0.0795774715459476678f

/* Real: float (the estimator, bit-exact with the oracle) or double (the
   same samples with every medium-dependent quantity in binary64 - the
   geometry, which does not depend on the medium, stays float) */
template <typename Real>
struct DmLookup {
    uint32_t idx[8];
    float w[8];
    Real rho;
};

ER_D uint32_t dm_index(const Params& P, int x, int y, int z)
{
    const int cx = x < 0 ? 0 : (x > P.res[0] - 1 ? P.res[0] - 1 : x);
    const int cy = y < 0 ? 0 : (y > P.res[1] - 1 ? P.res[1] - 1 : y);
    const int cz = z < 0 ? 0 : (z > P.res[2] - 1 ? P.res[2] - 1 : z);
    return (uint32_t)cz * (uint32_t)P.res[0] * (uint32_t)P.res[1] + (uint32_t)cy * (uint32_t)P.res[0] + (uint32_t)cx;
}

template <typename Real>
ER_D void dm_density(const Params& P, const DmParams& M, v3 p, DmLookup<Real>& k)
{
    const v3 off = V3(p.x - P.minp[0], p.y - P.minp[1], p.z - P.minp[2]);
    const float Lx = off.x * P.inv_size[0] * (float)P.res[0];
    const float Ly = off.y * P.inv_size[1] * (float)P.res[1];
    const float Lz = off.z * P.inv_size[2] * (float)P.res[2];
    const int vx = (int)floorf(Lx), vy = (int)floorf(Ly), vz = (int)floorf(Lz);
    const float dx = Lx - (float)vx, dy = Ly - (float)vy, dz = Lz - (float)vz;
    const float ex = 1.0f - dx, ey = 1.0f - dy, ez = 1.0f - dz;
    Real r = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int ox = c & 1, oy = (c >> 1) & 1, oz = (c >> 2) & 1;
        k.idx[c] = dm_index(P, vx + ox, vy + oy, vz + oz);
        k.w[c] = (ox ? dx : ex) * (oy ? dy : ey) * (oz ? dz : ez);
        r = r + (Real)k.w[c] * (Real)__ldg(M.rho + k.idx[c]);
    }
    k.rho = r;
}

template <typename Real>
struct DmTf {
    Real alpha, dalpha;
    int i0;
    Real b[4];
};

template <typename Real>
ER_D void dm_opacity(const DmParams& M, Real rho, DmTf<Real>& o)
{
    const int n = M.tf_n;
    const Real du = (Real)(n - 5);
    Real u = (Real)2.0f + rho * du;
    int slope = 1;
    if (u < (Real)1.0f) { u = 1.0f; slope = 0; }
    if (u > (Real)(n - 2)) { u = (Real)(n - 2); slope = 0; }
    int i = (int)floor(u);
    if (i > n - 3) i = n - 3;
    const Real f = u - (Real)i;
    const Real g = (Real)1.0f - f;
    const Real f2 = f * f, f3 = f2 * f;
    o.b[0] = g * g * g / (Real)6.0f;
    o.b[1] = ((Real)3.0f * f3 - (Real)6.0f * f2 + (Real)4.0f) / (Real)6.0f;
    o.b[2] = ((Real)-3.0f * f3 + (Real)3.0f * f2 + (Real)3.0f * f + (Real)1.0f) / (Real)6.0f;
    o.b[3] = f3 / (Real)6.0f;
    const Real d0 = (Real)-0.5f * g * g, d1 = (Real)1.5f * f2 - (Real)2.0f * f, d2 = (Real)-1.5f * f2 + f + (Real)0.5f,
               d3 = (Real)0.5f * f2;
    o.i0 = i - 1;
    const Real v0 = __ldg(M.tf + i - 1), v1 = __ldg(M.tf + i), v2 = __ldg(M.tf + i + 1), v3 = __ldg(M.tf + i + 2);
    o.alpha = o.b[0] * v0 + o.b[1] * v1 + o.b[2] * v2 + o.b[3] * v3;
    o.dalpha = slope ? du * (d0 * v0 + d1 * v1 + d2 * v2 + d3 * v3) : (Real)0.0f;
}

/* dLoss/dsigma = a at one lookup, scattered into the gradients */
ER_D void dm_scatter(const DmParams& M, const DmLookup<float>& k, const DmTf<float>& o, float a, float* g_rho, float* s_tf)
{
    const float as = a * M.scale;
    if (s_tf) {
#pragma unroll
        for (int j = 0; j < 4; j++) atomicAdd(s_tf + o.i0 + j, as * o.b[j]);
    }
    if (g_rho && o.dalpha != 0.0f) {
        const float ar = as * o.dalpha;
#pragma unroll
        for (int c = 0; c < 8; c++) atomicAdd(g_rho + k.idx[c], ar * k.w[c]);
    }
}

ER_D bool dm_segment(const Params& P, const Ray& R, float& t0, float& t1)
{
    Isect Int; Int.invalid();
    intersect_box(R, vload(P.minp), vload(P.half_size), Int, false);
    if (!Int.valid) return false;
    t0 = smax(Int.near_t, R.MinT);
    t1 = smin(Int.far_t, R.MaxT);
    return t0 < t1;
}

/* ratio-tracked shadow transmittance; ADJ scatters -a_scale / (mu - sigma) */
template <bool ADJ, typename Real = float>
ER_D Real dm_shadow(const Params& P, const DmParams& M, v3 P1, v3 P2, Rng& rng, float a_scale, float* g_rho, float* s_tf)
{
    if (!P.shadows) return 1.0f;
    const v3 W = vnorm(vsub(P2, P1));
    Ray R;
    R.O = vadd(P1, vscale(W, ER_RAY_EPS));
    R.D = W;
    R.MinT = 0.0f;
    R.MaxT = smin(vlen(vsub(P2, P1)) - 2.0f * ER_RAY_EPS, P.max_shadow_distance);
    float t0, t1;
    if (!dm_segment(P, R, t0, t1)) return 1.0f;
    Dda d;
    dda_init(P, R, t0, t1, d);
    Real Tr = 1.0f;
    float tau = -er_logf(rng.get1());
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(d);
        const float mu = dda_majorant(P, d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 Pt = vadd(R.O, vscale(R.D, t));
                DmLookup<Real> k;
                dm_density(P, M, Pt, k);
                DmTf<Real> o;
                dm_opacity(M, k.rho, o);
                const Real sig = (Real)M.scale * o.alpha;
                if constexpr (ADJ) dm_scatter(M, k, o, -a_scale / (mu - sig), g_rho, s_tf);
                Tr = Tr * ((Real)1.0f - sig / (Real)mu);
                if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); return Tr; }
                tau = -er_logf(rng.get1());
            }
        }
        dda_advance(P, d, e);
    }
    return Tr;
}

/* next-event estimate at Pt without the collision weight and the shadow */
ER_D c3 dm_nee(const Params& P, const DmParams& M, v3 Pt, Rng& rng, v3& S, bool& has)
{
    has = false;
    const float pick = rng.get1();
    const v3 uvw = rng.get3();
    if (P.light_count <= 0) return C3(0, 0, 0);
    int idx = (int)floorf(pick * (float)P.light_count);
    if (idx >= P.light_count) idx = P.light_count - 1;
    if (idx < 0 || !P.light_valid[idx]) return C3(0, 0, 0);
    const Light& L = P.lights[idx];
    Event SE;
    SE.type = 0; SE.valid = false; SE.T = 0.0f; SE.Le = C3(0, 0, 0);
    SE.P = Pt; SE.N = V3(0, 0, 0); SE.Wo = V3(0, 0, 0);
    v3 Wi;
    c3 Li;
    Surf SS;
    sample_light(P, L, uvw, SS, SE, Wi, Li);
    S = SS.P;
    if (cblack(Li)) return C3(0, 0, 0);
    const float LightPdf = vlen2(vsub(Pt, SS.P)) / (vabsdot(SS.N, vneg(Wi)) * L.area);
    if (!(LightPdf > 0.0f)) return C3(0, 0, 0);
    has = true;
    return cscale(cmul(C3(M.albedo[0], M.albedo[1], M.albedo[2]), Li), DM_INV_4PI * (float)P.light_count / (LightPdf * M.q));
}

/* the sample's value; Real = double returns it in L64 (L is then unused) */
template <bool ADJ, typename Real = float>
ER_D c3 dm_sample(const Params& P, const DmParams& M, int x, int y, Rng& rng, c3 g, c3 Ltot, float* g_rho, float* s_tf,
                  double* L64 = nullptr)
{
    c3 L = C3(0, 0, 0);
    double Ld[3] = {0.0, 0.0, 0.0};
    double Td = 1.0;
    const v2 film_uv = rng.get2();
    const v2 lens_uv = rng.get2();
    const Ray R = sample_camera(P, x, y, film_uv, lens_uv);
    float t0, t1;
    if (!dm_segment(P, R, t0, t1)) return L;
    Dda d;
    dda_init(P, R, t0, t1, d);
    float T = 1.0f;
    float tau = -er_logf(rng.get1());
    int guard = 0;
    while (!d.done) {
        const float e = dda_exit(d);
        const float mu = dda_majorant(P, d);
        float t = d.t;
        if (mu > 0.0f) {
            for (;;) {
                const float dt = tau / mu;
                if (!(t + dt < e)) {
                    tau = tau - mu * (e - t);
                    if (tau < 0.0f) tau = 0.0f;
                    break;
                }
                t = t + dt;
                const v3 Pt = vadd(R.O, vscale(R.D, t));
                DmLookup<Real> k;
                dm_density(P, M, Pt, k);
                DmTf<Real> o;
                dm_opacity(M, k.rho, o);
                if constexpr (sizeof(Real) == 8) {
                    /* binary64 evaluation of the same sample: the draws are those of the float path */
                    const double sig = (double)M.scale * o.alpha;
                    const double w = sig / (double)mu;
                    if (rng.get1() < M.q) {
                        v3 S;
                        bool has;
                        const c3 A0 = dm_nee(P, M, Pt, rng, S, has);
                        if (has) {
                            const double Tr = dm_shadow<false, double>(P, M, Pt, S, rng, 0.0f, nullptr, nullptr);
                            Ld[0] += (double)A0.r * Tr * Td * w;
                            Ld[1] += (double)A0.g * Tr * Td * w;
                            Ld[2] += (double)A0.b * Tr * Td * w;
                        }
                    }
                    Td = Td * (1.0 - w);
                    if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); break; }
                    tau = -er_logf(rng.get1());
                    continue;
                } else {
                const float sig = M.scale * o.alpha;
                if (!(sig < mu)) atomicOr(P.err, 4);     /* the majorant no longer bounds sigma */
                const float w = sig / mu;
                c3 A = C3(0, 0, 0);
                if (rng.get1() < M.q) {
                    v3 S;
                    bool has;
                    const c3 A0 = dm_nee(P, M, Pt, rng, S, has);
                    if (has) {
                        if constexpr (ADJ) {
                            const Rng keep = rng;
                            const float Tr = dm_shadow<false>(P, M, Pt, S, rng, 0.0f, nullptr, nullptr);
                            A = cscale(A0, Tr);
                            const c3 c = cscale(A, T * w);
                            const float gc = g.r * c.r + g.g * c.g + g.b * c.b;
                            if (gc != 0.0f) {
                                Rng r2 = keep;
                                dm_shadow<true>(P, M, Pt, S, r2, gc, g_rho, s_tf);
                            }
                        } else {
                            A = cscale(A0, dm_shadow<false>(P, M, Pt, S, rng, 0.0f, nullptr, nullptr));
                        }
                    }
                }
                const c3 c = cscale(A, T * w);
                L = cadd(L, c);
                if constexpr (ADJ) {
                    const c3 rest = csub(Ltot, L);
                    const c3 dLds = csub(cscale(A, T / mu), cdivs(rest, mu - sig));
                    const float a = g.r * dLds.r + g.g * dLds.g + g.b * dLds.b;
                    if (a != 0.0f) dm_scatter(M, k, o, a, g_rho, s_tf);
                }
                T = T * (1.0f - w);
                if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); return L; }
                tau = -er_logf(rng.get1());
                }
            }
        }
        dda_advance(P, d, e);
    }
    if (L64) { L64[0] = Ld[0]; L64[1] = Ld[1]; L64[2] = Ld[2]; }
    return L;
}

__global__ void __launch_bounds__(256) k_dm_forward(const Params P, const DmParams M, int spp, uint32_t view, uint32_t first,
                                                    uint32_t npix, float* __restrict__ samples)
{
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < items; i += stride) {
        const uint32_t s = (uint32_t)(i / npix);
        const uint32_t pix = (uint32_t)(i - (uint64_t)s * npix);
        Rng rng;
        er_seed_lanes(P.seed, view, pix, first + s, &rng.s0, &rng.s1);
        const int x = (int)(pix % (uint32_t)P.film[0]), y = (int)(pix / (uint32_t)P.film[0]);
        const c3 L = dm_sample<false>(P, M, x, y, rng, C3(0, 0, 0), C3(0, 0, 0), nullptr, nullptr);
        samples[3 * i] = L.r;
        samples[3 * i + 1] = L.g;
        samples[3 * i + 2] = L.b;
    }
}

/* the binary64 evaluation: per-sample values in double (finite differences) */
__global__ void __launch_bounds__(256) k_dm_forward64(const Params P, const DmParams M, int spp, uint32_t view, uint32_t first,
                                                      uint32_t npix, double* __restrict__ samples)
{
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < items; i += stride) {
        const uint32_t s = (uint32_t)(i / npix);
        const uint32_t pix = (uint32_t)(i - (uint64_t)s * npix);
        Rng rng;
        er_seed_lanes(P.seed, view, pix, first + s, &rng.s0, &rng.s1);
        const int x = (int)(pix % (uint32_t)P.film[0]), y = (int)(pix / (uint32_t)P.film[0]);
        double L[3];
        dm_sample<false, double>(P, M, x, y, rng, C3(0, 0, 0), C3(0, 0, 0), nullptr, nullptr, L);
        samples[3 * i] = L[0];
        samples[3 * i + 1] = L[1];
        samples[3 * i + 2] = L[2];
    }
}

__global__ void k_dm_reduce64(const double* __restrict__ samples, int spp, uint32_t npix, double* __restrict__ sum)
{
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int s = 0; s < spp; s++) {
        const size_t q = 3 * ((size_t)s * npix + pix);
        a0 += samples[q];
        a1 += samples[q + 1];
        a2 += samples[q + 2];
    }
    sum[3 * pix] = a0;
    sum[3 * pix + 1] = a1;
    sum[3 * pix + 2] = a2;
}

/* per-pixel sums over the samples in sample order */
__global__ void k_dm_reduce(const float* __restrict__ samples, int spp, uint32_t npix, float* __restrict__ sum)
{
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    for (int s = 0; s < spp; s++) {
        const size_t q = 3 * ((size_t)s * npix + pix);
        a0 += samples[q];
        a1 += samples[q + 1];
        a2 += samples[q + 2];
    }
    sum[3 * pix] = a0;
    sum[3 * pix + 1] = a1;
    sum[3 * pix + 2] = a2;
}

__global__ void __launch_bounds__(256) k_dm_adjoint(const Params P, const DmParams M, int spp, uint32_t view, uint32_t first,
                                                    uint32_t npix, const float* __restrict__ dimg,
                                                    const float* __restrict__ fwd, float* __restrict__ g_rho,
                                                    float* __restrict__ g_tf)
{
    __shared__ float s_tf[ER_MAX_TF_NODES];
    for (int j = threadIdx.x; j < ER_MAX_TF_NODES; j += blockDim.x) s_tf[j] = 0.0f;
    __syncthreads();
    float* stf = g_tf ? s_tf : nullptr;
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < items; i += stride) {
        const uint32_t s = (uint32_t)(i / npix);
        const uint32_t pix = (uint32_t)(i - (uint64_t)s * npix);
        const c3 g = C3(dimg[3 * pix], dimg[3 * pix + 1], dimg[3 * pix + 2]);
        if (g.r == 0.0f && g.g == 0.0f && g.b == 0.0f) continue;
        const int x = (int)(pix % (uint32_t)P.film[0]), y = (int)(pix / (uint32_t)P.film[0]);
        Rng rng;
        c3 Lt;
        if (fwd) {
            Lt = C3(fwd[3 * i], fwd[3 * i + 1], fwd[3 * i + 2]);
        } else {
            er_seed_lanes(P.seed, view, pix, first + s, &rng.s0, &rng.s1);
            Lt = dm_sample<false>(P, M, x, y, rng, C3(0, 0, 0), C3(0, 0, 0), nullptr, nullptr);
        }
        er_seed_lanes(P.seed, view, pix, first + s, &rng.s0, &rng.s1);
        dm_sample<true>(P, M, x, y, rng, g, Lt, g_rho, stf);
    }
    __syncthreads();
    if (g_tf)
        for (int j = threadIdx.x; j < M.tf_n; j += blockDim.x)
            if (s_tf[j] != 0.0f) atomicAdd(g_tf + j, s_tf[j]);
}

/* per-brick bound: the largest spline control value over the segments the
   brick's density range (1-voxel apron) covers, times margin, plus floor;
   one warp per brick */
__global__ void k_dm_majorant(const float* __restrict__ rho, int rx, int ry, int rz, int B, int nbx, int nby, int nbz,
                              const float* __restrict__ tf, int n, float scale, float margin, float floor_, float* __restrict__ out)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nbt = nbx * nby * nbz;
    if (warp >= nbt) return;
    const int bx = warp % nbx, by = (warp / nbx) % nby, bz = warp / (nbx * nby);
    const int x0 = max(bx * B - 1, 0), x1 = min((bx + 1) * B + 1, rx);
    const int y0 = max(by * B - 1, 0), y1 = min((by + 1) * B + 1, ry);
    const int z0 = max(bz * B - 1, 0), z1 = min((bz + 1) * B + 1, rz);
    const int wx = x1 - x0, wy = y1 - y0, wz = z1 - z0;
    const int total = wx * wy * wz;
    float lo = FLT_MAX, hi = -FLT_MAX;
    for (int k = lane; k < total; k += 32) {
        const int x = x0 + k % wx, y = y0 + (k / wx) % wy, z = z0 + k / (wx * wy);
        const float v = __ldg(rho + ((size_t)z * ry + y) * rx + x);
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if (lane != 0) return;
    float u0 = 2.0f + lo * (float)(n - 5), u1 = 2.0f + hi * (float)(n - 5);
    u0 = fminf(fmaxf(u0, 1.0f), (float)(n - 2));
    u1 = fminf(fmaxf(u1, 1.0f), (float)(n - 2));
    const int i0 = min((int)floorf(u0), n - 3), i1 = min((int)floorf(u1), n - 3);
    float vmax = -FLT_MAX;
    for (int i = i0 - 1; i <= i1 + 2; i++) vmax = fmaxf(vmax, __ldg(tf + i));
    out[warp] = scale * (vmax * margin + floor_);
}

int sm_count()
{
    int sm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    return sm > 0 ? sm : 132;
}

}  // namespace

cudaError_t er_launch_dm_forward(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, float* samples,
                                 float* sum, cudaStream_t s)
{
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t want = (items + 255) / 256, cap = (uint64_t)sm_count() * 32;
    k_dm_forward<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(P, M, spp, view, first, npix, samples);
    if (sum) k_dm_reduce<<<(npix + 255) / 256, 256, 0, s>>>(samples, spp, npix, sum);
    return cudaGetLastError();
}

cudaError_t er_launch_dm_forward64(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, double* samples,
                                   double* sum, cudaStream_t s)
{
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t want = (items + 255) / 256, cap = (uint64_t)sm_count() * 32;
    k_dm_forward64<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(P, M, spp, view, first, npix, samples);
    k_dm_reduce64<<<(npix + 255) / 256, 256, 0, s>>>(samples, spp, npix, sum);
    return cudaGetLastError();
}

cudaError_t er_launch_dm_adjoint(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, const float* dimg,
                                 const float* fwd, float* g_rho, float* g_tf, cudaStream_t s)
{
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    const uint64_t items = (uint64_t)spp * npix;
    const uint64_t want = (items + 255) / 256, cap = (uint64_t)sm_count() * 8;
    k_dm_adjoint<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(P, M, spp, view, first, npix, dimg, fwd, g_rho, g_tf);
    return cudaGetLastError();
}

cudaError_t er_launch_dm_majorant(const float* rho, const int res[3], int B, const float* tf, int n, float scale, float margin,
                                  float floor_, float* out, cudaStream_t s)
{
    const int nbx = (res[0] + B - 1) / B, nby = (res[1] + B - 1) / B, nbz = (res[2] + B - 1) / B;
    const long long warps = (long long)nbx * nby * nbz;
    const unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
    k_dm_majorant<<<blocks, 256, 0, s>>>(rho, res[0], res[1], res[2], B, nbx, nby, nbz, tf, n, scale, margin, floor_, out);
    return cudaGetLastError();
}
