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
    int i0, nb;          /* the nb parameters the opacity depends on, from i0 */
    Real b[4];
};

/* PiecewiseLinearFunction::Evaluate (Source/plf.h:68-91) with the node
   values `vals` at the positions of p: the value, the segment's slope d/dx
   (0 where it clamps), and the one or two values it blends with their
   weights (none at x equal to the last node, where Evaluate returns 0) */
template <typename Real>
ER_D Real dm_plf(const Plf& p, const float* vals, Real x, int& i0, int& nb, Real* b, Real& slope)
{
    const int n = p.count;
    slope = 0.0f;
    nb = 0;
    i0 = 0;
    if (n <= 0) return 0.0f;
    if (x < (Real)p.range0) { nb = 1; b[0] = 1.0f; return (Real)__ldg(vals); }
    if (x > (Real)p.range1) { nb = 1; i0 = n - 1; b[0] = 1.0f; return (Real)__ldg(vals + n - 1); }
    for (int i = 1; i < n; i++) {
        const Real P1 = p.pos[i - 1];
        const Real P2 = p.pos[i];
        const Real DeltaP = P2 - P1;
        const Real LerpT = (x - P1) / DeltaP;
        if (x >= P1 && x < P2) {
            const Real v0 = __ldg(vals + i - 1), v1 = __ldg(vals + i);
            i0 = i - 1;
            nb = 2;
            b[0] = (Real)1.0f - LerpT;
            b[1] = LerpT;
            slope = (v1 - v0) / DeltaP;
            return v0 + LerpT * (v1 - v0);
        }
    }
    return 0.0f;
}

/* a transfer function of the tracer (its own node values) at x, and its slope */
template <typename Real>
ER_D Real dm_tf_value(const Plf& p, Real x)
{
    if constexpr (sizeof(Real) == sizeof(float)) {
        return plf_eval(p, x);
    } else {
        const int n = p.count;
        if (n <= 0) return 0.0;
        if (x < (Real)p.range0) return p.val[0];
        if (x > (Real)p.range1) return p.val[n - 1];
        for (int i = 1; i < n; i++) {
            const Real P1 = p.pos[i - 1], P2 = p.pos[i];
            const Real LerpT = (x - P1) / (P2 - P1);
            if (x >= P1 && x < P2) return (Real)p.val[i - 1] + LerpT * ((Real)p.val[i] - (Real)p.val[i - 1]);
        }
        return 0.0;
    }
}

ER_D float dm_tf_slope(const Plf& p, float x)
{
    if (p.count <= 0 || x < p.range0 || x > p.range1) return 0.0f;
    for (int i = 1; i < p.count; i++) {
        const float P1 = p.pos[i - 1], P2 = p.pos[i];
        if (x >= P1 && x < P2) return (p.val[i] - p.val[i - 1]) / (P2 - P1);
    }
    return 0.0f;
}

ER_D float dm_pow(float x, float y) { return er_powf(x, y); }
ER_D double dm_pow(double x, double y) { return pow(x, y); }
ER_D float dm_exp(float x) { return er_expf(x); }
ER_D double dm_exp(double x) { return exp(x); }
ER_D float dm_sqrt(float x) { return sqrtf(x); }
ER_D double dm_sqrt(double x) { return sqrt(x); }

template <typename Real, int MODEL>
ER_D void dm_opacity(const Params& P, const DmParams& M, Real rho, DmTf<Real>& o)
{
    if (MODEL == 1) {
        o.alpha = dm_plf<Real>(P.tfs->opacity, M.tf, rho, o.i0, o.nb, o.b, o.dalpha);
        return;
    }
    o.nb = 4;
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
        for (int j = 0; j < 4; j++)
            if (j < o.nb) atomicAdd(s_tf + o.i0 + j, as * o.b[j]);
    }
    if (g_rho && o.dalpha != 0.0f) {
        const float ar = as * o.dalpha;
#pragma unroll
        for (int c = 0; c < 8; c++) atomicAdd(g_rho + k.idx[c], ar * k.w[c]);
    }
}

ER_D void dm_scatter_rho(const DmLookup<float>& k, float a, float* g_rho)
{
    if (!g_rho || a == 0.0f) return;
#pragma unroll
    for (int c = 0; c < 8; c++) atomicAdd(g_rho + k.idx[c], a * k.w[c]);
}

/* ---- model 1: the tracer's shading at a tentative collision ----------
   At the grid's float intensity I: Kd = Diffuse1D(I), Ks = Specular1D(I),
   exponent = 1e6 Glossiness1D(I)^7 and the volume IOR
   (Source/transport.h:136-139, Source/utilities.h:28-31); the normal from
   central differences of the grid at +-MinStep (Source/volumes.h:31-91);
   the BRDF (also without apply_shading_type, as the live reference),
   isotropic phase, or hybrid (Source/scatterevent.h:155-212) with its
   random shader choice replaced by the expected value P_brdf BRDF +
   (1 - P_brdf) phase, so that samples stay smooth in the parameters.  The
   next-event estimate is S(Wo, Wi) Li LightCount / (LightPdf q), S = F
   |Wi . N| for the BRDF and F for the phase function (Source/transport.h:
   58-84 without the MIS weight: the estimator samples lights only). */
template <typename Real>
struct DmShade {
    Real Kd[3], Ks[3];
    Real gl, e;          /* Glossiness1D(I) and its exponent */
    int type;            /* 0 BRDF, 1 isotropic phase, 2 hybrid (expected value) */
    Real g6[6];          /* I(P - d), I(P + d) per axis, d = MinStep */
    Real N[3];
    Real gm, pb;         /* gradient magnitude, probability of the BRDF */
};

template <typename Real>
ER_D void dm_shade_prepare(const Params& P, const DmParams& M, v3 Pt, Real I, const DmTf<Real>& o, DmShade<Real>& h)
{
    const Tfs& T = *P.tfs;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        h.Kd[c] = dm_tf_value<Real>(T.diffuse[c], I);
        h.Ks[c] = dm_tf_value<Real>(T.specular[c], I);
    }
    h.gl = dm_tf_value<Real>(T.glossiness, I);
    h.e = (Real)1000000.0f * dm_pow(h.gl, (Real)7.0f);
    h.type = !P.apply_shading_type ? 0 : (P.shading_type == 1 ? 1 : (P.shading_type == 2 ? 2 : 0));
    h.pb = h.type == 0 ? (Real)1.0f : (Real)0.0f;
    h.gm = 0.0f;
    h.N[0] = h.N[1] = h.N[2] = 0.0f;
    if (h.type == 1) return;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const v3 d = gdelta(P, i);
        DmLookup<Real> a, b;
        dm_density<Real>(P, M, vsub(Pt, d), a);
        dm_density<Real>(P, M, vadd(Pt, d), b);
        h.g6[2 * i] = a.rho;
        h.g6[2 * i + 1] = b.rho;
    }
    /* Normalize(V) = V / Length(V) (Source/vector.h:469-475); where the grid
       is flat the normal is undefined and the BRDF term is taken as 0 (the
       hybrid's P_brdf is 0 there anyway) */
    const Real gx = h.g6[0] - h.g6[1], gy = h.g6[2] - h.g6[3], gz = h.g6[4] - h.g6[5];
    const Real L = dm_sqrt(gx * gx + gy * gy + gz * gz);
    if (L > (Real)0.0f) { h.N[0] = gx / L; h.N[1] = gy / L; h.N[2] = gz / L; }
    if (h.type != 2) return;
    Real sum = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        Real D = h.g6[2 * i] - h.g6[2 * i + 1];
        D *= (Real)(0.5f / P.spacing[i]);
        sum += D * D;
    }
    h.gm = dm_sqrt(sum);
    const Real NGM = h.gm * (Real)M.gm_inv;
    const Real Exponent = (Real)25.0f * dm_pow((Real)P.gradient_factor, (Real)3.0f) * NGM;
    h.pb = P.opacity_modulated ? o.alpha * ((Real)1.0f - dm_exp(-Exponent)) : (Real)1.0f - dm_exp(-Exponent);
}

/* binary64 copies of the BRDF's functions (Source/shader.h), for the
   binary64 evaluation of the estimator; the float path calls er_path.cuh's */
struct dv3 { double x, y, z; };
ER_D dv3 DV3(double x, double y, double z) { dv3 r; r.x = x; r.y = y; r.z = z; return r; }
ER_D double ddot(dv3 a, dv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
ER_D dv3 dcross(dv3 a, dv3 b) { return DV3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)); }
ER_D dv3 dnorm(dv3 a) { const double L = sqrt(ddot(a, a)); return DV3(a.x / L, a.y / L, a.z / L); }

ER_D double dm_fresnel64(double ei_, double et_, double cosi)
{
    cosi = cosi < -1.0 ? -1.0 : (cosi > 1.0 ? 1.0 : cosi);
    const bool entering = cosi > 0.0;
    double ei = ei_, et = et_;
    if (!entering) { const double t = ei; ei = et; et = t; }
    const double s2 = 1.0 - cosi * cosi;
    const double sint = ei / et * sqrt(s2 > 0.0 ? s2 : 0.0);
    if (sint >= 1.0) return 1.0;
    const double c2 = 1.0 - sint * sint;
    const double cost = sqrt(c2 > 0.0 ? c2 : 0.0);
    const double ci = fabs(cosi);
    const double Rparl = ((et * ci) - (ei * cost)) / ((et * ci) + (ei * cost));
    const double Rperp = ((ei * ci) - (et * cost)) / ((ei * ci) + (et * cost));
    return (Rparl * Rparl + Rperp * Rperp) / 2.0;
}

/* BRDF::F (Lambertian + microfacet) times |Wi . N|, per channel, binary64 */
ER_D void dm_brdf64(const DmShade<double>& h, double ior, v3 Wo_, v3 Wi_, double out[3])
{
    const dv3 N = DV3(h.N[0], h.N[1], h.N[2]);
    const dv3 Wo = DV3(Wo_.x, Wo_.y, Wo_.z), Wi = DV3(Wi_.x, Wi_.y, Wi_.z);
    const dv3 Nn = dnorm(N);
    const dv3 Nu = dnorm(dcross(N, Wo));
    const dv3 Nv = dnorm(dcross(N, Nu));
    const dv3 Wol = DV3(ddot(Wo, Nu), ddot(Wo, Nv), ddot(Wo, Nn));
    const dv3 Wil = DV3(ddot(Wi, Nu), ddot(Wi, Nv), ddot(Wi, Nn));
    double m = 0.0;
    const double co = fabs(Wol.z), ci = fabs(Wil.z);
    dv3 Wh = DV3(Wil.x + Wol.x, Wil.y + Wol.y, Wil.z + Wol.z);
    if (ci != 0.0 && co != 0.0 && !(Wh.x == 0.0 && Wh.y == 0.0 && Wh.z == 0.0)) {
        Wh = dnorm(Wh);
        const double F = dm_fresnel64(1.0, ior, ddot(Wil, Wh));
        const double NdotWh = fabs(Wh.z);
        const double WOdotWh = fabs(ddot(Wol, Wh));
        const double g1 = 2.0 * NdotWh * co / WOdotWh, g2 = 2.0 * NdotWh * ci / WOdotWh;
        const double gmin = (g2 < g1) ? g2 : g1;
        const double G = (gmin < 1.0) ? gmin : 1.0;
        const double D = (h.e + 2.0) * 0.15915494309189533577 * pow(NdotWh, h.e);
        m = D * G * F / (4.0 * ci * co);
    }
    const double cosw = fabs(ddot(Wi, Nn));
    for (int c = 0; c < 3; c++) out[c] = (h.Kd[c] * 0.31830988618379067154 + h.Ks[c] * m) * cosw;
}

/* S(Wo, Wi) per channel, and its BRDF and phase parts */
template <typename Real>
ER_D void dm_shade_eval(const Params& P, const DmShade<Real>& h, v3 Wo, v3 Wi, Real S[3], Real Sb[3], Real Sp[3])
{
#pragma unroll
    for (int c = 0; c < 3; c++) {
        Sp[c] = h.Kd[c] * (Real)ER_INV_PI_F;
        Sb[c] = 0.0f;
    }
    if (h.type != 1 && !(h.N[0] == (Real)0.0f && h.N[1] == (Real)0.0f && h.N[2] == (Real)0.0f)) {
        if constexpr (sizeof(Real) == sizeof(float)) {
            Shader sh;
            shader_init(sh, 0, V3(h.N[0], h.N[1], h.N[2]), Wo, C3(h.Kd[0], h.Kd[1], h.Kd[2]), C3(h.Ks[0], h.Ks[1], h.Ks[2]),
                        P.volume_ior, h.e);
            const c3 f = cscale(shader_f(sh, Wo, Wi), vabsdot(Wi, V3(h.N[0], h.N[1], h.N[2])));
            Sb[0] = f.r; Sb[1] = f.g; Sb[2] = f.b;
        } else {
            dm_brdf64(h, (double)P.volume_ior, Wo, Wi, Sb);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
        S[c] = h.type == 1 ? Sp[c] : (h.type == 0 ? Sb[c] : Sb[c] * h.pb + Sp[c] * ((Real)1.0f - h.pb));
}

ER_D float dm_sgn(float x) { return x < 0.0f ? -1.0f : 1.0f; }

/* adjoint of S: aS = dLoss/dS; adds dLoss/dI to aI, dLoss/d(opacity at I)
   through the hybrid's modulation to aop, and returns dLoss/d(each of the
   six gradient lookups) in ag.  The microfacet term depends on the normal
   only through a = Wh.N, b = Wo.N and c = Wi.N (the Fresnel term and
   |Wo.Wh| do not). */
ER_D void dm_shade_adjoint(const Params& P, const DmParams& M, const DmShade<float>& h, const DmTf<float>& o, float I, v3 Wo, v3 Wi,
                           const float aS[3], float& aI, float& aop, float ag[6])
{
#pragma unroll
    for (int i = 0; i < 6; i++) ag[i] = 0.0f;
    float S[3], Sb[3], Sp[3];
    dm_shade_eval<float>(P, h, Wo, Wi, S, Sb, Sp);
    float aSb[3] = { aS[0], aS[1], aS[2] }, aSp[3] = { aS[0], aS[1], aS[2] };
    float angm = 0.0f;
    const Tfs& T = *P.tfs;
    if (h.type == 2) {
        const float apb = aS[0] * (Sb[0] - Sp[0]) + aS[1] * (Sb[1] - Sp[1]) + aS[2] * (Sb[2] - Sp[2]);
        const float GF3 = er_powf(P.gradient_factor, 3.0f);
        const float ex = er_expf(-25.0f * GF3 * h.gm * M.gm_inv);
        const float mod = P.opacity_modulated ? o.alpha : 1.0f;
        if (P.opacity_modulated) aop += apb * (1.0f - ex);
        angm = apb * mod * ex * 25.0f * GF3;
#pragma unroll
        for (int c = 0; c < 3; c++) { aSb[c] = aS[c] * h.pb; aSp[c] = aS[c] * (1.0f - h.pb); }
    }
    if (h.type != 0) {
#pragma unroll
        for (int c = 0; c < 3; c++) aI += aSp[c] * dm_tf_slope(T.diffuse[c], I) * ER_INV_PI_F;
    }
    if (h.type == 1) return;
    /* BRDF: Sb = (Kd / pi + Ks m(a, b, c, e)) |c| */
    const v3 N = V3(h.N[0], h.N[1], h.N[2]);
    const v3 Wsum = vadd(Wi, Wo);
    const float b = vdot(Wo, N), c = vdot(Wi, N);
    const float ab = fabsf(b), ac = fabsf(c);
    float m = 0.0f, dmda = 0.0f, dmdb = 0.0f, dmdc = 0.0f, dmde = 0.0f;
    v3 Wh = V3(0.0f, 0.0f, 0.0f);
    if (ab > 0.0f && ac > 0.0f && !(Wsum.x == 0.0f && Wsum.y == 0.0f && Wsum.z == 0.0f)) {
        Wh = vnorm(Wsum);
        const float a = vdot(Wh, N), aa = fabsf(a);
        const float k = vabsdot(Wo, Wh);
        const float F = fresnel_eval(1.0f, P.volume_ior, vdot(Wi, Wh));
        const float D = (h.e + 2.0f) * ER_INV_TWO_PI_F * er_powf(aa, h.e);
        const float g1 = 2.0f * aa * ab / k, g2 = 2.0f * aa * ac / k;
        const float gmin = (g2 < g1) ? g2 : g1;
        float G = 1.0f, dGda = 0.0f, dGdb = 0.0f, dGdc = 0.0f;
        if (gmin < 1.0f) {
            G = gmin;
            if (g2 < g1) { dGda = 2.0f * ac / k * dm_sgn(a); dGdc = 2.0f * aa / k * dm_sgn(c); }
            else { dGda = 2.0f * ab / k * dm_sgn(a); dGdb = 2.0f * aa / k * dm_sgn(b); }
        }
        const float den = 4.0f * ac * ab;
        m = D * G * F / den;
        const float dDda = aa > 0.0f ? D * h.e / aa * dm_sgn(a) : 0.0f;
        dmda = (dDda * G + D * dGda) * F / den;
        dmdb = D * F / (4.0f * ac) * (dGdb / ab - G * dm_sgn(b) / (ab * ab));
        dmdc = D * F / (4.0f * ab) * (dGdc / ac - G * dm_sgn(c) / (ac * ac));
        dmde = aa > 0.0f ? m * (1.0f / (h.e + 2.0f) + er_logf(aa)) : 0.0f;
    }
    /* through I: Kd', Ks' and the exponent's 7e6 gl^6 gl' */
    const float dedI = 7000000.0f * er_powf(h.gl, 6.0f) * dm_tf_slope(T.glossiness, I);
    float ks_dot = 0.0f, f_dot = 0.0f;
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
        aI += aSb[ch] * (dm_tf_slope(T.diffuse[ch], I) * ER_INV_PI_F + dm_tf_slope(T.specular[ch], I) * m + h.Ks[ch] * dmde * dedI) * ac;
        ks_dot += aSb[ch] * h.Ks[ch];
        f_dot += aSb[ch] * (h.Kd[ch] * ER_INV_PI_F + h.Ks[ch] * m);
    }
    /* through the normal N = g / |g|, g = (I(P - d) - I(P + d)) per axis */
    v3 aN = vscale(vadd(vadd(vscale(Wh, dmda), vscale(Wo, dmdb)), vscale(Wi, dmdc)), ks_dot * ac);
    aN = vadd(aN, vscale(Wi, f_dot * dm_sgn(c)));
    const v3 gv = V3(h.g6[0] - h.g6[1], h.g6[2] - h.g6[3], h.g6[4] - h.g6[5]);
    const float glen = vlen(gv);
    float aG[3] = { 0.0f, 0.0f, 0.0f };
    if (glen > 0.0f) {
        const float an = vdot(aN, N);
        aG[0] = (aN.x - an * N.x) / glen;
        aG[1] = (aN.y - an * N.y) / glen;
        aG[2] = (aN.z - an * N.z) / glen;
    }
    if (h.type == 2 && h.gm > 0.0f) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float hi = 0.5f / P.spacing[i];
            aG[i] += angm * M.gm_inv * vget(gv, i) * hi * hi / h.gm;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ag[2 * i] = aG[i];
        ag[2 * i + 1] = -aG[i];
    }
}

/* the six gradient lookups' adjoints into the density gradient */
ER_D void dm_scatter_gradient_lookups(const Params& P, const DmParams& M, v3 Pt, const float ag[6], float* g_rho)
{
    if (!g_rho) return;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const v3 d = gdelta(P, i);
        if (ag[2 * i] != 0.0f) {
            DmLookup<float> a;
            dm_density<float>(P, M, vsub(Pt, d), a);
            dm_scatter_rho(a, ag[2 * i], g_rho);
        }
        if (ag[2 * i + 1] != 0.0f) {
            DmLookup<float> b;
            dm_density<float>(P, M, vadd(Pt, d), b);
            dm_scatter_rho(b, ag[2 * i + 1], g_rho);
        }
    }
}

ER_D bool dm_segment(const Params& P, const Ray& R, float& t0, float& t1)
{
    Isect Int; Int.invalid();
    intersect_volume(P, R, Int);
    if (!Int.valid) return false;
    t0 = smax(Int.near_t, R.MinT);
    t1 = smin(Int.far_t, R.MaxT);
    return t0 < t1;
}

/* ratio-tracked shadow transmittance; ADJ scatters -a_scale / (mu - sigma) */
template <bool ADJ, int MODEL, typename Real = float>
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
                dm_opacity<Real, MODEL>(P, M, k.rho, o);
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

/* next-event estimate at Pt without the collision weight and the shadow:
   model 0 returns it (albedo, isotropic phase); model 1 returns the light
   sample's direction Wi and Li LightCount / (LightPdf q) in LiK, which the
   caller multiplies by the shading */
ER_D c3 dm_nee(const Params& P, const DmParams& M, v3 Pt, Rng& rng, v3& S, bool& has, v3& Wi_out, c3& LiK)
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
    if (M.model == 1) {
        Wi_out = Wi;
        LiK = cscale(Li, (float)P.light_count / (LightPdf * M.q));
        return LiK;
    }
    return cscale(cmul(C3(M.albedo[0], M.albedo[1], M.albedo[2]), Li), DM_INV_4PI * (float)P.light_count / (LightPdf * M.q));
}

/* random stream of the k-th next-event shadow segment of a sample: its own
   lanes, so the camera ray's draws do not depend on the segments' */
ER_D void dm_shadow_stream(uint32_t seed, uint32_t view, uint32_t pix, uint32_t sample, uint32_t k, Rng& r)
{
    er_seed_lanes(seed ^ er_hash32(0x51ED2705u + k), view ^ 0x6A09E667u, pix, sample, &r.s0, &r.s1);
}

/* one tentative collision of the camera ray, as the walker hands it over */
template <typename Real>
struct DmHit {
    v3 Pt;
    float mu;
    bool nee, has;       /* next-event estimate drawn here; it found a light sample */
    uint32_t k_nee;      /* index of the estimate along the ray (its shadow stream) */
    Real A0[3];          /* unshadowed next-event estimate */
    v3 S;                /* light sample point */
    Real Le[3];          /* model 1: the emission at the collision */
    v3 Wo;               /* model 1: minus the camera ray's direction */
    v3 Wi;               /* model 1: light sample direction */
    c3 LiK;              /* model 1: Li LightCount / (LightPdf q) */
};

/* the camera ray's tentative collisions in order; visit(hit, lookup,
   opacity, sigma, w, T, shading) sees each with the throughput T before
   it (shading: model 1's, prepared where a next-event estimate is drawn) */
template <typename Real, int MODEL, typename Visit>
ER_D void dm_walk(const Params& P, const DmParams& M, int x, int y, Rng& rng, Visit& visit)
{
    const v2 film_uv = rng.get2();
    const v2 lens_uv = rng.get2();
    const Ray R = sample_camera(P, x, y, film_uv, lens_uv);
    float t0, t1;
    if (!dm_segment(P, R, t0, t1)) return;
    Dda d;
    dda_init(P, R, t0, t1, d);
    Real T = 1.0f;
    float tau = -er_logf(rng.get1());
    uint32_t nee = 0;
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
                DmHit<Real> h;
                h.Pt = vadd(R.O, vscale(R.D, t));
                h.mu = mu;
                h.Wo = vneg(R.D);
                DmLookup<Real> k;
                dm_density(P, M, h.Pt, k);
                DmTf<Real> o;
                dm_opacity<Real, MODEL>(P, M, k.rho, o);
                const Real sig = (Real)M.scale * o.alpha;
                if (!(sig < (Real)mu)) atomicOr(P.err, 4);   /* the majorant no longer bounds sigma */
                const Real w = sig / (Real)mu;
                DmShade<Real> sd;
                sd.type = -1;
#pragma unroll
                for (int c = 0; c < 3; c++) h.Le[c] = 0.0f;
                if (MODEL == 1 && M.emissive) {
#pragma unroll
                    for (int c = 0; c < 3; c++) h.Le[c] = dm_tf_value<Real>(P.tfs->emission[c], k.rho);
                }
                h.has = false;
                h.nee = rng.get1() < M.q;
                if (h.nee) {
                    if (MODEL == 1) dm_shade_prepare<Real>(P, M, h.Pt, k.rho, o, sd);
                    const c3 a0 = dm_nee(P, M, h.Pt, rng, h.S, h.has, h.Wi, h.LiK);
                    if (MODEL == 1 && h.has) {
                        Real S[3], Sb[3], Sp[3];
                        dm_shade_eval<Real>(P, sd, h.Wo, h.Wi, S, Sb, Sp);
                        h.A0[0] = S[0] * (Real)a0.r;
                        h.A0[1] = S[1] * (Real)a0.g;
                        h.A0[2] = S[2] * (Real)a0.b;
                    } else {
                        h.A0[0] = a0.r; h.A0[1] = a0.g; h.A0[2] = a0.b;
                    }
                    h.k_nee = nee++;
                }
                visit(h, k, o, sig, w, T, sd);
                T = T * ((Real)1.0f - w);
                if (++guard > ER_DELTA_MAX_COLLISIONS) { atomicOr(P.err, 2); return; }
                tau = -er_logf(rng.get1());
            }
        }
        dda_advance(P, d, e);
    }
}

/* ---- the wavefront estimator ------------------------------------------
   A window of items (item = s * npix + pixel, s counted from the window's
   first sample row):
     k_dm_count   : walk, count the item's shadow jobs, reserve their slots
     k_dm_jobs    : walk again, write the jobs in order (point, light
                    sample, unshadowed estimate, T * w, stream index)
     k_dm_shadow  : one thread per job: the ratio-tracked transmittance
     k_dm_gather  : per item, L = sum over its jobs in order of (A0 Tr) (T w)
   adjoint (after the four above):
     k_dm_adj_primary : walk again with each job's transmittance: the
                        collision terms, and g . c per job
     k_dm_adj_shadow  : one thread per job: the shadow-segment terms
   Every float operation and its order are the oracle's. */

struct DmJobs {
    float4* P;         /* Pt, T * w */
    float4* S;         /* light sample, g . c (adjoint) */
    float4* A;         /* A0, transmittance */
    uint2* id;         /* item in the window, k_nee */
    uint32_t* off;     /* per item: first job */
    uint32_t* cnt;     /* per item: jobs */
    uint32_t* total;   /* jobs of the window */
    uint32_t cap;      /* job slots */
    float4* E;         /* model 1: per item, the emission summed along the walk (NULL for model 0) */
};

struct DmWindow {
    uint32_t npix;
    uint32_t s0;       /* first sample row of the window */
    uint32_t items;
    uint32_t view, first;
};

ER_D void dm_item(const Params& P, const DmWindow& W, uint32_t i, uint32_t& pix, uint32_t& sample, int& x, int& y)
{
    const uint32_t s = W.s0 + i / W.npix;
    pix = i % W.npix;
    sample = W.first + s;
    x = (int)(pix % (uint32_t)P.film[0]);
    y = (int)(pix / (uint32_t)P.film[0]);
}

template <int MODEL>
__global__ void __launch_bounds__(256) k_dm_count(const Params P, const DmParams M, const DmWindow W, DmJobs J)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < W.items; base += stride) {
        const uint32_t i = base + threadIdx.x;
        uint32_t n = 0;
        if (i < W.items) {
            uint32_t pix, sample;
            int x, y;
            dm_item(P, W, i, pix, sample, x, y);
            Rng rng;
            er_seed_lanes(P.seed, W.view, pix, sample, &rng.s0, &rng.s1);
            auto count = [&](const DmHit<float>& h, const DmLookup<float>&, const DmTf<float>&, float, float, float,
                             const DmShade<float>&) { n += h.has ? 1u : 0u; };
            dm_walk<float, MODEL>(P, M, x, y, rng, count);
        }
        /* warp-aggregated reservation of the item's job slots */
        const int lane = threadIdx.x & 31;
        uint32_t incl = n;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t base_slot = 0;
        if (lane == 31) base_slot = atomicAdd(J.total, incl);
        base_slot = __shfl_sync(0xffffffffu, base_slot, 31);
        if (i < W.items) {
            J.off[i] = base_slot + incl - n;
            J.cnt[i] = n;
        }
    }
}

template <int MODEL>
__global__ void __launch_bounds__(256) k_dm_jobs(const Params P, const DmParams M, const DmWindow W, DmJobs J)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < W.items; i += stride) {
        uint32_t pix, sample;
        int x, y;
        dm_item(P, W, i, pix, sample, x, y);
        Rng rng;
        er_seed_lanes(P.seed, W.view, pix, sample, &rng.s0, &rng.s1);
        uint32_t j = J.off[i];
        const uint32_t end = j + J.cnt[i];
        c3 E = C3(0, 0, 0);
        auto write = [&](const DmHit<float>& h, const DmLookup<float>&, const DmTf<float>&, float, float w, float T,
                         const DmShade<float>&) {
            if (MODEL == 1) E = cadd(E, cscale(C3(h.Le[0], h.Le[1], h.Le[2]), T * w));
            if (!h.has || j >= end || j >= J.cap) return;
            J.P[j] = make_float4(h.Pt.x, h.Pt.y, h.Pt.z, T * w);
            J.S[j] = make_float4(h.S.x, h.S.y, h.S.z, 0.0f);
            J.A[j] = make_float4(h.A0[0], h.A0[1], h.A0[2], 0.0f);
            J.id[j] = make_uint2(i, h.k_nee);
            j++;
        };
        dm_walk<float, MODEL>(P, M, x, y, rng, write);
        if (J.E) J.E[i] = make_float4(E.r, E.g, E.b, 0.0f);
    }
}

template <int MODEL>
__global__ void __launch_bounds__(256) k_dm_shadow(const Params P, const DmParams M, const DmWindow W, DmJobs J)
{
    const uint32_t n = min(*J.total, J.cap);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const uint2 id = J.id[j];
        uint32_t pix, sample;
        int x, y;
        dm_item(P, W, id.x, pix, sample, x, y);
        Rng sh;
        dm_shadow_stream(P.seed, W.view, pix, sample, id.y, sh);
        const float4 p = J.P[j], s = J.S[j];
        const float Tr = dm_shadow<false, MODEL>(P, M, V3(p.x, p.y, p.z), V3(s.x, s.y, s.z), sh, 0.0f, nullptr, nullptr);
        J.A[j].w = Tr;
    }
}

/* L of every item of the window in sample order; out = the item's slot of the
   whole launch's samples (window item i is launch item base + i) */
__global__ void k_dm_gather(const DmWindow W, const DmJobs J, uint64_t base, float* __restrict__ samples)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.items) return;
    c3 L = C3(0, 0, 0);
    const uint32_t j0 = J.off[i], j1 = j0 + J.cnt[i];
    for (uint32_t j = j0; j < j1 && j < J.cap; j++) {
        const float4 a = J.A[j];
        const float Tw = J.P[j].w;
        const c3 A = cscale(C3(a.x, a.y, a.z), a.w);
        L = cadd(L, cscale(A, Tw));
    }
    if (J.E) {
        /* model 1: the emission after the next-event estimates */
        const float4 e = J.E[i];
        L = cadd(L, C3(e.x, e.y, e.z));
    }
    const uint64_t q = 3 * (base + i);
    samples[q] = L.r;
    samples[q + 1] = L.g;
    samples[q + 2] = L.b;
}

/* one opacity-gradient row per warp: no block barrier, so a warp that
   finishes its items does not wait for the block's slowest */
#define DM_WARPS (256 / 32)

ER_D float* dm_tf_row(float (*rows)[ER_MAX_TF_NODES])
{
    float* r = rows[threadIdx.x >> 5];
    for (int j = threadIdx.x & 31; j < ER_MAX_TF_NODES; j += 32) r[j] = 0.0f;
    __syncwarp();
    return r;
}

ER_D void dm_tf_flush(const DmParams& M, const float* row, float* g_tf)
{
    __syncwarp();
    for (int j = threadIdx.x & 31; j < M.tf_n; j += 32)
        if (row[j] != 0.0f) atomicAdd(g_tf + j, row[j]);
}

template <int MODEL>
__global__ void __launch_bounds__(256) k_dm_adj_primary(const Params P, const DmParams M, const DmWindow W, DmJobs J, uint64_t base,
                                                        const float* __restrict__ dimg, const float* __restrict__ fwd,
                                                        float* __restrict__ g_rho, float* __restrict__ g_tf)
{
    __shared__ float rows[DM_WARPS][ER_MAX_TF_NODES];
    float* row = dm_tf_row(rows);
    float* s_tf = g_tf ? row : nullptr;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < W.items; i += stride) {
        uint32_t pix, sample;
        int x, y;
        dm_item(P, W, i, pix, sample, x, y);
        const c3 g = C3(dimg[3 * pix], dimg[3 * pix + 1], dimg[3 * pix + 2]);
        if (g.r == 0.0f && g.g == 0.0f && g.b == 0.0f) continue;
        const uint64_t q = 3 * (base + i);
        const c3 Lt = C3(fwd[q], fwd[q + 1], fwd[q + 2]);
        Rng rng;
        er_seed_lanes(P.seed, W.view, pix, sample, &rng.s0, &rng.s1);
        uint32_t j = J.off[i];
        const uint32_t end = j + J.cnt[i];
        c3 L = C3(0, 0, 0), E = C3(0, 0, 0);
        auto adj = [&](const DmHit<float>& h, const DmLookup<float>& k, const DmTf<float>& o, float sig, float w, float T,
                       const DmShade<float>& sd) {
            c3 A = C3(0, 0, 0);
            float Tr = 0.0f;
            bool shaded = false;
            if (h.has && j < end && j < J.cap) {
                const float4 a = J.A[j];
                Tr = a.w;
                A = cscale(C3(a.x, a.y, a.z), a.w);
                const c3 c = cscale(A, T * w);
                L = cadd(L, c);
                J.S[j].w = g.r * c.r + g.g * c.g + g.b * c.b;
                j++;
                shaded = MODEL == 1;
            }
            /* dL/dsigma = T A / mu - (Ltot - L_<=k) / (mu - sigma), A the
               collision's whole contribution before T w */
            const c3 Le = C3(h.Le[0], h.Le[1], h.Le[2]);
            if (MODEL == 1) E = cadd(E, cscale(Le, T * w));
            const c3 Ak = MODEL == 1 ? cadd(Le, A) : A;
            const c3 rest = csub(Lt, MODEL == 1 ? cadd(L, E) : L);
            const c3 dLds = csub(cscale(Ak, T / h.mu), cdivs(rest, h.mu - sig));
            const float a = g.r * dLds.r + g.g * dLds.g + g.b * dLds.b;
            if (MODEL == 1) {
                /* through the emission and shading at I, and the hybrid's
                   opacity modulation */
                const c3 gA = cscale(g, T * w);
                float aI = 0.0f, aop = 0.0f;
                if (M.emissive)
                    aI += gA.r * dm_tf_slope(P.tfs->emission[0], k.rho) + gA.g * dm_tf_slope(P.tfs->emission[1], k.rho) +
                          gA.b * dm_tf_slope(P.tfs->emission[2], k.rho);
                if (shaded) {
                    float ag[6];
                    const float aS[3] = { gA.r * Tr * h.LiK.r, gA.g * Tr * h.LiK.g, gA.b * Tr * h.LiK.b };
                    dm_shade_adjoint(P, M, sd, o, k.rho, h.Wo, h.Wi, aS, aI, aop, ag);
                    if (sd.type != 1) dm_scatter_gradient_lookups(P, M, h.Pt, ag, g_rho);
                }
                dm_scatter_rho(k, aI, g_rho);
                const float at = a + aop / M.scale;
                if (at != 0.0f) dm_scatter(M, k, o, at, g_rho, s_tf);
            } else if (a != 0.0f) {
                dm_scatter(M, k, o, a, g_rho, s_tf);
            }
        };
        dm_walk<float, MODEL>(P, M, x, y, rng, adj);
    }
    if (g_tf) dm_tf_flush(M, row, g_tf);
}

template <int MODEL>
__global__ void __launch_bounds__(256) k_dm_adj_shadow(const Params P, const DmParams M, const DmWindow W, DmJobs J,
                                                       float* __restrict__ g_rho, float* __restrict__ g_tf)
{
    __shared__ float rows[DM_WARPS][ER_MAX_TF_NODES];
    float* row = dm_tf_row(rows);
    float* s_tf = g_tf ? row : nullptr;
    const uint32_t n = min(*J.total, J.cap);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const float gc = J.S[j].w;
        if (gc == 0.0f) continue;
        const uint2 id = J.id[j];
        uint32_t pix, sample;
        int x, y;
        dm_item(P, W, id.x, pix, sample, x, y);
        Rng sh;
        dm_shadow_stream(P.seed, W.view, pix, sample, id.y, sh);
        const float4 p = J.P[j], s = J.S[j];
        dm_shadow<true, MODEL>(P, M, V3(p.x, p.y, p.z), V3(s.x, s.y, s.z), sh, gc, g_rho, s_tf);
    }
    if (g_tf) dm_tf_flush(M, row, g_tf);
}

/* the binary64 evaluation: one thread per sample, every medium-dependent
   quantity in double */
template <int MODEL>
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
        double L0 = 0.0, L1 = 0.0, L2 = 0.0;
        double E0 = 0.0, E1 = 0.0, E2 = 0.0;
        auto acc = [&](const DmHit<double>& h, const DmLookup<double>&, const DmTf<double>&, double, double w, double T,
                       const DmShade<double>&) {
            if (MODEL == 1) {
                E0 += h.Le[0] * T * w;
                E1 += h.Le[1] * T * w;
                E2 += h.Le[2] * T * w;
            }
            if (!h.has) return;
            Rng sh;
            dm_shadow_stream(P.seed, view, pix, first + s, h.k_nee, sh);
            const double Tr = dm_shadow<false, MODEL, double>(P, M, h.Pt, h.S, sh, 0.0f, nullptr, nullptr);
            L0 += h.A0[0] * Tr * T * w;
            L1 += h.A0[1] * Tr * T * w;
            L2 += h.A0[2] * Tr * T * w;
        };
        dm_walk<double, MODEL>(P, M, x, y, rng, acc);
        samples[3 * i] = L0 + E0;
        samples[3 * i + 1] = L1 + E1;
        samples[3 * i + 2] = L2 + E2;
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

/* per-brick bound: the largest spline control value over the segments the
   brick's density range (1-voxel apron) covers, times margin, plus floor;
   one warp per brick */
__global__ void k_dm_majorant(const float* __restrict__ rho, int rx, int ry, int rz, int B, int nbx, int nby, int nbz,
                              const float* __restrict__ tf, int n, const Plf* plf, float scale, float margin, float floor_,
                              float* __restrict__ out)
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
    if (plf) {
        /* model 1: the opacity PLF's maximum over [lo, hi] - its values at
           both ends and at the nodes inside */
        int i0, nb;
        float b[2], sl;
        float vmax = fmaxf(dm_plf<float>(*plf, tf, lo, i0, nb, b, sl), dm_plf<float>(*plf, tf, hi, i0, nb, b, sl));
        for (int i = 0; i < plf->count; i++)
            if (plf->pos[i] >= lo && plf->pos[i] <= hi) vmax = fmaxf(vmax, __ldg(tf + i));
        out[warp] = scale * (fmaxf(vmax, 0.0f) * margin + floor_);
        return;
    }
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

unsigned grid_for(uint64_t items, int per_sm)
{
    const uint64_t want = (items + 255) / 256, cap = (uint64_t)sm_count() * per_sm;
    return (unsigned)(want < cap ? want : cap);
}

}  // namespace

/* job storage of the wavefront medium estimator, grown on demand */
struct DmWorkspace {
    float4 *P = nullptr, *S = nullptr, *A = nullptr;
    uint2* id = nullptr;
    uint32_t *off = nullptr, *cnt = nullptr, *total = nullptr, *host_total = nullptr;
    float4* E = nullptr;       /* model 1: per item emission sums */
    size_t cap = 0, item_cap = 0;
    /* the call whose jobs the arrays hold (dm_windows): 0 = none, or not
       reusable (several windows, or a failed call) */
    uint64_t key = 0;
    cudaStream_t key_stream = nullptr;
    uint32_t kept_jobs = 0;    /* the kept walk's job count */
    ~DmWorkspace()
    {
        cudaFree(P); cudaFree(S); cudaFree(A); cudaFree(id); cudaFree(off); cudaFree(cnt); cudaFree(total); cudaFree(E);
        if (host_total) cudaFreeHost(host_total);
    }
    cudaError_t ensure_items(size_t n)
    {
        if (!total) {
            cudaError_t e = cudaMalloc(&total, sizeof(uint32_t));
            if (e == cudaSuccess) e = cudaMallocHost(&host_total, sizeof(uint32_t));
            if (e != cudaSuccess) return e;
        }
        if (n <= item_cap) return cudaSuccess;
        cudaFree(off); cudaFree(cnt); cudaFree(E);
        off = cnt = nullptr;
        E = nullptr;
        cudaError_t e = cudaMalloc(&off, n * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&cnt, n * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&E, n * sizeof(float4));
        item_cap = e == cudaSuccess ? n : 0;
        return e;
    }
    cudaError_t ensure_jobs(size_t n)
    {
        if (n <= cap) return cudaSuccess;
        n = n + n / 4;
        cudaFree(P); cudaFree(S); cudaFree(A); cudaFree(id);
        P = S = A = nullptr;
        id = nullptr;
        cudaError_t e = cudaMalloc(&P, n * sizeof(float4));
        if (e == cudaSuccess) e = cudaMalloc(&S, n * sizeof(float4));
        if (e == cudaSuccess) e = cudaMalloc(&A, n * sizeof(float4));
        if (e == cudaSuccess) e = cudaMalloc(&id, n * sizeof(uint2));
        cap = e == cudaSuccess ? n : 0;
        return e;
    }
};

/* one workspace per device (callers hold the library lock) */
static DmWorkspace& dm_workspace()
{
    static DmWorkspace* w[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev < 0 ? 0 : (dev > 63 ? 63 : dev);
    if (!w[dev]) w[dev] = new DmWorkspace();
    return *w[dev];
}

/* the four forward stages (and the two adjoint stages when dimg != NULL)
   over windows of whole sample rows; synchronises once per window to size
   the job storage.  key (nonzero) names the walk: tracer build, medium
   buffers and values, spp, view, first sample.  When the whole call is one
   window, the job arrays keep that walk's jobs after the call; an adjoint
   whose key and stream match the last call's skips the count, jobs and
   shadow stages and replays against the kept jobs (the same kernels would
   write the same jobs, in an order only the slot atomics decide). */
static cudaError_t dm_windows(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, float* samples,
                              const float* dimg, float* g_rho, float* g_tf, uint64_t key, cudaStream_t s)
{
    DmWorkspace& ws = dm_workspace();
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    uint32_t rows = (uint32_t)((1u << 21) / (npix ? npix : 1));
    if (rows < 1) rows = 1;
    cudaError_t e = ws.ensure_items((size_t)rows * npix);
    if (e != cudaSuccess) return e;
    const bool one_window = (uint32_t)spp <= rows;
    const bool reuse = dimg && one_window && key != 0 && ws.key == key && ws.key_stream == s;
    ws.key = 0;
    for (uint32_t s0 = 0; s0 < (uint32_t)spp; s0 += rows) {
        DmWindow W;
        W.npix = npix;
        W.s0 = s0;
        W.items = ((uint32_t)spp - s0 < rows ? (uint32_t)spp - s0 : rows) * npix;
        W.view = view;
        W.first = first;
        DmJobs J;
        J.P = ws.P; J.S = ws.S; J.A = ws.A; J.id = ws.id; J.off = ws.off; J.cnt = ws.cnt; J.total = ws.total;
        J.E = M.model == 1 ? ws.E : nullptr;
        J.cap = (uint32_t)ws.cap;
        const uint64_t base = (uint64_t)s0 * npix;
        uint32_t njobs = ws.kept_jobs;
        if (!reuse) {
            if ((e = cudaMemsetAsync(ws.total, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
            if (M.model == 1) k_dm_count<1><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J);
            else k_dm_count<0><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J);
            if ((e = cudaMemcpyAsync(ws.host_total, ws.total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
            njobs = *ws.host_total;
            if ((e = ws.ensure_jobs(njobs)) != cudaSuccess) return e;
            J.P = ws.P; J.S = ws.S; J.A = ws.A; J.id = ws.id; J.cap = (uint32_t)ws.cap;
            if (M.model == 1) k_dm_jobs<1><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J);
            else k_dm_jobs<0><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J);
            if (njobs && M.model == 1) k_dm_shadow<1><<<grid_for(njobs, 16), 256, 0, s>>>(P, M, W, J);
            else if (njobs) k_dm_shadow<0><<<grid_for(njobs, 16), 256, 0, s>>>(P, M, W, J);
            ws.kept_jobs = njobs;
        }
        if (!dimg || samples) {
            /* forward values: written by the forward, read by the adjoint */
            if (!dimg) k_dm_gather<<<(W.items + 255) / 256, 256, 0, s>>>(W, J, base, samples);
        }
        if (dimg) {
            if (M.model == 1) k_dm_adj_primary<1><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J, base, dimg, samples, g_rho, g_tf);
            else k_dm_adj_primary<0><<<grid_for(W.items, 16), 256, 0, s>>>(P, M, W, J, base, dimg, samples, g_rho, g_tf);
            if (njobs && M.model == 1) k_dm_adj_shadow<1><<<grid_for(njobs, 16), 256, 0, s>>>(P, M, W, J, g_rho, g_tf);
            else if (njobs) k_dm_adj_shadow<0><<<grid_for(njobs, 16), 256, 0, s>>>(P, M, W, J, g_rho, g_tf);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (one_window && key != 0) {
        ws.key = key;
        ws.key_stream = s;
    }
    return cudaSuccess;
}

cudaError_t er_launch_dm_forward(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, float* samples,
                                 float* sum, uint64_t key, cudaStream_t s)
{
    cudaError_t e = dm_windows(P, M, spp, view, first, samples, nullptr, nullptr, nullptr, key, s);
    if (e != cudaSuccess) return e;
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    if (sum) k_dm_reduce<<<(npix + 255) / 256, 256, 0, s>>>(samples, spp, npix, sum);
    return cudaGetLastError();
}

cudaError_t er_launch_dm_forward64(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, double* samples,
                                   double* sum, cudaStream_t s)
{
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    if (M.model == 1) k_dm_forward64<1><<<grid_for((uint64_t)spp * npix, 32), 256, 0, s>>>(P, M, spp, view, first, npix, samples);
    else k_dm_forward64<0><<<grid_for((uint64_t)spp * npix, 32), 256, 0, s>>>(P, M, spp, view, first, npix, samples);
    k_dm_reduce64<<<(npix + 255) / 256, 256, 0, s>>>(samples, spp, npix, sum);
    return cudaGetLastError();
}

/* fwd: the forward samples (spp * npix * 3); without them a scratch buffer
   receives the recomputed values window by window */
cudaError_t er_launch_dm_adjoint(const Params& P, const DmParams& M, int spp, uint32_t view, uint32_t first, const float* dimg,
                                 const float* fwd, float* g_rho, float* g_tf, uint64_t key, cudaStream_t s)
{
    float* samples = const_cast<float*>(fwd);
    float* scratch = nullptr;
    const uint32_t npix = (uint32_t)P.film[0] * (uint32_t)P.film[1];
    if (!fwd) {
        cudaError_t e = cudaMallocAsync(&scratch, (size_t)spp * npix * 3 * sizeof(float), s);
        if (e != cudaSuccess) return e;
        e = dm_windows(P, M, spp, view, first, scratch, nullptr, nullptr, nullptr, key, s);
        if (e != cudaSuccess) { cudaFreeAsync(scratch, s); return e; }
        samples = scratch;
    }
    cudaError_t e = dm_windows(P, M, spp, view, first, samples, dimg, g_rho, g_tf, key, s);
    if (scratch) cudaFreeAsync(scratch, s);
    return e;
}

cudaError_t er_launch_dm_majorant(const float* rho, const int res[3], int B, const float* tf, int n, const erd::Plf* plf, float scale,
                                  float margin, float floor_, float* out, cudaStream_t s)
{
    const int nbx = (res[0] + B - 1) / B, nby = (res[1] + B - 1) / B, nbz = (res[2] + B - 1) / B;
    const long long warps = (long long)nbx * nby * nbz;
    const unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
    k_dm_majorant<<<blocks, 256, 0, s>>>(rho, res[0], res[1], res[2], B, nbx, nby, nbz, tf, n, plf, scale, margin, floor_, out);
    return cudaGetLastError();
}
