/*
 * er_math.h - portable, bit-reproducible elementary functions.
 *
 * The transport code of Exposure Render calls logf/log (free-flight
 * distance, Source/raymarching.h:45,89), sinf/cosf (disk, ring and sphere
 * samplers, Source/montecarlo.h:136, Source/disk.h:64, Source/sphere.h:157),
 * powf (Blinn lobe and glossiness exponent, Source/shader.h:145,174,185,
 * Source/utilities.h:30), expf (Gauss weights and tone map,
 * Source/filterframeestimate.cuh:30, Source/tonemap.cuh:34), tanf (camera
 * set-up, Source/camera.h:75) and acosf/atan2f (sphere UVs,
 * Source/geometry.h:72,77).  Every one of those results feeds a threshold
 * test (`Sum < S`, `U <= P`) somewhere downstream, so a one-ulp difference
 * between the host C library and the CUDA library changes whole paths.
 *
 * This header gives one implementation of each function that produces the
 * same bits on an x86-64 or AArch64 host (compiled with -ffp-contract=off)
 * and on the GPU (compiled with --fmad=false): only IEEE-754 add, subtract,
 * multiply, divide, sqrt, floor and integer bit manipulation are used, in a
 * fixed order, and no fused multiply-add is relied upon.
 *
 * Methods (all written from the mathematics, constants derived here):
 *   - log:  x = 2^e * m with m in [sqrt(1/2), sqrt(2)); log(m) = 2 atanh(s),
 *           s = (m-1)/(m+1), odd Taylor series of atanh (coefficients 2/(2k+1)),
 *           arranged as log(1+f) = f - (f^2/2 - s (f^2/2 + R(s^2))).
 *   - exp:  Cody & Waite additive range reduction x = k ln2 + r with a two-part
 *           ln2 whose leading part has 12 trailing zero bits (k*LN2_HI exact),
 *           Taylor polynomial of e^r in Horner form, exact scaling by 2^k.
 *   - sin/cos: Cody & Waite reduction by pi/2 with a three-part pi/2
 *           (products with the quadrant index are exact for |x| < 6000),
 *           Taylor polynomials on [-pi/4, pi/4], quadrant table.
 *   - pow:  exp(y log|x|) with log|x| and the product y*log|x| carried in
 *           double-single arithmetic (Dekker's exact product with Veltkamp
 *           splitting, no FMA), so large exponents such as the 1e6*g^7 Blinn
 *           exponent keep float accuracy without binary64 instructions.
 *   - atan/atan2/acos: atan reduced to |v| <= tan(pi/12) with
 *           atan(u) = pi/6 + atan((sqrt3 u - 1)/(u + sqrt3)) and an odd Taylor
 *           series; acos(x) = atan2(sqrt((1-x)(1+x)), x).
 *
 * Accuracy (checked against float64 numpy in tests/test_math.py): log, exp,
 * sin, cos, pow, atan2, acos within a few ulp on the ranges the renderer
 * uses (the test states each bound).
 */
#ifndef ER_MATH_H
#define ER_MATH_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define ER_MATH_FN static __host__ __device__ __forceinline__
#else
#define ER_MATH_FN static inline
#endif

#ifdef __cplusplus
extern "C++" {
#endif

ER_MATH_FN float er_u2f(uint32_t u) { union { uint32_t u; float f; } v; v.u = u; return v.f; }
ER_MATH_FN uint32_t er_f2u(float f) { union { uint32_t u; float f; } v; v.f = f; return v.u; }
ER_MATH_FN double er_u2d(uint64_t u) { union { uint64_t u; double d; } v; v.u = u; return v.d; }
ER_MATH_FN uint64_t er_d2u(double d) { union { uint64_t u; double d; } v; v.d = d; return v.u; }

#define ER_F_INF er_u2f(0x7f800000u)
#define ER_F_NAN er_u2f(0x7fc00000u)
#define ER_D_INF er_u2d(0x7ff0000000000000ull)
#define ER_D_NAN er_u2d(0x7ff8000000000000ull)

/* ln2 = ER_LN2_HI + ER_LN2_LO; ER_LN2_HI has its 12 low mantissa bits clear. */
#define ER_LN2_HI 0.693115234375f
#define ER_LN2_LO 3.194618329871446e-05f
#define ER_LOG2E  1.44269504088896341f

/* natural logarithm, binary32 */
ER_MATH_FN float er_logf(float x)
{
    uint32_t b = er_f2u(x);
    if (b >= 0x7f800000u) {                 /* +inf, nan, or sign bit set */
        if (b == 0x7f800000u) return x;     /* log(+inf) = +inf */
        if ((b & 0x7fffffffu) == 0u) return -ER_F_INF; /* log(-0) */
        if ((b & 0x7fffffffu) > 0x7f800000u) return x;  /* nan */
        return ER_F_NAN;                    /* negative */
    }
    if (b == 0u) return -ER_F_INF;
    int e = 0;
    if (b < 0x00800000u) {                  /* subnormal: scale by 2^25 */
        x = x * 33554432.0f;
        b = er_f2u(x);
        e = -25;
    }
    e += (int)(b >> 23) - 127;
    float m = er_u2f((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float f = m - 1.0f;               /* exact */
    const float s = f / (2.0f + f);
    const float z = s * s;
    const float R = z * (0.666666667f + z * (0.4f + z * (0.285714286f + z * 0.222222222f)));
    const float hfsq = 0.5f * f * f;
    const float lm = f - (hfsq - s * (hfsq + R));
    const float fe = (float)e;
    return fe * ER_LN2_HI + (lm + fe * ER_LN2_LO);
}

/* exponential, binary32 */
ER_MATH_FN float er_expf(float x)
{
    if (x != x) return x;
    if (x > 88.7228394f) return ER_F_INF;
    if (x < -103.972084f) return 0.0f;
    const float kf = floorf(x * ER_LOG2E + 0.5f);
    const int k = (int)kf;
    const float r = (x - kf * ER_LN2_HI) - kf * ER_LN2_LO;
    const float p = 1.0f + r * (1.0f + r * (0.5f + r * (1.66666667e-1f + r * (4.16666667e-2f +
                    r * (8.33333333e-3f + r * (1.38888889e-3f + r * (1.98412698e-4f + r * 2.48015873e-5f)))))));
    const int k1 = k / 2;
    const int k2 = k - k1;
    return (p * er_u2f((uint32_t)(k1 + 127) << 23)) * er_u2f((uint32_t)(k2 + 127) << 23);
}

/* pi/2 = ER_PIO2_1 + ER_PIO2_2 + ER_PIO2_3; first part has 8 significant bits,
   second 12, so k*ER_PIO2_1 and k*ER_PIO2_2 are exact for |k| < 4096. */
#define ER_PIO2_1 1.5703125f
#define ER_PIO2_2 4.837512969970703e-04f
#define ER_PIO2_3 7.549790126404332e-08f
#define ER_TWO_OVER_PI 0.636619772367581343f

ER_MATH_FN void er_sincosf(float x, float* ps, float* pc)
{
    const float ax = fabsf(x);
    if (!(ax < ER_F_INF)) { *ps = ER_F_NAN; *pc = ER_F_NAN; return; }
    float kf = floorf(x * ER_TWO_OVER_PI + 0.5f);
    float r;
    if (ax < 6000.0f) {
        r = ((x - kf * ER_PIO2_1) - kf * ER_PIO2_2) - kf * ER_PIO2_3;
    } else {
        /* large arguments (never produced by the renderer): binary64 reduction */
        const double kd = floor((double)x * 0.63661977236758134 + 0.5);
        kf = (float)kd;
        const double rd = (((double)x - kd * 1.5707963109016418) - kd * 1.5893254712295857e-08) - kd * 6.123233995736766e-17;
        r = (float)rd;
        const double kmod = kd - 4.0 * floor(kd * 0.25);
        kf = (float)kmod;
    }
    const float z = r * r;
    const float sp = r + (r * z) * (-1.66666667e-1f + z * (8.33333333e-3f + z * (-1.98412698e-4f +
                     z * (2.75573192e-6f + z * -2.50521084e-8f))));
    const float cp = (1.0f - 0.5f * z) + (z * z) * (4.16666667e-2f + z * (-1.38888889e-3f +
                     z * (2.48015873e-5f + z * (-2.75573192e-7f + z * 2.08767570e-9f))));
    const int q = ((int)kf) & 3;
    float s, c;
    if (q == 0)      { s = sp;  c = cp;  }
    else if (q == 1) { s = cp;  c = -sp; }
    else if (q == 2) { s = -sp; c = -cp; }
    else             { s = -cp; c = sp;  }
    *ps = s;
    *pc = c;
}

ER_MATH_FN float er_sinf(float x) { float s, c; er_sincosf(x, &s, &c); return s; }
ER_MATH_FN float er_cosf(float x) { float s, c; er_sincosf(x, &s, &c); return c; }
ER_MATH_FN float er_tanf(float x) { float s, c; er_sincosf(x, &s, &c); return s / c; }

/* ---- double-single (float-float) helpers for pow / atan2 / acos ----
   All binary32: the GPU's binary64 rate is a small fraction of its binary32
   rate.  Exact products use Dekker's algorithm with Veltkamp splitting, which
   needs no fused multiply-add (valid while no product overflows). */

/* a * b = *p + *e exactly */
ER_MATH_FN void er_two_prod(float a, float b, float* p, float* e)
{
    const float ca = 4097.0f * a;
    const float ah = ca - (ca - a);
    const float al = a - ah;
    const float cb = 4097.0f * b;
    const float bh = cb - (cb - b);
    const float bl = b - bh;
    const float pp = a * b;
    *p = pp;
    *e = ((ah * bh - pp) + ah * bl + al * bh) + al * bl;
}

/* a + b = *s + *e exactly, for |a| >= |b| (or a == 0) */
ER_MATH_FN void er_fast_two_sum(float a, float b, float* s, float* e)
{
    const float ss = a + b;
    *s = ss;
    *e = b - (ss - a);
}

/* log(x) = *hi + *lo for finite x > 0 (about 2^-40 relative): the atanh
   series of er_logf with s = f / (2 + f) carried in double-single */
ER_MATH_FN void er_log_ds(float x, float* hi, float* lo)
{
    uint32_t b = er_f2u(x);
    int e = 0;
    if (b < 0x00800000u) {
        x = x * 33554432.0f;
        b = er_f2u(x);
        e = -25;
    }
    e += (int)(b >> 23) - 127;
    float m = er_u2f((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float f = m - 1.0f;                          /* exact */
    float dh, dl;
    er_fast_two_sum(2.0f, f, &dh, &dl);                /* 2 + f */
    const float sh = f / dh;
    float p, pe;
    er_two_prod(sh, dh, &p, &pe);
    const float sl = (((f - p) - pe) - sh * dl) / dh;  /* f/(2+f) - sh */
    const float z = sh * sh;
    const float poly = sh * (z * (0.666666667f + z * (0.4f + z * (0.285714286f + z * (0.222222222f + z * 0.181818182f)))));
    float h, l;
    er_fast_two_sum(2.0f * sh, poly, &h, &l);
    l = l + 2.0f * sl;
    /* + e * ln2 (ER_LN2_HI * e is exact) */
    const float fe = (float)e;
    float h2, l2;
    er_fast_two_sum(fe * ER_LN2_HI, h, &h2, &l2);
    if (fe == 0.0f) { h2 = h; l2 = 0.0f; }
    l2 = l2 + (l + fe * ER_LN2_LO);
    er_fast_two_sum(h2, l2, hi, lo);
}

/* exp(hi + lo) for |lo| <= ulp(hi) */
ER_MATH_FN float er_exp_ds(float hi, float lo)
{
    if (hi != hi) return hi;
    if (hi > 88.7228394f) return ER_F_INF;
    if (hi < -103.972084f) return 0.0f;
    const float kf = floorf(hi * ER_LOG2E + 0.5f);
    const int k = (int)kf;
    const float r = ((hi - kf * ER_LN2_HI) - kf * ER_LN2_LO) + lo;
    const float q = 1.0f + r * (1.0f + r * (0.5f + r * (1.66666667e-1f + r * (4.16666667e-2f +
                    r * (8.33333333e-3f + r * (1.38888889e-3f + r * (1.98412698e-4f + r * 2.48015873e-5f)))))));
    const int k1 = k / 2;
    const int k2 = k - k1;
    return (q * er_u2f((uint32_t)(k1 + 127) << 23)) * er_u2f((uint32_t)(k2 + 127) << 23);
}

/* x^y: exp(y log|x|) with the logarithm and the product in double-single,
   so large exponents such as the 1e6*g^7 Blinn exponent keep float accuracy */
ER_MATH_FN float er_powf(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (x == 1.0f) return 1.0f;
    if (x != x || y != y) return ER_F_NAN;
    const float ax = fabsf(x);
    const float ay = fabsf(y);
    const int yint = (floorf(y) == y);
    const int yodd = yint && ay < 16777216.0f && ((((int64_t)ay) & 1) != 0);
    if (ay == ER_F_INF) {
        if (ax == 1.0f) return 1.0f;
        if ((ax < 1.0f) == (y > 0.0f)) return 0.0f;
        return ER_F_INF;
    }
    if (x < 0.0f && !yint) return ER_F_NAN;
    if (ax == 0.0f) {
        if (y > 0.0f) return yodd ? x : 0.0f;
        return yodd ? (x < 0.0f || er_f2u(x) == 0x80000000u ? -ER_F_INF : ER_F_INF) : ER_F_INF;
    }
    if (ax == ER_F_INF) {
        float r = (y > 0.0f) ? ER_F_INF : 0.0f;
        return (x < 0.0f && yodd) ? -r : r;
    }
    float lh, ll;
    er_log_ds(ax, &lh, &ll);
    float th, tl;
    er_two_prod(y, lh, &th, &tl);
    tl = tl + y * ll;
    float h, l;
    er_fast_two_sum(th, tl, &h, &l);
    const float r = er_exp_ds(h, l);
    return (x < 0.0f && yodd) ? -r : r;
}

/* atan(u) for 0 <= u <= 1: u > tan(pi/12) is reduced with
   atan(u) = pi/6 + atan((sqrt3 u - 1)/(u + sqrt3)); odd Taylor series */
ER_MATH_FN float er_atan01f(float u)
{
    float base = 0.0f;
    float v = u;
    if (u > 0.267949194f) {
        v = (u * 1.73205081f - 1.0f) / (u + 1.73205081f);
        base = 0.523598776f;
    }
    const float z = v * v;
    const float p = v - (v * z) * (0.333333333f - z * (0.2f - z * (0.142857143f - z * (0.111111111f - z * (0.0909090909f -
                    z * 0.0769230769f)))));
    return base + p;
}

/* atan2(y, x) for finite and zero arguments */
ER_MATH_FN float er_atan2f(float y, float x)
{
    if (x != x || y != y) return ER_F_NAN;
    const float ax = fabsf(x), ay = fabsf(y);
    float a;
    if (ax == 0.0f && ay == 0.0f) a = 0.0f;
    else if (ay <= ax) a = er_atan01f(ay / ax);
    else a = (1.57079637f - er_atan01f(ax / ay)) + -4.37113883e-08f;
    if (x < 0.0f) a = (3.14159274f - a) + -8.74227766e-08f;
    return (y < 0.0f) ? -a : a;
}

ER_MATH_FN float er_acosf(float x)
{
    if (x != x || x > 1.0f || x < -1.0f) return ER_F_NAN;
    return er_atan2f(sqrtf((1.0f - x) * (1.0f + x)), x);
}

/* Counter-based seeding: 32-bit integer finaliser "lowbias32" from
   C. Wellons' hash-prospector (public domain); pure integer arithmetic. */
ER_MATH_FN uint32_t er_hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

/* Seed the two multiply-with-carry lanes of one sample (Source/rng.h:35-51)
   from (seed, view, pixel, sample).  A lane at 0 or at the map's fixed point
   (36969 resp. 18000 multiplier) would never move, so those values are
   replaced. */
ER_MATH_FN void er_seed_lanes(uint32_t seed, uint32_t view, uint32_t pixel, uint32_t sample,
                              uint32_t* lane0, uint32_t* lane1)
{
    uint32_t h = er_hash32(seed * 0x9e3779b9u + 0x632be5abu);
    h = er_hash32(h ^ (view * 0x85ebca6bu));
    h = er_hash32(h + pixel);
    h = er_hash32(h ^ (sample * 0xc2b2ae35u));
    uint32_t a = h;
    uint32_t b = er_hash32(h ^ 0x68e31da4u);
    if (a == 0u || a == 0x9068ffffu) a = 0x2545f491u;
    if (b == 0u || b == 0x464fffffu) b = 0x4f6cdd1du;
    *lane0 = a;
    *lane1 = b;
}

/* Stratified sample dimensions (er_render_settings.stratify).  For sample
   `sample` of `pixel` in `view`, the seven stratified dimensions are one
   point of the 7-dimensional Kronecker sequence R7 over the sample index
   (generator k = frac(g^-k) * 2^32, k = 1..7, g the positive root of
   x^8 = x + 1), shifted per pixel and dimension by a hash of (seed, view,
   pixel) (a Cranley-Patterson rotation).  The generators are distinct, so
   a pixel's points fill the 7-cube evenly as the samples grow and its
   estimate converges to the integral; dimensions sharing a generator would
   keep every point of the pixel on a lower-dimensional torus, and the
   pixel would converge to the integral along that torus instead.  Each
   sample alone is uniform, so estimates stay unbiased.  Integer arithmetic,
   23-bit mantissas in (0, 1): identical on every host and device.
     out[0], out[1]: point on the light (MetroSample light u, v)
     out[2]        : light choice
     out[3], out[4]: BSDF direction
     out[5]        : BSDF component
     out[6]        : the first free-flight draw of delta tracking */
ER_MATH_FN float er_lattice_unit(uint32_t x) { return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f); }

ER_MATH_FN void er_stratified_sample(uint32_t seed, uint32_t view, uint32_t pixel, uint32_t sample, float out[7])
{
    uint32_t h = er_hash32(seed * 0x9e3779b9u + 0x1b873593u);
    h = er_hash32(h ^ (view * 0x85ebca6bu));
    h = er_hash32(h + pixel);
    out[0] = er_lattice_unit(er_hash32(h ^ 0x3c6ef372u) + sample * 3915259345u);
    out[1] = er_lattice_unit(er_hash32(h ^ 0xa54ff53au) + sample * 3569120481u);
    out[2] = er_lattice_unit(er_hash32(h ^ 0x510e527fu) + sample * 3253582939u);
    out[3] = er_lattice_unit(er_hash32(h ^ 0x9b05688cu) + sample * 2965941329u);
    out[4] = er_lattice_unit(er_hash32(h ^ 0x1f83d9abu) + sample * 2703729436u);
    out[5] = er_lattice_unit(er_hash32(h ^ 0x5be0cd19u) + sample * 2464699080u);
    out[6] = er_lattice_unit(er_hash32(h ^ 0xcbbb9d5du) + sample * 2246800835u);
}

#ifdef __cplusplus
}
#endif

#endif /* ER_MATH_H */
