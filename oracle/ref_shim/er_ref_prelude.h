/*
 * er_ref_prelude.h - force-included (-include) before the reference's own
 * headers when oracle/Makefile builds the reference transport code for the
 * host (TEST INFRASTRUCTURE ONLY).  Nothing of the reference is copied; its
 * headers are compiled where they lie.  This prelude does three things:
 *
 * 1. Rvalue overloads of `float * Color` and `Color * float`.
 *    Source/color.h:260-284 declares these operators with a non-const
 *    reference to the colour, which MSVC binds to temporaries as an extension
 *    but g++ rejects (e.g. Source/lights.h:50, Source/color.h:262).  The
 *    templates below are viable only for rvalue colours, so lvalue calls keep
 *    the reference's own functions; for rvalues they compute X[i] *= F, the
 *    same products the reference computes.
 *
 * 2. Routes the elementary functions the transport code calls (logf via
 *    std::log(float), expf, powf, sinf, cosf, tanf, acosf, atan2f) to the
 *    bit-reproducible implementations of include/er_math.h, so the host build
 *    of the reference, the C restatement and the GPU parity kernel evaluate
 *    identical paths.  Define ER_REF_STOCK_LIBM to keep the C library instead.
 *
 * 3. Pulls in every standard header the reference includes, so the macros of
 *    (2) cannot reach a standard-library declaration.
 */
#ifndef ER_REF_PRELUDE_H
#define ER_REF_PRELUDE_H

#include <type_traits>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <cfloat>
#include <float.h>
#include <cmath>
#include <math.h>
#include <algorithm>
#include <map>
#include <cuda_runtime.h>

#include "er_math.h"

namespace ExposureRender {
class ColorRGBf;
class ColorXYZf;
class ColorXYZAf;
class ColorRGBuc;
class ColorRGBAuc;

template <class T> struct er_is_color : std::false_type {};
template <> struct er_is_color<ColorRGBf> : std::true_type {};
template <> struct er_is_color<ColorXYZf> : std::true_type {};
template <> struct er_is_color<ColorXYZAf> : std::true_type {};
template <> struct er_is_color<ColorRGBuc> : std::true_type {};
template <> struct er_is_color<ColorRGBAuc> : std::true_type {};

template <class T, class = typename std::enable_if<er_is_color<T>::value>::type>
inline T operator*(const float& F, T&& X) { T R(X); R *= F; return R; }

template <class T, class = typename std::enable_if<er_is_color<T>::value>::type>
inline T operator*(T&& X, const float& F) { T R(X); R *= F; return R; }
}

#ifndef ER_REF_STOCK_LIBM
static inline float er_ref_log(float x) { return er_logf(x); }
static inline double er_ref_log(double x) { return (double)er_logf((float)x); }
static inline float er_ref_exp(float x) { return er_expf(x); }
static inline double er_ref_exp(double x) { return (double)er_expf((float)x); }
#define logf er_logf
#define log er_ref_log
#define expf er_expf
#define exp er_ref_exp
#define powf er_powf
#define sinf er_sinf
#define cosf er_cosf
#define tanf er_tanf
#define acosf er_acosf
#define atan2f er_atan2f
#endif

#endif
