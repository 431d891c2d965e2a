/*
 * gbns_fmath.h -- fp32 elementary functions of the slice sampler built only from IEEE-754
 * basic operations (+, -, *, /, sqrt, fused multiply-add) and exact bit manipulation.
 *
 * Every operation used here is correctly rounded on the GPU (nvcc without fast-math:
 * -prec-div, -prec-sqrt, no flush to zero) and in C on an IEEE host (gcc with
 * -ffp-contract=off; fmaf from libm is correctly rounded), so a function evaluates to the
 * same bits on both.  That lets a CPU model of the kernels' fp32 arithmetic reproduce the
 * device chains bit for bit.  Their accuracy against FP64 references is tested separately.
 *
 *   gbns_fm_exp       exp(x): Cody-Waite reduction x = k ln2 + r (two-part ln2), degree-7
 *                     Taylor polynomial of exp(r) on |r| <= ln2/2, exact scaling by 2^k.
 *   gbns_fm_log       log(x): x = 2^e m with m in [sqrt(2)/2, sqrt(2)), s = (m-1)/(m+1),
 *                     log m = 2 atanh(s) = 2s + s^3 (2/3 + 2/5 s^2 + 2/7 s^4 + 2/9 s^6).
 *   gbns_fm_log1p     log1p(x) = log(u) x / (u - 1) with u = fl(1 + x) (D. Goldberg, "What
 *                     every computer scientist should know about floating-point arithmetic",
 *                     ACM Computing Surveys 23(1), 1991, theorem 4).
 *   gbns_fm_ndtri_*   standard normal quantile: M. J. Wichura, "Algorithm AS 241: the
 *                     percentage points of the normal distribution", Applied Statistics 37
 *                     (1988) 477-484, the single-precision rational approximations PPND7
 *                     (about 1e-7 relative).
 *   gbns_fm_normal_from_mantissa  jax.random.normal (float64) of one 52-bit mantissa M:
 *                     sqrt(2) erfinv(u) with u = (4M + 1 - 2^53) 2^-53 = 2p - 1, so the
 *                     quantile of p = (4M + 1) 2^-54, whose offset from 1/2 and whose tail
 *                     mass are formed exactly in integers and rounded once to fp32.
 *   gbns_fm_log64, gbns_fm_ndtri64  the FP64 log (the reduction of gbns_fm_log with a longer
 *                     atanh series) and the AS 241 double-precision quantile PPND16, for the
 *                     results' U -> X transform and prior density.
 */
#ifndef GBNS_FMATH_H
#define GBNS_FMATH_H

#include <stdint.h>
#include <math.h>
#if !defined(__CUDACC__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define GBNS_FM_FN __host__ __device__ __forceinline__
#else
#define GBNS_FM_FN static inline
#endif

GBNS_FM_FN uint32_t gbns_fm_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

GBNS_FM_FN float gbns_fm_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

/* Round-to-nearest-even conversion of a 64-bit unsigned integer to fp32.  On the device it
 * uses 32-bit operations only (the native 64-bit conversion runs on the FP64 pipe, which is
 * scarce on GB300): normalise, keep the top 32 bits with a sticky bit for the rest, convert,
 * rescale exactly.  The host conversion is correctly rounded as well. */
GBNS_FM_FN float gbns_fm_u64_to_float(uint64_t x) {
#if defined(__CUDA_ARCH__)
    if (x == 0ull) return 0.0f;
    const int nz = __clzll(x);
    const uint64_t y = x << nz;
    const uint32_t top = (uint32_t)(y >> 32) | ((uint32_t)y != 0u ? 1u : 0u);
    const float f = __uint2float_rn(top);
    return f * __int_as_float((127 + 32 - nz) << 23); /* 32 - nz in [-31, 32] */
#else
    return (float)x;
#endif
}

/* exp(x) */
GBNS_FM_FN float gbns_fm_exp(float x) {
    if (!(x == x)) return x;
    if (x > 0x1.62e430p+6f) return INFINITY; /* above log(FLT_MAX) */
    if (x < -0x1.9fe368p+6f) return 0.0f;    /* below log of half the smallest subnormal */
    const float kf = fmaf(x, 0x1.715476p+0f, 0x1.8p+23f) - 0x1.8p+23f; /* nearest integer to x / ln2 */
    float r = fmaf(kf, -0x1.62e400p-1f, x);
    r = fmaf(kf, -0x1.7f7d1cp-20f, r);
    float p = 0x1.a01a02p-13f; /* 1/7! */
    p = fmaf(p, r, 0x1.6c16c2p-10f);
    p = fmaf(p, r, 0x1.111112p-7f);
    p = fmaf(p, r, 0x1.555556p-5f);
    p = fmaf(p, r, 0x1.555556p-3f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int k = (int)kf;
    if (k > 127) return (p * 2.0f) * gbns_fm_from_bits((uint32_t)(k - 1 + 127) << 23);
    if (k < -125) return (p * gbns_fm_from_bits((uint32_t)(k + 64 + 127) << 23)) * 0x1p-64f;
    return p * gbns_fm_from_bits((uint32_t)(k + 127) << 23);
}

/* log(x) */
GBNS_FM_FN float gbns_fm_log(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    int e = 0;
    uint32_t ix = gbns_fm_bits(x);
    if (ix < 0x00800000u) { /* subnormal: scale into the normal range first */
        ix = gbns_fm_bits(x * 0x1p+24f);
        e = -24;
    }
    e += (int)(ix >> 23) - 127;
    ix = (ix & 0x007FFFFFu) | 0x3F800000u; /* m in [1, 2) */
    if (ix > 0x3FB504F3u) {                /* m > sqrt(2): use m / 2 */
        ix -= 0x00800000u;
        e += 1;
    }
    const float m = gbns_fm_from_bits(ix);
    const float f = m - 1.0f; /* exact */
    const float s = f / (2.0f + f);
    const float z = s * s;
    float P = 0x1.c71c72p-3f; /* 2/9 */
    P = fmaf(P, z, 0x1.24924ap-2f);
    P = fmaf(P, z, 0x1.99999ap-2f);
    P = fmaf(P, z, 0x1.555556p-1f);
    const float lm = fmaf(s * z, P, 2.0f * s);
    const float ef = (float)e;
    return fmaf(ef, 0x1.62e400p-1f, fmaf(ef, 0x1.7f7d1cp-20f, lm));
}

/* log(1 + x), x > -1 */
GBNS_FM_FN float gbns_fm_log1p(float x) {
    const float u = 1.0f + x;
    if (u == 1.0f) return x;
    if (u == INFINITY) return u;
    return gbns_fm_log(u) * (x / (u - 1.0f));
}

/* Phi^-1(1/2 + q) for |q| <= 0.425 (AS 241, PPND7, central region) */
GBNS_FM_FN float gbns_fm_ndtri_center(float q) {
    const float r = fmaf(-q, q, 0.180625f);
    float a = fmaf(59.109374720f, r, 159.29113202f);
    a = fmaf(a, r, 50.434271938f);
    a = fmaf(a, r, 3.3871327179f);
    float b = fmaf(67.187563600f, r, 78.757757664f);
    b = fmaf(b, r, 17.895169469f);
    b = fmaf(b, r, 1.0f);
    return (q * a) / b;
}

/* -Phi^-1(p) = Phi^-1(1 - p) for 0 < p <= 0.075 (AS 241, PPND7, tails) */
GBNS_FM_FN float gbns_fm_ndtri_upper(float p) {
    if (!(p == p)) return p;
    if (!(p > 0.0f)) return INFINITY;
    float r = sqrtf(-gbns_fm_log(p));
    float a, b;
    if (r <= 5.0f) {
        r = r - 1.6f;
        a = fmaf(0.17023821103f, r, 1.3067284816f);
        a = fmaf(a, r, 2.7568153900f);
        a = fmaf(a, r, 1.4234372777f);
        b = fmaf(0.12021132975f, r, 0.73700164250f);
        b = fmaf(b, r, 1.0f);
    } else {
        r = r - 5.0f;
        a = fmaf(0.017337203997f, r, 0.42868294337f);
        a = fmaf(a, r, 3.0812263860f);
        a = fmaf(a, r, 6.6579051150f);
        b = fmaf(0.012258202635f, r, 0.24197894225f);
        b = fmaf(b, r, 1.0f);
    }
    return a / b;
}

/* Phi^-1(u) of an fp32 u in [0, 1] (the Normal prior quantile) */
GBNS_FM_FN float gbns_fm_ndtri(float u) {
    const float q = u - 0.5f;
    if (fabsf(q) <= 0.425f) return gbns_fm_ndtri_center(q);
    const float z = gbns_fm_ndtri_upper(q < 0.0f ? u : 1.0f - u); /* 1 - u is exact here */
    return q < 0.0f ? -z : z;
}

/* Phi^-1(u) of an FP64 u: the offset from 1/2 and the tail mass are formed in FP64 and
 * rounded once, so u within 1e-12 of 0 or 1 keeps its own quantile. */
GBNS_FM_FN float gbns_fm_ndtri_d(double u) {
    const double q = u - 0.5;
    if (fabs(q) <= 0.425) return gbns_fm_ndtri_center((float)q);
    const float z = gbns_fm_ndtri_upper((float)(q < 0.0 ? u : 1.0 - u));
    return q < 0.0 ? -z : z;
}

/* ---- FP64: the results' prior transform (U -> X) ---------------------------------------- */

GBNS_FM_FN uint64_t gbns_fm_bits64(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

GBNS_FM_FN double gbns_fm_from_bits64(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

/* log(x) in FP64: x = 2^e m with m in [sqrt(2)/2, sqrt(2)), s = (m-1)/(m+1),
 * log m = 2 atanh(s) = 2s + s^3 sum_{k>=1} 2/(2k+1) s^(2k-2) through k = 10 (|s| <= 0.1716, so the
 * next term is below 2^-60 of the sum), e ln2 with ln2 split into a 32-bit head and a tail. */
GBNS_FM_FN double gbns_fm_log64(double x) {
    if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    int e = 0;
    uint64_t ix = gbns_fm_bits64(x);
    if ((ix >> 52) == 0) { /* subnormal */
        ix = gbns_fm_bits64(x * 0x1p+54);
        e = -54;
    }
    e += (int)(ix >> 52) - 1023;
    ix = (ix & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull; /* m in [1, 2) */
    if (ix > 0x3FF6A09E667F3BCCull) {                           /* m > sqrt(2): use m / 2 */
        ix -= 0x0010000000000000ull;
        e += 1;
    }
    const double m = gbns_fm_from_bits64(ix);
    const double f = m - 1.0; /* exact */
    const double s = f / (2.0 + f);
    const double z = s * s;
    double P = 2.0 / 21.0;
    P = fma(P, z, 2.0 / 19.0);
    P = fma(P, z, 2.0 / 17.0);
    P = fma(P, z, 2.0 / 15.0);
    P = fma(P, z, 2.0 / 13.0);
    P = fma(P, z, 2.0 / 11.0);
    P = fma(P, z, 2.0 / 9.0);
    P = fma(P, z, 2.0 / 7.0);
    P = fma(P, z, 2.0 / 5.0);
    P = fma(P, z, 2.0 / 3.0);
    const double lm = fma(s * z, P, 2.0 * s);
    const double ef = (double)e;
    return fma(ef, 0x1.62e42ffp-1, fma(ef, -0x1.718432a1b0e26p-35, lm));
}

/* Phi^-1(p) in FP64, p in [0, 1]: AS 241 (Wichura 1988), the double-precision rational
 * approximations PPND16 (about 1e-16 relative): a degree-7 / degree-7 rational in
 * r = 0.180625 - q^2 for |q| = |p - 1/2| <= 0.425, else two degree-7 / degree-7 rationals in
 * r = sqrt(-log(min(p, 1 - p))), split at r = 5.  Horner steps are explicit FMAs, so host and
 * device give the same bits. */
GBNS_FM_FN double gbns_fm_ndtri64(double p) {
    if (!(p == p)) return p;
    const double q = p - 0.5;
    if (fabs(q) <= 0.425) {
        const double r = fma(-q, q, 0.180625);
        double a = 2.5090809287301226727e+3;
        a = fma(a, r, 3.3430575583588128105e+4);
        a = fma(a, r, 6.7265770927008700853e+4);
        a = fma(a, r, 4.5921953931549871457e+4);
        a = fma(a, r, 1.3731693765509461125e+4);
        a = fma(a, r, 1.9715909503065514427e+3);
        a = fma(a, r, 1.3314166789178437745e+2);
        a = fma(a, r, 3.3871328727963666080e+0);
        double b = 5.2264952788528545610e+3;
        b = fma(b, r, 2.8729085735721942674e+4);
        b = fma(b, r, 3.9307895800092710610e+4);
        b = fma(b, r, 2.1213794301586595867e+4);
        b = fma(b, r, 5.3941960214247511077e+3);
        b = fma(b, r, 6.8718700749205790830e+2);
        b = fma(b, r, 4.2313330701600911252e+1);
        b = fma(b, r, 1.0);
        return (q * a) / b;
    }
    const double t = q < 0.0 ? p : 1.0 - p; /* 1 - p is exact for p > 0.925 */
    if (!(t > 0.0)) return q < 0.0 ? -INFINITY : INFINITY;
    double r = sqrt(-gbns_fm_log64(t));
    double a, b;
    if (r <= 5.0) {
        r = r - 1.6;
        a = 7.74545014278341407640e-4;
        a = fma(a, r, 2.27238449892691845833e-2);
        a = fma(a, r, 2.41780725177450611770e-1);
        a = fma(a, r, 1.27045825245236838258e+0);
        a = fma(a, r, 3.64784832476320460504e+0);
        a = fma(a, r, 5.76949722146069140550e+0);
        a = fma(a, r, 4.63033784615654529590e+0);
        a = fma(a, r, 1.42343711074968357734e+0);
        b = 1.05075007164441684324e-9;
        b = fma(b, r, 5.47593808499534494600e-4);
        b = fma(b, r, 1.51986665636164571966e-2);
        b = fma(b, r, 1.48103976427480074590e-1);
        b = fma(b, r, 6.89767334985100004550e-1);
        b = fma(b, r, 1.67638483018380384940e+0);
        b = fma(b, r, 2.05319162663775882187e+0);
        b = fma(b, r, 1.0);
    } else {
        r = r - 5.0;
        a = 2.01033439929228813265e-7;
        a = fma(a, r, 2.71155556874348757815e-5);
        a = fma(a, r, 1.24266094738807843860e-3);
        a = fma(a, r, 2.65321895265761230930e-2);
        a = fma(a, r, 2.96560571828504891230e-1);
        a = fma(a, r, 1.78482653991729133580e+0);
        a = fma(a, r, 5.46378491116411436990e+0);
        a = fma(a, r, 6.65790464350110377720e+0);
        b = 2.04426310338993978564e-15;
        b = fma(b, r, 1.42151175831644588870e-7);
        b = fma(b, r, 1.84631831751005468180e-5);
        b = fma(b, r, 7.86869131145613259100e-4);
        b = fma(b, r, 1.48753612908506148525e-2);
        b = fma(b, r, 1.36929880922735805310e-1);
        b = fma(b, r, 5.99832206555887937690e-1);
        b = fma(b, r, 1.0);
    }
    const double z = a / b;
    return q < 0.0 ? -z : z;
}

/* jax.random.normal (float64) from the 52-bit mantissa M of one 64-bit draw */
GBNS_FM_FN float gbns_fm_normal_from_mantissa(uint64_t M) {
    const uint64_t a = 4ull * M + 1ull; /* 2^54 p, odd, never 2^53 */
    const int upper = a > (1ull << 53);
    const uint64_t dq = upper ? a - (1ull << 53) : (1ull << 53) - a; /* 2^54 |p - 1/2| */
    const float q = gbns_fm_u64_to_float(dq) * 0x1p-54f;
    if (q <= 0.425f) {
        const float v = gbns_fm_ndtri_center(q);
        return upper ? v : -v;
    }
    const uint64_t pt = upper ? (1ull << 54) - a : a; /* 2^54 min(p, 1 - p) */
    const float z = gbns_fm_ndtri_upper(gbns_fm_u64_to_float(pt) * 0x1p-54f);
    return upper ? z : -z;
}

#endif /* GBNS_FMATH_H */
