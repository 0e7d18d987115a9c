/*
 * nt2_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of NT2's scalar float algorithms for the fused-expression
 * and reduction hot path, plus FP64 reference formulas and an exact
 * superaccumulator.  It is the checker for the CUDA library and the timed CPU
 * baseline; nothing in the product links or calls it.
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline leg load this
 * file (as liboracle.so through ctypes).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -fPIC -shared.
 * -ffp-contract=off matters: NT2's generic fma/fnms and its Horner scheme are
 * unfused (a*b+c with two roundings), and GCC defaults to contraction on
 * aarch64.
 *
 * Parity pinning: the elementary functions are checked against the golden
 * values in NT2's own unit tests (tests/golden/nt2_unit_vectors.json).
 * Whole-expression outputs have no golden vectors in the reference (its demos
 * assert nothing), so for those this restatement plus the FP64 formulas are
 * the oracle.
 *
 * Citations are paths inside the NT2 source tree:
 *   EXP  = modules/core/exponential/include/nt2/exponential/functions
 *   EUL  = modules/core/euler/include/nt2/euler/functions
 *   STAT = modules/core/statistics/include/nt2/statistics/functions
 *   BSIMD= modules/boost/simd/base/include/boost/simd
 *   TRIG = modules/core/trigonometric/include/nt2/trigonometric/functions
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

static inline float bf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t fb(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* NT2 float constants (hex as in the NT2 constant headers). */
#define C_MAXLOG      0x42b0c0a5u /* EXP/../constants/maxlog.hpp:29  88.3763 */
#define C_MINLOG      0xc2b0c0a5u /* minlog.hpp:29 */
#define C_INVLOG_2    0x3fb8aa3bu /* invlog_2.hpp:29 */
#define C_LOG_2HI     0x3f318000u /* log_2hi.hpp:29  0.693359375 */
#define C_LOG_2LO     0xb95e8083u /* log_2lo.hpp:29 -2.1219444e-4 */
#define C_SQRT_2O_2   0x3F3504F3u /* BSIMD/constant/constants/sqrt_2o_2.hpp:30 */
#define C_SMALLESTPOS 0x00800000u /* smallestposval.hpp:30 */
#define C_TWOTONMB    0x4B000000u /* twotonmb.hpp:30  2^23 */
#define C_MLOGTWO2NMB 0xc17f1402u /* mlogtwo2nmb.hpp:29 */
#define C_TWOTHIRD    0x3f2aaaabu /* twothird.hpp:30 */
#define C_INVSQRT_2PI 0x3ecc422au /* invsqrt_2pi.hpp:28 */

/* Static Horner, NT2 order: c[0] is the highest degree; each step is
 * x*acc + c (unfused fma).  POLY/scalar/impl/horner.hpp:37-53. */
static inline float horner(float x, const uint32_t *c, int n)
{
    float r = bf(c[0]);
    for (int i = 1; i < n; ++i) r = x * r + bf(c[i]);
    return r;
}

/* round2even: BSIMD/arithmetic/functions/scalar/round2even.hpp:29-36 */
static inline float round2even(float a0)
{
    const float v = fabsf(a0), t2n = bf(C_TWOTONMB);
    volatile float d0 = v + t2n; /* volatile keeps the add/sub pair literal */
    float d = d0 - t2n;
    d = (v < t2n) ? d : v;
    return a0 < 0.0f ? -d : d;
}

/* ---------------------------------------------------------------- exp ----
 * EXP/scalar/impl/expo/expo_base.hpp:58-69 (driver),
 * EXP/scalar/impl/expo/f_expo_reduction.hpp:52-85 (reduce + approx),
 * EXP/scalar/impl/expo/expo_scale.hpp:27-35 (2^k by exponent bits). */
static const uint32_t EXP_P[5] = {0x3ab778cf, 0x3c098d8b, 0x3d2aa957, 0x3e2aa9a5, 0x3f000000};

EXPORT float o_exp(float a0)
{
    if (a0 >= bf(C_MAXLOG)) return INFINITY;
    if (a0 <= bf(C_MINLOG)) return 0.0f;
    if (a0 != a0) return a0;
    float k = round2even(bf(C_INVLOG_2) * a0);
    float x = a0 - k * bf(C_LOG_2HI);
    x = x - k * bf(C_LOG_2LO);
    float y = horner(x, EXP_P, 5);
    float c = (y * (x * x) + x) + 1.0f;
    int32_t ik = (int32_t)k + 127;
    ik = (int32_t)((uint32_t)ik << 23);
    return c * bf((uint32_t)ik);
}

/* ---------------------------------------------------------------- log ----
 * EXP/scalar/impl/logs/f_log.hpp:59-88, kernel f_kernel.hpp:43-75,
 * fast_frexp BSIMD/ieee/functions/scalar/fast_frexp.hpp:52-58. */
static const uint32_t LOG_P[8] = {0xbda5dff0, 0x3e0229f9, 0xbe04d6b7, 0x3e116e80,
                                  0xbe2a6aa0, 0x3e4cd0a3, 0xbe800064, 0x3eaaaaa9};

/* The reduction every float logarithm shares (logs/f_kernel.hpp:43-75):
 * a0 = 2^fe (1 + x), x2 = x*x, y = P8(x)*x*x2; denormals scaled by 2^23 first,
 * with t = the matching -23 log_b(2) (f_log.hpp:70-78). */
static void log_reduce(float a0, uint32_t mlog_two2nmb, float *fe, float *x, float *x2, float *y, float *t)
{
    float z = a0;
    *t = 0.0f;
    if (fabsf(z) < bf(C_SMALLESTPOS)) { z *= bf(C_TWOTONMB); *t = bf(mlog_two2nmb); }
    uint32_t u = fb(z);
    int32_t e = (int32_t)((u & 0x7f800000u) >> 23) - 126;
    float m = bf((u & ~0x7f800000u) | 0x3f000000u);
    int lt = m < bf(C_SQRT_2O_2);
    *fe = lt ? (float)e + (-1.0f) : (float)e;
    *x = (lt ? m + m : m) - 1.0f;
    *x2 = *x * *x;
    *y = horner(*x, LOG_P, 8) * *x * *x2;
}

#define LOG_SPECIALS(a0)                          \
    if (a0 == INFINITY) return a0;                \
    if (a0 == 0.0f) return -INFINITY;             \
    if (a0 != a0 || a0 < 0.0f) return NAN;

/* log: f_log.hpp:59-88 */
EXPORT float o_log(float a0)
{
    LOG_SPECIALS(a0)
    float fe, x, x2, y, t;
    log_reduce(a0, C_MLOGTWO2NMB, &fe, &x, &x2, &y, &t);
    y = fe * bf(C_LOG_2LO) + y;
    y = -0.5f * x2 + y;
    return bf(C_LOG_2HI) * fe + ((x + y) + t);
}

/* log2: f_log.hpp:90-119, Log2_em1 = 0x3ee2a8ed, Mlog2two2nmb = 0xc1b80000 */
EXPORT float o_log2(float a0)
{
    LOG_SPECIALS(a0)
    float fe, x, x2, y, t;
    log_reduce(a0, 0xc1b80000u, &fe, &x, &x2, &y, &t);
    y = -0.5f * x2 + y;
    float z = x * bf(0x3ee2a8edu) + y * bf(0x3ee2a8edu);
    return (((z + y) + x) + fe) + t;
}

/* log10: f_log.hpp:121-153 (amul(a,b,c) = b*c + a), Log10_ehi = 0x3ede0000,
 * Log10_elo = 0x3a37b152, Log10_2hi = 0x3e9a0000, Log10_2lo = 0x39826a14,
 * Mlog10two2nmb = 0xc0dd8ede */
EXPORT float o_log10(float a0)
{
    LOG_SPECIALS(a0)
    float fe, x, x2, y, t;
    log_reduce(a0, 0xc0dd8edeu, &fe, &x, &x2, &y, &t);
    y = -0.5f * x2 + y;
    float z = (x + y) * bf(0x3a37b152u);
    z = y * bf(0x3ede0000u) + z;
    z = x * bf(0x3ede0000u) + z;
    z = fe * bf(0x3e9a0000u) + z;
    return fe * bf(0x39826a14u) + (z + t);
}

/* -------------------------------------------------------------- log1p ----
 * EXP/scalar/log1p.hpp:35-45 */
EXPORT float o_log1p(float a0)
{
    if (-1.0f > a0) return NAN;
    if (a0 == INFINITY) return INFINITY;
    if (a0 == -1.0f) return -INFINITY;
    float u = 1.0f + a0;
    return o_log(u) + (a0 - (u - 1.0f)) / u;
}

/* --------------------------------------------------------------- erfc ----
 * EUL/scalar/erfc.hpp:83-104, polynomials EUL/details/erf_kernel.hpp:48-91 */
static const uint32_t ERFC2_P[11] = {0xc0283611, 0x40d67e3b, 0xc0cd1a85, 0x4050b063,
                                     0xbfaea865, 0x3e2006f0, 0x3e1175c7, 0x3ec4ca6e,
                                     0x3e243828, 0xbf918a62, 0x3f0a0e8b};
static const uint32_t ERFC3_P[9] = {0x41aa8e55, 0x401b5680, 0xc010d956, 0x3f2cff3b,
                                    0xc016c985, 0xbffc9284, 0xbfa11698, 0xbe036d7e,
                                    0x3f7ffffe};

/* erfc(|a0|) before the sign fold; shared by erfc, normcdf and the fused
 * call/put pairs, which in NT2 differ only in the final 2-r select. */
static inline float erfc_core(float x)
{
    float z = x / (1.0f + x);
    if (x < bf(C_TWOTHIRD)) return (1.0f - z) * horner(z, ERFC3_P, 9);
    if (x == INFINITY) return 0.0f;
    z -= 0.4f;
    return o_exp(-(x * x)) * horner(z, ERFC2_P, 11);
}

EXPORT float o_erfc(float a0)
{
    float r1 = erfc_core(fabsf(a0));
    return (a0 < 0.0f) ? 2.0f - r1 : r1;
}

/* erf EUL/scalar/erf.hpp (single_), erf1 kernel EUL/details/erf_kernel.hpp:34-44 */
static const uint32_t ERF1_P[6] = {0xba1fc83b, 0x3ba4468d, 0xbcdb61f4, 0x3de70f22, 0xbec0937e, 0x3f906eba};
EXPORT float o_exp(float a0);

EXPORT float o_erf(float a0)
{
    if (isnan(a0)) return a0;
    if (isinf(a0)) return a0 > 0.0f ? 1.0f : -1.0f;
    float x = fabsf(a0);
    if (x < bf(C_TWOTHIRD)) return a0 * horner(x * x, ERF1_P, 6);
    float z = x / (1.0f + x) - 0.4f;
    float r2 = 1.0f - o_exp(-(x * x)) * horner(z, ERFC2_P, 11);
    return (a0 < 0.0f) ? -r2 : r2;
}

/* expx2 EXP/scalar/expx2.hpp (one argument): exp(x^2) as exp(m^2) exp(2mf + f^2)
 * with m = Expx2c1 floor(Expx2c2 x + 1/2) (float constants 32 and 1/32) */
EXPORT float o_expx2(float a0)
{
    if (isinf(a0)) return INFINITY;
    float x = fabsf(a0);
    float m = 32.0f * floorf(0.03125f * x + 0.5f);
    x -= m;
    float u = m * m;
    float u1 = (2.0f * m) * x + x * x;
    if (u + u1 > bf(C_MAXLOG)) return INFINITY;
    return o_exp(u) * o_exp(u1);
}

/* erfcx EUL/scalar/erfcx.hpp (single_): exp(x^2) erfc(x) below 2/3, else the erfc2 kernel */
EXPORT float o_erfcx(float a0)
{
    if (a0 == INFINITY) return 0.0f;
    if (isnan(a0)) return a0;
    if (a0 < bf(C_TWOTHIRD)) return o_expx2(a0) * o_erfc(a0);
    float z = a0 / (1.0f + a0) - 0.4f;
    return horner(z, ERFC2_P, 11);
}

/* normcdf: STAT/generic/normcdf.hpp:34  Half*erfc(-Sqrt_2o_2*a0) */
EXPORT float o_normcdf(float a0) { return 0.5f * o_erfc(-bf(C_SQRT_2O_2) * a0); }

/* fastnormcdf: STAT/generic/fastnormcdf.hpp:39-54 (A&S 26.2.17 form) */
static const uint32_t FNCDF_P[5] = {0x3faa466f, 0xbfe91eea, 0x3fe40778, 0xbeb68f87, 0x3ea385fa};

EXPORT float o_fastnormcdf(float a0)
{
    float l = fabsf(a0);
    float k = 1.0f / (0.2316419f * l + 1.0f);
    float w = horner(k, FNCDF_P, 5);
    w *= k * bf(C_INVSQRT_2PI) * o_exp(-(l * l) * 0.5f);
    return (a0 > 0.0f) ? 1.0f - w : w;
}

/* ------------------------------------------------- exp2, exp10, expm1 --
 * NT2's float algorithms, every operation rounded: the two_tag and ten_tag
 * reductions (EXP/scalar/impl/expo/f_expo_reduction.hpp:88-126, 129-168)
 * under the float driver expo_base.hpp:55-69 and the scale expo_scale.hpp:34
 * (a multiply by the bits (k+127)<<23); expm1 per EXP/scalar/expm1.hpp:33-41
 * and EXP/details/expm1_kernel.hpp:49-73. */
static float o_pow2i(float k) { return bf((uint32_t)((int32_t)k + 127) << 23); }

EXPORT float o_exp2(float a0)
{
    if (a0 >= bf(0x42fe0000u)) return INFINITY;
    if (a0 <= bf(0xc2fe0000u)) return 0.0f;
    if (a0 != a0) return a0;
    const float k = rintf(a0);
    const float x = a0 - k;
    float y = bf(0x3922c8c4u);
    y = y * x + bf(0x3ab01218u);
    y = y * x + bf(0x3c1d9422u);
    y = y * x + bf(0x3d6356ebu);
    y = y * x + bf(0x3e75fdf1u);
    const float c = (y * (x * x) + x * bf(0x3f317218u)) + 1.0f;
    return c * o_pow2i(k);
}

EXPORT float o_exp10(float a0)
{
    if (a0 >= bf(0x4218ec59u)) return INFINITY;
    if (a0 <= bf(0xc2179999u)) return 0.0f;
    if (a0 != a0) return a0;
    const float k = rintf(bf(0x40549a78u) * a0);
    float x = a0 - k * bf(0x3e9a0000u);
    x = x - k * bf(0x39826a14u);
    float y = bf(0x3e54dff1u);
    y = y * x + bf(0x3f0aacefu);
    y = y * x + bf(0x3f95eb4cu);
    y = y * x + bf(0x400237dau);
    y = y * x + bf(0x4029a926u);
    y = y * x + bf(0x40135d8eu);
    return (y * x + 1.0f) * o_pow2i(k);
}

EXPORT float o_expm1(float a0)
{
    if (a0 != a0) return bf(0x7fc00000u);
    if (a0 < bf(0xc17f1402u)) return -1.0f;
    if (a0 > bf(C_MAXLOG)) return INFINITY;
    const float k = rintf(bf(C_INVLOG_2) * a0);
    float x = a0 - k * bf(C_LOG_2HI);
    x = x - k * bf(C_LOG_2LO);
    const float hx = x * 0.5f;
    const float hxs = x * hx;
    float r1 = bf(0x3acf6db4u);
    r1 = r1 * hxs + bf(0xbd08887fu);
    r1 = r1 * hxs + 1.0f;
    const float t = 3.0f - r1 * hx;
    float e = hxs * ((r1 - t) / (6.0f - x * t));
    e = x * e - hxs;
    const int32_t ik = (int32_t)k;
    const float two2mk = bf((uint32_t)(127 - ik) << 23);
    const float y = (1.0f - two2mk) - (e - x);
    return y * o_pow2i(k);
}

/* --------------------------------------------------------- hyperbolic ----
 * HYP = modules/core/hyperbolic/include/nt2/hyperbolic/functions:
 * sinh HYP/scalar/sinh.hpp:35-58 + HYP/details/sinh_kernel.hpp:24-35,
 * cosh HYP/generic/cosh.hpp:33-43 (average(a,b) = a*0.5 + b*0.5),
 * tanh HYP/scalar/tanh.hpp:33-50 + HYP/details/tanh_kernel.hpp:27-40. */
static const uint32_t SINH_P[4] = {0x39559e2f, 0x3c087bbe, 0x3e2aaacc, 0x3f800000};
static const uint32_t TANH_P[5] = {0xbbbaf0ea, 0x3ca9134e, 0xbd5c1e2d, 0x3e088393, 0xbeaaaa99};

EXPORT float o_sinh(float a0)
{
    float x = fabsf(a0), r;
    if (x < 1.0f) return horner(x * x, SINH_P, 4) * a0;
    if (x > bf(C_MAXLOG) - bf(0x3f317218u)) {
        float t = o_exp(0.5f * x);
        r = (0.5f * t) * t;
    } else {
        float t = o_exp(x);
        r = t * 0.5f - 0.5f * (1.0f / t);
    }
    return bf(fb(r) ^ (fb(a0) & 0x80000000u));
}

EXPORT float o_cosh(float a0)
{
    float x = fabsf(a0);
    int big = x > bf(C_MAXLOG) - bf(0x3f317218u);
    float t = o_exp(x * (big ? 0.5f : 1.0f));
    if (big) return (0.5f * t) * t;
    return t * 0.5f + (1.0f / t) * 0.5f;
}

EXPORT float o_tanh(float a0)
{
    float x = fabsf(a0);
    if (x < 0.625f) {
        float x2 = x * x;
        return (horner(x2, TANH_P, 5) * x2) * a0 + a0;
    }
    float r = -2.0f * (1.0f / (1.0f + o_exp(x + x))) + 1.0f;
    return bf(fb(r) ^ (fb(a0) & 0x80000000u));
}

/* coth HYP/scalar/coth.hpp (tanh_kernel::coth = rec(tanh kernel)) */
EXPORT float o_coth(float a0)
{
    float x = fabsf(a0), r;
    if (x < 0.625f) {
        float x2 = x * x;
        r = 1.0f / ((horner(x2, TANH_P, 5) * x2) * x + x);
    } else {
        r = 2.0f * (1.0f / (o_exp(x + x) - 1.0f)) + 1.0f;
    }
    return bf(fb(r) ^ (fb(a0) & 0x80000000u));
}

/* sinhc HYP/scalar/sinhc.hpp + HYP/details/sinhc_kernel.hpp (the sinh kernel's coefficients) */
EXPORT float o_sinhc(float a0)
{
    float x = fabsf(a0);
    if (isinf(x)) return x;
    if (x < 1.0f) return horner(x * x, SINH_P, 4);
    int big = x > bf(C_MAXLOG) - bf(0x3f317218u);
    float t = o_exp(x * (big ? 0.5f : 1.0f));
    if (big) return ((0.5f * t) / x) * t;
    return (t * 0.5f + (-(1.0f / t)) * 0.5f) / x;
}

/* sech, csch, asech, acsch, acoth: HYP/generic/{sech,csch,asech,acsch,acoth}.hpp */
EXPORT float o_asinh(float a0);
EXPORT float o_acosh(float a0);
EXPORT float o_atanh(float a0);
EXPORT float o_sech(float a0) { return 1.0f / o_cosh(a0); }
EXPORT float o_csch(float a0) { return 1.0f / o_sinh(a0); }
EXPORT float o_asech(float a0) { return o_acosh(1.0f / a0); }
EXPORT float o_acsch(float a0) { return o_asinh(1.0f / a0); }
EXPORT float o_acoth(float a0) { return o_atanh(1.0f / a0); }

/* --------------------------------------------------------- cbrt, hypot ----
 * cbrt: EXP/scalar/cbrt.hpp (float overload, Cephes' cbrtf); hypot:
 * BSIMD/arithmetic/functions/scalar/hypot.hpp:27-40 with NT2's exponent()
 * (0 for zero, inf, NaN, else ::ilogbf, BSIMD/ieee/functions/scalar/exponent.hpp). */
static const uint32_t CBRT_P[5] = {0xbe09e49a, 0x3f0bf0fe, 0xbf745265, 0x3f91eb77, 0x3ece0609};
static float nt2_ldexpf(float a, int e);

EXPORT float o_cbrt(float a0)
{
    float z = fabsf(a0);
    if (z == INFINITY || z == 0.0f) return a0;
    float f = 1.0f;
    if (z < bf(0x00800000u)) { z *= 8388608.0f; f = bf(0x3ba14518u); }
    uint32_t u = fb(z);
    int e = (int)((u & 0x7f800000u) >> 23) - 126;
    float x = bf((u & ~0x7f800000u) | 0x3f000000u);
    x = horner(x, CBRT_P, 5);
    int flag = e >= 0, e1 = e < 0 ? -e : e, rem = e1;
    e1 /= 3;
    rem -= e1 * 3;
    e = e < 0 ? -e1 : e1;
    float cbrt2 = flag ? bf(0x3fa14518u) : bf(0x3f4b2ff5u), cbrt4 = flag ? bf(0x3fcb2ff5u) : bf(0x3f214518u);
    float fact = rem == 1 ? cbrt2 : 1.0f;
    fact = rem == 2 ? cbrt4 : fact;
    x = (x * fact) * bf((uint32_t)(e + 127) << 23);
    x = x - (x - z / (x * x)) * bf(0x3eaaaaabu);
    return bf(fb(x) | (fb(a0) & 0x80000000u)) * f;
}

static int nt2_exponent(float x)
{
    if (x != x || fabsf(x) == INFINITY || x == 0.0f) return 0;
    return ilogbf(x);
}

EXPORT float o_hypot(float a0, float a1)
{
    if ((a0 != a0 && fabsf(a1) == INFINITY) || (fabsf(a0) == INFINITY && a1 != a1)) return INFINITY;
    float r = fabsf(a0), i = fabsf(a1);
    int e = nt2_exponent((i > r) ? i : r);
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    float a = nt2_ldexpf(r, -e), b = nt2_ldexpf(i, -e);
    return nt2_ldexpf(sqrtf(a * a + b * b), e);
}

EXPORT void o_hypot_f32(const float *x, const float *y, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = o_hypot(x[i], y[i]);
}

EXPORT void o_hypot_f64(const float *x, const float *y, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = hypot((double)x[i], (double)y[i]);
}

/* ------------------------------------------------- inverse hyperbolic ----
 * HYP/scalar/asinh.hpp (float overload, Cephes' asinhf polynomial), acosh.hpp,
 * atanh.hpp; hypot per BSIMD/arithmetic/functions/scalar/hypot.hpp:27-40
 * (both operands scaled by 2^-e, e the larger one's exponent clamped to
 * [-126, 126]). */
static const uint32_t ASINH_P[5] = {0x3ca4d6e6, 0xbd2ee581, 0x3d9949b1, 0xbe2aa9ad, 0x3f800000};
static float nt2_ldexpf(float a, int e);

static float hypot_nt2(float r, float i)
{
    float m = (i > r) ? i : r;
    int e = (int)((fb(m) >> 23) & 0xff) - 127;
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    float a = nt2_ldexpf(r, -e), b = nt2_ldexpf(i, -e);
    return nt2_ldexpf(sqrtf(a * a + b * b), e);
}

EXPORT float o_asinh(float a0)
{
    float x = fabsf(a0), z;
    if (x < 0.5f) z = horner(x * x, ASINH_P, 5) * x;
    else if (x > bf(0x453504f3u)) z = o_log(x) + bf(0x3f317218u);
    else z = o_log(x + hypot_nt2(1.0f, x));
    return bf(fb(z) ^ (fb(a0) & 0x80000000u));
}

EXPORT float o_acosh(float a0)
{
    float t = a0 - 1.0f;
    if (t <= bf(0x4a800000u)) return o_log1p(t + sqrtf((t + t) + t * t));
    return o_log(t) + bf(0x3f317218u);
}

EXPORT float o_atanh(float a0)
{
    float x = fabsf(a0), t = x + x, z1 = 1.0f - x;
    float u = (x < 0.5f) ? t * (x / z1) + t : t / z1;
    return bf(fb(0.5f * o_log1p(u)) ^ (fb(a0) & 0x80000000u));
}

/* ------------------------------------------------ inverse trigonometry ----
 * TRIG/scalar/impl/invtrig/f_invtrig.hpp:33-128 (Cephes asinf / atanf),
 * atan2 TRIG/scalar/atan2.hpp:30-46 */
static const uint32_t ASIN_P[5] = {0x3d2cb352, 0x3cc617e3, 0x3d3a3ec7, 0x3d9980f6, 0x3e2aaae4};
static const uint32_t ATAN_P[4] = {0x3da4f0d1, 0xbe0e1b85, 0x3e4c925f, 0xbeaaaa2a};

EXPORT float o_asin(float a0)
{
    float x = fabsf(a0), z;
    uint32_t sign = fb(a0) & 0x80000000u;
    if (x < bf(0x38d1b717u)) return a0;
    if (x > 1.0f) return NAN;
    int big = x > 0.5f;
    if (big) { z = 0.5f * (1.0f - x); x = sqrtf(z); }
    else z = x * x;
    float z1 = horner(z, ASIN_P, 5);
    z1 = z1 * (z * x) + x;
    if (big) { z1 = z1 + z1; z1 = bf(0x3fc90fdbu) - z1; }
    return bf(fb(z1) ^ sign);
}

EXPORT float o_acos(float a0)
{
    if (a0 < -0.5f) return bf(0x40490fdbu) - o_asin(sqrtf((a0 + 1.0f) * 0.5f)) * 2.0f;
    if (a0 > 0.5f) return o_asin(sqrtf((1.0f - a0) * 0.5f)) * 2.0f;
    return bf(0x3fc90fdbu) - o_asin(a0);
}

static float atan_kernel(float a0)
{
    if (a0 == 0.0f) return 0.0f;
    if (fabsf(a0) == INFINITY) return bf(0x3fc90fdbu);
    float x = fabsf(a0), y = 0.0f, more = 0.0f;
    if (x > bf(0x401a827au)) { y = bf(0x3fc90fdbu); more = bf(0xb33bbd2eu); x = -(1.0f / x); }
    else if (x > bf(0x3ed413cdu)) { y = bf(0x3f490fdbu); more = bf(0xb2bbbd2eu); x = (x - 1.0f) / (x + 1.0f); }
    float z = x * x;
    float z1 = horner(z, ATAN_P, 4);
    z1 = x * (z1 * z) + x;
    return y + (z1 + more);
}

EXPORT float o_atan(float a0) { return bf(fb(atan_kernel(a0)) ^ (fb(a0) & 0x80000000u)); }

EXPORT float o_atan2(float a0, float a1)
{
    if (a0 != a0 || a1 != a1) return NAN;
    if (fabsf(a0) == INFINITY && fabsf(a1) == INFINITY) { a0 = copysignf(1.0f, a0); a1 = copysignf(1.0f, a1); }
    float z = atan_kernel(a0 / a1);
    z = (a1 > 0.0f) ? z : bf(0x40490fdbu) - z;
    z = z * ((fb(a0) & 0x80000000u) ? -1.0f : 1.0f);
    if (a0 == 0.0f) return (a1 < 0.0f) ? bf(0x40490fdbu) : 0.0f;
    return z;
}

EXPORT void o_atan2_f32(const float *x, const float *y, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = o_atan2(x[i], y[i]);
}

EXPORT void o_atan2_f64(const float *x, const float *y, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = atan2((double)x[i], (double)y[i]);
}

/* ---------------------------------------------------------------- pow ----
 * EXP/scalar/pow.hpp:28-36, EXP/scalar/pow_abs.hpp:31-84 and the float
 * kernel EXP/details/pow_kernel.hpp:43-125 (Cephes powf: a 2^(-i/16) table,
 * b log2|a| carried as multiples of 1/16 plus remainders), ldexp per
 * BSIMD/ieee/functions/scalar/ldexp.hpp:37-51, frexp per frexp.hpp:30-60. */
static const uint32_t POW_A[17] = {0x3f800000, 0x3f75257d, 0x3f6ac0c7, 0x3f60ccdf, 0x3f5744fd, 0x3f4e248c,
                                   0x3f45672a, 0x3f3d08a4, 0x3f3504f3, 0x3f2d583f, 0x3f25fed7, 0x3f1ef532,
                                   0x3f1837f0, 0x3f11c3d3, 0x3f0b95c2, 0x3f05aac3, 0x3f000000};
static const uint32_t POW_B[9] = {0x0, 0xb1c116de, 0xb254a58a, 0x318aa837, 0x324fe77a,
                                  0xb2ac9d5e, 0x32a31b71, 0xb1e0aba1, 0x0};
static const uint32_t POW1_P[4] = {0xbe2a61b2, 0x3e4d2fa3, 0xbe800015, 0x3eaaaaa3};
static const uint32_t POW2_P[4] = {0x3c1a49bc, 0x3d634d38, 0x3e75fde1, 0x3f317218};

static float reduc16(float x) { return 0.0625f * floorf(16.0f * x); }

static float nt2_ldexpf(float a, int e)
{
    float f = 1.0f;
    if (e < -126) { e -= -126; f = bf(0x00800000u); }
    int b = e == 128;
    f += (float)b;
    e -= b;
    e += 127;
    return a * bf((uint32_t)e << 23) * f;
}

static float pow_abs(float a0, float a1)
{
    float x = fabsf(a0);
    if (x == 1.0f) return x;
    if (x == 0.0f) return (float)(a1 == 0.0f);
    if (x == a1 && a1 == INFINITY) return INFINITY;
    if (x == INFINITY && a1 == -INFINITY) return 0.0f;
    if (a1 == INFINITY) return (x < 1.0f) ? 0.0f : INFINITY;
    if (a1 == -INFINITY) return (x > 1.0f) ? 0.0f : INFINITY;
    if (x == INFINITY) return (a1 < 0.0f) ? 0.0f : ((a1 == 0.0f) ? 1.0f : INFINITY);
    if (a0 != a0 || a1 != a1) return NAN;
    int e = 0, t = 0;
    uint32_t u = fb(x);
    if ((u & 0x7f800000u) == 0) { x *= 8388608.0f; u = fb(x); t = 23; }
    e = (int)((u & 0x7f800000u) >> 23) - 126 - t;
    x = bf((u & ~0x7f800000u) | 0x3f000000u);
    int i = 1;
    if (x <= bf(POW_A[9])) i = 9;
    if (x <= bf(POW_A[i + 4])) i += 4;
    if (x <= bf(POW_A[i + 2])) i += 2;
    if (x >= bf(POW_A[1])) i = -1;
    i += 1;
    float tmp = bf(POW_A[i]);
    x -= tmp;
    x -= bf(POW_B[i >> 1]);
    x /= tmp;
    float z = x * x;
    float w = z * x * horner(x, POW1_P, 4);
    w = -0.5f * z + w;
    w = bf(0x3ee2a8edu) * w + w;
    z = bf(0x3ee2a8edu) * x + w;
    z += x;
    w = (float)(-i) * 0.0625f + (float)e;
    float ya = reduc16(a1), yb = a1 - ya;
    float W = z * a1 + w * yb;
    float Wa = reduc16(W), Wb = W - Wa;
    W = w * ya + Wa;
    Wa = reduc16(W);
    float uu = W - Wa;
    W = Wb + uu;
    Wb = reduc16(W);
    w = 16.0f * (Wa + Wb);
    if (w > bf(0x44ffe000u)) return INFINITY;
    if (w < bf(0xc5160000u)) return 0.0f;
    e = (int)w;
    Wb = W - Wb;
    if (Wb > 0.0f) { ++e; Wb -= 0.0625f; }
    z = horner(Wb, POW2_P, 4) * Wb;
    i = e / 16 + (e >= 0);
    e = i * 16 - e;
    w = bf(POW_A[e]);
    z = w * z + w;
    return nt2_ldexpf(z, i);
}

static int flint(float x) { return (x - truncf(x)) == 0.0f; }

EXPORT float o_pow(float a0, float a1)
{
    int ltz = a0 < 0.0f;
    if (ltz && !flint(a1)) return NAN;
    float z = pow_abs(a0, a1);
    return (ltz && flint((a1 - 1.0f) * 0.5f)) ? -z : z;
}

EXPORT void o_pow_f32(const float *x, const float *y, float *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = o_pow(x[i], y[i]);
}

/* FP64 reference: libm pow on the float inputs */
EXPORT void o_pow_f64(const float *x, const float *y, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) out[i] = pow((double)x[i], (double)y[i]);
}

/* ------------------------------------------------------- trigonometry ----
 * NT2's float sin/cos/tan (TRIG/scalar/impl/trigo/trig_base.hpp:131-176,
 * regular style, big_ mode) and sinpi/cospi (pi_tag), every operation rounded:
 *   reduction cascade trig_reduction.hpp:76-251 --
 *     |x| <= pi/4 as is; <= pi/2 rem_pio2_straight.hpp:60-66; <= 20 pi
 *     rem_pio2_cephes.hpp:65-72; <= 2^6 pi rem_pio2_medium.hpp:68-84 in float;
 *     <= 2^18 pi the same in double (use_conversion, :235-244); beyond, fdlibm's
 *     __ieee754_rem_pio2f / __kernel_rem_pio2f (TRIG/scalar/rem_pio2.hpp).
 *   evaluation f_trig_evaluation.hpp:40-72; pi_tag reduction
 *   trig_reduction.hpp:303-317.
 * Beyond 2^18 pi this oracle reduces exactly (a 2/pi table and 128-bit integer
 * products) and rounds r once to float; NT2's fdlibm float kernel is taken to
 * give that same rounded r.  That band is checked against FP64 libm only. */
static const uint32_t TWOOPI[9] = {0u, 0xA2F9836Eu, 0x4E441529u, 0xFC2757D1u, 0xF534DDC0u,
                                   0xDB629599u, 0x3C439041u, 0xFE5163ABu, 0xDEBBC561u};

EXPORT uint32_t o_twoopi_word(int i) { return (i >= 0 && i < 9) ? TWOOPI[i] : 0u; }

/* x = m 2^e; x (2/pi) = sum_i b_i m 2^(e-i).  Bits b_i with i <= e-2 add
 * multiples of 4: start the 128-bit window at i = e-1 (table bit i+31). */
static int big_reduce(float x, float *xr)
{
    uint32_t u = fb(x);
    uint64_t m = (u & 0x7fffffu) | 0x800000u;
    int e = (int)(u >> 23) - 150;
    int j = e + 30;
    unsigned __int128 win = 0;
    for (int k = 0; k < 128; ++k) {  /* bit by bit: slow and plain */
        int bit = j + k, w = bit >> 5, o = 31 - (bit & 31);
        uint32_t word = (w >= 0 && w < 9) ? TWOOPI[w] : 0u;
        win = (win << 1) | ((word >> o) & 1u);
    }
    /* window bit k is b_(e-1+k) with weight 2^(1-k): x 2/pi = m * win * 2^-126
     * (mod 4), so the quadrant is bits 126..127 of the product and the fraction
     * its 126 bits below (wrap-around above bit 127 only drops multiples of 4) */
    unsigned __int128 plo = (unsigned __int128)m * (uint64_t)win + (((unsigned __int128)m * (uint64_t)(win >> 64)) << 64);
    int n = (int)(plo >> 126) & 3;
    unsigned __int128 frac = plo << 2;                                 /* fraction scaled by 2^128 */
    long double q;
    if (frac >> 127) { n = (n + 1) & 3; frac = ~frac + 1; q = -(long double)frac; }
    else q = (long double)frac;
    double qd = (double)(q * 0x1p-128L);
    *xr = (float)(qd * 1.5707963267948966);
    return n;
}

static double dmul(double a, double b) { volatile double r = a * b; return r; }
static double dsub(double a, double b) { volatile double r = a - b; return r; }

static int medium_f(float t, float *xr)
{
    float fn = rintf(t * bf(0x3f22f984u));
    float r = t - fn * bf(0x3fc90f80u), t2, w;
    t2 = r; w = fn * bf(0x37354400u); r = t2 - w; w = fn * bf(0x2e85a308u) - ((t2 - r) - w);
    t2 = r; w = fn * bf(0x2e85a300u); r = t2 - w; w = fn * bf(0x248d3132u) - ((t2 - r) - w);
    *xr = r - w;
    return (int)fn & 3;
}

static double bd(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }

static int medium_d(double t, float *xr)
{
    double fn = rint(dmul(t, bd(0x3FE45F306DC9C883ull)));
    double r = dsub(t, dmul(fn, bd(0x3FF921FB54400000ull))), t2, w;
    t2 = r; w = dmul(fn, bd(0x3DD0B4611A600000ull)); r = dsub(t2, w);
    w = dsub(dmul(fn, bd(0x3BA3198A2E037073ull)), dsub(dsub(t2, r), w));
    t2 = r; w = dmul(fn, bd(0x3BA3198A2E000000ull)); r = dsub(t2, w);
    w = dsub(dmul(fn, bd(0x397B839A252049C1ull)), dsub(dsub(t2, r), w));
    *xr = (float)dsub(r, w);
    return (int)(int64_t)fn & 3;
}

static int trig_reduce(float x, float *xr)
{
    if (!(x > bf(0x3f490fdbu))) { *xr = x; return 0; }
    if (!(x > bf(0x3fc90fdbu))) { *xr = ((x - bf(0x3fc90f80u)) - bf(0x37354400u)) - bf(0x2e85a300u); return 1; }
    if (!(x > bf(0x427b53d1u))) {
        float xi = rintf(x * bf(0x3f22f983u));
        float r = x - xi * bf(0x3fc90f80u);
        r = r - xi * bf(0x37354400u);
        *xr = r - xi * bf(0x2e85a300u);
        return (int)xi & 3;
    }
    if (!(x > bf(0x43490fdbu))) return medium_f(x, xr);
    if (!((double)x > bd(0x412921fb54442d18ull))) return medium_d((double)x, xr);
    return big_reduce(x, xr);
}

static int trig_reduce_pi(float x, float *xr)
{
    float xi = rintf(x * 2.0f);
    float x2 = x - xi * 0.5f;
    *xr = x2 * bf(0x40490fdbu);
    return (fabsf(xi) < 0x1p62f) ? (int)((int64_t)xi & 3) : 0;
}

static const uint32_t COS_P[3] = {0x37ccf5ce, 0xbab60619, 0x3d2aaaa5};
static const uint32_t SIN_P[3] = {0xb94ca1f9, 0x3c08839d, 0xbe2aaaa2};
static const uint32_t TAN_P[6] = {0x3c19c53b, 0x3b4c779c, 0x3cc821b5, 0x3d5ac5c9, 0x3e0896dd, 0x3eaaaa6f};

static float cos_eval(float z) { float y = horner(z, COS_P, 3); return 1.0f + (z * -0.5f + y * (z * z)); }
static float sin_eval(float z, float x) { float y1 = horner(z, SIN_P, 3); return (y1 * z) * x + x; }
static float tan_eval(float z) { float zz = z * z; return (horner(zz, TAN_P, 6) * zz) * z + z; }

static int invalid(float a) { return !(fabsf(a) < INFINITY); }

/* degree_tag (TRIG/scalar/impl/trigo/trig_reduction.hpp:254-266): k = round(x/90),
 * xr = (x - 90 k) * Deginrad; the quadrant k mod 4, 0 once k leaves int32 (x86's
 * conversion gives INT_MIN there) */
static int trig_reduce_deg(float x, float *xr)
{
    float xi = rintf(x * bf(0x3c360b61u));
    float x2 = x - xi * 90.0f;
    *xr = x2 * bf(0x3c8efa35u);
    return (fabsf(xi) < 2147483648.0f) ? ((int)xi & 3) : 0;
}

static int reduce_unit(float x, float *xr, int unit)
{
    return unit == 1 ? trig_reduce_pi(x, xr) : unit == 2 ? trig_reduce_deg(x, xr) : trig_reduce(x, xr);
}

static float cos_any(float a0, int pi)
{
    if (invalid(a0)) return NAN;
    float xr;
    int n = reduce_unit(fabsf(a0), &xr, pi);
    int swap = n & 1;
    float z = xr * xr;
    float v = swap ? sin_eval(z, xr) : cos_eval(z);
    return bf(fb(v) ^ ((uint32_t)(swap ^ ((n & 2) >> 1)) << 31));
}

static float sin_any(float a0, int pi)
{
    if (invalid(a0)) return NAN;
    float xr;
    int n = reduce_unit(fabsf(a0), &xr, pi);
    float z = xr * xr;
    float v = (n & 1) ? cos_eval(z) : sin_eval(z, xr);
    return bf(fb(v) ^ (fb(a0) & 0x80000000u) ^ ((uint32_t)(n & 2) << 30));
}

EXPORT float o_cos(float a0) { return cos_any(a0, 0); }
EXPORT float o_sin(float a0) { return sin_any(a0, 0); }
EXPORT float o_cospi(float a0) { return cos_any(a0, 1); }
EXPORT float o_sinpi(float a0) { return sin_any(a0, 1); }

/* NT2's is_flint (frac(x) == 0, false for +-inf and NaN) and is_odd(x) =
 * is_flint((x - 1)/2) (BSIMD/predicates/functions/scalar/is_odd.hpp:50,
 * is_even.hpp:50, is_flint.hpp:50) */
static int flintf(float x) { return (x - truncf(x)) == 0.0f; }
static int oddf(float x) { return flintf((x - 1.0f) * 0.5f); }

/* tan_invalid / cot_invalid per unit (trig_reduction.hpp:89-90, 268-269, 308-309) */
static int tan_invalid_u(float a0, int unit)
{
    if (unit == 1) return flintf(a0 - 0.5f);
    if (unit == 2) return flintf((a0 - 90.0f) * bf(0x3bb60b61u));
    return 0;
}
static int cot_invalid_u(float a0, int unit)
{
    if (unit == 1) return a0 != 0.0f && flintf(a0);
    if (unit == 2) return a0 != 0.0f && flintf(a0 * bf(0x3bb60b61u));
    return 0;
}

static float tan_any(float a0, int unit)
{
    if (invalid(a0)) return NAN;
    if (tan_invalid_u(a0, unit)) return NAN;
    if (a0 == 0.0f) return a0;
    float xr;
    int n = reduce_unit(fabsf(a0), &xr, unit);
    float y = tan_eval(xr);
    if (n & 1) y = -(1.0f / y);
    return bf(fb(y) ^ (fb(a0) & 0x80000000u));
}

EXPORT float o_tan(float a0) { return tan_any(a0, 0); }
EXPORT float o_tand(float a0) { return tan_any(a0, 2); }
EXPORT float o_sind(float a0) { return sin_any(a0, 2); }
EXPORT float o_cosd(float a0) { return cos_any(a0, 2); }
/* sec = rec(cos), csc = rec(sin) (TRIG/generic/sec.hpp, csc.hpp) */
EXPORT float o_sec(float a0) { return 1.0f / o_cos(a0); }
EXPORT float o_csc(float a0) { return 1.0f / o_sin(a0); }

/* cot, cotpi, cotd: TRIG/scalar/impl/trigo/trig_base.hpp:178-188 */
static float cot_any(float a0, int unit)
{
    if (invalid(a0) || cot_invalid_u(a0, unit)) return NAN;
    uint32_t bos = fb(a0) & 0x80000000u;
    if (a0 == 0.0f) return bf(0x7f800000u | bos);
    float xr;
    int n = reduce_unit(fabsf(a0), &xr, unit);
    float y = tan_eval(xr);
    y = (n & 1) ? -y : 1.0f / y;
    return bf(fb(y) ^ bos);
}
EXPORT float o_cot(float a0) { return cot_any(a0, 0); }
EXPORT float o_cotpi(float a0) { return cot_any(a0, 1); }
EXPORT float o_cotd(float a0) { return cot_any(a0, 2); }
EXPORT float o_tanpi(float a0) { return tan_any(a0, 1); }

/* mod boost/simd/arithmetic/functions/generic/mod.hpp:22-31 (float divfloor
 * scalar/divfloor.hpp:89-100 = floor(a/b)): b != 0 ? a - floor(a/b)*b : a;
 * rem scalar/rem.hpp:27-37 (idivfix generic/idivfix.hpp:38-49 = itrunc(a/b),
 * toints scalar/toints.hpp:36-46: NaN -> 0, saturating): b != 0 ? a - b*q : a */
EXPORT float o_mod(float a, float b) { return b != 0.0f ? a - floorf(a / b) * b : a; }
static int32_t o_toints(float v)
{
    if (v != v) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
EXPORT float o_rem(float a, float b) { return b != 0.0f ? a - b * (float)o_toints(a / b) : a; }

/* boost.simd's scalar float selects, minmod and negate:
 * ieee/functions/scalar/maxnum.hpp, minnum.hpp (is_nan(a) ? b : max/min(b, a),
 * max(x, y) = x > y ? x : y), maxmag.hpp, minmag.hpp (by magnitude, ties to
 * max/min), arithmetic/functions/scalar/minmod.hpp (is_nltz(a*b) ? min : 0),
 * ieee/functions/scalar/negate.hpp (a * sign(b)) */
EXPORT float o_sign(float a0);
static float o_max2(float x, float y) { return x > y ? x : y; }
static float o_min2(float x, float y) { return x < y ? x : y; }
EXPORT float o_maxnum(float a, float b) { return (a != a) ? b : o_max2(b, a); }
EXPORT float o_minnum(float a, float b) { return (a != a) ? b : o_min2(b, a); }
EXPORT float o_maxmag(float a, float b)
{
    float x = fabsf(a), y = fabsf(b);
    return x > y ? a : y > x ? b : o_max2(a, b);
}
EXPORT float o_minmag(float a, float b)
{
    float x = fabsf(a), y = fabsf(b);
    return x < y ? a : y < x ? b : o_min2(a, b);
}
EXPORT float o_minmod(float a, float b) { return !(a * b < 0.0f) ? o_min2(a, b) : 0.0f; }
EXPORT float o_negate(float a, float b) { return a * o_sign(b); }
/* divfloor, divceil, divfix, divround, divround2even for floats
 * (arithmetic/functions/scalar/div*.hpp): the rounding of a/b */
EXPORT float o_round2even(float a0);
EXPORT float o_divfloor(float a, float b) { return floorf(a / b); }
EXPORT float o_divceil(float a, float b) { return ceilf(a / b); }
EXPORT float o_divfix(float a, float b) { return truncf(a / b); }
EXPORT float o_divround(float a, float b) { return roundf(a / b); }
EXPORT float o_divround2even(float a, float b) { return o_round2even(a / b); }

/* pow2 EXP/generic/pow2.hpp:21-70: fast_ldexp(a, toint(b)) =
 * a * bits((n + 127) << 23) in wrapping int32 arithmetic
 * (boost/simd/ieee/functions/scalar/fast_ldexp.hpp:33-43); toint truncates,
 * INT_MIN outside int32 and for NaN (x86's conversion) */
EXPORT float o_pow2(float a, float b)
{
    int32_t n = (b >= -2147483648.0f && b < 2147483648.0f) ? (int32_t)b : INT32_MIN;
    return a * bf(((uint32_t)n + 127u) << 23);
}

/* proper_tanpi TRIG/scalar/proper_tanpi.hpp:25-36: NaN outside [-1/2, 1/2];
 * the fast-style tana of trig_base.hpp:236-242 (clipped_pio4_: the tangent
 * polynomial at |x| * Pi, no reduction) for |x| <= 1/4, else the reciprocal
 * of it at 1/2 - |x|, x's sign applied before the reciprocal */
EXPORT float o_proper_tanpi(float a0)
{
    if (a0 != a0) return a0;
    float ab = fabsf(a0);
    if (ab > 0.5f) return NAN;
    int test = ab <= 0.25f;
    ab = test ? ab : 0.5f - ab;
    float t = tan_eval(ab * bf(0x40490fdbu));
    t = a0 < 0.0f ? -t : t;
    return test ? t : 1.0f / t;
}
EXPORT void o_proper_tanpi_f32(const float *x, float *out, int64_t m)
{
    for (int64_t i = 0; i < m; ++i) out[i] = o_proper_tanpi(x[i]);
}

/* secpi TRIG/generic/secpi.hpp, cscpi TRIG/generic/cscpi.hpp, secd
 * TRIG/generic/secd.hpp, cscd TRIG/generic/cscd.hpp */
EXPORT float o_secpi(float a0) { float r = 1.0f / o_cospi(a0); return oddf(a0 * 2.0f) ? NAN : r; }
EXPORT float o_cscpi(float a0) { float r = 1.0f / o_sinpi(a0); return (flintf(a0) && a0 != 0.0f) ? NAN : r; }
EXPORT float o_secd(float a0) { float c = o_cosd(a0); return 1.0f / (c == 0.0f ? NAN : c); }
EXPORT float o_cscd(float a0) { return o_cscpi(bf(0x3bb60b61u) * a0); }

/* sinc TRIG/scalar/sinc.hpp, sincpi TRIG/scalar/sincpi.hpp (Eps = 2^-23) */
EXPORT float o_sinc(float a0)
{
    if (isinf(a0)) return 0.0f;
    return (fabsf(a0) < bf(0x34000000u)) ? 1.0f : o_sin(a0) / a0;
}
EXPORT float o_sincpi(float a0)
{
    if (isinf(a0)) return 0.0f;
    return (fabsf(a0) < bf(0x34000000u)) ? 1.0f : (bf(0x3ea2f983u) * o_sinpi(a0)) / a0;
}

/* indeg TRIG/generic/indeg.hpp (Radindeg, Radindegr), inrad TRIG/generic/inrad.hpp */
EXPORT float o_indeg(float a0) { return a0 * bf(0x42652ee1u) - a0 * bf(0xb53387c1u); }
EXPORT float o_inrad(float a0) { return a0 * bf(0x3c8efa35u); }

/* acotd TRIG/generic/acotd.hpp */
EXPORT float o_acotd(float a0)
{
    float z = 90.0f - (a0 != 0.0f ? o_indeg(o_atan(fabsf(a0))) : 0.0f);
    if (isinf(a0)) z = 0.0f;
    return bf(fb(z) | (fb(a0) & 0x80000000u));
}

/* acsc TRIG/generic/acsc.hpp; asec TRIG/scalar/asec.hpp (single_ overload) */
EXPORT float o_acsc(float a0) { return o_asin(1.0f / a0); }
EXPORT float o_asec(float a0)
{
    float ax = fabsf(a0);
    if (ax < 1.0f) return NAN;
    float ax1 = ax - 1.0f;
    if (ax1 < 0.001f) {
        float t = sqrtf(2.0f * ax1) * (1.0f - ax1 * ((5 / 12.0f) + ax1 * ((43 / 160.0f) - ax1 * ((177 / 896.0f)
                                                                           + ax1 * (2867 / 18432.0f)))));
        return (a0 < 0.0f) ? bf(0x40490fdbu) - t : t;
    }
    if (a0 == 1.0f) return 0.0f;
    return bf(0x3fc90fdbu) - o_acsc(a0);
}

/* the inverse functions in degrees and in multiples of pi, and acot
 * (TRIG/generic/{asind,acosd,atand,asecd,acscd,asinpi,acospi,atanpi,acot}.hpp) */
EXPORT float o_asind(float a0) { return o_indeg(o_asin(a0)); }
EXPORT float o_acosd(float a0) { return o_indeg(o_acos(a0)); }
EXPORT float o_atand(float a0) { return o_indeg(o_atan(a0)); }
EXPORT float o_asecd(float a0) { return o_indeg(o_asec(a0)); }
EXPORT float o_acscd(float a0) { return o_indeg(o_acsc(a0)); }
EXPORT float o_asinpi(float a0) { return bf(0x3ea2f983u) * o_asin(a0); }
EXPORT float o_acospi(float a0) { return bf(0x3ea2f983u) * o_acos(a0); }
EXPORT float o_atanpi(float a0) { return bf(0x3ea2f983u) * o_atan(a0); }
EXPORT float o_acot(float a0) { return o_atan(1.0f / a0); }
EXPORT float o_atan2d(float a0, float a1) { return o_indeg(o_atan2(a0, a1)); }

/* ------------------------------------------------------ gamma family ----
 * stirling EUL/scalar/stirling.hpp + EUL/details/stirling_kernel.hpp (float),
 * gamma EUL/scalar/gamma.hpp + EUL/details/gamma_kernel.hpp (float),
 * gammaln EUL/scalar/gammaln.hpp (single_) + EUL/details/gammaln_kernel.hpp. */
static const uint32_t STIRLING_P[4] = {0xb970b359, 0xbb2fb930, 0x3b638e39, 0x3daaaaab};
static const uint32_t GAMMA1_P[8] = {0x3ad28b22, 0x3ba90c99, 0x3b91db14, 0x3d93ae7c,
                                     0x3da82a34, 0x3ed2d411, 0x3ed87799, 0x3f800000};
static const uint32_t GAMMALNB_P[8] = {0x3a1ebb94, 0xbaabeab1, 0x3b3ba883, 0xbbf164fd,
                                       0x3ca89ed8, 0xbd89f07e, 0x3ea51a64, 0x3ed87730};
static const uint32_t GAMMALNC_P[8] = {0x3e0c3c4f, 0xbe22d329, 0x3e2d4dab, 0xbe53c04f,
                                       0x3e8a898b, 0xbecd27a8, 0x3f528d34, 0xbf13c468};
static const uint32_t GAMMALN2_P[3] = {0x3a31fd69, 0xbb358701, 0x3daaaa94};

EXPORT float o_stirling(float a0)
{
    if (isnan(a0)) return a0;
    if (a0 > bf(0x420c28f3u)) return INFINITY;  /* Stirlinglargelim */
    float w = 1.0f / a0;
    w = w * horner(w, STIRLING_P, 4) + 1.0f;
    float y = o_exp(-a0);
    if (y == 0.0f) return INFINITY;
    float z = a0 - 0.5f;
    if (a0 >= bf(0x41d628f6u)) {  /* Stirlingsplitlim */
        float v = o_pow(a0, z * 0.5f);
        y *= v;
        y *= v;
    } else {
        y *= o_pow(a0, z);
    }
    return y * (bf(0x40206c99u) * w);  /* Sqrt_2pi */
}

EXPORT float o_gamma(float a0)
{
    if (a0 == 0.0f) return copysignf(INFINITY, a0);
    if (isnan(a0) || a0 == -INFINITY) return NAN;
    if (a0 == INFINITY) return a0;
    float x = a0, q = fabsf(x);
    if (x < -33.0f) {
        float st = o_stirling(q);
        float p = floorf(q);
        if (p == q) return NAN;
        int iseven = (((int32_t)p) & 1) == 0;
        float z = q - p;
        if (z > 0.5f) {
            p += 1.0f;
            z = q - p;
        }
        z = q * o_sinpi(z);
        if (z == 0.0f) return NAN;
        st = bf(0x40490fdbu) / (fabsf(z) * st);
        return iseven ? -st : st;
    }
    /* NT2 counts x down one by one; its product is +inf long before x = 64
     * is reached (and from 2^24 on, x - 1 == x and the loop never ends) */
    if (x > 64.0f) return INFINITY;
    float z = 1.0f;
    while (x >= 3.0f) {
        x -= 1.0f;
        z *= x;
    }
    while (x < 0.0f) {
        z /= x;
        x += 1.0f;
    }
    while (x < 2.0f) {
        if (x == 0.0f) return NAN;
        z /= x;
        x += 1.0f;
    }
    if (x == 2.0f) return z;
    x -= 2.0f;
    return z * horner(x, GAMMA1_P, 8);
}

EXPORT float o_gammaln(float a0)
{
    if (a0 > bf(0x7bc3f8eau) || a0 == 0.0f) return INFINITY;  /* Maxgammaln */
    float x = a0, q = fabsf(x);
    if (x < 0.0f) {
        if (q > bf(0x7bc3f8eau)) return NAN;
        float w = o_gammaln(q);
        float p = floorf(q);
        if (p == q) return INFINITY;
        float z = q - p;
        if (z > 0.5f) {
            p += 1.0f;
            z = p - q;
        }
        z = q * o_sinpi(z);
        if (z == 0.0f) return INFINITY;
        return -o_log(bf(0x3ea2f983u) * fabsf(z)) - w;
    }
    if (x < 6.5f) {
        float z = 1.0f, tx = x, nx = 0.0f;
        if (x >= 1.5f) {
            while (tx > 2.5f) {
                nx = nx - 1.0f;
                tx = x + nx;
                z *= tx;
            }
            x += nx - 2.0f;
            return x * horner(x, GAMMALNB_P, 8) + o_log(z);
        }
        if (x >= 1.25f) {
            z *= x;
            x = x - 1.0f;
            return x * horner(x, GAMMALNB_P, 8) - o_log(z);
        }
        if (x >= 0.75f) {
            x = x - 1.0f;
            return x * horner(x, GAMMALNC_P, 8);
        }
        while (tx < 1.5f) {
            if (tx == 0.0f) return INFINITY;
            z *= tx;
            nx = nx + 1.0f;
            tx = x + nx;
        }
        x += nx - 2.0f;
        float p = x * horner(x, GAMMALNB_P, 8);
        return p - o_log(z);
    }
    float r = (x - 0.5f) * o_log(x) + (bf(0x3f6b3f8eu) - x);  /* Logsqrt2pi */
    if (x <= 1.0e4f) {
        float z = 1.0f / x;
        float p = z * z;
        r = z * horner(p, GAMMALN2_P, 3) + r;
    }
    return r;
}

/* signgam EUL/scalar/signgam.hpp (floating_): NaN at the non-positive
 * integers and -inf, 1 - 2 is_odd(floor(x)) below zero (boost.simd's float
 * is_odd(f) = is_even(f - 1) = is_flint((f - 1) * 1/2), is_flint(y) = frac(y) == 0),
 * NaN through, 1 above zero. */
EXPORT float o_signgam(float a0)
{
    if (a0 <= 0.0f) {
        if (a0 - truncf(a0) == 0.0f || a0 == -INFINITY) return NAN;
        float h = (floorf(a0) - 1.0f) * 0.5f;
        return (h - truncf(h) == 0.0f) ? -1.0f : 1.0f;
    }
    return isnan(a0) ? a0 : 1.0f;
}

/* digamma EUL/scalar/digamma.hpp: the float overload returns the double
 * algorithm rounded (double_ overload), which reflects below zero
 * (pi / tanpi of the fractional part of 1 - x), uses digamma_imp_large from
 * Digammalargelim = 20 on, else reduces to [1, 2] and evaluates digamma_1_2
 * (EUL/details/digamma_kernel.hpp, double coefficients by bit pattern).  The
 * double log and tanpi are libm's (NT2's own double versions differ from
 * them by an ulp of double at most). */
static double horner_bd(double x, const uint64_t *c, int n)
{
    double acc = bd(c[0]);
    for (int i = 1; i < n; ++i) acc = x * acc + bd(c[i]);
    return acc;
}
EXPORT double o_digamma_d(double a0)
{
    static const uint64_t LARGE[8] = {0xbfdc5e5e5e5e5e5eull, 0x3fb5555555555555ull, 0xbf95995995995996ull,
                                      0x3f7f07c1f07c1f08ull, 0xbf71111111111111ull, 0x3f70410410410410ull,
                                      0xbf81111111111111ull, 0x3fb5555555555555ull};
    static const uint64_t P6[6] = {0xbf60f7e5f66c2537ull, 0xbfa72b2e63723c78ull, 0xbfd2821c13c5e2bfull,
                                   0xbfe4cf68d26e295aull, 0xbfd4d5d0f9ab412full, 0x3fd04e9e69894978ull};
    static const uint64_t Q7[7] = {0xbea2b84f95bbf448ull, 0x3f616fc90a0a1908ull, 0x3fabb9c8cc612ca3ull,
                                   0x3fdbe65d28de361cull, 0x3ff75eb79397c930ull, 0x40009d1b06674d41ull,
                                   0x3ff0000000000000ull};
    const double pi = bd(0x400921fb54442d18ull);
    double result = 0.0, x = a0;
    if (a0 == 0.0) return copysign(INFINITY, a0);
    if (x < 0.0) {
        x = 1.0 - x;
        result = x - floor(x);
        if (result > 0.5) result -= 1.0;
        if (result == 0.5) result = 0.0;
        else if (result != 0.0) result = pi / (sin(pi * result) / cos(pi * result));
        else result = NAN;
    }
    if (x >= 20.0) {
        double xm = x - 1.0, r = log(xm);
        r += 1.0 / (2.0 * xm);
        double z = 1.0 / (xm * xm);
        r -= z * horner_bd(z, LARGE, 8);
        return r + result;
    }
    while (x > 2.0) {
        x -= 1.0;
        result += 1.0 / x;
    }
    if (x < 1.0) {
        result = -1.0 / x;
        x += 1.0;
    }
    const double Y = (double)0.99558162689208984f;
    const double root1 = 1569415565.0 / 1073741824.0, root2 = (381566830.0 / 1073741824.0) / 1073741824.0,
                 root3 = 0.9016312093258695918615325266959189453125e-19;
    double g = x - root1;
    g -= root2;
    g -= root3;
    double xm = x - 1.0;
    double r = horner_bd(xm, P6, 6) / horner_bd(xm, Q7, 7);
    return (g * Y + g * r) + result;
}
EXPORT float o_digamma(float a0) { return (float)o_digamma_d((double)a0); }

/* beta EUL/scalar/beta.hpp: sign*exp(gammaln(a0)+gammaln(a1)-gammaln(y)),
 * y = a0+a1, sign = signgam(a0)*signgam(a1)*signgam(y); betaln
 * EUL/simd/common/betaln.hpp: gammaln(a0)+gammaln(a1)-gammaln(a0+a1). */
EXPORT float o_beta(float a0, float a1)
{
    float y = a0 + a1;
    float sign = o_signgam(a0) * o_signgam(a1) * o_signgam(y);
    return sign * o_exp(o_gammaln(a0) + o_gammaln(a1) - o_gammaln(y));
}
EXPORT float o_betaln(float a0, float a1) { return o_gammaln(a0) + o_gammaln(a1) - o_gammaln(a0 + a1); }

/* dawson EUL/scalar/dawson.hpp:27-55 with the float rational approximations
 * of EUL/details/dawson_kernel.hpp:22-107 (NT2_HORNER_RAT = horner(P)/horner(Q),
 * POLY/scalar/impl/horner.hpp:107-110). */
static const uint32_t DAW1_P[10] = {0x2d47fd98, 0x30697185, 0x32a70489, 0x357fdc17, 0x364e9480,
                                    0x39b8d18b, 0xba5edc97, 0x3d2d1abc, 0xbdbbe665, 0x3f800000};
static const uint32_t DAW1_Q[11] = {0x2dd36efb, 0x30cc991a, 0x335fe1b9, 0x35aacdae, 0x37c306e7, 0x39aaab31,
                                    0x3b6497e8, 0x3ce4ec9b, 0x3e22afee, 0x3f132dde, 0x3f800000};
static const uint32_t DAW2_N[11] = {0x3f024ae3, 0xbe7aa0e7, 0x3dc0d25d, 0xbcb32b13, 0x3b6fff71, 0xb9dde22a,
                                    0x3816d831, 0xb6100aef, 0x33c36c5f, 0xb1251d8a, 0x2e1dfe15};
static const uint32_t DAW2_D[11] = {0x3f800000, 0xbf21c042, 0x3e726344, 0xbd59d3f0, 0x3c0af173, 0xba7882fc,
                                    0x38a3cafe, 0xb698f761, 0x344b0b83, 0xb1a8d160, 0x2e9dfe10};
static const uint32_t DAW3_N[5] = {0xbf173118, 0x3f211590, 0xbe3101f1, 0x3c8708d6, 0xb9ff3ce5};
static const uint32_t DAW3_D[6] = {0x3f800000, 0xc02caf51, 0x3fddc960, 0xbec9942c, 0x3d0d0443, 0xba7f3ce5};

EXPORT float o_dawson(float a0)
{
    float x = fabsf(a0), xx = x * x;
    if (x < 3.25f) return a0 * (horner(xx, DAW1_P, 10) / horner(xx, DAW1_Q, 11));
    xx = 1.0f / xx;
    if (x < 6.25f) {
        float y = 1.0f / x + xx * horner(xx, DAW2_N, 11) / (horner(xx, DAW2_D, 11) * x);
        return copysignf(0.5f * y, a0);
    }
    if (x > 1.0e9f) return 0.5f * copysignf(1.0f / x, a0);
    float y = 1.0f / x + xx * horner(xx, DAW3_N, 5) / (horner(xx, DAW3_D, 6) * x);
    return copysignf(0.5f * y, a0);
}

/* spence EUL/scalar/spence.hpp:27-70 (Cephes spencef, the float coefficients
 * by bit pattern; Pi2o_6 = 0x3fd28d33). */
static const uint32_t SPENCE_P[11] = {0x3c80e79e, 0xbc8a8ad6, 0x3c1f4a7f, 0xbc604c2f, 0x3caa7af5, 0xbce56409,
                                      0x3d23ba15, 0xbd7ff525, 0x3de38e97, 0xbe800004, 0x3f800000};
EXPORT float o_spence(float a0)
{
    float x = a0;
    const float pi2o6 = bf(0x3fd28d33u);
    if (x < 0.0f) return NAN;
    if (x == 1.0f) return 0.0f;
    if (x == 0.0f) return pi2o6;
    int flag = 0;
    if (x > 2.0f) {
        x = 1.0f / x;
        flag |= 2;
    }
    float w;
    if (x > 1.5f) {
        w = 1.0f / x - 1.0f;
        flag |= 2;
    } else if (x < 0.5f) {
        w = -x;
        flag |= 1;
    } else {
        w = x - 1.0f;
    }
    float y = -w * horner(w, SPENCE_P, 11);
    if (flag & 1) y = pi2o6 - o_log(x) * o_log(1.0f - x) - y;
    if (flag & 2) {
        float z = o_log(x);
        y = -0.5f * (z * z) - y;
    }
    return y;
}

/* An integer operand carried in a float: truncated toward zero, saturated
 * to int32, NaN as 0 (the library's convention for nthroot's and expni's n). */
static int32_t int_operand(float b)
{
    if (isnan(b)) return 0;
    if (b >= 2147483648.0f) return INT32_MAX;
    if (b <= -2147483648.0f) return INT32_MIN;
    return (int32_t)b;
}

/* pow(float, int) EXP/generic/pow.hpp:111-140: binary powering of |n|, the
 * base squared after each bit; the reciprocal for n < 0. */
static float powi(float a0, int32_t n)
{
    uint32_t e = n < 0 ? 0u - (uint32_t)n : (uint32_t)n;
    float base = a0, r = 1.0f;
    for (; e; e >>= 1) {
        if (e & 1u) r *= base;
        base = base * base;
    }
    return n < 0 ? 1.0f / r : r;
}

EXPORT float o_sign(float a0);

/* nthroot EXP/scalar/nthroot.hpp:29-49 */
EXPORT float o_nthroot(float a0, int32_t n)
{
    int ltz = a0 < 0.0f, odd = (n % 2) != 0;
    if (ltz && !odd) return NAN;
    float x = fabsf(a0);
    if (x == 1.0f) return a0;
    if (n == 0) return (x < 1.0f) ? 0.0f : o_sign(a0) * INFINITY;
    if (a0 == 0.0f) return 0.0f;
    if (isinf(a0)) return a0;
    float an = (float)n;
    float y = o_pow(x, 1.0f / an);
    if (y != 0.0f) y -= (powi(y, n) - x) / (an * powi(y, n - 1));
    return (ltz && odd) ? -y : y;
}

/* expni EUL/scalar/expni.hpp:37-127 (Cephes expn in float).  NT2's two
 * loops end when the relative change reaches Halfeps = 2^-24; like the
 * library, this stops them after 10000 terms as well. */
EXPORT float o_expni(int32_t n, float x)
{
    const float halfeps = bf(0x33800000u), big = bf(0x4b800000u), euler = bf(0x3f13c468u);
    if (n < 0 || x < 0.0f) return NAN;
    if (x > bf(C_MAXLOG)) return 0.0f;
    if (x == 0.0f) return (n < 2) ? INFINITY : 1.0f / ((float)n - 1.0f);
    if (n == 0) return o_exp(-x) / x;
    if (n > 5000) {
        float xk = x + (float)n, yk = 1.0f / (xk * xk), t = (float)n;
        float ans = yk * t * (6.0f * (x * x) - 8.0f * t * x + t * t);
        ans = yk * (ans + t * (t - 2.0f * x));
        ans = yk * (ans + t);
        return (1.0f + ans) * o_exp(-x) / xk;
    }
    if (x <= 1.0f) {
        float psi = -euler - o_log(x);
        for (int32_t i = n - 1; i; --i) psi += 1.0f / (float)i;
        float z = -x, xk = 0.0f, yk = 1.0f, pk = 1.0f - (float)n, t;
        float ans = (n == 1) ? 0.0f : 1.0f / pk;
        int it = 0;
        do {
            xk += 1.0f;
            yk *= z / xk;
            pk += 1.0f;
            if (pk != 0.0f) ans += yk / pk;
            t = (ans != 0.0f) ? fabsf(yk / ans) : 1.0f;
        } while (t > halfeps && ++it < 10000);
        return (o_pow(z, (float)(n - 1)) * psi / o_gamma((float)n)) - ans;
    }
    int32_t k = 1;
    float t, pkm2 = 1.0f, qkm2 = x, pkm1 = 1.0f, qkm1 = x + (float)n;
    float ans = pkm1 / qkm1;
    int it = 0;
    do {
        int odd = (++k) % 2 != 0;
        float yk = odd ? 1.0f : x;
        float xk = odd ? (float)(n + (k - 1) / 2) : (float)(k / 2);
        float pk = pkm1 * yk + pkm2 * xk;
        float qk = qkm1 * yk + qkm2 * xk;
        if (qk != 0.0f) {
            float r = pk / qk;
            t = fabsf((ans - r) / r);
            ans = r;
        } else {
            t = 1.0f;
        }
        pkm2 = pkm1;
        pkm1 = pk;
        qkm2 = qkm1;
        qkm1 = qk;
        if (fabsf(pk) > big) {
            pkm2 *= halfeps;
            pkm1 *= halfeps;
            qkm2 *= halfeps;
            qkm1 *= halfeps;
        }
    } while (t > halfeps && ++it < 10000);
    return ans * o_exp(-x);
}

EXPORT void o_nthroot_f32(const float *x, const float *n, float *out, int64_t m)
{
    for (int64_t i = 0; i < m; ++i) out[i] = o_nthroot(x[i], int_operand(n[i]));
}
EXPORT void o_expni_f32(const float *n, const float *x, float *out, int64_t m)
{
    for (int64_t i = 0; i < m; ++i) out[i] = o_expni(int_operand(n[i]), x[i]);
}

/* erfinv EUL/scalar/erfinv.hpp, erfcinv EUL/scalar/erfcinv.hpp (single_, Giles),
 * kernels EUL/details/erfinv_kernel.hpp */
static const uint32_t ERFINV1_P[9] = {0x32f16588, 0x34b84b36, 0xb66c7357, 0xb6935ac1, 0x396532db,
                                      0xbaa45408, 0xbb88e4ef, 0x3e7c8f63, 0x3fc02e2f};
static const uint32_t ERFINV2_P[9] = {0xb951f09b, 0x38d3b56b, 0x3ab0dc72, 0xbb70bde7, 0x3bbc127b,
                                      0xbbf9c5d7, 0x3c1aa57e, 0x3f8036db, 0x40354f7e};
static const uint32_t ERFCINV2_P[5] = {0x3b3a8aee, 0x3ba62c57, 0xbc8bcf63, 0x3c98e17c, 0xbbaf8bfe};
static const uint32_t ERFCINV2_Q[5] = {0x321631b2, 0x3b3a73c1, 0x3ba9025f, 0xbc5d80aa, 0x3c2f4022};

EXPORT float o_erfinv(float a0)
{
    float w = -o_log((1.0f - a0) * (a0 + 1.0f));
    if (w == INFINITY) return copysignf(1.0f, a0) * w;
    if (w < 5.0f) return a0 * horner(w - 2.5f, ERFINV1_P, 9);
    return a0 * horner(sqrtf(w) - 3.0f, ERFINV2_P, 9);
}
EXPORT float o_erfcinv(float a0)
{
    float a00 = 1.0f - a0;
    float w = -o_log(a0 * (2.0f - a0));
    if (w == INFINITY) return copysignf(1.0f, a00) * w;
    if (w < 5.0f) return a00 * horner(w - 2.5f, ERFINV1_P, 9);
    w = sqrtf(w);
    return copysignf(horner(w, ERFCINV2_P, 5) / horner(w, ERFCINV2_Q, 5), a00);
}

/* exprecneg, exprecnegc EXP/generic/{exprecneg,exprecnegc}.hpp; sqrt1pm1
 * EXP/generic/sqrt1pm1.hpp (compositions the front ends build as programs) */
EXPORT float o_exprecneg(float a0) { return o_exp(-(1.0f / a0)); }
EXPORT float o_exprecnegc(float a0) { return -o_expm1(-(1.0f / a0)); }
EXPORT float o_sqrt1pm1(float a0)
{
    float t = sqrtf(1.0f + a0);
    return (fabsf(a0) < 0.5f) ? a0 / (1.0f + t) : t - 1.0f;
}

/* rounding and sign: BSIMD/arithmetic/functions/scalar/{floor,ceil,round,round2even,trunc}.hpp,
 * BSIMD/ieee/functions/scalar/{frac,sign,signnz,copysign}.hpp; oneplus, oneminus, minusone, sqr_abs,
 * dist, average: BSIMD/arithmetic/functions/{generic,scalar}/ */
EXPORT float o_floor(float a0) { return floorf(a0); }
EXPORT float o_ceil(float a0) { return ceilf(a0); }
EXPORT float o_trunc(float a0) { return truncf(a0); }
EXPORT float o_fix(float a0) { return truncf(a0); }
EXPORT float o_round(float a0) { return roundf(a0); }
EXPORT float o_round2even(float a0)
{
    float v = fabsf(a0), t2n = 8388608.0f;
    float d = (v + t2n) - t2n;
    d = (v < t2n) ? d : v;
    return (a0 < 0.0f) ? -d : d;
}
EXPORT float o_frac(float a0) { return a0 - truncf(a0); }
EXPORT float o_sign(float a0) { return isnan(a0) ? a0 : (float)(a0 > 0.0f) - (float)(a0 < 0.0f); }
EXPORT float o_signnz(float a0) { return isnan(a0) ? a0 : bf(0x3f800000u | (fb(a0) & 0x80000000u)); }
EXPORT float o_oneplus(float a0) { return a0 + 1.0f; }
EXPORT float o_oneminus(float a0) { return 1.0f - a0; }
EXPORT float o_minusone(float a0) { return a0 - 1.0f; }
EXPORT float o_sqr_abs(float a0) { return a0 * a0; }
EXPORT float o_copysign(float a0, float a1) { return copysignf(a0, a1); }
EXPORT float o_dist(float a0, float a1) { return fabsf(a0 - a1); }
EXPORT float o_average(float a0, float a1) { return a0 * 0.5f + a1 * 0.5f; }

/* realsqrt, reallog: EXP/generic/{realsqrt,reallog}.hpp (sqrt and log behind an assertion) */
EXPORT float o_realsqrt(float a0) { return sqrtf(a0); }
EXPORT float o_reallog(float a0) { return o_log(a0); }

/* logspace_add, logspace_sub EXP/scalar/{logspace_add,logspace_sub}.hpp;
 * NT2's max(a, b) is a > b ? a : b */
EXPORT float o_logspace_add(float a0, float a1)
{
    float t = -fabsf(a0 - a1);
    float r = (a0 > a1 ? a0 : a1) + o_log1p(o_exp(t));
    return isnan(t) ? a0 + a1 : r;
}
EXPORT float o_logspace_sub(float a0, float a1)
{
    float x = a1 - a0;
    float t = (x > -bf(0x3f317218u)) ? o_log(-o_expm1(x)) : o_log1p(-o_exp(x));
    return a0 + t;
}

/* ------------------------------------------------- elementwise maps ---- */
enum { FN_EXP = 0, FN_LOG, FN_LOG1P, FN_ERFC, FN_NORMCDF, FN_FASTNORMCDF, FN_SQRT, FN_EXP2 = 8, FN_EXP10,
       FN_EXPM1, FN_LOG2, FN_LOG10, FN_SIN, FN_COS, FN_TAN, FN_SINPI, FN_COSPI, FN_SINH, FN_COSH, FN_TANH,
       FN_ASIN, FN_ACOS, FN_ATAN, FN_ASINH, FN_ACOSH, FN_ATANH, FN_CBRT, FN_COT, FN_SEC, FN_CSC, FN_SIND,
       FN_COSD, FN_TAND, FN_TANPI, FN_COTPI, FN_COTD, FN_SECPI, FN_CSCPI, FN_SECD, FN_CSCD, FN_SINC, FN_SINCPI,
       FN_ACOTD, FN_ASEC, FN_COTH, FN_SINHC, FN_ACSC, FN_ASECH, FN_ACOTH, FN_ACSCH,
       FN_ERF = 64, FN_ERFCX, FN_EXPX2, FN_GAMMA, FN_GAMMALN, FN_ERFINV, FN_ERFCINV, FN_DIGAMMA, FN_SIGNGAM, FN_DAWSON, FN_SPENCE, FN_STIRLING,
       FN_EXPRECNEG = 80, FN_EXPRECNEGC,
       FN_SQRT1PM1,
       /* compositions of the above, oracle only (the front ends lower them to programs) */
       FN_SECH = 51, FN_CSCH, FN_ACOT, FN_ASIND, FN_ACOSD, FN_ATAND, FN_ASECD, FN_ACSCD, FN_ASINPI, FN_ACOSPI,
       FN_ATANPI, FN_INDEG, FN_INRAD };

EXPORT void o_map_f32(int fn, const float *x, float *y, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) {
        float a = x[i];
        switch (fn) {
        case FN_EXP: y[i] = o_exp(a); break;
        case FN_LOG: y[i] = o_log(a); break;
        case FN_LOG1P: y[i] = o_log1p(a); break;
        case FN_ERFC: y[i] = o_erfc(a); break;
        case FN_NORMCDF: y[i] = o_normcdf(a); break;
        case FN_FASTNORMCDF: y[i] = o_fastnormcdf(a); break;
        case FN_EXP2: y[i] = o_exp2(a); break;
        case FN_EXP10: y[i] = o_exp10(a); break;
        case FN_EXPM1: y[i] = o_expm1(a); break;
        case FN_LOG2: y[i] = o_log2(a); break;
        case FN_LOG10: y[i] = o_log10(a); break;
        case FN_SIN: y[i] = o_sin(a); break;
        case FN_COS: y[i] = o_cos(a); break;
        case FN_TAN: y[i] = o_tan(a); break;
        case FN_SINPI: y[i] = o_sinpi(a); break;
        case FN_COSPI: y[i] = o_cospi(a); break;
        case FN_SINH: y[i] = o_sinh(a); break;
        case FN_COSH: y[i] = o_cosh(a); break;
        case FN_TANH: y[i] = o_tanh(a); break;
        case FN_ASIN: y[i] = o_asin(a); break;
        case FN_ACOS: y[i] = o_acos(a); break;
        case FN_ATAN: y[i] = o_atan(a); break;
        case FN_ASINH: y[i] = o_asinh(a); break;
        case FN_ACOSH: y[i] = o_acosh(a); break;
        case FN_ATANH: y[i] = o_atanh(a); break;
        case FN_CBRT: y[i] = o_cbrt(a); break;
        case FN_COT: y[i] = o_cot(a); break;
        case FN_SEC: y[i] = o_sec(a); break;
        case FN_CSC: y[i] = o_csc(a); break;
        case FN_SIND: y[i] = o_sind(a); break;
        case FN_COSD: y[i] = o_cosd(a); break;
        case FN_TAND: y[i] = o_tand(a); break;
        case FN_TANPI: y[i] = o_tanpi(a); break;
        case FN_COTPI: y[i] = o_cotpi(a); break;
        case FN_COTD: y[i] = o_cotd(a); break;
        case FN_SECPI: y[i] = o_secpi(a); break;
        case FN_CSCPI: y[i] = o_cscpi(a); break;
        case FN_SECD: y[i] = o_secd(a); break;
        case FN_CSCD: y[i] = o_cscd(a); break;
        case FN_SINC: y[i] = o_sinc(a); break;
        case FN_SINCPI: y[i] = o_sincpi(a); break;
        case FN_ACOTD: y[i] = o_acotd(a); break;
        case FN_ASEC: y[i] = o_asec(a); break;
        case FN_COTH: y[i] = o_coth(a); break;
        case FN_SINHC: y[i] = o_sinhc(a); break;
        case FN_SECH: y[i] = o_sech(a); break;
        case FN_CSCH: y[i] = o_csch(a); break;
        case FN_ASECH: y[i] = o_asech(a); break;
        case FN_ACSCH: y[i] = o_acsch(a); break;
        case FN_ACOTH: y[i] = o_acoth(a); break;
        case FN_ACOT: y[i] = o_acot(a); break;
        case FN_ACSC: y[i] = o_acsc(a); break;
        case FN_ASIND: y[i] = o_asind(a); break;
        case FN_ACOSD: y[i] = o_acosd(a); break;
        case FN_ATAND: y[i] = o_atand(a); break;
        case FN_ASECD: y[i] = o_asecd(a); break;
        case FN_ACSCD: y[i] = o_acscd(a); break;
        case FN_ASINPI: y[i] = o_asinpi(a); break;
        case FN_ACOSPI: y[i] = o_acospi(a); break;
        case FN_ATANPI: y[i] = o_atanpi(a); break;
        case FN_INDEG: y[i] = o_indeg(a); break;
        case FN_INRAD: y[i] = o_inrad(a); break;
        case FN_ERF: y[i] = o_erf(a); break;
        case FN_ERFCX: y[i] = o_erfcx(a); break;
        case FN_EXPX2: y[i] = o_expx2(a); break;
        case FN_GAMMA: y[i] = o_gamma(a); break;
        case FN_GAMMALN: y[i] = o_gammaln(a); break;
        case FN_DIGAMMA: y[i] = o_digamma(a); break;
        case FN_SIGNGAM: y[i] = o_signgam(a); break;
        case FN_DAWSON: y[i] = o_dawson(a); break;
        case FN_SPENCE: y[i] = o_spence(a); break;
        case FN_STIRLING: y[i] = o_stirling(a); break;
        case FN_ERFINV: y[i] = o_erfinv(a); break;
        case FN_ERFCINV: y[i] = o_erfcinv(a); break;
        case FN_EXPRECNEG: y[i] = o_exprecneg(a); break;
        case FN_EXPRECNEGC: y[i] = o_exprecnegc(a); break;
        case FN_SQRT1PM1: y[i] = o_sqrt1pm1(a); break;
        default: y[i] = sqrtf(a); break;
        }
    }
}

/* sin(pi a), cos(pi a) in FP64 for a float a: a mod 2 is exact in double
 * (fmod), then |r| <= 1/2 keeps the product pi r within an ulp. */
static double sinpi_d(double a)
{
    double r = fmod(a, 2.0);           /* exact, sign of a */
    if (r > 1.0) r -= 2.0; else if (r < -1.0) r += 2.0;
    if (r > 0.5) return sin(M_PI * (1.0 - r));
    if (r < -0.5) return -sin(M_PI * (1.0 + r));
    return sin(M_PI * r);
}
static double cospi_d(double a)
{
    double r = fabs(fmod(a, 2.0));
    if (r > 1.0) r = 2.0 - r;          /* [0, 1] */
    if (r > 0.5) return -sin(M_PI * (r - 0.5));
    return sin(M_PI * (0.5 - r));
}

/* sin and cos of a float angle in degrees: a mod 360 is exact in double */
static double sind_d(double a)
{
    double r = fmod(a, 360.0);
    if (r == 0.0 || fabs(r) == 180.0) return copysign(0.0, a);
    return sin(r * (M_PI / 180.0));
}
static double cosd_d(double a)
{
    double r = fabs(fmod(a, 360.0));
    if (r == 90.0 || r == 270.0) return 0.0;
    return cos(r * (M_PI / 180.0));
}

/* exp(x^2) erfc(x): the product below 2, the continued fraction of erfc above
 * (A&S 7.1.14: exp(x^2) erfc(x) = (1/sqrt(pi)) 1/(x + 1/2/(x + 1/(x + 3/2/(x + ...))))) */
static double erfcx_d(double a)
{
    if (a < 2.0) return exp(a * a) * erfc(a);
    double f = a;
    for (int k = 200; k >= 1; --k) f = a + (k * 0.5) / f;
    return 1.0 / (f * sqrt(M_PI));
}
/* inverse error functions by Newton's method on erf / erfc in FP64 from a
 * bracket-free start (the float algorithm's own result, refined) */
static double erfinv_d(double y)
{
    if (!(fabs(y) <= 1.0)) return NAN;
    if (fabs(y) == 1.0) return copysign(INFINITY, y);
    double x = (double)o_erfinv((float)y);
    if (!isfinite(x)) x = copysign(4.0, y);
    for (int k = 0; k < 6; ++k) x -= (erf(x) - y) / (1.1283791670955126 * exp(-x * x));
    return x;
}
static double erfcinv_d(double y)
{
    if (!(y >= 0.0 && y <= 2.0)) return NAN;
    if (y == 0.0) return INFINITY;
    if (y == 2.0) return -INFINITY;
    double x = (double)o_erfcinv((float)y);
    if (!isfinite(x)) x = y < 1.0 ? 10.0 : -4.0;
    for (int k = 0; k < 8; ++k) x += (erfc(x) - y) / (1.1283791670955126 * exp(-x * x));
    return x;
}
/* sqrt(1 + x) - 1 without cancellation */
static double sqrt1pm1_d(double a) { return a / (1.0 + sqrt(1.0 + a)); }

/* acot in degrees: 90 - atan|x| in degrees with x's sign (+-90 at +-0) */
static double acotd_d(double a)
{
    if (isinf(a)) return copysign(0.0, a);
    double t = fabs(a) >= 1.0 ? atan(1.0 / fabs(a)) * (180.0 / M_PI) : 90.0 - atan(fabs(a)) * (180.0 / M_PI);
    return copysign(t, a);
}

/* FP64 reference of the same functions on float inputs (glibc double libm). */
EXPORT void o_map_f64(int fn, const float *x, double *y, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) {
        double a = (double)x[i];
        switch (fn) {
        case FN_EXP: y[i] = exp(a); break;
        case FN_LOG: y[i] = log(a); break;
        case FN_LOG1P: y[i] = log1p(a); break;
        case FN_ERFC: y[i] = erfc(a); break;
        case FN_NORMCDF:
        case FN_FASTNORMCDF: y[i] = 0.5 * erfc(-a / sqrt(2.0)); break;
        case FN_EXP2: y[i] = exp2(a); break;
        case FN_EXP10: y[i] = pow(10.0, a); break;
        case FN_EXPM1: y[i] = expm1(a); break;
        case FN_LOG2: y[i] = log2(a); break;
        case FN_LOG10: y[i] = log10(a); break;
        case FN_SIN: y[i] = sin(a); break;
        case FN_COS: y[i] = cos(a); break;
        case FN_TAN: y[i] = tan(a); break;
        case FN_SINPI: y[i] = sinpi_d(a); break;
        case FN_COSPI: y[i] = cospi_d(a); break;
        case FN_SINH: y[i] = sinh(a); break;
        case FN_COSH: y[i] = cosh(a); break;
        case FN_TANH: y[i] = tanh(a); break;
        case FN_ASIN: y[i] = asin(a); break;
        case FN_ACOS: y[i] = acos(a); break;
        case FN_ATAN: y[i] = atan(a); break;
        case FN_ASINH: y[i] = asinh(a); break;
        case FN_ACOSH: y[i] = acosh(a); break;
        case FN_ATANH: y[i] = atanh(a); break;
        case FN_CBRT: y[i] = cbrt(a); break;
        case FN_COT: y[i] = cos(a) / sin(a); break;
        case FN_SEC: y[i] = 1.0 / cos(a); break;
        case FN_CSC: y[i] = 1.0 / sin(a); break;
        case FN_SIND: y[i] = sind_d(a); break;
        case FN_COSD: y[i] = cosd_d(a); break;
        case FN_TAND: y[i] = sind_d(a) / cosd_d(a); break;
        case FN_TANPI: y[i] = sinpi_d(a) / cospi_d(a); break;
        case FN_COTPI: y[i] = cospi_d(a) / sinpi_d(a); break;
        case FN_COTD: y[i] = cosd_d(a) / sind_d(a); break;
        case FN_SECPI: y[i] = 1.0 / cospi_d(a); break;
        case FN_CSCPI: y[i] = 1.0 / sinpi_d(a); break;
        case FN_SECD: y[i] = 1.0 / cosd_d(a); break;
        case FN_CSCD: y[i] = 1.0 / sind_d(a); break;
        case FN_SINC: y[i] = a == 0.0 ? 1.0 : isinf(a) ? 0.0 : sin(a) / a; break;
        case FN_SINCPI: y[i] = a == 0.0 ? 1.0 : isinf(a) ? 0.0 : sinpi_d(a) / (M_PI * a); break;
        case FN_ACOTD: y[i] = acotd_d(a); break;
        case FN_ASEC: y[i] = fabs(a) < 1.0 ? NAN : acos(1.0 / a); break;
        case FN_COTH: y[i] = 1.0 / tanh(a); break;
        case FN_SINHC: y[i] = a == 0.0 ? 1.0 : isinf(a) ? INFINITY : sinh(a) / a; break;
        case FN_SECH: y[i] = 1.0 / cosh(a); break;
        case FN_CSCH: y[i] = 1.0 / sinh(a); break;
        case FN_ASECH: y[i] = acosh(1.0 / a); break;
        case FN_ACSCH: y[i] = asinh(1.0 / a); break;
        case FN_ACOTH: y[i] = atanh(1.0 / a); break;
        case FN_ACOT: y[i] = atan(1.0 / a); break;
        case FN_ACSC: y[i] = asin(1.0 / a); break;
        case FN_ASIND: y[i] = asin(a) * (180.0 / M_PI); break;
        case FN_ACOSD: y[i] = acos(a) * (180.0 / M_PI); break;
        case FN_ATAND: y[i] = atan(a) * (180.0 / M_PI); break;
        case FN_ASECD: y[i] = (fabs(a) < 1.0 ? NAN : acos(1.0 / a)) * (180.0 / M_PI); break;
        case FN_ACSCD: y[i] = asin(1.0 / a) * (180.0 / M_PI); break;
        case FN_ASINPI: y[i] = asin(a) / M_PI; break;
        case FN_ACOSPI: y[i] = acos(a) / M_PI; break;
        case FN_ATANPI: y[i] = atan(a) / M_PI; break;
        case FN_INDEG: y[i] = a * (180.0 / M_PI); break;
        case FN_INRAD: y[i] = a * (M_PI / 180.0); break;
        case FN_ERF: y[i] = erf(a); break;
        case FN_ERFCX: y[i] = erfcx_d(a); break;
        case FN_EXPX2: y[i] = exp(a * a); break;
        case FN_GAMMA: y[i] = tgamma(a); break;
        case FN_GAMMALN: y[i] = lgamma(a); break;
        case FN_DIGAMMA: y[i] = o_digamma_d(a); break;
        case FN_SIGNGAM: y[i] = o_signgam((float)a); break;
        case FN_ERFINV: y[i] = erfinv_d(a); break;
        case FN_ERFCINV: y[i] = erfcinv_d(a); break;
        case FN_EXPRECNEG: y[i] = exp(-1.0 / a); break;
        case FN_EXPRECNEGC: y[i] = -expm1(-1.0 / a); break;
        case FN_SQRT1PM1: y[i] = sqrt1pm1_d(a); break;
        default: y[i] = sqrt(a); break;
        }
    }
}

/* ------------------------------------------------ Black-Scholes --------
 * Textbook call+put written as the NT2 expression a user would assign
 * through tie():
 *   d1 = (log(S/K) + fma(sqr(sig),0.5,r)*T) / (sig*sqrt(T))
 *   d2 = fnms(sig, sqrt(T), d1)
 *   e  = K*exp(-r*T)
 *   call = fnms(e, normcdf(d2), S*normcdf(d1))
 *   put  = fnms(S, normcdf(-d1), e*normcdf(-d2))
 * Operator semantics follow the demo (demo/blackscholes/nt2/
 * blackandscholes_nt2.cpp:55-59): fma/fnms unfused, -r*T is (-r)*T.
 * sig and r are either per-option tables (pointer non-NULL) or scalars. */
static inline void bs_one(float S, float K, float T, float sig, float r, float *call, float *put)
{
    float sq = sqrtf(T);
    float d1 = (o_log(S / K) + ((sig * sig) * 0.5f + r) * T) / (sig * sq);
    float d2 = d1 - sig * sq;
    float e = K * o_exp((-r) * T);
    float n1 = o_normcdf(d1), n2 = o_normcdf(d2);
    float m1 = o_normcdf(-d1), m2 = o_normcdf(-d2);
    *call = S * n1 - e * n2;
    *put = e * m2 - S * m1;
}

EXPORT void o_bs_f32(const float *S, const float *K, const float *T, const float *sig_tab,
                     float sig, const float *r_tab, float r, float *call, float *put, int64_t n,
                     int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i)
        bs_one(S[i], K[i], T[i], sig_tab ? sig_tab[i] : sig, r_tab ? r_tab[i] : r, &call[i], &put[i]);
}

/* NT2 demo form, call only, fastnormcdf, non-textbook d1 (log term not
 * divided): demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59. */
EXPORT void o_bs_demo_f32(const float *S, const float *K, const float *T, const float *r_tab, float r,
                          const float *v_tab, float v, float *R, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        float ri = r_tab ? r_tab[i] : r, vi = v_tab ? v_tab[i] : v;
        float da = sqrtf(T[i]);
        float d1 = o_log(S[i] / K[i]) + (((vi * vi) * 0.5f + ri) * T[i]) / (vi * da);
        float d2 = d1 - vi * da;
        R[i] = S[i] * o_fastnormcdf(d1) - (K[i] * o_exp((-ri) * T[i])) * o_fastnormcdf(d2);
    }
}

/* FP64 textbook BS on the float inputs.  terms (optional, 4 per option):
 * S*N(d1), K e^{-rT} N(d2), K e^{-rT} N(-d2), S*N(-d1) -- the magnitudes the
 * conditioned error metric scales by. */
static inline double ncdf64(double x) { return 0.5 * erfc(-x / sqrt(2.0)); }

EXPORT void o_bs_f64(const float *S, const float *K, const float *T, const float *sig_tab, float sig,
                     float r, double *call, double *put, double *terms, int64_t n)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = S[i], k = K[i], t = T[i], v = sig_tab ? sig_tab[i] : sig, rr = r;
        double sq = sqrt(t);
        double d1 = (log(s / k) + (rr + 0.5 * v * v) * t) / (v * sq);
        double d2 = d1 - v * sq;
        double e = k * exp(-rr * t);
        double a = s * ncdf64(d1), b = e * ncdf64(d2), c = e * ncdf64(-d2), d = s * ncdf64(-d1);
        call[i] = a - b;
        put[i] = c - d;
        if (terms) { terms[4 * i] = a; terms[4 * i + 1] = b; terms[4 * i + 2] = c; terms[4 * i + 3] = d; }
    }
}

/* Analytic FP64 vector-Jacobian product of (call, put) w.r.t. S, K, T, sigma,
 * r, given upstream gradients gc, gp.  Used to check the adjoint kernel. */
EXPORT void o_bs_vjp_f64(const float *S, const float *K, const float *T, const float *sig_tab, float sig,
                         float r, const float *gc, const float *gp, double *dS, double *dK, double *dT,
                         double *dsig, double *dr, int64_t n)
{
    const double inv_sqrt_2pi = 0.398942280401432677939946059934;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = S[i], k = K[i], t = T[i], v = sig_tab ? sig_tab[i] : sig, rr = r;
        double sq = sqrt(t);
        double d1 = (log(s / k) + (rr + 0.5 * v * v) * t) / (v * sq);
        double d2 = d1 - v * sq;
        double df = exp(-rr * t);
        double pdf1 = inv_sqrt_2pi * exp(-0.5 * d1 * d1);
        double n1 = ncdf64(d1), n2 = ncdf64(d2), m1 = ncdf64(-d1), m2 = ncdf64(-d2);
        double gC = gc[i], gP = gp[i];
        dS[i] = gC * n1 - gP * m1;
        dK[i] = -gC * df * n2 + gP * df * m2;
        double thetaC = s * pdf1 * v / (2.0 * sq) + rr * k * df * n2;
        double thetaP = s * pdf1 * v / (2.0 * sq) - rr * k * df * m2;
        dT[i] = gC * thetaC + gP * thetaP;
        dsig[i] = (gC + gP) * s * pdf1 * sq;
        dr[i] = gC * k * t * df * n2 - gP * k * t * df * m2;
    }
}

/* Term-magnitude scale of each VJP component (the sum of the absolute values
 * of the terms the analytic gradient adds): the yardstick for relative
 * gradient error when the seeds make a gradient cancel to near zero. */
EXPORT void o_bs_vjp_scale_f64(const float *S, const float *K, const float *T, const float *sig_tab, float sig,
                               float r, const float *gc, const float *gp, double *sS, double *sK, double *sT,
                               double *ssig, double *sr, int64_t n)
{
    const double inv_sqrt_2pi = 0.398942280401432677939946059934;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = S[i], k = K[i], t = T[i], v = sig_tab ? sig_tab[i] : sig, rr = r;
        double sq = sqrt(t);
        double d1 = (log(s / k) + (rr + 0.5 * v * v) * t) / (v * sq);
        double d2 = d1 - v * sq;
        double df = exp(-rr * t);
        double pdf1 = inv_sqrt_2pi * exp(-0.5 * d1 * d1);
        double n1 = ncdf64(d1), n2 = ncdf64(d2), m1 = ncdf64(-d1), m2 = ncdf64(-d2);
        double aC = fabs((double)gc[i]), aP = fabs((double)gp[i]);
        double e2 = aC * n2 + aP * m2;
        sS[i] = aC * n1 + aP * m1;
        sK[i] = df * e2;
        sT[i] = (aC + aP) * s * pdf1 * v / (2.0 * sq) + fabs(rr) * k * df * e2;
        ssig[i] = (aC + aP) * s * pdf1 * sq;
        sr[i] = k * t * df * e2;
    }
}

/* FP64 forward used by the central finite-difference check (same formula as
 * o_bs_f64, parameters in double so a perturbation h is not rounded away). */
EXPORT void o_bs_point_f64(double s, double k, double t, double v, double rr, double *call, double *put)
{
    double sq = sqrt(t);
    double d1 = (log(s / k) + (rr + 0.5 * v * v) * t) / (v * sq);
    double d2 = d1 - v * sq;
    double e = k * exp(-rr * t);
    *call = s * ncdf64(d1) - e * ncdf64(d2);
    *put = e * ncdf64(-d2) - s * ncdf64(-d1);
}

/* ------------------------------------------------ other expressions ---- */
/* saxpy: demo/saxpy/nt2/saxpy_nt2.cpp:41  Y = alpha*X + Y (two roundings) */
EXPORT void o_saxpy_f32(float alpha, const float *X, float *Y, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) Y[i] = alpha * X[i] + Y[i];
}

/* expr3 = exp(-sqr(x))*sqrt(abs(y)) + log1p(abs(z)) */
EXPORT void o_expr3_f32(const float *x, const float *y, const float *z, float *out, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i)
        out[i] = o_exp(-(x[i] * x[i])) * sqrtf(fabsf(y[i])) + o_log1p(fabsf(z[i]));
}

EXPORT void o_expr3_f64(const float *x, const float *y, const float *z, double *out, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) {
        double a = x[i], b = y[i], c = z[i];
        out[i] = exp(-a * a) * sqrt(fabs(b)) + log1p(fabs(c));
    }
}

/* rgb2yuv: demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:30-32 (three statements; u and v
 * re-read the stored y). */
EXPORT void o_rgb2yuv_f32(const float *r, const float *g, const float *b, float *y, float *u, float *v,
                          int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        float yy = 0.299f * r[i] + 0.587f * g[i] + 0.114f * b[i];
        y[i] = yy;
        u[i] = 0.492f * (b[i] - yy);
        v[i] = 0.877f * (r[i] - yy);
    }
}

/* Sigma-delta step on uint8 pixels: demo/sigmadelta/nt2/sigmadelta_nt2.cpp:38-57
 * with selinc/seldec (BSIMD/boolean/functions/scalar/selinc.hpp:27,
 * seldec.hpp:27), saturating adds for unsigned
 * (BSIMD/arithmetic/functions/scalar/adds.hpp:54-66) and if_zero_else_one on a
 * logical (BSIMD/boolean/functions/scalar/if_zero_else_one.hpp:21-29).
 * The diff and mul temporaries are not stored. */
static inline uint8_t adds_u8(uint8_t a, uint8_t b)
{
    unsigned s = (unsigned)a + (unsigned)b;
    return (uint8_t)(s > 255u ? 255u : s);
}

EXPORT void o_sigmadelta_u8(const uint8_t *fr, uint8_t *bkg, uint8_t *var, uint8_t *label, int64_t n,
                            int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        uint8_t f = fr[i], b = bkg[i], v = var[i];
        b = (b < f) ? (uint8_t)(b + 1) : ((b > f) ? (uint8_t)(b - 1) : b);
        uint8_t d = (uint8_t)((b > f ? b : f) - (b < f ? b : f));
        uint8_t m = adds_u8(adds_u8(d, d), d);
        if (d != 0) v = (v < m) ? (uint8_t)(v + 1) : ((v > m) ? (uint8_t)(v - 1) : v);
        bkg[i] = b;
        var[i] = v;
        label[i] = (d < v) ? 0 : 1;
    }
}

/* ------------------------------------------------------- reductions ----
 * NT2 fold schedule (OMP/spawner/fold.hpp:37-81 with the shared_memory
 * inner_fold worker, SHM/sdk/shared_memory/worker/inner_fold.hpp:64-98):
 * grain = top_cache_line_size(2)/sizeof(float) = 16 elements; each block of
 * 16 is folded naively in FP32 from zero, then added to the total inside an
 * omp critical section (combine order is thread-timing dependent); the tail
 * n % 16 is folded serially afterwards.  dot(x,y) = sum(x*y) with the
 * product rounded to float (RED/reduction/functions/expr/dot.hpp:22-42). */
static int64_t nt2_line_grain(void)
{
    /* top_cache_line_size(2): the L3 line when an L3 size is reported, else
     * the L2 line.  NT2 would divide by zero when both read 0 (common on
     * aarch64 glibc); the restatement uses a 64-byte line there. */
    long line = sysconf(_SC_LEVEL3_CACHE_SIZE) > 0 ? sysconf(_SC_LEVEL3_CACHE_LINESIZE)
                                                   : sysconf(_SC_LEVEL2_CACHE_LINESIZE);
    if (line <= 0) line = 64;
    return line / (long)sizeof(float);
}

EXPORT float o_sum_nt2_f32(const float *x, const float *y, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    int64_t grain = nt2_line_grain();
    int64_t nblocks = n / grain;
    float total = 0.0f;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t b = 0; b < nblocks; ++b) {
        float out = 0.0f;
        const int64_t o = b * grain;
        if (y) for (int64_t j = 0; j < grain; ++j) out = out + x[o + j] * y[o + j];
        else for (int64_t j = 0; j < grain; ++j) out = out + x[o + j];
#pragma omp critical
        total = total + out;
    }
    for (int64_t i = nblocks * grain; i < n; ++i) total = total + (y ? x[i] * y[i] : x[i]);
    return total;
}

/* Same blocks, one private partial per thread, combined once: the plain
 * all-cores schedule reported beside the NT2-rule one. */
EXPORT float o_sum_plain_f32(const float *x, const float *y, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    float total = 0.0f;
#pragma omp parallel for schedule(static) num_threads(nthreads) reduction(+ : total)
    for (int64_t i = 0; i < n; ++i) total += y ? x[i] * y[i] : x[i];
    return total;
}

/* globalsum: serial accumulation (RED/core/functions/scalar/global.hpp:17-43) */
EXPORT float o_globalsum_f32(const float *x, int64_t n)
{
    float s = 0.0f;
    for (int64_t i = 0; i < n; ++i) s = s + x[i];
    return s;
}

/* Exact superaccumulator.  Every float and every float*float product is an
 * integer m (<= 53 bits) times 2^e with e >= -351; digits hold signed sums of
 * 32-bit chunks at weight 2^(32*i + ACC_BASE), covering 2^-416 .. 2^352. */
#define ACC_BASE (-416)
#define ACC_DIGITS 24
typedef struct { int64_t d[ACC_DIGITS]; } superacc;

static void acc_norm(superacc *a)
{
    for (int i = 0; i < ACC_DIGITS - 1; ++i) {
        int64_t c = a->d[i] >> 32; /* arithmetic shift: floor division */
        a->d[i] -= c * ((int64_t)1 << 32);
        a->d[i + 1] += c;
    }
}

static inline void acc_add(superacc *a, double v)
{
    if (v == 0.0) return;
    int ex;
    double f = frexp(fabs(v), &ex);
    uint64_t m = (uint64_t)ldexp(f, 53);
    int p = ex - 53 - ACC_BASE;
    int i = p >> 5, s = p & 31;
    /* m << s is at most 85 bits: three 32-bit digits */
    unsigned __int128 w = (unsigned __int128)m << s;
    int64_t c0 = (int64_t)(uint32_t)w, c1 = (int64_t)(uint32_t)(w >> 32), c2 = (int64_t)(uint64_t)(w >> 64);
    if (v < 0) { a->d[i] -= c0; a->d[i + 1] -= c1; a->d[i + 2] -= c2; }
    else { a->d[i] += c0; a->d[i + 1] += c1; a->d[i + 2] += c2; }
}

static double acc_value(superacc a)
{
    acc_norm(&a);
    int neg = a.d[ACC_DIGITS - 1] < 0;
    if (neg) {
        for (int i = 0; i < ACC_DIGITS; ++i) a.d[i] = -a.d[i];
        acc_norm(&a);
    }
    long double r = 0.0L;
    for (int i = ACC_DIGITS - 1; i >= 0; --i) r += ldexpl((long double)a.d[i], 32 * i + ACC_BASE);
    return neg ? -(double)r : (double)r;
}

/* Exact sum (y == NULL) or exact dot.  Returns the exact value rounded to
 * double; abs_sum receives sum |x_i| (or |x_i*y_i|) for the condition number. */
EXPORT double o_exact_sum(const float *x, const float *y, int64_t n, int nthreads, double *abs_sum)
{
    if (nthreads < 1) nthreads = 1;
    superacc total;
    memset(&total, 0, sizeof total);
    double asum = 0.0;
#pragma omp parallel num_threads(nthreads) reduction(+ : asum)
    {
        superacc a;
        memset(&a, 0, sizeof a);
        int64_t cnt = 0;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double v = y ? (double)x[i] * (double)y[i] : (double)x[i];
            acc_add(&a, v);
            asum += fabs(v);
            if (++cnt == (1 << 24)) { acc_norm(&a); cnt = 0; }
        }
        acc_norm(&a);
#pragma omp critical
        {
            for (int i = 0; i < ACC_DIGITS; ++i) total.d[i] += a.d[i];
            acc_norm(&total);
        }
    }
    if (abs_sum) *abs_sum = asum;
    return acc_value(total);
}

/* median / medianad along a dimension (core/reduction/include/nt2/core/
 * functions/expr/median.hpp:37-50, expr/medianad.hpp:38-54): each slice of
 * the [lo, inner, hi] view sorted ascending (NT2's sort, std::sort with
 * operator<), the middle element for odd inner, meanof of the two middle ones
 * for even inner (boost.simd generic/meanof.hpp:21-33: m + (max - m) * 1/2
 * for finite values, else average = a0 * 1/2 + a1 * 1/2, unfused).  NT2's
 * result for a slice holding a NaN is unspecified (operator< orders no NaN);
 * here it is NaN, as for an empty slice.  medianad is the median of
 * |x - median| per slice. */
static int cmp_float_lt(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return x < y ? -1 : (y < x ? 1 : 0);
}

static float nt2_meanof_f(float a0, float a1)
{
    float m = a0 < a1 ? a0 : a1, M = a0 > a1 ? a0 : a1;
    if (a0 - a0 == 0.0f && a1 - a1 == 0.0f) return m + (M - m) * 0.5f;
    return a0 * 0.5f + a1 * 0.5f;
}

static float median_of(float *v, int64_t n)
{
    if (n == 0) return NAN;
    for (int64_t k = 0; k < n; ++k)
        if (isnan(v[k])) return NAN;
    qsort(v, (size_t)n, sizeof(float), cmp_float_lt);
    int64_t mid = n >> 1;
    return (n & 1) ? v[mid] : nt2_meanof_f(v[mid - 1], v[mid]);
}

/* trapz (core/functions/expr/trapz.hpp:24-50): per slice the float sums of
 * neighbours y_k + y_(k+1) (adjfun(plus)), folded in index order, times 1/2. */
EXPORT void o_trapz_nt2_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, float *out)
{
    for (int64_t h = 0; h < hi; ++h)
        for (int64_t l = 0; l < lo; ++l) {
            const float *b = x + l + lo * inner * h;
            float s = 0.0f;
            for (int64_t k = 0; k + 1 < inner; ++k) s += b[lo * k] + b[lo * (k + 1)];
            out[l + lo * h] = 0.5f * s;
        }
}

EXPORT void o_median_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int ad, float *out)
{
    float *v = (float *)malloc((size_t)(inner > 0 ? inner : 1) * sizeof(float));
    for (int64_t h = 0; h < hi; ++h)
        for (int64_t l = 0; l < lo; ++l) {
            const float *base = x + l + lo * inner * h;
            for (int64_t k = 0; k < inner; ++k) v[k] = base[lo * k];
            float m = median_of(v, inner);
            if (ad) {
                for (int64_t k = 0; k < inner; ++k) v[k] = fabsf(base[lo * k] - m);
                m = median_of(v, inner);
            }
            out[l + lo * h] = m;
        }
    free(v);
}

/* Reductions along one dimension, the table viewed as [lo, inner, hi]
 * (core/reduction/include/nt2/dsl/functions/reduction/run.hpp:51-89).
 * op: 0 sum, 1 prod, 2 max, 3 min, 4 mean, 5 asum1, 6 asum2, 7 norm2.
 *
 * o_fold_nt2_f32: each output folded in index order from the neutral element
 * with unfused float operations, fold_step's acc = bop(acc, x)
 * (core/reduction/include/nt2/core/functions/details/fold_step.hpp:31-43) as
 * NT2's per-segment workers run it (arch/shared_memory/include/nt2/sdk/
 * shared_memory/worker/inner_fold.hpp:47-80, worker/outer_fold.hpp);
 * max = (a0 > a1) ? a0 : a1 (boost/simd/arithmetic/functions/scalar/max.hpp),
 * mean = rec(float(n)) * sum (core/functions/expr/mean.hpp:22-33),
 * asum2 = sum(sqr_abs), norm2 = sqrt(asum2), var = f * asum2(a - mean(a)) with
 * f = rec(n - 1) (ops 8, 9; rec(n) for 10, 11; 1 when n <= 1) and stdev = sqrt(var)
 * (core/functions/expr/var.hpp, expr/stdev.hpp), meanad = mean(abs(a - mean(a)))
 * (op 18, core/functions/expr/meanad.hpp).  index: first position equal to
 * the result (common/globalmax.hpp:36-48), -1 if none. */
EXPORT void o_fold_nt2_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, float *out,
                           int64_t *index, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t o = 0; o < lo * hi; ++o) {
        const int64_t h = o / lo, l = o - h * lo;
        const float *p = x + l + lo * inner * h;
        float acc = op == 1 ? 1.0f : op == 2 ? -INFINITY : op == 3 ? INFINITY : 0.0f;
        if (op == 18) {  /* meanad = mean(abs(center(a))) (expr/meanad.hpp): NT2's mean, then in order */
            float sm = 0.0f;
            for (int64_t k = 0; k < inner; ++k) sm = sm + p[lo * k];
            const float m = (1.0f / (float)inner) * sm;
            for (int64_t k = 0; k < inner; ++k) acc = acc + fabsf(p[lo * k] - m);
            out[o] = (1.0f / (float)inner) * acc;
            continue;
        }
        if (op >= 12) {  /* nbtrue, all/any/none (sum of is_nez), nansum, nanmean (expr/nansum.hpp, nanmean.hpp) */
            float cnt = 0.0f, sm = 0.0f, ok = 0.0f;
            for (int64_t k = 0; k < inner; ++k) {
                const float v = p[lo * k];
                cnt = cnt + (v != 0.0f ? 1.0f : 0.0f);
                ok = ok + (v == v ? 1.0f : 0.0f);
                sm = sm + (v == v ? v : 0.0f);
            }
            const float n = (float)inner;
            out[o] = op == 12 ? cnt : op == 13 ? (cnt == n ? 1.0f : 0.0f) : op == 14 ? (cnt != 0.0f ? 1.0f : 0.0f)
                   : op == 15 ? (cnt == 0.0f ? 1.0f : 0.0f) : op == 16 ? sm : (1.0f / (ok > 1.0f ? ok : 1.0f)) * sm;
            continue;
        }
        if (op >= 8) {  /* var / stdev: f * asum2(a - mean(a)) (expr/var.hpp, expr/stdev.hpp) */
            float sm = 0.0f;
            for (int64_t k = 0; k < inner; ++k) sm = sm + p[lo * k];
            const float m = (1.0f / (float)inner) * sm;
            for (int64_t k = 0; k < inner; ++k) { const float d = p[lo * k] - m; acc = acc + d * d; }
            const float n = (float)inner;
            const float f = (n <= 1.0f) ? 1.0f : 1.0f / ((op == 10 || op == 11) ? n : n - 1.0f);
            acc = f * acc;
            out[o] = (op == 9 || op == 11) ? sqrtf(acc) : acc;
            continue;
        }
        for (int64_t k = 0; k < inner; ++k) {
            const float v = p[lo * k];
            switch (op) {
            case 1: acc = acc * v; break;
            case 2: acc = (acc > v) ? acc : v; break;
            case 3: acc = (acc < v) ? acc : v; break;
            case 5: acc = acc + fabsf(v); break;
            case 6: case 7: acc = acc + v * v; break;
            default: acc = acc + v; break;
            }
        }
        if (op == 4) acc = (1.0f / (float)inner) * acc;
        if (op == 7) acc = sqrtf(acc);
        out[o] = acc;
        if (index && (op == 2 || op == 3)) {
            int64_t f = -1;
            for (int64_t k = 0; k < inner && f < 0; ++k)
                if (p[lo * k] == acc) f = k;
            index[o] = f;
        }
    }
}

/* Reference values for the fast policy: sum-type ops exactly (superaccumulator;
 * x*x is exact in double), rounded to double, with sum |term| for the error
 * bound; prod in long double; max/min in NT2's order with NaN propagation
 * (the first NaN), index = first position equal to the result. */
EXPORT void o_fold_ref(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, double *out, double *abs_sum,
                       int64_t *index, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (int64_t o = 0; o < lo * hi; ++o) {
        const int64_t h = o / lo, l = o - h * lo;
        const float *p = x + l + lo * inner * h;
        if (op == 1) {
            long double r = 1.0L;
            for (int64_t k = 0; k < inner; ++k) r *= p[lo * k];
            out[o] = (double)r;
            if (abs_sum) abs_sum[o] = fabs((double)r);
        } else if (op == 2 || op == 3) {
            float best = op == 2 ? -INFINITY : INFINITY;
            int nan = 0;
            for (int64_t k = 0; k < inner; ++k) {
                const float v = p[lo * k];
                if (v != v) { best = v; nan = 1; break; }
                if (op == 2 ? !(best > v) : !(best < v)) best = v;  /* NT2's order: an equal later value wins */
            }
            out[o] = best;
            if (index) {
                int64_t f = -1;
                for (int64_t k = 0; k < inner && f < 0; ++k) {
                    const float v = p[lo * k];
                    if (nan ? v != v : v == best) f = k;
                }
                index[o] = f;
            }
        } else if (op == 18) {  /* meanad: exact mean, then |x - mu| in long double, / n */
            superacc a;
            memset(&a, 0, sizeof a);
            int64_t cnt = 0;
            for (int64_t k = 0; k < inner; ++k) {
                acc_add(&a, (double)p[lo * k]);
                if (++cnt == (1 << 24)) { acc_norm(&a); cnt = 0; }
            }
            const long double mu = inner > 0 ? (long double)acc_value(a) / (long double)inner : 0.0L;
            long double sa = 0.0L;
            for (int64_t k = 0; k < inner; ++k) sa += fabsl((long double)p[lo * k] - mu);
            out[o] = (double)(sa / (long double)inner);
            if (abs_sum) abs_sum[o] = out[o];
        } else if (op >= 12) {  /* counts exactly; nansum exactly; nanmean = nansum / max(count, 1) */
            superacc a;
            memset(&a, 0, sizeof a);
            int64_t cnt = 0, nz = 0, ok = 0;
            double as = 0.0;
            for (int64_t k = 0; k < inner; ++k) {
                const float v = p[lo * k];
                nz += v != 0.0f;
                if (v == v) { ++ok; acc_add(&a, (double)v); as += fabs((double)v); }
                if (++cnt == (1 << 24)) { acc_norm(&a); cnt = 0; }
            }
            const double sm = acc_value(a);
            out[o] = op == 12 ? (double)nz : op == 13 ? (double)(nz == inner) : op == 14 ? (double)(nz != 0)
                   : op == 15 ? (double)(nz == 0) : op == 16 ? sm : sm / (double)(ok > 1 ? ok : 1);
            if (abs_sum) abs_sum[o] = op == 17 ? as / (double)(ok > 1 ? ok : 1) : op == 16 ? as : 0.0;
        } else if (op >= 8) {  /* var / stdev: exact mean (superaccumulator), then deviations in long double */
            superacc a;
            memset(&a, 0, sizeof a);
            int64_t cnt = 0;
            for (int64_t k = 0; k < inner; ++k) {
                acc_add(&a, (double)p[lo * k]);
                if (++cnt == (1 << 24)) { acc_norm(&a); cnt = 0; }
            }
            const long double mu = inner > 0 ? (long double)acc_value(a) / (long double)inner : 0.0L;
            long double ss = 0.0L;
            for (int64_t k = 0; k < inner; ++k) { const long double d = (long double)p[lo * k] - mu; ss += d * d; }
            const long double n = (long double)inner;
            if (inner > 1) ss /= (op == 10 || op == 11) ? n : n - 1.0L;
            out[o] = (op == 9 || op == 11) ? (double)sqrtl(ss) : (double)ss;
            if (abs_sum) abs_sum[o] = fabs(out[o]);
        } else {
            superacc a;
            memset(&a, 0, sizeof a);
            double as = 0.0;
            int64_t cnt = 0;
            for (int64_t k = 0; k < inner; ++k) {
                const double v = p[lo * k];
                const double t = op == 5 ? fabs(v) : (op == 6 || op == 7) ? v * v : v;
                acc_add(&a, t);
                as += fabs(t);
                if (++cnt == (1 << 24)) { acc_norm(&a); cnt = 0; }
            }
            double r = acc_value(a);
            if (op == 4) r = r / (double)inner;
            if (op == 7) r = sqrt(r);
            out[o] = r;
            if (abs_sum) abs_sum[o] = as;
        }
    }
}

/* Cumulative functions, the table viewed as [lo, inner, hi]: each segment in
 * order from the neutral element, summary = bop(summary, x); out = summary
 * (core/swar/include/nt2/core/functions/details/scan_step.hpp:27-43).
 * op: 0 cumsum, 1 cumprod, 2 cummax, 3 cummin. */
EXPORT void o_scan_nt2_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, float *out, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t s = 0; s < lo * hi; ++s) {
        const int64_t h = s / lo, l = s - h * lo;
        const int64_t base = l + lo * inner * h;
        float acc = op == 1 ? 1.0f : op == 2 ? -INFINITY : op == 3 ? INFINITY : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = x[base + lo * k];
            switch (op) {
            case 1: acc = acc * v; break;
            case 2: acc = (acc > v) ? acc : v; break;
            case 3: acc = (acc < v) ? acc : v; break;
            default: acc = acc + v; break;
            }
            out[base + lo * k] = acc;
        }
    }
}

/* Exact prefix sums (superaccumulator), rounded to double, for the fast
 * policy's cumsum; |prefix| bound: running sum of |x|. */
EXPORT void o_cumsum_exact(const float *x, int64_t lo, int64_t inner, int64_t hi, double *out, double *abs_run,
                           int nthreads)
{
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int64_t s = 0; s < lo * hi; ++s) {
        const int64_t h = s / lo, l = s - h * lo;
        const int64_t base = l + lo * inner * h;
        superacc a;
        memset(&a, 0, sizeof a);
        double as = 0.0;
        for (int64_t k = 0; k < inner; ++k) {
            const double v = x[base + lo * k];
            acc_add(&a, v);
            acc_norm(&a);
            as += fabs(v);
            out[base + lo * k] = acc_value(a);
            abs_run[base + lo * k] = as;
        }
    }
}

/* NT2 grain for transform on Linux without cpuid: top_cache_size(2) reads
 * cache_sizes_[2], which the sysconf path fills with the L3 size in bytes
 * (modules/sdk/config/include/nt2/sdk/config/details/cache.hpp:26-39,
 * .../config/cache.hpp:46-58); transform goes parallel only when
 * n > 8*grain (SHM/core/functions/shared_memory/transform.hpp:39-49). */
EXPORT int64_t o_nt2_transform_grain(int64_t elem_size)
{
    long c = sysconf(_SC_LEVEL3_CACHE_SIZE);
    if (c <= 0) c = sysconf(_SC_LEVEL2_CACHE_SIZE);
    int64_t g = c > 0 ? (int64_t)c / elem_size : 0;
    return g ? g : 1;
}

EXPORT int o_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
