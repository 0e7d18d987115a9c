// nt2g_math.cuh -- FP32 element math for the fused evaluator.
//
// Every function is a template on an arithmetic policy:
//
//  * Nt2  -- NT2's own scalar float algorithms with NT2's operation order:
//            fma/fnms/Horner unfused (a*b then +c, two roundings), IEEE
//            division and square root.  On the GPU the intrinsics __fmul_rn /
//            __fadd_rn / __fdiv_rn / __fsqrt_rn stop the compiler from
//            contracting, so results are bit-identical to NT2's scalar CPU
//            evaluation.
//  * Fast -- the default hot path: fused multiply-add, a reciprocal-approx
//            division refined by one Newton step, and an erfc/normcdf built
//            on an exact split of x^2 so the tail keeps FP32 accuracy (NT2's
//            float erfc loses up to ~75 ulp there).
//
// The header also compiles as plain C++ (host), with std::fma, so the
// accuracy of the Fast policy can be studied on a CPU; only the division
// differs (host: IEEE division, device: rcp.approx + Newton, <= 1 ulp apart).
//
// NT2 sources followed (paths inside the NT2 tree):
//   exp   modules/core/exponential/include/nt2/exponential/functions/
//           scalar/impl/expo/{expo_base.hpp:58-69, f_expo_reduction.hpp:52-85,
//           expo_scale.hpp:27-35}
//   log   .../scalar/impl/logs/{f_log.hpp:59-88, f_kernel.hpp:43-75}
//   log1p .../scalar/log1p.hpp:35-45
//   erfc  modules/core/euler/include/nt2/euler/functions/scalar/erfc.hpp:83-104,
//           details/erf_kernel.hpp:48-91
//   normcdf / fastnormcdf  modules/core/statistics/include/nt2/statistics/
//           functions/generic/{normcdf.hpp:34, fastnormcdf.hpp:39-54}
#pragma once
#if defined(__CUDACC_RTC__)
// run-time compilation (the JIT path embeds this header): no host headers
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
#else
#include <stdint.h>
#include <string.h>
#include <math.h>
#endif

#if defined(__CUDACC__)
#define NT2G_HD __host__ __device__ __forceinline__
#else
#define NT2G_HD inline
#endif

namespace nt2g {

NT2G_HD float bits_f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}
NT2G_HD uint32_t f_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}

// ----------------------------------------------------------- policies ----
struct Nt2 {
    static constexpr bool exact = true;
#if defined(__CUDA_ARCH__)
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
#else
    static inline float mul(float a, float b) { volatile float r = a * b; return r; }
    static inline float add(float a, float b) { volatile float r = a + b; return r; }
    static inline float sub(float a, float b) { volatile float r = a - b; return r; }
    static inline float div(float a, float b) { return a / b; }
    static inline float sqrt(float a) { return sqrtf(a); }
#endif
    static NT2G_HD float fdiv(float a, float b) { return div(a, b); }
    // NT2's generic fma is a*b+c with two roundings.
    static NT2G_HD float fma(float a, float b, float c) { return add(mul(a, b), c); }
};

struct Fast {
    static constexpr bool exact = false;
#if defined(__CUDA_ARCH__)
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float rcp(float b)
    {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
        return r;
    }
    // IEEE division for user-visible '/', where operands are arbitrary.
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    // q0 = a*rcp(b), one Newton correction on the residual a - q0*b (<= 1 ulp
    // from the rounded quotient).  Valid for finite normal b whose reciprocal
    // is normal; used only inside kernels whose operands are known to be so.
    static __device__ __forceinline__ float fdiv(float a, float b)
    {
        float r = rcp(b);
        float q = a * r;
        float e = __fmaf_rn(-q, b, a);
        return __fmaf_rn(e, r, q);
    }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
#else
    static inline float mul(float a, float b) { return a * b; }
    static inline float add(float a, float b) { return a + b; }
    static inline float sub(float a, float b) { return a - b; }
    static inline float fma(float a, float b, float c) { return fmaf(a, b, c); }
    static inline float rcp(float b) { return 1.0f / b; }
    static inline float div(float a, float b) { return a / b; }
    static inline float fdiv(float a, float b) { return a / b; }
    static inline float sqrt(float a) { return sqrtf(a); }
#endif
};

// Horner with NT2's coefficient order: first argument after x is the
// highest degree; each step is fma(x, acc, c).
template <class P> NT2G_HD float horner(float, float acc) { return acc; }
template <class P, class... R>
NT2G_HD float horner(float x, float acc, float c, R... rest)
{
    return horner<P>(x, P::fma(x, acc, c), rest...);
}

// ------------------------------------------------------------ constants --
// NT2 float constants, by bit pattern (modules/core/exponential/include/nt2/
// exponential/constants/*.hpp, modules/boost/simd/base/include/boost/simd/
// constant/constants/*.hpp).
#define NT2G_MAXLOG      0x42b0c0a5u
#define NT2G_MINLOG      0xc2b0c0a5u
#define NT2G_INVLOG_2    0x3fb8aa3bu
#define NT2G_LOG_2HI     0x3f318000u
#define NT2G_LOG_2LO     0xb95e8083u
#define NT2G_SQRT_2O_2   0x3F3504F3u
#define NT2G_SMALLESTPOS 0x00800000u
#define NT2G_TWOTONMB    0x4B000000u
#define NT2G_MLOGTWO2NMB 0xc17f1402u
#define NT2G_TWOTHIRD    0x3f2aaaabu
#define NT2G_INVSQRT_2PI 0x3ecc422au
#define NT2G_MAXLOG2     0x42fe0000u
#define NT2G_MINLOG2     0xc2fe0000u
#define NT2G_MAXLOG10    0x4218ec59u
#define NT2G_MINLOG10    0xc2179999u
#define NT2G_LOG_2       0x3f317218u
#define NT2G_INVLOG10_2  0x40549a78u
#define NT2G_LOG10_2HI   0x3e9a0000u
#define NT2G_LOG10_2LO   0x39826a14u
#define NT2G_LOGEPS      0xc17f1402u
#define NT2G_LOG2_EM1    0x3ee2a8edu
#define NT2G_LOG10_EHI   0x3ede0000u
#define NT2G_LOG10_ELO   0x3a37b152u
#define NT2G_MLOG2TWO2NMB  0xc1b80000u
#define NT2G_MLOG10TWO2NMB 0xc0dd8edeu

NT2G_HD float f_inf() { return bits_f(0x7f800000u); }
NT2G_HD float f_nan() { return bits_f(0x7fc00000u); }
NT2G_HD bool is_nan(float x) { return x != x; }

// ------------------------------------------------------------------ exp --
// NT2: k = round2even(x/ln2); r = x - k*ln2hi - k*ln2lo (unfused fnms);
// degree-4 Remez for (e^r-1-r)/r^2; 2^k built in the exponent field.
// Fast: same reduction with FMAs, k from the 1.5*2^23 shifter (round to
// nearest even, so k equals NT2's except on exact ties), and its own degree-5
// fit of q(r) = (e^r-1-r)/r^2 on |r| <= ln2/2 (truncation < 0.02 ulp).
// exp_fast_parts returns e^x = (1 + s) * 2^k unassembled so that callers can
// fold the "+1" into a following product (one rounding instead of two).
NT2G_HD float exp_fast_parts(float a0, float &scale)
{
    const float shifter = 12582912.0f;  // 1.5 * 2^23
    float kf = Fast::fma(a0, bits_f(NT2G_INVLOG_2), shifter);
    float k = Fast::sub(kf, shifter);
    int32_t ik = (int32_t)(f_bits(kf) - 0x4B400000u);
    float x = Fast::fma(-k, bits_f(NT2G_LOG_2HI), a0);
    x = Fast::fma(-k, bits_f(NT2G_LOG_2LO), x);
    float q = horner<Fast>(x, 0x1.a157b2p-13f, 0x1.6d4926p-10f, 0x1.1110c4p-7f, 0x1.5554e4p-5f,
                           0x1.555556p-3f, 0.5f);
    scale = bits_f((uint32_t)(ik + 127) << 23);
    return Fast::fma(q, Fast::mul(x, x), x);
}

template <class P> NT2G_HD float exp(float a0)
{
    if (P::exact) {
        if (a0 >= bits_f(NT2G_MAXLOG)) return f_inf();
        if (a0 <= bits_f(NT2G_MINLOG)) return 0.0f;
        if (is_nan(a0)) return a0;
        float k = rintf(P::mul(bits_f(NT2G_INVLOG_2), a0));
        float x = P::sub(a0, P::mul(k, bits_f(NT2G_LOG_2HI)));
        x = P::sub(x, P::mul(k, bits_f(NT2G_LOG_2LO)));
        float y = horner<P>(x, bits_f(0x3ab778cfu), bits_f(0x3c098d8bu), bits_f(0x3d2aa957u),
                            bits_f(0x3e2aa9a5u), bits_f(0x3f000000u));
        float c = P::add(P::fma(y, P::mul(x, x), x), 1.0f);
        return P::mul(c, bits_f((uint32_t)((int32_t)k + 127) << 23));
    }
    float scale;
    float s = exp_fast_parts(a0, scale);
    float r = Fast::mul(Fast::add(s, 1.0f), scale);
    r = (a0 >= bits_f(NT2G_MAXLOG)) ? f_inf() : r;
    r = (a0 <= bits_f(NT2G_MINLOG)) ? 0.0f : r;
    return is_nan(a0) ? a0 : r;
}

// float(p) rounded to nearest for a position 0 <= p < 2^46 (NT2's
// enumerate<float>(p)), without the 64-bit integer conversion: with
// p = hi 2^23 + lo, float(hi) and float(lo) are exact (the 2^23 bit-pattern
// trick) and one fused hi * 2^23 + lo rounds the exact sum once.
NT2G_HD float pos_to_float(long long p)
{
#if defined(__CUDA_ARCH__)
    if (p >= (1ll << 46)) return __ll2float_rn(p);
    const uint32_t lo = (uint32_t)p & 0x7fffffu, hi = (uint32_t)(p >> 23);
    const float flo = __fsub_rn(__uint_as_float(0x4B000000u | lo), 8388608.0f);
    const float fhi = __fsub_rn(__uint_as_float(0x4B000000u | hi), 8388608.0f);
    return __fmaf_rn(fhi, 8388608.0f, flo);
#else
    return (float)p;
#endif
}

// 2^k for k in [-126, 127] built in the exponent field (expo_scale.hpp:27-35)
NT2G_HD float pow2i(float k) { return bits_f((uint32_t)((int32_t)k + 127) << 23); }

// ----------------------------------------------------------- exp2, exp10 --
// NT2: the float exponential driver of scalar/impl/expo/expo_base.hpp:55-69
// with the two_ / ten_tag reductions of f_expo_reduction.hpp:88-126, 129-168:
//   exp2:  k = round2even(x), r = x - k, 2^r = 1 + (P5(r) r^2 + r ln2);
//   exp10: k = round2even(x log2(10)), r = x - k log10(2)hi - k log10(2)lo,
//          10^r = 1 + P6(r) r;
// each result scaled by 2^k; +inf from Maxlog2 / Maxlog10, 0 at Minlog2 /
// Minlog10 and below.  Fast: the same steps with FMAs, specials by select.
template <class P> NT2G_HD float exp2(float a0)
{
    if (P::exact) {
        if (a0 >= bits_f(NT2G_MAXLOG2)) return f_inf();
        if (a0 <= bits_f(NT2G_MINLOG2)) return 0.0f;
        if (is_nan(a0)) return a0;
    }
    const float k = rintf(a0);
    const float x = P::sub(a0, k);
    const float y = horner<P>(x, bits_f(0x3922c8c4u), bits_f(0x3ab01218u), bits_f(0x3c1d9422u),
                              bits_f(0x3d6356ebu), bits_f(0x3e75fdf1u));
    const float c = P::add(P::fma(y, P::mul(x, x), P::mul(x, bits_f(NT2G_LOG_2))), 1.0f);
    if (P::exact) return P::mul(c, pow2i(k));
    float r = P::mul(c, pow2i(fminf(fmaxf(k, -127.0f), 127.0f)));
    r = (a0 >= bits_f(NT2G_MAXLOG2)) ? f_inf() : r;
    r = (a0 <= bits_f(NT2G_MINLOG2)) ? 0.0f : r;
    return is_nan(a0) ? a0 : r;
}

template <class P> NT2G_HD float exp10(float a0)
{
    if (P::exact) {
        if (a0 >= bits_f(NT2G_MAXLOG10)) return f_inf();
        if (a0 <= bits_f(NT2G_MINLOG10)) return 0.0f;
        if (is_nan(a0)) return a0;
    }
    const float k = rintf(P::mul(bits_f(NT2G_INVLOG10_2), a0));
    float x = P::fma(-k, bits_f(NT2G_LOG10_2HI), a0);
    x = P::sub(x, P::mul(k, bits_f(NT2G_LOG10_2LO)));
    const float y = horner<P>(x, bits_f(0x3e54dff1u), bits_f(0x3f0aacefu), bits_f(0x3f95eb4cu),
                              bits_f(0x400237dau), bits_f(0x4029a926u), bits_f(0x40135d8eu));
    const float c = P::add(P::mul(y, x), 1.0f);
    if (P::exact) return P::mul(c, pow2i(k));
    float r = P::mul(c, pow2i(fminf(fmaxf(k, -127.0f), 127.0f)));
    r = (a0 >= bits_f(NT2G_MAXLOG10)) ? f_inf() : r;
    r = (a0 <= bits_f(NT2G_MINLOG10)) ? 0.0f : r;
    return is_nan(a0) ? a0 : r;
}

// ----------------------------------------------------------------- expm1 --
// NT2 (scalar/expm1.hpp:33-41, details/expm1_kernel.hpp:49-73): NaN -> NaN,
// x < Logeps -> -1, x > Maxlog -> +inf, else k = round2even(x/ln2), r by
// Cody-Waite, hx = r/2, hxs = r*hx, r1 = 1 + hxs*(c2 + hxs*c1),
// t = 3 - r1*hx, e = hxs*((r1 - t)/(6 - r*t)), e = r*e - hxs,
// y = (1 - 2^-k) - (e - r), expm1 = y * 2^k.
template <class P> NT2G_HD float expm1(float a0)
{
    if (P::exact) {
        if (is_nan(a0)) return f_nan();
        if (a0 < bits_f(NT2G_LOGEPS)) return -1.0f;
        if (a0 > bits_f(NT2G_MAXLOG)) return f_inf();
    }
    // out-of-range arguments take a harmless value through the kernel (fast: selected away)
    const float a = P::exact ? a0 : fminf(fmaxf(a0, bits_f(NT2G_LOGEPS)), bits_f(NT2G_MAXLOG));
    const float k = rintf(P::mul(bits_f(NT2G_INVLOG_2), a));
    float x = P::fma(-k, bits_f(NT2G_LOG_2HI), a);
    x = P::fma(-k, bits_f(NT2G_LOG_2LO), x);
    const float hx = P::mul(x, 0.5f);
    const float hxs = P::mul(x, hx);
    const float r1 = horner<P>(hxs, bits_f(0x3acf6db4u), bits_f(0xbd08887fu), bits_f(0x3f800000u));
    const float t = P::fma(-r1, hx, 3.0f);
    float e = P::mul(hxs, P::div(P::sub(r1, t), P::fma(-x, t, 6.0f)));
    e = P::fma(x, e, -hxs);
    const int32_t ik = (int32_t)k;
    const float two2mk = bits_f((uint32_t)(127 - ik) << 23);
    const float y = P::sub(P::sub(1.0f, two2mk), P::sub(e, x));
    float r = P::mul(y, pow2i(k));  // fast_ldexp: y * 2^k (boost/simd/ieee/functions/scalar/fast_ldexp.hpp)
    if (!P::exact) {
        r = (a0 < bits_f(NT2G_LOGEPS)) ? -1.0f : r;
        r = (a0 > bits_f(NT2G_MAXLOG)) ? f_inf() : r;
        r = is_nan(a0) ? f_nan() : r;
    }
    return r;
}

// ------------------------------------------------------------------ log --
// NT2's float logarithms (scalar/impl/logs/f_log.hpp:59-153) share one
// reduction (f_kernel.hpp:43-75): a0 = 2^fe * (1 + x) with 1 + x in
// [sqrt(1/2), sqrt(2)), x2 = x^2, y = P8(x) * x * x2.  Denormal arguments are
// first scaled by 2^23 and the matching -23 log_b(2) is added back as t.
struct LogParts { float fe, x, x2, y, t; };

template <class P> NT2G_HD LogParts log_reduce(float a0, uint32_t mlog_two2nmb)
{
    LogParts r;
    float z = a0;
    r.t = 0.0f;
    bool den = fabsf(z) < bits_f(NT2G_SMALLESTPOS);
    if (P::exact) {
        if (den) { z = P::mul(z, bits_f(NT2G_TWOTONMB)); r.t = bits_f(mlog_two2nmb); }
    } else {
        z = den ? P::mul(z, bits_f(NT2G_TWOTONMB)) : z;
        r.t = den ? bits_f(mlog_two2nmb) : 0.0f;
    }
    uint32_t u = f_bits(z);
    int32_t e = (int32_t)((u & 0x7f800000u) >> 23) - 126;
    float x = bits_f((u & ~0x7f800000u) | 0x3f000000u);
    bool lt = x < bits_f(NT2G_SQRT_2O_2);
    r.fe = lt ? P::add((float)e, -1.0f) : (float)e;
    r.x = P::sub(lt ? P::add(x, x) : x, 1.0f);
    r.x2 = P::mul(r.x, r.x);
    float y = horner<P>(r.x, bits_f(0xbda5dff0u), bits_f(0x3e0229f9u), bits_f(0xbe04d6b7u),
                        bits_f(0x3e116e80u), bits_f(0xbe2a6aa0u), bits_f(0x3e4cd0a3u),
                        bits_f(0xbe800064u), bits_f(0x3eaaaaa9u));
    r.y = P::mul(P::mul(y, r.x), r.x2);
    return r;
}

// The special values of every float logarithm: log_b(+inf) = +inf,
// log_b(0) = -inf, NaN for NaN and negative arguments.
template <class P> NT2G_HD float log_specials(float a0, float r)
{
    r = (a0 == f_inf()) ? a0 : r;
    r = (a0 == 0.0f) ? -f_inf() : r;
    return (is_nan(a0) || a0 < 0.0f) ? f_nan() : r;
}

#define NT2G_LOG_SPECIALS_EXACT(a0)                                   \
    if (P::exact) {                                                   \
        if (a0 == f_inf()) return a0;                                 \
        if (a0 == 0.0f) return -f_inf();                              \
        if (is_nan(a0) || a0 < 0.0f) return f_nan();                  \
    }

template <class P> NT2G_HD float log(float a0)
{
    NT2G_LOG_SPECIALS_EXACT(a0)
    const LogParts k = log_reduce<P>(a0, NT2G_MLOGTWO2NMB);
    float y = P::fma(k.fe, bits_f(NT2G_LOG_2LO), k.y);
    y = P::fma(-0.5f, k.x2, y);
    float r = P::fma(bits_f(NT2G_LOG_2HI), k.fe, P::add(P::add(k.x, y), k.t));
    return P::exact ? r : log_specials<P>(a0, r);
}

// log2 (f_log.hpp:90-119): y += -x2/2, z = x*log2(e)-1 + y*(log2(e)-1),
// log2 = ((z + y) + x) + fe (+ t)
template <class P> NT2G_HD float log2(float a0)
{
    NT2G_LOG_SPECIALS_EXACT(a0)
    const LogParts k = log_reduce<P>(a0, NT2G_MLOG2TWO2NMB);
    const float y = P::fma(-0.5f, k.x2, k.y);
    const float z = P::fma(k.x, bits_f(NT2G_LOG2_EM1), P::mul(y, bits_f(NT2G_LOG2_EM1)));
    float r = P::add(P::add(P::add(P::add(z, y), k.x), k.fe), k.t);
    return P::exact ? r : log_specials<P>(a0, r);
}

// log10 (f_log.hpp:121-153): with log10(e) = ehi + elo and log10(2) = 2hi + 2lo,
// z = (x + y)*elo + y*ehi + x*ehi + fe*2hi, log10 = (z + t) + fe*2lo
template <class P> NT2G_HD float log10(float a0)
{
    NT2G_LOG_SPECIALS_EXACT(a0)
    const LogParts k = log_reduce<P>(a0, NT2G_MLOG10TWO2NMB);
    const float y = P::fma(-0.5f, k.x2, k.y);
    float z = P::mul(P::add(k.x, y), bits_f(NT2G_LOG10_ELO));
    z = P::fma(y, bits_f(NT2G_LOG10_EHI), z);
    z = P::fma(k.x, bits_f(NT2G_LOG10_EHI), z);
    z = P::fma(k.fe, bits_f(NT2G_LOG10_2HI), z);
    float r = P::fma(k.fe, bits_f(NT2G_LOG10_2LO), P::add(z, k.t));
    return P::exact ? r : log_specials<P>(a0, r);
}
#undef NT2G_LOG_SPECIALS_EXACT

// ---------------------------------------------------------------- log1p --
template <class P> NT2G_HD float log1p(float a0)
{
    if (P::exact) {
        if (-1.0f > a0) return f_nan();
        if (a0 == f_inf()) return f_inf();
        if (a0 == -1.0f) return -f_inf();
    }
    float u = P::add(1.0f, a0);
    float r;
    if (P::exact) {
        r = P::add(log<P>(u), P::div(P::sub(a0, P::sub(u, 1.0f)), u));
    } else {
        // u == 1 exactly (tiny a0): log(u) = 0, correction a0/1; the division
        // runs only on normal u, so rcp.approx stays in range.
        float uu = (u > 0.0f && u < f_inf()) ? u : 1.0f;
        r = P::add(log<P>(u), P::div(P::sub(a0, P::sub(u, 1.0f)), uu));
        r = (a0 == f_inf()) ? f_inf() : r;
        r = (a0 == -1.0f) ? -f_inf() : r;
        r = (-1.0f > a0 || is_nan(a0)) ? f_nan() : r;
    }
    return r;
}

// ------------------------------------------------------- NT2 erfc core --
// erfc(|x|) before the sign fold (EUL/scalar/erfc.hpp:85-101).
template <class P> NT2G_HD float erfc_core_nt2(float x)
{
    float z = P::div(x, P::add(x, 1.0f));
    if (x < bits_f(NT2G_TWOTHIRD))
        return P::mul(P::sub(1.0f, z),
                      horner<P>(z, bits_f(0x41aa8e55u), bits_f(0x401b5680u), bits_f(0xc010d956u),
                                bits_f(0x3f2cff3bu), bits_f(0xc016c985u), bits_f(0xbffc9284u),
                                bits_f(0xbfa11698u), bits_f(0xbe036d7eu), bits_f(0x3f7ffffeu)));
    if (x == f_inf()) return 0.0f;
    z = P::sub(z, 0.4f);
    return P::mul(exp<P>(-P::mul(x, x)),
                  horner<P>(z, bits_f(0xc0283611u), bits_f(0x40d67e3bu), bits_f(0xc0cd1a85u),
                            bits_f(0x4050b063u), bits_f(0xbfaea865u), bits_f(0x3e2006f0u),
                            bits_f(0x3e1175c7u), bits_f(0x3ec4ca6eu), bits_f(0x3e243828u),
                            bits_f(0xbf918a62u), bits_f(0x3f0a0e8bu)));
}

// ----------------------------------------------------- fast erfc tail --
// For t >= 0:  erfc(t) = exp(-t^2) * w * R(w),  w = 1/(1 + t/2).
// R is a degree-10 fit in w - 1/2 (coefficients from fit_erfc.py, highest
// degree first).  exp(-t^2) is evaluated as exp(-hi) * (1 - lo) with hi + lo = t^2
// exactly (FMA split), so the rounding of t^2 is not amplified in the tail.
NT2G_HD float erfc_tail_poly(float w)
{
    // polynomial in d = w - 1/2 (exact for w >= 1/4; below that the rounding
    // is an absolute 2^-26 that R barely feels)
    float d = Fast::sub(w, 0.5f);
    return horner<Fast>(d, 0x1.5af3d4p-5f, -0x1.38d8fcp-6f, -0x1.382c16p-4f, 0x1.c51560p-5f,
                        0x1.908f48p-4f, -0x1.a94032p-4f, -0x1.604ccep-3f, 0x1.2a8c2ep-3f,
                        0x1.1e2dc2p-1f, 0x1.5fd384p-1f, 0x1.058672p-1f);
}

// Tail value T(a) for a >= 0 with scale s:
//   s = 1      : T = erfc(a)
//   s = 1/sqrt2: T = erfc(a/sqrt2) = 2*normcdf(-a)
// computed as exp(-(s*a)^2) * w * R(w), w = 1/(1 + (s/2)*a).  The square is
// the exact split a^2 = hi + lo times s^2 (1 or 1/2: exact), and
// exp(-s^2*hi) = (1 + e) * 2^k with e corrected for lo, so the result is
// 2^k * fma(e, wR, wR): one rounding for the exponential's "+1" and the
// product together.
template <bool HALF_SQ> NT2G_HD float erfc_tail_fast(float a)
{
    const float q = HALF_SQ ? 0.353553390593273762f : 0.5f;  // (1/2)*s
    // w ~ 1/den, den = 1 + q*a held as den + dlo.  The polynomial takes the
    // rounded w; the multiplier uses w*(1 + r), r the residual of w against
    // den + dlo, so the rounding of w and of den only reaches the result
    // through R(w), whose log-derivative is <= 1.3 (<= 2.3 for w itself).
    float den = Fast::fma(q, a, 1.0f);
    float dlo = Fast::fma(q, a, Fast::sub(1.0f, den));
    float w = Fast::rcp(den);
    w = Fast::fma(w, Fast::fma(-den, w, 1.0f), w);
    float r = Fast::fma(-dlo, w, Fast::fma(-den, w, 1.0f));
    float hi = Fast::mul(a, a);
    float lo = Fast::fma(a, a, -hi);
    const float s2 = HALF_SQ ? -0.5f : -1.0f;
    float scale;
    float e = exp_fast_parts(Fast::mul(s2, hi), scale);
    // fold the square's low part L = s2*lo (|L| < 2^-18) and the reciprocal
    // residual r into the small term: (1+e)(1+L)(1+r) - 1 = e + c + c*e,
    // c = L + r (c*e and L*r are below 2^-40 relative)
    float c = Fast::fma(s2, lo, r);
    e = Fast::add(e, Fast::fma(c, e, c));
    float wr = Fast::mul(w, erfc_tail_poly(w));
    float res = Fast::mul(Fast::fma(e, wr, wr), scale);
    // past amax the exponential leaves the normal range (its 2^k scale would
    // underflow) and the true value is subnormal; the guard also keeps inf*0
    // out of the split for a = inf.
    const float amax = HALF_SQ ? 13.2f : 9.3f;
    return (a < amax) ? res : 0.0f;
}

// ---------------------------------------------------------------- erfc --
template <class P> NT2G_HD float erfc(float a0)
{
    if (P::exact) {
        float r1 = erfc_core_nt2<P>(fabsf(a0));
        return (a0 < 0.0f) ? P::sub(2.0f, r1) : r1;
    }
    float r1 = erfc_tail_fast<false>(fabsf(a0));
    r1 = (a0 < 0.0f) ? Fast::sub(2.0f, r1) : r1;
    return is_nan(a0) ? a0 : r1;
}

// -------------------------------------------------------------- normcdf --
// NT2: Half*erfc(-Sqrt_2o_2*x).  Both the call and the put of a fused
// Black-Scholes need N(d) and N(-d): normcdf_pair returns both from one erfc
// core, which in NT2 arithmetic is bit-identical to two separate calls
// (|-c*d| == |c*d|; only the final 2-r select differs).
template <class P> NT2G_HD void normcdf_pair(float x, float &n_pos, float &n_neg)
{
    if (P::exact) {
        float t = P::mul(-bits_f(NT2G_SQRT_2O_2), x);
        float r1 = erfc_core_nt2<P>(fabsf(t));
        float r2 = P::sub(2.0f, r1);
        // erfc(t): t<0 -> 2-r1.  normcdf(x) = 0.5*erfc(t), normcdf(-x) = 0.5*erfc(-t)
        n_pos = P::mul(0.5f, (t < 0.0f) ? r2 : r1);
        n_neg = P::mul(0.5f, (-t < 0.0f) ? r2 : r1);
        return;
    }
    float half_tail = Fast::mul(0.5f, erfc_tail_fast<true>(fabsf(x)));  // normcdf(-|x|)
    float other = Fast::sub(1.0f, half_tail);
    bool neg = x < 0.0f;
    n_pos = neg ? half_tail : other;
    n_neg = neg ? other : half_tail;
    if (is_nan(x)) { n_pos = x; n_neg = x; }
}

template <class P> NT2G_HD float normcdf(float x)
{
    float a, b;
    normcdf_pair<P>(x, a, b);
    return a;
}

// ---------------------------------------------------------- fastnormcdf --
// NT2's Abramowitz-Stegun 26.2.17 form, identical in both policies except
// for fusion.  (Its absolute error is ~7.5e-8 by construction.)
template <class P> NT2G_HD float fastnormcdf(float a0)
{
    // Fast: clamp |x| (the result saturates long before 100) so the
    // approximate reciprocal never sees inf; NaN is restored at the end.
    float l = P::exact ? fabsf(a0) : fminf(fabsf(a0), 100.0f);
    float k = P::fdiv(1.0f, P::fma(0.2316419f, l, 1.0f));
    float w = horner<P>(k, bits_f(0x3faa466fu), bits_f(0xbfe91eeau), bits_f(0x3fe40778u),
                        bits_f(0xbeb68f87u), bits_f(0x3ea385fau));
    w = P::mul(w, P::mul(P::mul(k, bits_f(NT2G_INVSQRT_2PI)),
                         exp<P>(P::mul(-P::mul(l, l), 0.5f))));
    float r = (a0 > 0.0f) ? P::sub(1.0f, w) : w;
    return (!P::exact && is_nan(a0)) ? a0 : r;
}

template <class P> NT2G_HD float sqr(float x) { return P::mul(x, x); }

// exp(-sqr(x)).  NT2: the rounded square is exponentiated (its rounding is
// amplified by x^2).  Fast: exp(-hi) * (1 - lo) with hi + lo = x^2 exactly.
template <class P> NT2G_HD float exp_neg_sqr(float x)
{
    if (P::exact) return exp<P>(-P::mul(x, x));
    float hi = Fast::mul(x, x);
    float lo = Fast::fma(x, x, -hi);
    float scale;
    float s = exp_fast_parts(-hi, scale);
    s = Fast::add(s, Fast::fma(-lo, s, -lo));  // (1+s)(1-lo) - 1
    float r = Fast::mul(Fast::add(s, 1.0f), scale);
    r = (-hi <= bits_f(NT2G_MINLOG)) ? 0.0f : r;
    return is_nan(x) ? x : r;
}

// ------------------------------------------------------------------- pow --
// NT2's float pow (exponential/functions/scalar/pow.hpp:28-36 over
// pow_abs.hpp:31-84 and details/pow_kernel.hpp:43-125, Cephes' powf): x = |a|
// split by frexp, log2 of the significand against a 2^(-i/16) table, the
// product with b carried in multiples of 1/16 plus remainders, then 2^w from a
// degree-4 polynomial, the table and ldexp.  Special values as NT2 has them:
// pow(+-1 magnitude ...) = 1, pow(0, b) = (b == 0), NaN for a < 0 and a
// non-integer b, the sign of a for odd integer b.
NT2G_HD float pow_twomio16(int i)  // 2^(-i/16) rounded to 24 bits, i in [0, 16]
{
    switch (i) {
    case 0: return bits_f(0x3f800000u);  case 1: return bits_f(0x3f75257du);
    case 2: return bits_f(0x3f6ac0c7u);  case 3: return bits_f(0x3f60ccdfu);
    case 4: return bits_f(0x3f5744fdu);  case 5: return bits_f(0x3f4e248cu);
    case 6: return bits_f(0x3f45672au);  case 7: return bits_f(0x3f3d08a4u);
    case 8: return bits_f(0x3f3504f3u);  case 9: return bits_f(0x3f2d583fu);
    case 10: return bits_f(0x3f25fed7u); case 11: return bits_f(0x3f1ef532u);
    case 12: return bits_f(0x3f1837f0u); case 13: return bits_f(0x3f11c3d3u);
    case 14: return bits_f(0x3f0b95c2u); case 15: return bits_f(0x3f05aac3u);
    default: return bits_f(0x3f000000u);
    }
}

NT2G_HD float pow_continuation(int i)  // 2^(i/8) - twomio16(2i), i in [0, 8]
{
    switch (i) {
    case 1: return bits_f(0xb1c116deu); case 2: return bits_f(0xb254a58au);
    case 3: return bits_f(0x318aa837u); case 4: return bits_f(0x324fe77au);
    case 5: return bits_f(0xb2ac9d5eu); case 6: return bits_f(0x32a31b71u);
    case 7: return bits_f(0xb1e0aba1u); default: return 0.0f;
    }
}

// NT2's ldexp (boost/simd/ieee/functions/scalar/ldexp.hpp:37-51): a * 2^e * f,
// with f = 2^-126 carrying exponents below -126 and f = 2 the exponent 128.
template <class P> NT2G_HD float nt2_ldexp(float a, int e)
{
    float f = 1.0f;
    if (e < -126) { e += 126; f = bits_f(0x00800000u); }
    const int b = e == 128;
    f = P::add(f, (float)b);
    e = e - b + 127;
    return P::mul(P::mul(a, bits_f((uint32_t)e << 23)), f);
}

NT2G_HD bool is_flint(float x) { return (x - truncf(x)) == 0.0f; }      // false for +-inf, NaN
NT2G_HD bool is_odd_f(float x) { return is_flint((x - 1.0f) * 0.5f); }

// Fast: this file's own pow for finite x > 0, x != 1: log2(x) in float-float
// (x = 2^e m, m in [sqrt(1/2), sqrt(2)], log m = 2 atanh(s), s = (m-1)/(m+1)
// carried as s_hi + s_lo, the series tail in float), times b in float-float,
// then 2^(k + f) with k = round(p_hi), a degree-7 Taylor polynomial of 2^f and
// the scale applied in two exact halves so subnormal results round once.
NT2G_HD float pow_core_fast(float x, float y)
{
    int e = 0;
    if (x < 1.17549435e-38f) { x = Fast::mul(x, 8388608.0f); e = -23; }
    const uint32_t u = f_bits(x);
    e += (int)(u >> 23) - 127;
    float m = bits_f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421354f) { m = Fast::mul(m, 0.5f); e += 1; }
    const float num = Fast::sub(m, 1.0f);                       // exact
    const float den = Fast::add(m, 1.0f);
    const float den_lo = Fast::sub(m, Fast::sub(den, 1.0f));    // m + 1 = den + den_lo exactly
    const float r = Fast::div(1.0f, den);
    const float s_hi = Fast::mul(num, r);
    const float res = Fast::fma(-s_hi, den_lo, Fast::fma(-s_hi, den, num));
    const float s_lo = Fast::mul(res, r);
    // log m = 2 s + (2/3) s^3 + s^5 R(s^2): s^3 and its (2/3) in float-float, the
    // rest in float (it is below 2e-4 of log m)
    const float q_hi = Fast::mul(s_hi, s_hi);
    const float q_lo = Fast::fma(s_hi, s_hi, -q_hi);
    const float c3_hi = Fast::mul(s_hi, q_hi);
    const float c3_lo = Fast::fma(s_hi, q_lo, Fast::fma(s_hi, q_hi, -c3_hi));
    const float TT_hi = 0x1.555556p-1f, TT_lo = -0x1.555556p-26f;  // 2/3
    const float t3_hi = Fast::mul(c3_hi, TT_hi);
    const float t3_lo = Fast::fma(c3_lo, TT_hi, Fast::fma(c3_hi, TT_lo, Fast::fma(c3_hi, TT_hi, -t3_hi)));
    const float rest = Fast::mul(Fast::mul(c3_hi, q_hi),
                                 horner<Fast>(q_hi, 0x1.3b13b2p-3f, 0x1.745d18p-3f, 0x1.c71c72p-3f, 0x1.24924ap-2f,
                                              0x1.99999ap-2f));
    // 2 s_lo (1 + s^2) carries s_lo through the first two terms
    const float lo_sum = Fast::add(Fast::fma(2.0f * s_lo, q_hi, 2.0f * s_lo), Fast::add(t3_lo, rest));
    const float h0 = Fast::add(s_hi, s_hi);
    const float h = Fast::add(h0, t3_hi);
    const float l = Fast::add(Fast::add(Fast::sub(h0, h), t3_hi), lo_sum);
    const float l_hi = Fast::add(h, l);
    const float l_lo = Fast::add(Fast::sub(h, l_hi), l);
    // log2 m = log m * log2(e), log2(e) = C_hi + C_lo
    const float C_hi = 0x1.715476p+0f, C_lo = 0x1.4ae0c0p-26f;
    const float g_hi = Fast::mul(l_hi, C_hi);
    const float g_lo = Fast::add(Fast::fma(l_hi, C_hi, -g_hi), Fast::fma(l_lo, C_hi, Fast::mul(l_hi, C_lo)));
    // + e (|e| >= 1 > |g_hi| unless e = 0): fast two-sum
    const float fe = (float)e;
    const float t_hi = Fast::add(fe, g_hi);
    const float t_lo = Fast::add(Fast::add(Fast::sub(fe, t_hi), g_hi), g_lo);
    // p = y log2 x
    const float p_hi = Fast::mul(y, t_hi);
    const float p_lo = Fast::fma(y, t_lo, Fast::fma(y, t_hi, -p_hi));
    if (!(p_hi < 129.0f)) return f_inf();
    if (!(p_hi > -152.0f)) return 0.0f;
    const float k = rintf(p_hi);
    const float f = Fast::add(Fast::sub(p_hi, k), p_lo);       // |f| <= 1/2 + tiny
    const float c = horner<Fast>(f, 0x1.ffcbfcp-17f, 0x1.430912p-13f, 0x1.5d87fep-10f, 0x1.3b2ab6p-7f,
                                 0x1.c6b08ep-5f, 0x1.ebfbe0p-3f, 0x1.62e430p-1f);
    const float v = Fast::fma(c, f, 1.0f);
    const int ki = (int)k, k1 = ki >> 1, k2 = ki - k1;             // each within [-76, 65]
    return Fast::mul(Fast::mul(v, bits_f((uint32_t)(k1 + 127) << 23)), bits_f((uint32_t)(k2 + 127) << 23));
}

template <class P> NT2G_HD float pow_abs(float a0, float a1)
{
    float x = fabsf(a0);
    if (x == 1.0f) return x;
    if (x == 0.0f) return a1 == 0.0f ? 1.0f : 0.0f;
    if (x == a1 && a1 == f_inf()) return f_inf();
    if (x == f_inf() && a1 == -f_inf()) return 0.0f;
    if (a1 == f_inf()) return (x < 1.0f) ? 0.0f : f_inf();
    if (a1 == -f_inf()) return (x > 1.0f) ? 0.0f : f_inf();
    if (x == f_inf()) return (a1 < 0.0f) ? 0.0f : ((a1 == 0.0f) ? 1.0f : f_inf());
    if (is_nan(a0) || is_nan(a1)) return f_nan();
    if (!P::exact) return pow_core_fast(x, a1);
    // frexp: x = m 2^e, m in [1/2, 1) (denormals through a 2^23 scale)
    int e;
    {
        uint32_t u = f_bits(x);
        int t = 0;
        if ((u & 0x7f800000u) == 0) { u = f_bits(P::mul(x, 8388608.0f)); t = 23; }
        e = (int)((u & 0x7f800000u) >> 23) - 126 - t;
        x = bits_f((u & ~0x7f800000u) | 0x3f000000u);
    }
    // select: the table entry nearest below m (pow_kernel.hpp:111-125)
    int i = 1;
    if (x <= pow_twomio16(9)) i = 9;
    if (x <= pow_twomio16(i + 4)) i += 4;
    if (x <= pow_twomio16(i + 2)) i += 2;
    if (x >= pow_twomio16(1)) i = -1;
    i += 1;
    const float tmp = pow_twomio16(i);
    x = P::sub(x, tmp);
    x = P::sub(x, pow_continuation(i >> 1));
    x = P::div(x, tmp);
    float z = P::mul(x, x);
    float w = P::mul(P::mul(z, x), horner<P>(x, bits_f(0xbe2a61b2u), bits_f(0x3e4d2fa3u), bits_f(0xbe800015u),
                                                 bits_f(0x3eaaaaa3u)));
    w = P::fma(-0.5f, z, w);
    w = P::fma(bits_f(NT2G_LOG2_EM1), w, w);
    z = P::fma(bits_f(NT2G_LOG2_EM1), x, w);
    z = P::add(z, x);
    w = P::fma((float)(-i), 0.0625f, (float)e);
    // b log2(x) in multiples of 1/16 plus remainders (reduc: a multiple of 1/16 within 1/16)
    const float ya = P::mul(0.0625f, floorf(P::mul(16.0f, a1)));
    const float yb = P::sub(a1, ya);
    float W = P::fma(z, a1, P::mul(w, yb));
    float Wa = P::mul(0.0625f, floorf(P::mul(16.0f, W)));
    float Wb = P::sub(W, Wa);
    W = P::fma(w, ya, Wa);
    Wa = P::mul(0.0625f, floorf(P::mul(16.0f, W)));
    const float u = P::sub(W, Wa);
    W = P::add(Wb, u);
    Wb = P::mul(0.0625f, floorf(P::mul(16.0f, W)));
    w = P::mul(16.0f, P::add(Wa, Wb));
    if (w > bits_f(0x44ffe000u)) return f_inf();  // Powlargelim
    if (w < bits_f(0xc5160000u)) return 0.0f;     // Powlowlim
    e = (int)w;
    Wb = P::sub(W, Wb);
    if (Wb > 0.0f) { ++e; Wb = P::sub(Wb, 0.0625f); }
    z = P::mul(horner<P>(Wb, bits_f(0x3c1a49bcu), bits_f(0x3d634d38u), bits_f(0x3e75fde1u), bits_f(0x3f317218u)), Wb);
    i = e / 16 + (e >= 0);
    e = i * 16 - e;
    w = pow_twomio16(e);
    z = P::fma(w, z, w);
    return nt2_ldexp<P>(z, i);
}

template <class P> NT2G_HD float pow(float a0, float a1)
{
    const bool neg = a0 < 0.0f;
    if (neg && !is_flint(a1)) return f_nan();
    const float z = pow_abs<P>(a0, a1);
    return (neg && is_odd_f(a1)) ? -z : z;
}

// ------------------------------------------------------------ hyperbolic --
// NT2 (modules/core/hyperbolic/include/nt2/hyperbolic/functions/):
//   sinh  scalar/sinh.hpp:35-58, |x| < 1 by the degree-3 polynomial of
//         details/sinh_kernel.hpp:24-35, else (e - 1/e)/2 with e = exp|x|, or
//         (e^(x/2)/2) e^(x/2) beyond Maxlog - log 2; the sign of x
//   cosh  generic/cosh.hpp:33-43, average(e, 1/e) or (e^(x/2)/2) e^(x/2)
//   tanh  scalar/tanh.hpp:33-50, |x| < 5/8 by details/tanh_kernel.hpp:27-40,
//         else 1 - 2/(1 + e^(2|x|)); the sign of x
template <class P> NT2G_HD float sinh(float a0)
{
    const float x = fabsf(a0);
    if (x < 1.0f) {
        const float x2 = P::mul(x, x);
        return P::mul(horner<P>(x2, bits_f(0x39559e2fu), bits_f(0x3c087bbeu), bits_f(0x3e2aaaccu), 1.0f), a0);
    }
    float r;
    if (x > P::sub(bits_f(NT2G_MAXLOG), bits_f(NT2G_LOG_2))) {
        const float t = exp<P>(P::mul(0.5f, x));
        r = P::mul(P::mul(0.5f, t), t);
    } else {
        const float t = exp<P>(x);
        r = P::fma(t, 0.5f, -P::mul(0.5f, P::div(1.0f, t)));
    }
    return bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u));
}

template <class P> NT2G_HD float cosh(float a0)
{
    const float x = fabsf(a0);
    const bool big = x > P::sub(bits_f(NT2G_MAXLOG), bits_f(NT2G_LOG_2));
    const float t = exp<P>(P::mul(x, big ? 0.5f : 1.0f));
    if (big) return P::mul(P::mul(0.5f, t), t);
    return P::fma(t, 0.5f, P::mul(P::div(1.0f, t), 0.5f));
}

template <class P> NT2G_HD float tanh(float a0)
{
    const float x = fabsf(a0);
    if (x < 0.625f) {
        const float x2 = P::mul(x, x);
        const float y = horner<P>(x2, bits_f(0xbbbaf0eau), bits_f(0x3ca9134eu), bits_f(0xbd5c1e2du),
                                  bits_f(0x3e088393u), bits_f(0xbeaaaa99u));
        return P::fma(P::mul(y, x2), a0, a0);
    }
    const float r = P::fma(-2.0f, P::div(1.0f, P::add(1.0f, exp<P>(P::add(x, x)))), 1.0f);
    return bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u));
}

// coth (scalar/coth.hpp): below 5/8 the reciprocal of the tanh kernel, else
// 1 + 2/(e^(2|x|) - 1); the sign of x
template <class P> NT2G_HD float coth(float a0)
{
    const float x = fabsf(a0);
    float r;
    if (x < 0.625f) {
        const float x2 = P::mul(x, x);
        const float y = horner<P>(x2, bits_f(0xbbbaf0eau), bits_f(0x3ca9134eu), bits_f(0xbd5c1e2du),
                                  bits_f(0x3e088393u), bits_f(0xbeaaaa99u));
        r = P::div(1.0f, P::fma(P::mul(y, x2), x, x));
    } else {
        r = P::fma(2.0f, P::div(1.0f, P::sub(exp<P>(P::add(x, x)), 1.0f)), 1.0f);
    }
    return bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u));
}

// sinhc = sinh(x)/x (scalar/sinhc.hpp): +inf at +-inf; below 1 the degree-3
// polynomial of details/sinhc_kernel.hpp in x^2; else average(e, -1/e)/x with
// e = e^|x|, or ((e/2)/|x|) e with e = e^(|x|/2) beyond Maxlog - log 2
template <class P> NT2G_HD float sinhc(float a0)
{
    const float x = fabsf(a0);
    if (x == f_inf()) return x;
    if (x < 1.0f)
        return horner<P>(P::mul(x, x), bits_f(0x39559e2fu), bits_f(0x3c087bbeu), bits_f(0x3e2aaaccu), 1.0f);
    const bool big = x > P::sub(bits_f(NT2G_MAXLOG), bits_f(NT2G_LOG_2));
    const float t = exp<P>(P::mul(x, big ? 0.5f : 1.0f));
    if (big) return P::mul(P::div(P::mul(0.5f, t), x), t);
    const float avg = P::fma(t, 0.5f, P::mul(-P::div(1.0f, t), 0.5f));  // average(t, -1/t)
    return P::div(avg, x);
}

// ------------------------------------------------- inverse trigonometry --
// NT2 (trigonometric/functions/scalar/impl/invtrig/f_invtrig.hpp:33-128,
// Cephes' asinf/atanf): asin by a degree-4 polynomial in x^2 (|x| <= 1/2) or
// in (1-|x|)/2 with pi/2 - 2 asin(sqrt(.)); acos from asin in three bands;
// atan reduced at tan(3pi/8) and tan(pi/8) with pi/2 and pi/4 carried in two
// parts; atan2 (scalar/atan2.hpp:30-46) from the atan kernel of |a/b|.
template <class P> NT2G_HD float asin(float a0)
{
    float x = fabsf(a0);
    const uint32_t sign = f_bits(a0) & 0x80000000u;
    if (x < bits_f(0x38d1b717u)) return a0;  // 1e-4
    if (x > 1.0f) return f_nan();
    const bool big = x > 0.5f;
    float z;
    if (big) {
        z = P::mul(0.5f, P::sub(1.0f, x));
        x = P::sqrt(z);
    } else {
        z = P::mul(x, x);
    }
    float z1 = horner<P>(z, bits_f(0x3d2cb352u), bits_f(0x3cc617e3u), bits_f(0x3d3a3ec7u), bits_f(0x3d9980f6u),
                         bits_f(0x3e2aaae4u));
    if (!P::exact && big) {
        // Fast: pi/2 - 2 (s + s z p(z)) with s's rounding error (from the
        // residual z - s^2) and pi/2's low part carried, and the subtraction
        // from pi/2 split exactly (Fast2Sum: 2s <= 1 < pi/2): 2.3 -> 0.6 ulp
        const float slo = (z > 0.0f) ? P::mul(P::fma(-x, x, z), P::div(0.5f, x)) : 0.0f;
        const float t = P::fma(P::mul(z1, z), x, slo);
        const float hi = P::fma(-2.0f, x, bits_f(0x3fc90fdbu));
        const float err = P::fma(-2.0f, x, P::sub(bits_f(0x3fc90fdbu), hi));
        z1 = P::add(hi, P::add(err, P::fma(-2.0f, t, bits_f(0xb33bbd2eu))));
        return bits_f(f_bits(z1) ^ sign);
    }
    z1 = P::fma(z1, P::mul(z, x), x);
    if (big) {
        z1 = P::add(z1, z1);
        z1 = P::sub(bits_f(0x3fc90fdbu), z1);  // Pio_2
    }
    return bits_f(f_bits(z1) ^ sign);
}

template <class P> NT2G_HD float acos(float a0)
{
    if (a0 < -0.5f)
        return P::sub(bits_f(0x40490fdbu), P::mul(asin<P>(P::sqrt(P::mul(P::add(1.0f, a0), 0.5f))), 2.0f));
    if (a0 > 0.5f) return P::mul(asin<P>(P::sqrt(P::mul(P::sub(1.0f, a0), 0.5f))), 2.0f);
    return P::sub(bits_f(0x3fc90fdbu), asin<P>(a0));
}

// atan(|a0|) (NT2's kernel_atan: the sign is left to the caller)
// Fast: the reduced argument carried as xr + xl (the reciprocal's and the
// quotient's rounding errors from FMA residuals, (x-1)/(x+1) from exact sums)
// and the final y + xr split exactly, so that only the polynomial's own error
// and one rounding remain
NT2G_HD void two_sum_f(float a, float b, float &s, float &t)
{
    s = a + b;
    const float bb = s - a;
    t = (a - (s - bb)) + (b - bb);
}
NT2G_HD float atan_kernel_fast(float a0)
{
    if (a0 == 0.0f) return 0.0f;
    if (fabsf(a0) == f_inf()) return bits_f(0x3fc90fdbu);
    const float x = fabsf(a0);
    float y = 0.0f, more = 0.0f, xr = x, xl = 0.0f;
    if (x > bits_f(0x401a827au)) {  // tan(3 pi/8): pi/2 - atan(1/x)
        y = bits_f(0x3fc90fdbu);
        more = bits_f(0xb33bbd2eu);
        xr = Fast::div(-1.0f, x);
        xl = Fast::mul(Fast::fma(xr, x, 1.0f), xr);
    } else if (x > bits_f(0x3ed413cdu)) {  // tan(pi/8): pi/4 + atan((x-1)/(x+1))
        y = bits_f(0x3f490fdbu);
        more = bits_f(0xb2bbbd2eu);
        float nh, nl, dh, dl;
        two_sum_f(x, -1.0f, nh, nl);
        two_sum_f(x, 1.0f, dh, dl);
        xr = Fast::div(nh, dh);
        const float rho = Fast::fma(-xr, dh, nh);
        xl = Fast::div(Fast::fma(-xr, dl, Fast::add(rho, nl)), dh);
    }
    const float z = Fast::mul(xr, xr);
    const float p = horner<Fast>(z, bits_f(0x3da4f0d1u), bits_f(0xbe0e1b85u), bits_f(0x3e4c925fu), bits_f(0xbeaaaa2au));
    const float corr = Fast::fma(Fast::mul(p, z), xr, xl);
    const float sh = Fast::add(y, xr);
    const float sl = Fast::sub(xr, Fast::sub(sh, y));
    return Fast::add(sh, Fast::add(sl, Fast::add(corr, more)));
}

template <class P> NT2G_HD float atan_kernel(float a0)
{
    if (!P::exact) return atan_kernel_fast(a0);
    if (a0 == 0.0f) return 0.0f;
    if (fabsf(a0) == f_inf()) return bits_f(0x3fc90fdbu);
    float x = fabsf(a0), y = 0.0f, more = 0.0f;
    if (x > bits_f(0x401a827au)) {  // tan(3 pi/8)
        y = bits_f(0x3fc90fdbu);
        more = bits_f(0xb33bbd2eu);
        x = -P::div(1.0f, x);
    } else if (x > bits_f(0x3ed413cdu)) {  // tan(pi/8)
        y = bits_f(0x3f490fdbu);
        more = bits_f(0xb2bbbd2eu);
        x = P::div(P::sub(x, 1.0f), P::add(1.0f, x));
    }
    const float z = P::mul(x, x);
    float z1 = horner<P>(z, bits_f(0x3da4f0d1u), bits_f(0xbe0e1b85u), bits_f(0x3e4c925fu), bits_f(0xbeaaaa2au));
    z1 = P::fma(x, P::mul(z1, z), x);
    return P::add(y, P::add(z1, more));
}

template <class P> NT2G_HD float atan(float a0)
{
    return bits_f(f_bits(atan_kernel<P>(a0)) ^ (f_bits(a0) & 0x80000000u));
}

template <class P> NT2G_HD float atan2(float a0, float a1)
{
    if (is_nan(a0) || is_nan(a1)) return f_nan();
    if (fabsf(a0) == f_inf() && fabsf(a1) == f_inf()) {
        a0 = copysignf(1.0f, a0);
        a1 = copysignf(1.0f, a1);
    }
    float z = atan_kernel<P>(P::div(a0, a1));
    z = (a1 > 0.0f) ? z : P::sub(bits_f(0x40490fdbu), z);
    z = P::mul(z, (f_bits(a0) & 0x80000000u) ? -1.0f : 1.0f);  // signnz
    if (a0 == 0.0f) return (a1 < 0.0f) ? bits_f(0x40490fdbu) : 0.0f;
    return z;
}

// ------------------------------------------------------------ cbrt, hypot --
// cbrt (exponential/functions/scalar/cbrt.hpp, float overload, Cephes' cbrtf):
// x = m 2^e, a degree-4 polynomial for m^(1/3), 2^(e/3) from e / 3 and the
// remainder's 2^(1/3) or 2^(2/3), one Newton step, denormals through a 2^23
// scale; +-0 and +-inf return themselves.
template <class P> NT2G_HD float cbrt(float a0)
{
    float z = fabsf(a0);
    if (z == f_inf() || z == 0.0f) return a0;
    float f = 1.0f;
    if (z < bits_f(0x00800000u)) {
        z = P::mul(z, 8388608.0f);
        f = bits_f(0x3ba14518u);  // 2^(-23/3)
    }
    const uint32_t u = f_bits(z);
    int e = (int)((u & 0x7f800000u) >> 23) - 126;
    float x = bits_f((u & ~0x7f800000u) | 0x3f000000u);
    x = horner<P>(x, bits_f(0xbe09e49au), bits_f(0x3f0bf0feu), bits_f(0xbf745265u), bits_f(0x3f91eb77u),
                  bits_f(0x3ece0609u));
    const bool flag = e >= 0;
    int e1 = e < 0 ? -e : e;
    int rem = e1;
    e1 /= 3;
    rem -= e1 * 3;
    e = e < 0 ? -e1 : e1;
    const float cbrt2 = flag ? bits_f(0x3fa14518u) : bits_f(0x3f4b2ff5u);
    const float cbrt4 = flag ? bits_f(0x3fcb2ff5u) : bits_f(0x3f214518u);
    float fact = rem == 1 ? cbrt2 : 1.0f;
    fact = rem == 2 ? cbrt4 : fact;
    x = P::mul(P::mul(x, fact), pow2i((float)e));  // fast_ldexp
    x = P::sub(x, P::mul(P::sub(x, P::div(z, P::mul(x, x))), bits_f(0x3eaaaaabu)));
    return P::mul(bits_f(f_bits(x) | (f_bits(a0) & 0x80000000u)), f);
}

// NT2's exponent(): 0 for zero, inf and NaN, else ilogb (denormals included)
NT2G_HD int nt2_exponent(float x)
{
    const uint32_t u = f_bits(x) & 0x7fffffffu;
    if (u == 0 || u >= 0x7f800000u) return 0;
    if (u >= 0x00800000u) return (int)(u >> 23) - 127;
#if defined(__CUDA_ARCH__)
    return (31 - __clz((int)u)) - 149;
#else
    return (31 - __builtin_clz(u)) - 149;
#endif
}

// hypot (boost/simd/arithmetic/functions/scalar/hypot.hpp:27-40): inf when one
// operand is NaN and the other infinite, else both scaled by 2^-e, e the larger
// one's exponent clamped to [-126, 126], and the root scaled back.
template <class P> NT2G_HD float hypot(float a0, float a1)
{
    if ((is_nan(a0) && fabsf(a1) == f_inf()) || (fabsf(a0) == f_inf() && is_nan(a1))) return f_inf();
    const float r = fabsf(a0), i = fabsf(a1);
    int e = nt2_exponent((i > r) ? i : r);
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    const float a = nt2_ldexp<P>(r, -e), b = nt2_ldexp<P>(i, -e);
    const float ss = P::exact ? P::add(P::mul(a, a), P::mul(b, b)) : Fast::fma(a, a, Fast::mul(b, b));
    return nt2_ldexp<P>(P::sqrt(ss), e);
}

// -------------------------------------------------- inverse hyperbolic --
// NT2 (hyperbolic/functions/scalar/{asinh,acosh,atanh}.hpp):
//   asinh  |x| < 1/2: x P4(x^2) (Cephes' asinhf), |x| > 1/sqrt(eps): log|x| + log 2,
//          else log(|x| + hypot(1, |x|)); the sign of x
//   acosh  t = x - 1; t <= 1/(2 eps): log1p(t + sqrt(2t + t^2)), else log t + log 2
//   atanh  sign(x) (1/2) log1p(|x| < 1/2 ? 2|x| + 2|x| |x|/(1 - |x|) : 2|x|/(1 - |x|))
// hypot as NT2 computes it (arithmetic/functions/scalar/hypot.hpp:27-40): both
// operands scaled by 2^-e, e the larger one's exponent, sqrt of the sum of
// squares, scaled back (here for the finite, normal operands asinh gives it).
template <class P> NT2G_HD float hypot_scaled(float r, float i)
{
    const float m = (i > r) ? i : r;
    int e = (int)((f_bits(m) >> 23) & 0xff) - 127;
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    const float a = nt2_ldexp<P>(r, -e), b = nt2_ldexp<P>(i, -e);
    return nt2_ldexp<P>(P::sqrt(P::add(P::mul(a, a), P::mul(b, b))), e);
}

template <class P> NT2G_HD float asinh(float a0)
{
    const float x = fabsf(a0);
    float z;
    if (x < 0.5f) {
        const float x2 = P::mul(x, x);
        z = P::mul(horner<P>(x2, bits_f(0x3ca4d6e6u), bits_f(0xbd2ee581u), bits_f(0x3d9949b1u), bits_f(0xbe2aa9adu),
                             1.0f),
                   x);
    } else if (x > bits_f(0x453504f3u)) {  // 1/sqrt(eps)
        z = P::add(log<P>(x), bits_f(NT2G_LOG_2));
    } else {
        if (P::exact) {
            z = log<P>(P::add(x, hypot_scaled<P>(1.0f, x)));
        } else {
            // Fast: log1p(x + x^2 / (1 + sqrt(1 + x^2))) -- the same value, taken
            // through log1p so the rounding of x + sqrt(1 + x^2) is not felt
            const float h = Fast::sqrt(Fast::fma(x, x, 1.0f));  // x <= 2^11.5: no overflow
            z = log1p<P>(Fast::fma(x, Fast::div(x, Fast::add(1.0f, h)), x));
        }
    }
    return bits_f(f_bits(z) ^ (f_bits(a0) & 0x80000000u));
}

template <class P> NT2G_HD float acosh(float a0)
{
    const float t = P::sub(a0, 1.0f);
    if (t <= bits_f(0x4a800000u))  // 1/(2 eps)
        return log1p<P>(P::add(t, P::sqrt(P::add(P::add(t, t), P::mul(t, t)))));
    return P::add(log<P>(t), bits_f(NT2G_LOG_2));
}

template <class P> NT2G_HD float atanh(float a0)
{
    const float x = fabsf(a0);
    const float t = P::add(x, x);
    const float z1 = P::sub(1.0f, x);
    const float u = (x < 0.5f) ? P::fma(t, P::div(x, z1), t) : P::div(t, z1);
    const float r = P::mul(0.5f, log1p<P>(u));
    return bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u));
}

// asech, acoth (hyperbolic/functions/generic/asech.hpp, acoth.hpp): acosh(1/x)
// and atanh(1/x).  Fast: with u = (1 - x)/x (1 - x exact near 1),
// asech = log1p(u + sqrt(u (u + 2))), and log 2 - log x below 2^-12;
// acoth = log1p(2/(|x| - 1))/2 with x's sign.  Both keep NT2's domain: NaN
// outside (0, 1] (asech; +inf at +0) and inside (-1, 1) (acoth; +-inf at +-1).
template <class P> NT2G_HD float asech(float a0)
{
    if (P::exact) return acosh<P>(P::div(1.0f, a0));
    const float u = P::div(P::sub(1.0f, a0), a0);
    const float mid = log1p<P>(P::add(u, P::sqrt(P::mul(u, P::add(u, 2.0f)))));
    const float tiny = P::sub(bits_f(NT2G_LOG_2), log<P>(a0));
    const float r = (a0 < 0x1p-12f) ? tiny : mid;
    return (a0 >= 0.0f && a0 <= 1.0f && !(a0 == 0.0f && (f_bits(a0) >> 31))) ? r : f_nan();
}
// acsch (hyperbolic/functions/generic/acsch.hpp): asinh(1/x).  Fast: below
// 2^-12 in magnitude log 2 - log|x| (1/x would overflow for the smallest x)
template <class P> NT2G_HD float acsch(float a0)
{
    if (P::exact) return asinh<P>(P::div(1.0f, a0));
    const float ax = fabsf(a0);
    const float tiny = bits_f(f_bits(P::sub(bits_f(NT2G_LOG_2), log<P>(ax))) ^ (f_bits(a0) & 0x80000000u));
    const float r = asinh<P>(P::div(1.0f, a0));
    return (ax < 0x1p-12f) ? tiny : r;
}
template <class P> NT2G_HD float acoth(float a0)
{
    if (P::exact) return atanh<P>(P::div(1.0f, a0));
    const float ax = fabsf(a0);
    const float r = P::mul(0.5f, log1p<P>(P::div(2.0f, P::sub(ax, 1.0f))));
    return (ax >= 1.0f) ? bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u)) : f_nan();
}

// ----------------------------------------------------------- trigonometry --
// NT2 (modules/core/trigonometric/include/nt2/trigonometric/functions/):
//   sin/cos/tan   scalar/impl/trigo/trig_base.hpp:131-176 (regular style,
//                 big_ mode) over the radian cascade of trig_reduction.hpp:76-251:
//                 |x| <= pi/4 as is, <= pi/2 one subtraction of pi/2 in three
//                 parts (generic/rem_pio2_straight.hpp:60-66), <= 20 pi Cody-Waite
//                 with k = round(x 2/pi) (rem_pio2_cephes.hpp:65-72), <= 2^6 pi the
//                 error-compensated three-step form (rem_pio2_medium.hpp:68-84),
//                 <= 2^18 pi the same three-step form in double, beyond that
//                 fdlibm's Payne-Hanek reduction (scalar/rem_pio2.hpp).
//   evaluation    f_trig_evaluation.hpp:40-72: NT2's degree-3 sin/cos and
//                 degree-6 tan polynomials on [-pi/4, pi/4].
//   sinpi/cospi   the pi_tag reduction trig_reduction.hpp:303-317: k = round(2x),
//                 r = (x - k/2) pi.
// The Payne-Hanek step here is this file's own: the float's 24-bit significand
// times a 96-bit window of 2/pi in 64-bit integer pieces gives the quadrant and
// at least 64 fraction bits, so r is the exactly reduced argument rounded once.

// 2/pi in binary, 32 bits per word, after one word of zeros (word 1 holds the
// first 32 fraction bits).  gen_twoopi.py prints these words.
NT2G_HD uint32_t twoopi_word(int i)
{
    switch (i) {
    case 1: return 0xA2F9836Eu;
    case 2: return 0x4E441529u;
    case 3: return 0xFC2757D1u;
    case 4: return 0xF534DDC0u;
    case 5: return 0xDB629599u;
    case 6: return 0x3C439041u;
    case 7: return 0xFE5163ABu;
    case 8: return 0xDEBBC561u;
    default: return 0u;
    }
}

// Quadrant n (mod 4) and r = x - n pi/2 in double, |r| <= pi/4 (+2^-60), for a
// finite x >= 2^-6 (the window below starts inside the table for those).
NT2G_HD int trig_reduce_big(float x, double &r)
{
    const uint32_t u = f_bits(x);
    const uint64_t m = (u & 0x007fffffu) | 0x00800000u;  // x = m 2^e
    const int e = (int)(u >> 23) - 150;
    // x 2/pi mod 4 only needs the bits b_i of 2/pi with i >= e - 1 (earlier ones
    // contribute multiples of 4 m); b_i sits at bit i + 31 of the padded table.
    const int j = e + 30;
    const int w = j >> 5, sh = j & 31;
    const uint64_t a0 = twoopi_word(w), a1 = twoopi_word(w + 1), a2 = twoopi_word(w + 2), a3 = twoopi_word(w + 3);
    const uint64_t b2 = ((a0 << 32 | a1) << sh) >> 32;
    const uint64_t b1 = ((a1 << 32 | a2) << sh) >> 32;
    const uint64_t b0 = ((a2 << 32 | a3) << sh) >> 32;
    // P = m (b2 b1 b0) = t2 2^64 + (t1 mod 2^32) 2^32 + (t0 mod 2^32); x 2/pi = P 2^-94 (mod 4)
    const uint64_t t0 = m * b0;
    const uint64_t t1 = m * b1 + (t0 >> 32);
    const uint64_t t2 = m * b2 + (t1 >> 32);
    int n = (int)(t2 >> 30) & 3;
    const uint64_t f = (t2 << 34) | ((t1 & 0xffffffffu) << 2) | ((t0 & 0xffffffffu) >> 30);  // fraction bits 1..64
    const uint32_t lo = (uint32_t)(t0 & 0x3fffffffu);                                      // bits 65..94
    n = (n + (int)(f >> 63)) & 3;  // a fraction >= 1/2 rounds up to the next quadrant
    const double q = (double)(int64_t)f * 0x1p-64 + (double)lo * 0x1p-94;
    r = q * 0x1.921fb54442d18p+0;  // pi/2
    return n;
}

// NT2's double helpers for the 2^6 pi .. 2^18 pi band (unfused, like its floats)
#if defined(__CUDA_ARCH__)
NT2G_HD double nt2_dmul(double a, double b) { return __dmul_rn(a, b); }
NT2G_HD double nt2_dsub(double a, double b) { return __dsub_rn(a, b); }
#else
inline double nt2_dmul(double a, double b) { volatile double r = a * b; return r; }
inline double nt2_dsub(double a, double b) { volatile double r = a - b; return r; }
#endif

// rem_pio2_medium.hpp:68-84 in float or double.  The first correction term
// (fn * Pio2_1t) is computed and then overwritten in NT2, so it is not applied.
template <class P> NT2G_HD int trig_medium_f(float t, float &xr)
{
    const float fn = rintf(P::mul(t, bits_f(0x3f22f984u)));  // Invpio_2
    float r = P::sub(t, P::mul(fn, bits_f(0x3fc90f80u)));    // Pio2_1
    float t2 = r;
    float w = P::mul(fn, bits_f(0x37354400u));               // Pio2_2
    r = P::sub(t2, w);
    w = P::sub(P::mul(fn, bits_f(0x2e85a308u)), P::sub(P::sub(t2, r), w));  // Pio2_2t
    t2 = r;
    w = P::mul(fn, bits_f(0x2e85a300u));                     // Pio2_3
    r = P::sub(t2, w);
    w = P::sub(P::mul(fn, bits_f(0x248d3132u)), P::sub(P::sub(t2, r), w));  // Pio2_3t
    xr = P::sub(r, w);
    return (int)fn & 3;
}

NT2G_HD int trig_medium_d(double t, float &xr)
{
    const double fn = rint(nt2_dmul(t, 0x1.45f306dc9c883p-1));  // Invpio_2
    double r = nt2_dsub(t, nt2_dmul(fn, 0x1.921fb544p+0));      // Pio2_1
    double t2 = r;
    double w = nt2_dmul(fn, 0x1.0b4611a6p-34);                   // Pio2_2
    r = nt2_dsub(t2, w);
    w = nt2_dsub(nt2_dmul(fn, 0x1.3198a2e037073p-69), nt2_dsub(nt2_dsub(t2, r), w));  // Pio2_2t
    t2 = r;
    w = nt2_dmul(fn, 0x1.3198a2ep-69);                           // Pio2_3
    r = nt2_dsub(t2, w);
    w = nt2_dsub(nt2_dmul(fn, 0x1.b839a252049c1p-104), nt2_dsub(nt2_dsub(t2, r), w));  // Pio2_3t
    xr = (float)nt2_dsub(r, w);
    return (int)(int64_t)fn & 3;
}

// Fast: below this bound a three-float Cody-Waite with FMAs (pi/2 = C1 + C2 + C3,
// each the float nearest the remainder) keeps the reduced argument within an
// ulp; above it the exact reduction runs.
#define NT2G_TRIG_FAST_MAX 131072.0f

// Quadrant n (mod 4) and the reduced argument xr of x = |a0| (finite).
template <class P> NT2G_HD int trig_reduce(float x, float &xr)
{
    if (P::exact) {
        if (!(x > bits_f(0x3f490fdbu))) { xr = x; return 0; }  // pi/4
        if (!(x > bits_f(0x3fc90fdbu))) {                       // pi/2
            xr = P::sub(P::sub(P::sub(x, bits_f(0x3fc90f80u)), bits_f(0x37354400u)), bits_f(0x2e85a300u));
            return 1;
        }
        if (!(x > bits_f(0x427b53d1u))) {                       // 20 pi
            const float xi = rintf(P::mul(x, bits_f(0x3f22f983u)));  // Twoopi
            float r = P::sub(x, P::mul(xi, bits_f(0x3fc90f80u)));
            r = P::sub(r, P::mul(xi, bits_f(0x37354400u)));
            xr = P::sub(r, P::mul(xi, bits_f(0x2e85a300u)));
            return (int)xi & 3;
        }
        if (!(x > bits_f(0x43490fdbu))) return trig_medium_f<P>(x, xr);  // 2^6 pi
        if (!((double)x > 0x1.921fb54442d18p+19)) return trig_medium_d((double)x, xr);  // 2^18 pi in double
        double r;
        const int n = trig_reduce_big(x, r);
        xr = (float)r;
        return n;
    }
    if (x <= NT2G_TRIG_FAST_MAX) {
        const float k = rintf(Fast::mul(x, 0x1.45f306p-1f));
        float r = Fast::fma(-k, 0x1.921fb6p+0f, x);
        r = Fast::fma(-k, -0x1.777a5cp-25f, r);
        xr = Fast::fma(-k, -0x1.ee59dap-50f, r);
        return (int)k & 3;
    }
    double r;
    const int n = trig_reduce_big(x, r);
    xr = (float)r;
    return n;
}

template <class P> NT2G_HD float trig_cos_eval(float z)
{
    const float y = horner<P>(z, bits_f(0x37ccf5ceu), bits_f(0xbab60619u), bits_f(0x3d2aaaa5u));
    return P::add(1.0f, P::fma(z, -0.5f, P::mul(y, P::mul(z, z))));
}

template <class P> NT2G_HD float trig_sin_eval(float z, float x)
{
    const float y1 = horner<P>(z, bits_f(0xb94ca1f9u), bits_f(0x3c08839du), bits_f(0xbe2aaaa2u));
    return P::fma(P::mul(y1, z), x, x);
}

template <class P> NT2G_HD float trig_tan_eval(float z)
{
    const float zz = P::mul(z, z);
    const float y = horner<P>(zz, bits_f(0x3c19c53bu), bits_f(0x3b4c779cu), bits_f(0x3cc821b5u),
                              bits_f(0x3d5ac5c9u), bits_f(0x3e0896ddu), bits_f(0x3eaaaa6fu));
    return P::add(P::mul(P::mul(y, zz), z), z);
}

// Fast: tan(z) as the unevaluated sum hi + lo of z and its odd tail (Fast2Sum,
// |tail| < |z| on [-pi/4, pi/4]), so that a reciprocal sees the tail unrounded.
template <class P> NT2G_HD float trig_tan_eval_ff(float z, float &lo)
{
    const float zz = P::mul(z, z);
    const float y = horner<P>(zz, bits_f(0x3c19c53bu), bits_f(0x3b4c779cu), bits_f(0x3cc821b5u),
                              bits_f(0x3d5ac5c9u), bits_f(0x3e0896ddu), bits_f(0x3eaaaa6fu));
    const float t = P::mul(P::mul(y, zz), z);
    const float hi = P::add(t, z);
    lo = P::add(P::sub(z, hi), t);
    return hi;
}

// Fast: 1/(hi + lo) with one Newton step on the residual 1 - r (hi + lo);
// r itself where it is infinite (hi = 0 or subnormal).
template <class P> NT2G_HD float rec_ff(float hi, float lo)
{
    const float r = P::div(1.0f, hi);
    const float e = P::fma(-r, lo, P::fma(-r, hi, 1.0f));
    return (fabsf(r) < bits_f(0x7f800000u)) ? P::fma(r, e, r) : r;
}

// The shared tail of sin and cos: swap selects the other polynomial, sign is
// xor-ed into the result.  Fast evaluates both and selects (no divergence).
template <class P> NT2G_HD float trig_sincos_tail(float xr, bool use_cos, uint32_t sign)
{
    const float z = P::mul(xr, xr);
    float v;
    if (P::exact) v = use_cos ? trig_cos_eval<P>(z) : trig_sin_eval<P>(z, xr);
    else {
        const float c = trig_cos_eval<P>(z), s = trig_sin_eval<P>(z, xr);
        v = use_cos ? c : s;
    }
    return bits_f(f_bits(v) ^ sign);
}

NT2G_HD bool trig_invalid(float a0) { return !(fabsf(a0) < f_inf()); }  // NaN or +-inf

// pi_tag reduction: k = round(2x), xr = (x - k/2) pi.  The quadrant is k mod 4
// (k is an even integer, hence a multiple of 4, once it leaves the int64 range).
// NT2's 2x overflows for x >= 2^127 and its sinpi/cospi are NaN there; Fast
// clamps x to 2^24 first (every float from 2^24 on is an even integer, as 2^24
// is, so the results are unchanged below 2^127 and correct above).
template <class P> NT2G_HD int trig_reduce_pi(float x, float &xr)
{
    if (!P::exact) x = fminf(x, 0x1p24f);
    const float xi = rintf(P::mul(x, 2.0f));
    const float x2 = P::sub(x, P::mul(xi, 0.5f));
    xr = P::mul(x2, bits_f(0x40490fdbu));  // Pi
    // k mod 4 without a 64-bit conversion: exact below 2^24; in [2^24, 2^25) k
    // is even and k/2 is odd exactly when the significand's last bit is set;
    // from 2^25 on (and for inf, NaN) k is a multiple of 4
    if (fabsf(xi) < 16777216.0f) return (int)xi & 3;
    return ((f_bits(xi) & 1u) && fabsf(xi) < 33554432.0f) ? 2 : 0;
}

// degree_tag reduction (trig_reduction.hpp:254-266): k = round(x / 90),
// xr = (x - 90 k) pi/180; the quadrant is k mod 4 (0 once k leaves int32, as
// NT2's conversion gives on x86)
template <class P> NT2G_HD int trig_reduce_deg(float x, float &xr)
{
    const float xi = rintf(P::mul(x, bits_f(0x3c360b61u)));  // Oneo_90
    const float x2 = P::sub(x, P::mul(xi, 90.0f));
    xr = P::mul(x2, bits_f(0x3c8efa35u));  // Deginrad
    return (fabsf(xi) < 2147483648.0f) ? ((int)xi & 3) : 0;
}

// the unit of the argument: radians, multiples of pi, degrees
enum TrigUnit { kRad = 0, kPi = 1, kDeg = 2 };
template <class P, int U> NT2G_HD int trig_reduce_unit(float x, float &xr)
{
    if (U == kPi) return trig_reduce_pi<P>(x, xr);
    if (U == kDeg) return trig_reduce_deg<P>(x, xr);
    return trig_reduce<P>(x, xr);
}

template <class P, int U> NT2G_HD float cos_any(float a0)
{
    if (P::exact && trig_invalid(a0)) return f_nan();
    const float x = (P::exact || !trig_invalid(a0)) ? fabsf(a0) : 0.0f;
    float xr;
    const int n = trig_reduce_unit<P, U>(x, xr);
    const int swap = n & 1;
    const float r = trig_sincos_tail<P>(xr, !swap, (uint32_t)(swap ^ ((n & 2) >> 1)) << 31);
    return (!P::exact && trig_invalid(a0)) ? f_nan() : r;
}

template <class P, int U> NT2G_HD float sin_any(float a0)
{
    if (P::exact && trig_invalid(a0)) return f_nan();
    const float x = (P::exact || !trig_invalid(a0)) ? fabsf(a0) : 0.0f;
    float xr;
    const int n = trig_reduce_unit<P, U>(x, xr);
    const uint32_t sign = (f_bits(a0) & 0x80000000u) ^ ((uint32_t)(n & 2) << 30);
    const float r = trig_sincos_tail<P>(xr, (n & 1) != 0, sign);
    return (!P::exact && trig_invalid(a0)) ? f_nan() : r;
}

template <class P> NT2G_HD float cos(float a0) { return cos_any<P, kRad>(a0); }
template <class P> NT2G_HD float sin(float a0) { return sin_any<P, kRad>(a0); }
template <class P> NT2G_HD float cospi(float a0) { return cos_any<P, kPi>(a0); }
template <class P> NT2G_HD float sinpi(float a0) { return sin_any<P, kPi>(a0); }
template <class P> NT2G_HD float cosd(float a0) { return cos_any<P, kDeg>(a0); }
template <class P> NT2G_HD float sind(float a0) { return sin_any<P, kDeg>(a0); }
// sec = rec(cos), csc = rec(sin) (generic/sec.hpp, generic/csc.hpp)
template <class P> NT2G_HD float sec(float a0) { return P::div(1.0f, cos<P>(a0)); }
template <class P> NT2G_HD float csc(float a0) { return P::div(1.0f, sin<P>(a0)); }

// tan: NaN for NaN/inf, tan(+-0) = +-0, else tan(xr) or -1/tan(xr) by the
// quadrant's parity, with a0's sign.
// tand is NaN at 90 + 180 k (NT2's tan_invalid for degrees: (x - 90)/180 an integer)
NT2G_HD bool tand_invalid(float a0)
{
    const float q = (a0 - 90.0f) * bits_f(0x3bb60b61u);  // Oneo_180
    return (q - truncf(q)) == 0.0f;
}

// tan_invalid / cot_invalid of each unit (trig_reduction.hpp:89-90, 268-269,
// 308-309): radians none; pi: x - 1/2 integral, or x a nonzero integer;
// degrees: (x - 90)/180 integral, or x/180 a nonzero integer (in float)
template <int U> NT2G_HD bool tan_invalid_u(float a0)
{
    if (U == kPi) return is_flint(a0 - 0.5f);
    if (U == kDeg) return tand_invalid(a0);
    return false;
}
template <int U> NT2G_HD bool cot_invalid_u(float a0)
{
    if (U == kPi) return a0 != 0.0f && is_flint(a0);
    if (U == kDeg) return a0 != 0.0f && is_flint(a0 * bits_f(0x3bb60b61u));  // Oneo_180
    return false;
}

template <class P, int U> NT2G_HD float tan_any(float a0)
{
    const bool bad = trig_invalid(a0) || tan_invalid_u<U>(a0);
    if (P::exact) {
        if (bad) return f_nan();
        if (a0 == 0.0f) return a0;
    }
    const float x = (P::exact || !trig_invalid(a0)) ? fabsf(a0) : 0.0f;
    float xr;
    const int n = trig_reduce_unit<P, U>(x, xr);
    float y;
    if (P::exact) {
        y = trig_tan_eval<P>(xr);
        if (n & 1) y = -P::div(1.0f, y);
    } else {
        float lo;
        const float hi = trig_tan_eval_ff<P>(xr, lo);
        y = (n & 1) ? -rec_ff<P>(hi, lo) : hi;
    }
    float r = bits_f(f_bits(y) ^ (f_bits(a0) & 0x80000000u));
    if (!P::exact) {
        r = (a0 == 0.0f) ? a0 : r;
        r = bad ? f_nan() : r;
    }
    return r;
}

template <class P> NT2G_HD float tan(float a0) { return tan_any<P, kRad>(a0); }
template <class P> NT2G_HD float tand(float a0) { return tan_any<P, kDeg>(a0); }
template <class P> NT2G_HD float tanpi(float a0) { return tan_any<P, kPi>(a0); }

// mod (boost/simd/arithmetic/functions/generic/mod.hpp:22-31 with the float
// divfloor of scalar/divfloor.hpp:89-100): selsub(b != 0, a, floor(a/b)*b),
// each operation rounded once; rem (scalar/rem.hpp:27-37 with idivfix,
// generic/idivfix.hpp:38-49): b != 0 ? a - b*q : a, q = itrunc(a/b), the
// saturating float -> int32 conversion (NaN -> 0) converted back to float.
// Both policies compute NT2's sequence: a faster quotient could move floor or
// trunc across an integer.
template <class P> NT2G_HD float mod_(float a, float b)
{
    return b != 0.0f ? Nt2::sub(a, Nt2::mul(floorf(Nt2::div(a, b)), b)) : a;
}
NT2G_HD int32_t toints(float v)
{
    if (is_nan(v)) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v <= -2147483648.0f) return (int32_t)0x80000000u;
    return (int32_t)v;
}
template <class P> NT2G_HD float rem_(float a, float b)
{
    return b != 0.0f ? Nt2::sub(a, Nt2::mul(b, (float)toints(Nt2::div(a, b)))) : a;
}

// pow2 (EXP/generic/pow2.hpp:21-70): fast_ldexp(a, toint(b)), i.e. a times
// the float whose bits are (n + Maxexponent) << Nbmantissabits in wrapping
// int32 arithmetic (boost/simd/ieee/functions/scalar/fast_ldexp.hpp:33-43);
// toint is C's truncating conversion, INT_MIN outside the int32 range and for
// NaN (the x86 conversion NT2 runs on).  pow2(x) is pow2(1, x).
NT2G_HD int32_t toint_x86(float v)
{
    return (v >= -2147483648.0f && v < 2147483648.0f) ? (int32_t)v : (int32_t)0x80000000u;
}
template <class P> NT2G_HD float pow2_(float a, float b)
{
    return Nt2::mul(a, bits_f(((uint32_t)toint_x86(b) + 127u) << 23));
}

// proper_tanpi (TRIG/scalar/proper_tanpi.hpp:25-36): tan(pi x) for x in
// [-1/2, 1/2], NaN outside and +-inf at +-1/2.  NT2 evaluates the unreduced
// tangent polynomial at |x| pi (one rounded product: the fast-style tana of
// trig_base.hpp:236-242 under clipped_pio4_) for |x| <= 1/4, else at
// (1/2 - |x|) pi and takes the reciprocal; x's sign goes on before the
// reciprocal.  Fast: tanpi's reduction and float-float reciprocal, which
// agree with it inside the interval.
template <class P> NT2G_HD float proper_tanpi(float a0)
{
    float ab = fabsf(a0);
    if (P::exact) {
        if (is_nan(a0)) return a0;
        if (ab > 0.5f) return f_nan();
        const bool test = ab <= 0.25f;
        ab = test ? ab : P::sub(0.5f, ab);
        float t = trig_tan_eval<P>(P::mul(ab, bits_f(0x40490fdbu)));
        t = a0 < 0.0f ? -t : t;
        return test ? t : P::div(1.0f, t);
    }
    const float r = tanpi<P>(a0);
    const float inf = bits_f(0x7f800000u | (f_bits(a0) & 0x80000000u));
    return ab > 0.5f ? f_nan() : (ab == 0.5f ? inf : r);
}

// cot (trig_base.hpp:178-188): NaN for NaN/inf and the unit's poles, +-inf at
// +-0, else 1/tan(xr) or -tan(xr) by the quadrant's parity, with a0's sign
template <class P, int U> NT2G_HD float cot_any(float a0)
{
    const uint32_t bos = f_bits(a0) & 0x80000000u;
    const bool bad = trig_invalid(a0) || cot_invalid_u<U>(a0);
    if (P::exact) {
        if (bad) return f_nan();
        if (a0 == 0.0f) return bits_f(0x7f800000u | bos);
    }
    const float x = (P::exact || !trig_invalid(a0)) ? fabsf(a0) : 0.0f;
    float xr;
    const int n = trig_reduce_unit<P, U>(x, xr);
    float y;
    if (P::exact) {
        y = trig_tan_eval<P>(xr);
        y = (n & 1) ? -y : P::div(1.0f, y);
    } else {
        float lo;
        const float hi = trig_tan_eval_ff<P>(xr, lo);
        y = (n & 1) ? -hi : rec_ff<P>(hi, lo);
    }
    float r = bits_f(f_bits(y) ^ bos);
    if (!P::exact) {
        r = (a0 == 0.0f) ? bits_f(0x7f800000u | bos) : r;
        r = bad ? f_nan() : r;
    }
    return r;
}

template <class P> NT2G_HD float cot(float a0) { return cot_any<P, kRad>(a0); }
template <class P> NT2G_HD float cotpi(float a0) { return cot_any<P, kPi>(a0); }
template <class P> NT2G_HD float cotd(float a0) { return cot_any<P, kDeg>(a0); }

// secpi (generic/secpi.hpp): NaN where 2x is odd, else 1/cospi(x); cscpi
// (generic/cscpi.hpp): NaN at nonzero integers, else 1/sinpi(x); secd
// (generic/secd.hpp): 1/cosd(x), NaN where cosd(x) is zero; cscd
// (generic/cscd.hpp): cscpi(x/180).  NT2's is_odd(y) is is_flint((y - 1)/2).
template <class P> NT2G_HD float secpi(float a0)
{
    const float r = P::div(1.0f, cospi<P>(a0));
    return is_odd_f(P::mul(a0, 2.0f)) ? f_nan() : r;
}
template <class P> NT2G_HD float cscpi(float a0)
{
    const float r = P::div(1.0f, sinpi<P>(a0));
    return (is_flint(a0) && a0 != 0.0f) ? f_nan() : r;
}
template <class P> NT2G_HD float secd(float a0)
{
    const float c = cosd<P>(a0);
    return P::div(1.0f, (c == 0.0f) ? f_nan() : c);
}
template <class P> NT2G_HD float cscd(float a0)
{
    const float y = P::mul(bits_f(0x3bb60b61u), a0);
    if (P::exact) return cscpi<P>(y);
    // Fast: NT2's poles (x/180 a nonzero integer in float), the value from
    // sind, whose reduction is exact, instead of sinpi of the rounded x/180
    const float r = P::div(1.0f, sind<P>(a0));
    return (is_flint(y) && y != 0.0f) ? f_nan() : r;
}

// sinc, sincpi (scalar/sinc.hpp, scalar/sincpi.hpp): 0 at +-inf, 1 below Eps
// in magnitude, else sin(x)/x and (sinpi(x)/pi)/x
template <class P> NT2G_HD float sinc(float a0)
{
    const float ax = fabsf(a0);
    const float r = P::div(sin<P>(a0), a0);
    return (ax == f_inf()) ? 0.0f : (ax < bits_f(0x34000000u)) ? 1.0f : r;
}
template <class P> NT2G_HD float sincpi(float a0)
{
    const float ax = fabsf(a0);
    const float r = P::div(P::mul(bits_f(0x3ea2f983u), sinpi<P>(a0)), a0);  // Invpi
    return (ax == f_inf()) ? 0.0f : (ax < bits_f(0x34000000u)) ? 1.0f : r;
}

// acsc (generic/acsc.hpp): asin(1/x).  Fast: asin(1/|x|) from |x| = 2 on,
// below it atan(1/sqrt(x^2 - 1)) (x^2 - 1 by one FMA), which stays accurate
// at 1 where 1/x's rounding would be magnified by asin
template <class P> NT2G_HD float acsc(float a0)
{
    if (P::exact) return asin<P>(P::div(1.0f, a0));
    const float ax = fabsf(a0);
    const float near = atan<P>(P::div(1.0f, P::sqrt(P::fma(ax, ax, -1.0f))));
    const float r = (ax >= 2.0f) ? asin<P>(P::div(1.0f, ax)) : near;
    return (ax < 1.0f) ? f_nan() : bits_f(f_bits(r) ^ (f_bits(a0) & 0x80000000u));
}

// indeg (generic/indeg.hpp): x Radindeg - x Radindegr, the constant in two parts
template <class P> NT2G_HD float indeg(float a)
{
    return P::sub(P::mul(a, bits_f(0x42652ee1u)), P::mul(a, bits_f(0xb53387c1u)));
}

// acotd (generic/acotd.hpp): 90 - atand|x| (90 at 0, 0 at +-inf) with x's sign
template <class P> NT2G_HD float acotd(float a0)
{
    const float ax = fabsf(a0);
    float z;
    if (P::exact) {
        const float t = indeg<P>(atan<P>(ax));
        z = P::sub(90.0f, (a0 != 0.0f) ? t : 0.0f);
    } else {
        // Fast: atand(1/|x|) from 1 on, where 90 - atand|x| would cancel
        z = (ax >= 1.0f) ? indeg<P>(atan<P>(P::div(1.0f, ax))) : P::sub(90.0f, indeg<P>(atan<P>(ax)));
    }
    z = (ax == f_inf()) ? 0.0f : z;
    return bits_f(f_bits(z) | (f_bits(a0) & 0x80000000u));
}

// asec (float: scalar/asec.hpp, single_ overload): NaN inside (-1, 1); a
// series in sqrt(2(|x| - 1)) just above 1 (pi minus it for x < 0); 0 at 1;
// else pi/2 - acsc(x) with acsc(x) = asin(1/x)
template <class P> NT2G_HD float asec(float a0)
{
    const float ax = fabsf(a0);
    if (ax < 1.0f) return f_nan();
    if (!P::exact) {
        // Fast: atan(sqrt(x^2 - 1)) with x^2 - 1 rounded once (an FMA), pi
        // minus it for x < 0 with pi's low part carried; no cancellation at 1
        const float t = atan<P>(P::sqrt(P::fma(ax, ax, -1.0f)));
        return (a0 < 0.0f) ? P::add(P::sub(bits_f(0x40490fdbu), t), bits_f(0xb3bbbd2eu)) : t;
    }
    const float ax1 = P::sub(ax, 1.0f);
    if (ax1 < 0.001f) {
        const float c1 = 5 / 12.0f, c2 = 43 / 160.0f, c3 = 177 / 896.0f, c4 = 2867 / 18432.0f;
        const float q = P::add(c1, P::mul(ax1, P::sub(c2, P::mul(ax1, P::add(c3, P::mul(ax1, c4))))));
        const float t = P::mul(P::sqrt(P::mul(2.0f, ax1)), P::sub(1.0f, P::mul(ax1, q)));
        return (a0 < 0.0f) ? P::sub(bits_f(0x40490fdbu), t) : t;  // Pi
    }
    if (a0 == 1.0f) return 0.0f;
    return P::sub(bits_f(0x3fc90fdbu), asin<P>(P::div(1.0f, a0)));  // Pio_2
}

// ---------------------------------------------------- rounding, sign --
// boost/simd arithmetic/functions/scalar/{floor,ceil,round}.hpp (::floorf,
// ::ceilf, ::roundf), trunc = floor|x| with x's sign bit, round2even: |x| +
// 2^23 - 2^23 below 2^23 (ties to even) with the sign of x < 0 (so -0 gives
// +0), frac = x - trunc(x); ieee/functions/scalar/{sign,signnz,copysign}.hpp:
// sign = (x > 0) - (x < 0) (NaN kept), signnz = +-1 by the sign bit (NaN
// kept).  Exact in both policies.
NT2G_HD float nt2_round2even(float a0)
{
    const float v = fabsf(a0);
    const float d = (v < 8388608.0f) ? rintf(v) : v;
    return (a0 < 0.0f) ? -d : d;
}
template <class P> NT2G_HD float nt2_frac(float a0) { return P::sub(a0, truncf(a0)); }
NT2G_HD float nt2_sign(float a0)
{
    return is_nan(a0) ? a0 : (float)(a0 > 0.0f) - (float)(a0 < 0.0f);
}
NT2G_HD float nt2_signnz(float a0)
{
    return is_nan(a0) ? a0 : bits_f(0x3f800000u | (f_bits(a0) & 0x80000000u));
}

// ------------------------------------------------------------ euler --
// erf2 kernel: erfc(x) e^(x^2) for x >= 2/3 as a polynomial in x/(1+x) - 0.4
// (euler/functions/details/erf_kernel.hpp:48-66, the one erfc uses)
template <class P> NT2G_HD float erfc2_kernel(float z)
{
    return horner<P>(z, bits_f(0xc0283611u), bits_f(0x40d67e3bu), bits_f(0xc0cd1a85u), bits_f(0x4050b063u),
                     bits_f(0xbfaea865u), bits_f(0x3e2006f0u), bits_f(0x3e1175c7u), bits_f(0x3ec4ca6eu),
                     bits_f(0x3e243828u), bits_f(0xbf918a62u), bits_f(0x3f0a0e8bu));
}

// erf (euler/functions/scalar/erf.hpp, single_): x erf1(x^2) below 2/3, else
// 1 - e^(-x^2) erfc2(x/(1+x) - 0.4) with x's sign; +-1 at +-inf.  Fast: the
// same small branch with FMAs, 1 - erfc(|x|) from the fast erfc tail above it.
template <class P> NT2G_HD float erf(float a0)
{
    if (is_nan(a0)) return a0;
    const float x = fabsf(a0);
    if (x == f_inf()) return copysignf(1.0f, a0);
    if (x < bits_f(NT2G_TWOTHIRD))
        return P::mul(a0, horner<P>(P::mul(x, x), bits_f(0xba1fc83bu), bits_f(0x3ba4468du), bits_f(0xbcdb61f4u),
                                    bits_f(0x3de70f22u), bits_f(0xbec0937eu), bits_f(0x3f906ebau)));
    float r2;
    if (P::exact) {
        const float z = P::sub(P::div(x, P::add(x, 1.0f)), 0.4f);
        r2 = P::sub(1.0f, P::mul(exp<P>(-P::mul(x, x)), erfc2_kernel<P>(z)));
    } else {
        r2 = Fast::sub(1.0f, erfc_tail_fast<false>(x));
    }
    return (a0 < 0.0f) ? -r2 : r2;
}

// expx2 = e^(x^2) (exponential/functions/scalar/expx2.hpp, one argument):
// e^(m^2) e^(2mf + f^2) with m = 32 floor(x/32 + 1/2) (NT2's float constants
// Expx2c1 = 32, Expx2c2 = 1/32), +inf past Maxlog.  Fast: x^2 split exactly
// by an FMA, e^hi (1 + lo), so the rounding of x^2 is not magnified by e^.
template <class P> NT2G_HD float expx2(float a0)
{
    const float x = fabsf(a0);
    if (x == f_inf()) return f_inf();
    if (!P::exact) {
        const float hi = Fast::mul(x, x), lo = Fast::fma(x, x, -hi);
        const float e = exp<Fast>(hi);
        return (e < f_inf()) ? Fast::fma(e, lo, e) : e;
    }
    const float m = P::mul(32.0f, floorf(P::add(P::mul(0.03125f, x), 0.5f)));
    const float f = P::sub(x, m);
    const float u = P::mul(m, m);
    const float u1 = P::add(P::mul(P::mul(2.0f, m), f), P::mul(f, f));
    if (P::add(u, u1) > bits_f(NT2G_MAXLOG)) return f_inf();
    return P::mul(exp<P>(u), exp<P>(u1));
}

// erfcx = e^(x^2) erfc(x) (euler/functions/scalar/erfcx.hpp, single_):
// expx2(x) erfc(x) below 2/3, else the erfc2 kernel; 0 at +inf.  Fast: for
// x >= 0 the fast erfc tail without its exponential, w R(w) (1 + r); below 0,
// 2 e^(x^2) - erfcx(-x).
template <class P> NT2G_HD float erfcx(float a0)
{
    if (a0 == f_inf()) return 0.0f;
    if (is_nan(a0)) return a0;
    if (P::exact) {
        if (a0 < bits_f(NT2G_TWOTHIRD)) return P::mul(expx2<P>(a0), erfc<P>(a0));
        return erfc2_kernel<P>(P::sub(P::div(a0, P::add(a0, 1.0f)), 0.4f));
    }
    const float a = fabsf(a0);
    const float den = Fast::fma(0.5f, a, 1.0f);
    const float dlo = Fast::fma(0.5f, a, Fast::sub(1.0f, den));
    float w = Fast::div(1.0f, den);
    const float r = Fast::fma(-dlo, w, Fast::fma(-den, w, 1.0f));
    const float wr = Fast::mul(w, erfc_tail_poly(w));
    const float t = (a < f_inf()) ? Fast::fma(r, wr, wr) : 0.0f;
    return (a0 < 0.0f) ? Fast::fma(2.0f, expx2<Fast>(a0), -t) : t;
}

// exprecneg = e^(-1/x), exprecnegc = 1 - e^(-1/x) (exponential/functions/
// generic/exprecneg.hpp, exprecnegc.hpp: exp(-rec(x)), -expm1(-rec(x))).
// Fast: 1/x carried as hi + lo (the division's residual), so its rounding is
// not magnified by the exponential: e^(-hi) (1 - lo).
template <class P> NT2G_HD float exprecneg(float a0)
{
    const float hi = P::div(1.0f, a0);
    if (P::exact) return exp<P>(-hi);
    const bool fin = fabsf(hi) < f_inf() && fabsf(a0) < f_inf();
    const float lo = fin ? Fast::mul(Fast::fma(-hi, a0, 1.0f), hi) : 0.0f;
    const float e = exp<Fast>(-hi);
    return (e < f_inf()) ? Fast::fma(-e, lo, e) : e;
}
template <class P> NT2G_HD float exprecnegc(float a0)
{
    const float hi = P::div(1.0f, a0);
    if (P::exact) return -expm1<P>(-hi);
    const bool fin = fabsf(hi) < f_inf() && fabsf(a0) < f_inf();
    const float lo = fin ? Fast::mul(Fast::fma(-hi, a0, 1.0f), hi) : 0.0f;
    const float em1 = expm1<Fast>(-hi);
    // 1 - e^(-hi-lo) = -em1 + (em1 + 1) lo
    return (fabsf(em1) < f_inf()) ? Fast::fma(Fast::add(em1, 1.0f), lo, -em1) : -em1;
}

// sqrt1pm1 = sqrt(1+x) - 1 (exponential/functions/generic/sqrt1pm1.hpp):
// x/(1 + sqrt(1+x)) below 1/2 in magnitude, sqrt(1+x) - 1 above.  Fast: the
// quotient everywhere (no cancellation), +inf at +inf.
template <class P> NT2G_HD float sqrt1pm1(float a0)
{
    const float t = P::sqrt(P::add(a0, 1.0f));
    const float q = P::div(a0, P::add(t, 1.0f));
    if (P::exact) return (fabsf(a0) < 0.5f) ? q : P::sub(t, 1.0f);
    return (a0 == f_inf()) ? a0 : q;
}

// erfinv, erfcinv (euler/functions/scalar/erfinv.hpp, erfcinv.hpp, single_:
// Giles' approximation): w = -log((1-x)(1+x)) (erfcinv: -log(x(2-x)) and
// 1 - x as the argument), a degree-8 polynomial in w - 2.5 below 5, else a
// degree-8 polynomial in sqrt(w) - 3 (erfcinv: a 5/5 rational in sqrt(w))
// (details/erfinv_kernel.hpp); +-inf at the ends.  Fast: the same with FMAs
// and 1 - x^2 (2x - x^2) rounded once.
template <class P> NT2G_HD float erfinv1(float w)
{
    return horner<P>(w, bits_f(0x32f16588u), bits_f(0x34b84b36u), bits_f(0xb66c7357u), bits_f(0xb6935ac1u),
                     bits_f(0x396532dbu), bits_f(0xbaa45408u), bits_f(0xbb88e4efu), bits_f(0x3e7c8f63u),
                     bits_f(0x3fc02e2fu));
}
template <class P> NT2G_HD float erfinv2(float w)
{
    return horner<P>(w, bits_f(0xb951f09bu), bits_f(0x38d3b56bu), bits_f(0x3ab0dc72u), bits_f(0xbb70bde7u),
                     bits_f(0x3bbc127bu), bits_f(0xbbf9c5d7u), bits_f(0x3c1aa57eu), bits_f(0x3f8036dbu),
                     bits_f(0x40354f7eu));
}
template <class P> NT2G_HD float erfinv(float a0)
{
    const float q = P::exact ? P::mul(P::sub(1.0f, a0), P::add(a0, 1.0f)) : Fast::fma(-a0, a0, 1.0f);
    float w = -log<P>(q);
    if (w == f_inf()) return copysignf(1.0f, a0) * w;
    if (w < 5.0f) return P::mul(a0, erfinv1<P>(P::sub(w, 2.5f)));
    return P::mul(a0, erfinv2<P>(P::sub(P::sqrt(w), 3.0f)));
}
template <class P> NT2G_HD float erfcinv(float a0)
{
    const float a00 = P::sub(1.0f, a0);
    const float q = P::exact ? P::mul(a0, P::sub(2.0f, a0))
                             : ((a0 > 2.0f) ? f_nan() : Fast::fma(-a0, a0, Fast::add(a0, a0)));
    float w = -log<P>(q);
    if (w == f_inf()) return copysignf(1.0f, a00) * w;
    if (w < 5.0f) return P::mul(a00, erfinv1<P>(P::sub(w, 2.5f)));
    if (!P::exact && w < 16.0f)  // Fast: erfinv's second polynomial, where it holds, for both ends
        return Fast::mul(a00, erfinv2<Fast>(Fast::sub(Fast::sqrt(w), 3.0f)));
    w = P::sqrt(w);
    const float num = horner<P>(w, bits_f(0x3b3a8aeeu), bits_f(0x3ba62c57u), bits_f(0xbc8bcf63u), bits_f(0x3c98e17cu),
                                bits_f(0xbbaf8bfeu));
    const float den = horner<P>(w, bits_f(0x321631b2u), bits_f(0x3b3a73c1u), bits_f(0x3ba9025fu), bits_f(0xbc5d80aau),
                                bits_f(0x3c2f4022u));
    float r = P::div(num, den);
    if (!P::exact && r < 9.3f) {
        // Fast: one Newton step on erfc(r) = t (t = x, or 2 - x exactly at the
        // other end): r += (erfcx(r) - t e^(r^2)) sqrt(pi)/2, both factors
        // accurate where erfc itself would underflow
        const float t = (a00 > 0.0f) ? a0 : Fast::sub(2.0f, a0);
        r = Fast::fma(Fast::fma(-t, expx2<Fast>(r), erfcx<Fast>(r)), 0.886226925f, r);
    }
    return copysignf(r, a00);
}

// gamma (euler/functions/scalar/gamma.hpp): below -33 the reflection with
// Stirling's formula (scalar/stirling.hpp + details/stirling_kernel.hpp),
// else x stepped into [2, 3) one unit at a time, the product of the steps
// times the degree-7 polynomial of details/gamma_kernel.hpp.  NT2's steps from
// a large x make the product +inf long before the end (and never end from 2^24
// on, where x - 1 == x): from 64 on the result is +inf at once.  Fast: the
// product carried as a float-float pair (x - 1 and x + 1 are exact in this
// range, each multiply or divide adds only its residual), and the reflection
// below -33 from that same product for |x| instead of Stirling's formula.
template <class P> NT2G_HD float stirling(float a0)
{
    if (is_nan(a0)) return a0;
    if (a0 > bits_f(0x420c28f3u)) return f_inf();  // Stirlinglargelim
    float w = P::div(1.0f, a0);
    w = P::fma(w, horner<P>(w, bits_f(0xb970b359u), bits_f(0xbb2fb930u), bits_f(0x3b638e39u), bits_f(0x3daaaaabu)),
               1.0f);
    float y = exp<P>(-a0);
    if (y == 0.0f) return f_inf();
    const float z = P::sub(a0, 0.5f);
    if (a0 >= bits_f(0x41d628f6u)) {  // Stirlingsplitlim
        const float v = pow<P>(a0, P::mul(z, 0.5f));
        y = P::mul(y, v);
        y = P::mul(y, v);
    } else {
        y = P::mul(y, pow<P>(a0, z));
    }
    return P::mul(y, P::mul(bits_f(0x40206c99u), w));  // Sqrt_2pi
}

// Gamma(x) for x in [-33, 64] by NT2's stepping; Fast keeps the product as zh + zl
template <class P> NT2G_HD float gamma_steps(float x)
{
    float zh = 1.0f, zl = 0.0f;
    while (x >= 3.0f) {
        x = P::sub(x, 1.0f);
        if (P::exact) {
            zh = P::mul(zh, x);
        } else {
            const float p = Fast::mul(zh, x);
            zl = Fast::fma(zl, x, Fast::fma(zh, x, -p));
            zh = p;
        }
    }
    for (int k = 0; k < 2; ++k) {  // x < 0 steps, then up to two below 2
        while (k == 0 ? (x < 0.0f) : (x < 2.0f)) {
            if (k == 1 && x == 0.0f) return f_nan();
            if (P::exact) {
                zh = P::div(zh, x);
            } else {
                const float q = Fast::div(zh, x);
                zl = Fast::div(Fast::add(Fast::fma(-q, x, zh), zl), x);
                zh = q;
            }
            x = P::add(x, 1.0f);
        }
    }
    // (Fast: once the product is +inf its low part is NaN and is dropped)
    const bool fin = P::exact || fabsf(zh) < f_inf();
    if (x == 2.0f) return fin ? (P::exact ? zh : Fast::add(zh, zl)) : zh;
    x = P::sub(x, 2.0f);
    const float g = horner<P>(x, bits_f(0x3ad28b22u), bits_f(0x3ba90c99u), bits_f(0x3b91db14u), bits_f(0x3d93ae7cu),
                              bits_f(0x3da82a34u), bits_f(0x3ed2d411u), bits_f(0x3ed87799u), 1.0f);
    if (P::exact || !fin) return P::mul(zh, g);
    return Fast::fma(zh, g, Fast::mul(zl, g));
}

template <class P> NT2G_HD float gamma(float a0)
{
    if (a0 == 0.0f) return copysignf(f_inf(), a0);
    if (is_nan(a0) || a0 == -f_inf()) return f_nan();
    if (a0 == f_inf()) return a0;
    const float q = fabsf(a0);
    if (a0 < -33.0f) {
        float p = floorf(q);
        if (p == q) return f_nan();
        const bool iseven = !(((int)p) & 1);
        float z = P::sub(q, p);
        if (z > 0.5f) {
            p = P::add(p, 1.0f);
            z = P::sub(q, p);
        }
        z = P::mul(q, sinpi<P>(z));
        if (z == 0.0f) return f_nan();
        const float st = P::exact ? stirling<P>(q) : gamma_steps<P>(q);
        const float r = P::div(bits_f(0x40490fdbu), P::mul(fabsf(z), st));
        return iseven ? -r : r;
    }
    if (a0 > 64.0f) return f_inf();
    return gamma_steps<P>(a0);
}

// gammaln (euler/functions/scalar/gammaln.hpp, single_): the reflection for
// x < 0, the polynomials of details/gammaln_kernel.hpp around 1 and 2 below
// 6.5 (with up to four steps), else Stirling's series with its correction up
// to 1e4.  Both policies follow it (Fast with FMAs).
template <class P> NT2G_HD float gammaln_b(float x)
{
    return horner<P>(x, bits_f(0x3a1ebb94u), bits_f(0xbaabeab1u), bits_f(0x3b3ba883u), bits_f(0xbbf164fdu),
                     bits_f(0x3ca89ed8u), bits_f(0xbd89f07eu), bits_f(0x3ea51a64u), bits_f(0x3ed87730u));
}

template <class P> NT2G_HD float gammaln_pos(float x)
{
    if (!P::exact && x < 6.5f) {
        // Fast: NT2's steps into [1.5, 2.5] as four predicated iterations
        // (the same products, no data-dependent loop or branch), the log-gamma
        // polynomial around 2 with + or - log of the product, and the one
        // around 1 selected on [0.75, 1.25): one log, two polynomials
        float nx = 0.0f, t = x, z = 1.0f;
        const bool up = x < 1.5f;
        for (int k = 0; k < 4; ++k) {  // t = x + nx as NT2 forms it (fixed trip count: unrolled)
            const bool dn = t > 2.5f, rise = t < 1.5f;
            const float nd = Fast::sub(nx, 1.0f), td = Fast::add(x, nd);
            z = dn ? Fast::mul(z, td) : rise ? Fast::mul(z, t) : z;
            nx = dn ? nd : rise ? Fast::add(nx, 1.0f) : nx;
            t = dn ? td : rise ? Fast::add(x, nx) : t;
        }
        const float xb = Fast::add(x, Fast::sub(nx, 2.0f));
        const float lz = log<Fast>(z);
        const float rb = Fast::fma(xb, gammaln_b<Fast>(xb), up ? -lz : lz);
        const float xc = Fast::sub(x, 1.0f);
        const float rc = Fast::mul(xc, horner<Fast>(xc, bits_f(0x3e0c3c4fu), bits_f(0xbe22d329u), bits_f(0x3e2d4dabu),
                                                   bits_f(0xbe53c04fu), bits_f(0x3e8a898bu), bits_f(0xbecd27a8u),
                                                   bits_f(0x3f528d34u), bits_f(0xbf13c468u)));
        const float r = (x >= 0.75f && x < 1.25f) ? rc : rb;
        return (x == 0.0f) ? f_inf() : r;
    }
    if (x < 6.5f) {
        float z = 1.0f, tx = x, nx = 0.0f;
        if (x >= 1.5f) {
            while (tx > 2.5f) {
                nx = P::sub(nx, 1.0f);
                tx = P::add(x, nx);
                z = P::mul(z, tx);
            }
            x = P::add(x, P::sub(nx, 2.0f));
            return P::add(P::mul(x, gammaln_b<P>(x)), log<P>(z));
        }
        if (x >= 1.25f) {
            z = P::mul(z, x);
            x = P::sub(x, 1.0f);
            return P::sub(P::mul(x, gammaln_b<P>(x)), log<P>(z));
        }
        if (x >= 0.75f) {
            x = P::sub(x, 1.0f);
            return P::mul(x, horner<P>(x, bits_f(0x3e0c3c4fu), bits_f(0xbe22d329u), bits_f(0x3e2d4dabu),
                                          bits_f(0xbe53c04fu), bits_f(0x3e8a898bu), bits_f(0xbecd27a8u),
                                          bits_f(0x3f528d34u), bits_f(0xbf13c468u)));
        }
        while (tx < 1.5f) {
            if (tx == 0.0f) return f_inf();
            z = P::mul(z, tx);
            nx = P::add(nx, 1.0f);
            tx = P::add(x, nx);
        }
        x = P::add(x, P::sub(nx, 2.0f));
        const float p = P::mul(x, gammaln_b<P>(x));
        return P::sub(p, log<P>(z));
    }
    float r = P::fma(P::sub(x, 0.5f), log<P>(x), P::sub(bits_f(0x3f6b3f8eu), x));  // Logsqrt2pi
    if (x <= 1.0e4f) {
        const float z = P::div(1.0f, x);
        const float p = P::mul(z, z);
        r = P::fma(z, horner<P>(p, bits_f(0x3a31fd69u), bits_f(0xbb358701u), bits_f(0x3daaaa94u)), r);
    }
    return r;
}

template <class P> NT2G_HD float gammaln(float a0)
{
    if (a0 > bits_f(0x7bc3f8eau) || a0 == 0.0f) return f_inf();  // Maxgammaln
    const float q = fabsf(a0);
    // Fast: below 2^-20 in magnitude -log|x| (NT2's q sinpi(q) underflows to
    // 0 for the smallest negative x and gives +inf there)
    if (!P::exact && q < 0x1p-20f) return -log<P>(q);
    if (a0 < 0.0f) {
        if (q > bits_f(0x7bc3f8eau)) return f_nan();
        const float w = gammaln_pos<P>(q);
        float p = floorf(q);
        if (p == q) return f_inf();
        float z = P::sub(q, p);
        if (z > 0.5f) {
            p = P::add(p, 1.0f);
            z = P::sub(p, q);
        }
        z = P::mul(q, sinpi<P>(z));
        if (z == 0.0f) return f_inf();
        return P::sub(-log<P>(P::mul(bits_f(0x3ea2f983u), fabsf(z))), w);
    }
    return gammaln_pos<P>(a0);
}

// ------------------------------------------------------------- signgam --
// NT2's sign of Gamma (EUL/scalar/signgam.hpp): NaN at the non-positive
// integers and at -inf; below zero 1 - 2 is_odd(floor(x)), with boost.simd's
// float is_odd(f) = is_flint((f - 1) * 1/2) and is_flint(y) = frac(y) == 0;
// NaN passes through; 1 above zero.  Both policies.
NT2G_HD float signgam(float a0)
{
    if (a0 <= 0.0f) {
        if (a0 - truncf(a0) == 0.0f || a0 == -f_inf()) return f_nan();
        const float h = (floorf(a0) - 1.0f) * 0.5f;
        return (h - truncf(h) == 0.0f) ? -1.0f : 1.0f;
    }
    return is_nan(a0) ? a0 : 1.0f;
}

// ------------------------------------------------------------- digamma --
// NT2's float digamma evaluates its double algorithm and rounds the result
// (EUL/scalar/digamma.hpp: the single_ overload calls the double one), so
// both policies do the same here.  The double algorithm, with NT2's unfused
// double arithmetic: below 0 the reflection pi / tanpi(r) of the fractional
// part of 1 - x (NaN at the poles); from Digammalargelim = 20 on the
// asymptotic series of digamma_kernel::digamma_imp_large; otherwise down to
// [1, 2] by psi(x) = psi(x - 1) + 1/(x - 1) (or up by -1/x) and NT2's
// rational approximation digamma_1_2 about the root 1.4616..., held as three
// parts (EUL/details/digamma_kernel.hpp).  NT2's double log and tanpi are
// taken as the platform's double log and sinpi / cospi: the float result is
// NT2's unless the two double values straddle a float rounding boundary.
struct D64 {
#if defined(__CUDA_ARCH__)
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double tanpi(double r) { return __ddiv_rn(::sinpi(r), ::cospi(r)); }
#else
    static inline double mul(double a, double b) { volatile double r = a * b; return r; }
    static inline double add(double a, double b) { volatile double r = a + b; return r; }
    static inline double sub(double a, double b) { volatile double r = a - b; return r; }
    static inline double div(double a, double b) { volatile double r = a / b; return r; }
    static inline double tanpi(double r)
    {
        return div(::sin(3.14159265358979323846 * r), ::cos(3.14159265358979323846 * r));
    }
#endif
    static NT2G_HD double fma(double a, double b, double c) { return add(mul(a, b), c); }
};

NT2G_HD double bits_d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d; memcpy(&d, &u, 8); return d;
#endif
}

// Horner over NT2's coefficient order (highest degree first), unfused
template <int N> NT2G_HD double horner_d(double x, const uint64_t (&c)[N])
{
    double acc = bits_d(c[0]);
    for (int i = 1; i < N; ++i) acc = D64::fma(x, acc, bits_d(c[i]));
    return acc;
}

NT2G_HD double digamma_d(double a0)
{
    const double pi = bits_d(0x400921fb54442d18ull);
    double result = 0.0, x = a0;
    if (a0 == 0.0) return ::copysign(bits_d(0x7ff0000000000000ull), a0);
    if (x < 0.0) {
        x = D64::sub(1.0, x);
        result = D64::sub(x, ::floor(x));
        if (result > 0.5) result = D64::sub(result, 1.0);
        if (result == 0.5) result = 0.0;
        else if (result != 0.0) result = D64::div(pi, D64::tanpi(result));
        else result = bits_d(0x7ff8000000000000ull);
    }
    if (x >= 20.0) {  // digamma_imp_large
        const uint64_t c[8] = {0xbfdc5e5e5e5e5e5eull, 0x3fb5555555555555ull, 0xbf95995995995996ull,
                               0x3f7f07c1f07c1f08ull, 0xbf71111111111111ull, 0x3f70410410410410ull,
                               0xbf81111111111111ull, 0x3fb5555555555555ull};
        const double xm = D64::sub(x, 1.0);
        double r = ::log(xm);
        r = D64::add(r, D64::div(1.0, D64::mul(2.0, xm)));
        const double z = D64::div(1.0, D64::mul(xm, xm));
        r = D64::sub(r, D64::mul(z, horner_d(z, c)));
        return D64::add(r, result);
    }
    while (x > 2.0) {
        x = D64::sub(x, 1.0);
        result = D64::add(result, D64::div(1.0, x));
    }
    if (x < 1.0) {
        result = D64::div(-1.0, x);
        x = D64::add(x, 1.0);
    }
    // digamma_1_2
    const double Y = (double)0.99558162689208984f;
    const double root1 = 1569415565.0 / 1073741824.0, root2 = (381566830.0 / 1073741824.0) / 1073741824.0,
                 root3 = 0.9016312093258695918615325266959189453125e-19;
    const uint64_t P6[6] = {0xbf60f7e5f66c2537ull, 0xbfa72b2e63723c78ull, 0xbfd2821c13c5e2bfull,
                            0xbfe4cf68d26e295aull, 0xbfd4d5d0f9ab412full, 0x3fd04e9e69894978ull};
    const uint64_t Q7[7] = {0xbea2b84f95bbf448ull, 0x3f616fc90a0a1908ull, 0x3fabb9c8cc612ca3ull,
                            0x3fdbe65d28de361cull, 0x3ff75eb79397c930ull, 0x40009d1b06674d41ull,
                            0x3ff0000000000000ull};
    double g = D64::sub(x, root1);
    g = D64::sub(g, root2);
    g = D64::sub(g, root3);
    const double xm = D64::sub(x, 1.0);
    const double r = D64::div(horner_d(xm, P6), horner_d(xm, Q7));
    return D64::add(D64::fma(g, Y, D64::mul(g, r)), result);
}

template <class P> NT2G_HD float digamma(float a0) { return (float)digamma_d((double)a0); }

// -------------------------------------------------------------- dawson --
// NT2's float Dawson integral (EUL/scalar/dawson.hpp with the float rational
// approximations of EUL/details/dawson_kernel.hpp, Cephes' dawsnf): below
// |x| = 3.25 x P(x^2)/Q(x^2); below 6.25 and up to 1e9 copysign(y/2, x) with
// y = 1/|x| + x^-2 N(x^-2) / (D(x^-2) |x|); beyond, copysign(1/(2|x|), x).
template <class P> NT2G_HD float dawson(float a0)
{
    const float x = fabsf(a0);
    float xx = P::mul(x, x);
    if (x < 3.25f) {
        const float n = horner<P>(xx, bits_f(0x2d47fd98u), bits_f(0x30697185u), bits_f(0x32a70489u),
                                  bits_f(0x357fdc17u), bits_f(0x364e9480u), bits_f(0x39b8d18bu), bits_f(0xba5edc97u),
                                  bits_f(0x3d2d1abcu), bits_f(0xbdbbe665u), bits_f(0x3f800000u));
        const float d = horner<P>(xx, bits_f(0x2dd36efbu), bits_f(0x30cc991au), bits_f(0x335fe1b9u),
                                  bits_f(0x35aacdaeu), bits_f(0x37c306e7u), bits_f(0x39aaab31u), bits_f(0x3b6497e8u),
                                  bits_f(0x3ce4ec9bu), bits_f(0x3e22afeeu), bits_f(0x3f132ddeu), bits_f(0x3f800000u));
        return P::mul(a0, P::div(n, d));
    }
    xx = P::div(1.0f, xx);
    float n, d;
    if (x < 6.25f) {
        n = horner<P>(xx, bits_f(0x3f024ae3u), bits_f(0xbe7aa0e7u), bits_f(0x3dc0d25du), bits_f(0xbcb32b13u),
                      bits_f(0x3b6fff71u), bits_f(0xb9dde22au), bits_f(0x3816d831u), bits_f(0xb6100aefu),
                      bits_f(0x33c36c5fu), bits_f(0xb1251d8au), bits_f(0x2e1dfe15u));
        d = horner<P>(xx, bits_f(0x3f800000u), bits_f(0xbf21c042u), bits_f(0x3e726344u), bits_f(0xbd59d3f0u),
                      bits_f(0x3c0af173u), bits_f(0xba7882fcu), bits_f(0x38a3cafeu), bits_f(0xb698f761u),
                      bits_f(0x344b0b83u), bits_f(0xb1a8d160u), bits_f(0x2e9dfe10u));
    } else {
        if (x > 1.0e9f) return P::mul(0.5f, copysignf(P::div(1.0f, x), a0));
        n = horner<P>(xx, bits_f(0xbf173118u), bits_f(0x3f211590u), bits_f(0xbe3101f1u), bits_f(0x3c8708d6u),
                      bits_f(0xb9ff3ce5u));
        d = horner<P>(xx, bits_f(0x3f800000u), bits_f(0xc02caf51u), bits_f(0x3fddc960u), bits_f(0xbec9942cu),
                      bits_f(0x3d0d0443u), bits_f(0xba7f3ce5u));
    }
    const float y = P::add(P::div(1.0f, x), P::div(P::mul(xx, n), P::mul(d, x)));
    return copysignf(P::mul(0.5f, y), a0);
}

// -------------------------------------------------------------- spence --
// NT2's float dilogarithm (EUL/scalar/spence.hpp:27-70, Cephes' spencef):
// NaN below 0, 0 at 1, pi^2/6 at 0; x > 2 maps to 1/x and x > 1.5 to
// w = 1/x - 1 (flag 2), x < 1/2 to w = -x (flag 1), else w = x - 1;
// y = -w P(w) (degree 10), then pi^2/6 - log(x) log(1 - x) - y for flag 1 and
// -(1/2) log(x)^2 - y for flag 2.
template <class P> NT2G_HD float spence(float a0)
{
    float x = a0;
    if (x < 0.0f) return f_nan();
    if (x == 1.0f) return 0.0f;
    const float pi2o6 = bits_f(0x3fd28d33u);
    if (x == 0.0f) return pi2o6;
    int flag = 0;
    if (x > 2.0f) {
        x = P::div(1.0f, x);
        flag |= 2;
    }
    float w;
    if (x > 1.5f) {
        w = P::sub(P::div(1.0f, x), 1.0f);
        flag |= 2;
    } else if (x < 0.5f) {
        w = -x;
        flag |= 1;
    } else {
        w = P::sub(x, 1.0f);
    }
    float y = P::mul(-w, horner<P>(w, bits_f(0x3c80e79eu), bits_f(0xbc8a8ad6u), bits_f(0x3c1f4a7fu),
                                   bits_f(0xbc604c2fu), bits_f(0x3caa7af5u), bits_f(0xbce56409u),
                                   bits_f(0x3d23ba15u), bits_f(0xbd7ff525u), bits_f(0x3de38e97u),
                                   bits_f(0xbe800004u), bits_f(0x3f800000u)));
    if (flag & 1) y = P::sub(P::sub(pi2o6, P::mul(log<P>(x), log<P>(P::sub(1.0f, x)))), y);
    if (flag & 2) {
        const float z = log<P>(x);
        y = P::sub(P::mul(-0.5f, P::mul(z, z)), y);
    }
    return y;
}

// An integer operand carried in a float (nthroot's n, expni's n): truncated
// toward zero, saturated to the int32 range, NaN as 0.
NT2G_HD int32_t int_operand(float b)
{
    if (!(b == b)) return 0;
    if (b >= 2147483648.0f) return 2147483647;
    if (b <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)b;
}

// NT2's pow of a float by an integer (EXP/generic/pow.hpp:111-140): binary
// powering of |n| (the base squared after every bit, the last square
// unused), the reciprocal for n < 0.
template <class P> NT2G_HD float pow_int(float a0, int32_t n)
{
    uint32_t e = n < 0 ? 0u - (uint32_t)n : (uint32_t)n;
    float base = a0, r = 1.0f;
    while (e) {
        if (e & 1u) r = P::mul(r, base);
        e >>= 1;
        base = P::mul(base, base);
    }
    return n < 0 ? P::div(1.0f, r) : r;
}

// ------------------------------------------------------------- nthroot --
// NT2's float nthroot(x, n) (EXP/scalar/nthroot.hpp:29-49): NaN for x < 0
// and even n; x for |x| = 1; n = 0: 0 below |x| = 1, sign(x) inf above; 0 for
// x = 0; x for x = +-inf; else y = pow(|x|, 1/n) refined by one Newton step
// y -= (y^n - |x|) / (n y^(n-1)) (integer powers), negated for x < 0.
template <class P> NT2G_HD float nthroot(float a0, int32_t n)
{
    const bool neg = a0 < 0.0f, odd = (n & 1) != 0;
    if (neg && !odd) return f_nan();
    const float x = fabsf(a0);
    if (x == 1.0f) return a0;
    if (n == 0) return x < 1.0f ? 0.0f : P::mul(nt2_sign(a0), f_inf());
    if (a0 == 0.0f) return 0.0f;
    if (x == f_inf()) return a0;
    const float an = (float)n;
    float y = pow<P>(x, P::div(1.0f, an));
    if (y != 0.0f)
        y = P::sub(y, P::div(P::sub(pow_int<P>(y, n), x), P::mul(an, pow_int<P>(y, n - 1))));
    return (neg && odd) ? -y : y;
}

// --------------------------------------------------------------- expni --
// NT2's float exponential integral E_n(x) (EUL/scalar/expni.hpp:37-127,
// Cephes' expn in float): NaN for n < 0 or x < 0; 0 above Maxlog; at x = 0
// inf (n < 2) or 1/(n - 1); e^-x / x for n = 0; an asymptotic expansion for
// n > 5000; the power series with psi(n) for x <= 1; else the continued
// fraction, rescaled by Halfeps when |p_k| exceeds Expnibig = 2^24.  Both
// loops stop when the relative change falls to Halfeps = 2^-24 -- NT2's
// loops have no other bound; here they also stop after kExpniTerms terms.
constexpr int kExpniTerms = 10000;

template <class P> NT2G_HD float expni(int32_t n, float x)
{
    const float halfeps = bits_f(0x33800000u), big = bits_f(0x4b800000u);
    if (n < 0 || x < 0.0f) return f_nan();
    if (x > bits_f(NT2G_MAXLOG)) return 0.0f;
    if (x == 0.0f) return n < 2 ? f_inf() : P::div(1.0f, P::sub((float)n, 1.0f));
    if (n == 0) return P::div(exp<P>(-x), x);
    if (n > 5000) {
        const float xk = P::add(x, (float)n), yk = P::div(1.0f, P::mul(xk, xk)), t = (float)n;
        const float inner = P::add(P::sub(P::mul(6.0f, P::mul(x, x)), P::mul(P::mul(8.0f, t), x)), P::mul(t, t));
        float ans = P::mul(P::mul(yk, t), inner);
        ans = P::mul(yk, P::add(ans, P::mul(t, P::sub(t, P::mul(2.0f, x)))));
        ans = P::mul(yk, P::add(ans, t));
        return P::div(P::mul(P::add(1.0f, ans), exp<P>(-x)), xk);
    }
    if (x <= 1.0f) {
        float psi = P::sub(-bits_f(0x3f13c468u), log<P>(x));  // -Euler - log(x)
        for (int32_t i = n - 1; i; --i) psi = P::add(psi, P::div(1.0f, (float)i));
        const float z = -x;
        float xk = 0.0f, yk = 1.0f, pk = P::sub(1.0f, (float)n), t;
        float ans = (n == 1) ? 0.0f : P::div(1.0f, pk);
        int it = 0;
        do {
            xk = P::add(xk, 1.0f);
            yk = P::mul(yk, P::div(z, xk));
            pk = P::add(pk, 1.0f);
            if (pk != 0.0f) ans = P::add(ans, P::div(yk, pk));
            t = ans != 0.0f ? fabsf(P::div(yk, ans)) : 1.0f;
        } while (t > halfeps && ++it < kExpniTerms);
        const float tn = (float)n, r = (float)(n - 1);
        return P::sub(P::div(P::mul(pow<P>(z, r), psi), gamma<P>(tn)), ans);
    }
    int32_t k = 1;
    float t, pkm2 = 1.0f, qkm2 = x, pkm1 = 1.0f, qkm1 = P::add(x, (float)n);
    float ans = P::div(pkm1, qkm1);
    int it = 0;
    do {
        const bool odd = ((++k) & 1) != 0;
        const float yk = odd ? 1.0f : x;
        const float xk = odd ? (float)(n + (k - 1) / 2) : (float)(k / 2);
        const float pk = P::add(P::mul(pkm1, yk), P::mul(pkm2, xk));
        const float qk = P::add(P::mul(qkm1, yk), P::mul(qkm2, xk));
        if (qk != 0.0f) {
            const float r = P::div(pk, qk);
            t = fabsf(P::div(P::sub(ans, r), r));
            ans = r;
        } else {
            t = 1.0f;
        }
        pkm2 = pkm1;
        pkm1 = pk;
        qkm2 = qkm1;
        qkm1 = qk;
        if (fabsf(pk) > big) {
            pkm2 = P::mul(pkm2, halfeps);
            pkm1 = P::mul(pkm1, halfeps);
            qkm2 = P::mul(qkm2, halfeps);
            qkm1 = P::mul(qkm1, halfeps);
        }
    } while (t > halfeps && ++it < kExpniTerms);
    return P::mul(ans, exp<P>(-x));
}

// ------------------------------------------------------------ gammainc --
// NT2's gammainc(x, a) (EUL/scalar/gammainc.hpp:37-43) is 1 for a = 0 or
// x = +inf and otherwise Boost.Math's gamma_p(a, x), the regularised lower
// incomplete gamma function, which for float arguments works in double and
// rounds (Boost's default promote_float policy; domain errors -- a < 0,
// x < 0, a not finite -- give NaN under NT2's errno policy).  Boost.Math is
// not part of NT2's tree, so this is this library's own double evaluation,
// after the published methods: the power series
//   P = D sum_k x^k / ((a+1)...(a+k)),  D = x^a e^-x / Gamma(a+1),
// below x = a + 1; the continued fraction of Q = 1 - P (Legendre's, by the
// modified Lentz method) above; and for a > 1e6 Temme's uniform asymptotic
// expansion (DLMF 8.12.8-8.12.10, first correction term c0).  D is taken as
// exp(a log1pmx(t) - log(2 pi a)/2 - S(a)) with x = a(1 + t), S the Stirling
// series of log Gamma, so that it keeps double accuracy for large a.
NT2G_HD double log1pmx_d(double t)  // log(1 + t) - t
{
    if (fabs(t) > 0.5) return ::log1p(t) - t;
    double term = t, sum = 0.0;
    for (int k = 2; k < 80; ++k) {
        term *= -t;
        const double c = term / k;
        sum += c;
        if (fabs(c) <= 1e-17 * fabs(sum)) break;
    }
    return sum;
}

NT2G_HD double stirling_series_d(double a)  // log Gamma(a) - ((a - 1/2) log a - a + log(2 pi)/2), a >= 10
{
    const double r = 1.0 / a, r2 = r * r;
    return r * (1.0 / 12 - r2 * (1.0 / 360 - r2 * (1.0 / 1260 - r2 * (1.0 / 1680 - r2 * (1.0 / 1188)))));
}

NT2G_HD double gammainc_prefix_d(double x, double a)  // x^a e^-x / Gamma(a + 1)
{
    if (a < 10.0) return ::exp(a * ::log(x) - x - ::lgamma(a + 1.0));
    const double t = (x - a) / a;
    return ::exp(a * log1pmx_d(t) - 0.5 * ::log(6.283185307179586476925 * a) - stirling_series_d(a));
}

NT2G_HD double gammainc_d(double x, double a)
{
    if (a == 0.0 || x == (double)f_inf()) return 1.0;
    if (x != x || a != a || a < 0.0 || x < 0.0 || a == (double)f_inf()) return (double)f_nan();
    if (x == 0.0) return 0.0;
    if (a > 1.0e6) {  // Temme: P = erfc(-eta sqrt(a/2))/2 - e^(-a eta^2/2) c0(eta) / sqrt(2 pi a)
        const double lam = x / a, t = lam - 1.0;
        const double h = -log1pmx_d(t);  // lam - 1 - log(lam) >= 0
        const double eta = (t < 0.0 ? -1.0 : 1.0) * ::sqrt(2.0 * h);
        double c0;
        if (fabs(eta) < 1e-3)
            c0 = -1.0 / 3 + eta * (1.0 / 12 - eta * (2.0 / 135 - eta * (1.0 / 864)));
        else
            c0 = 1.0 / t - 1.0 / eta;
        const double e = ::exp(-a * h) / ::sqrt(6.283185307179586476925 * a);
        return 0.5 * ::erfc(-eta * ::sqrt(0.5 * a)) - e * c0;
    }
    const double d = gammainc_prefix_d(x, a);
    if (x < a + 1.0) {
        double term = 1.0, sum = 1.0;
        for (int k = 1; k < 100000; ++k) {
            term *= x / (a + k);
            sum += term;
            if (term <= 1e-17 * sum) break;
        }
        return d * sum;
    }
    // Q = a D h, h = 1/(x+1-a- 1(1-a)/(x+3-a- 2(2-a)/(x+5-a- ...)))
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, dd = 1.0 / b, h = dd;
    for (int i = 1; i < 100000; ++i) {
        const double an = -i * (i - a);
        b += 2.0;
        dd = an * dd + b;
        if (fabs(dd) < tiny) dd = tiny;
        c = b + an / c;
        if (fabs(c) < tiny) c = tiny;
        dd = 1.0 / dd;
        const double del = dd * c;
        h *= del;
        if (fabs(del - 1.0) <= 1e-16) break;
    }
    return 1.0 - a * d * h;
}

template <class P> NT2G_HD float gammainc(float x, float a) { return (float)gammainc_d((double)x, (double)a); }

// --------------------------------------------------------- gammaincinv --
// NT2's gammaincinv(p, a) (EUL/scalar/gammaincinv.hpp:37-43): +inf for p = 1,
// otherwise Boost.Math's gamma_p_inv(a, p), the x with P(a, x) = p, in double
// for float arguments (NaN outside p in [0, 1], a > 0 finite).  This
// library's own double evaluation: a starting point from the normal quantile
// (Abramowitz & Stegun 26.2.23) through Wilson and Hilferty's cube for
// a >= 1, or from P ~ x^a / Gamma(a + 1) near 0, then Halley steps on
// P(a, x) - p (P' = x^(a-1) e^-x / Gamma(a), P''/P' = (a - 1)/x - 1) kept
// inside the bracket the signs establish (bisected, or doubled while it is
// open above, when a step would leave it) until a step is below 4e-16 of x.
NT2G_HD double gammaincinv_d(double p, double a)
{
    if (p == 1.0) return (double)f_inf();
    if (p != p || a != a || p < 0.0 || p > 1.0 || !(a > 0.0) || a == (double)f_inf()) return (double)f_nan();
    if (p == 0.0) return 0.0;
    double x;
    if (a >= 1.0) {
        const double q = p < 0.5 ? p : 1.0 - p, t = ::sqrt(-2.0 * ::log(q));
        double z = t - (2.515517 + t * (0.802853 + t * 0.010328)) / (1.0 + t * (1.432788 + t * (0.189269 + t * 0.001308)));
        if (p < 0.5) z = -z;
        const double c = 1.0 / (9.0 * a), w = 1.0 - c + z * ::sqrt(c);
        x = a * w * w * w;
        if (!(x > 0.0)) x = 0.5 * a;
    } else {
        x = ::exp((::log(p) + ::lgamma(a + 1.0)) / a);
        if (!(x > 0.0)) x = 1e-300;
    }
    const double lga = ::lgamma(a);
    double lo = 0.0, hi = (double)f_inf();
    for (int it = 0; it < 200; ++it) {
        const double f = gammainc_d(x, a) - p;
        if (f == 0.0) break;
        if (f < 0.0) lo = x;
        else hi = x;
        const double d = ::exp((a - 1.0) * ::log(x) - x - lga);  // P'(x)
        double xn = x;
        if (d > 0.0) {
            const double u = f / d, h = u / (1.0 - 0.5 * u * ((a - 1.0) / x - 1.0));
            xn = x - (h == h ? h : u);
        }
        if (fabs(xn - x) <= 4e-16 * fabs(x)) {  // converged (the step may land on the bracket's end)
            x = xn;
            break;
        }
        if (!(xn > lo && xn < hi)) xn = hi == (double)f_inf() ? 2.0 * x : 0.5 * (lo + hi);
        x = xn;
    }
    return x;
}

template <class P> NT2G_HD float gammaincinv(float p, float a) { return (float)gammaincinv_d((double)p, (double)a); }

}  // namespace nt2g
