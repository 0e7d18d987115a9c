// nt2g_vjp.cuh -- derivatives the reverse sweep of a program needs beyond
// what the forward values give directly (nt2g_jit.cu emits the per-opcode
// adjoint rules; this header is embedded into the run-time compiled source
// after nt2g_math.cuh).
//
// NT2 has no reverse mode: these are the derivatives of the functions as the
// library computes them, written from their mathematical definitions.
#pragma once

namespace nt2g {
namespace vjp {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kLn2 = 0.693147180559945309417f;
constexpr float kLn10 = 2.30258509299404568402f;
constexpr float kTwoOverSqrtPi = 1.12837916709551257390f;
constexpr float kHalfSqrtPi = 0.886226925452758013649f;
constexpr float kInvSqrt2Pi = 0.398942280401432677940f;
constexpr float kDegToRad = 0.0174532925199432957692f;
constexpr float kRadToDeg = 57.2957795130823208768f;
constexpr float kInvLn2 = 1.44269504088896340736f;
constexpr float kInvLn10 = 0.434294481903251827651f;

// 1/x for the derivative arithmetic: the SFU's approximate reciprocal and one
// Newton step (within an ulp of 1/x); where the step would make a NaN (x = 0
// or +-inf) the approximation's own +-inf or 0.  Flushes subnormal x (and a
// subnormal 1/x) to zero first.
NT2G_HD float grcp(float x)
{
#if defined(__CUDA_ARCH__)
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x));
    const float r1 = __fmaf_rn(r0, __fmaf_rn(-x, r0, 1.0f), r0);
    return r1 == r1 ? r1 : r0;
#else
    return 1.0f / x;
#endif
}

// 1/sqrt(x) from the SFU (relative error below 2^-22): +inf at 0, NaN below.
NT2G_HD float grsqrt(float x)
{
#if defined(__CUDA_ARCH__)
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / sqrtf(x);
#endif
}

// d/dx of NT2's Abramowitz-Stegun 26.2.17 fastnormcdf (the approximation
// itself, not the normal density it approximates).  With l = |x|,
// k = 1/(1 + p l), w(l) = c k q(k) e^(-l^2/2) (q the quintic of the
// approximation, c = 1/sqrt(2 pi)): fastnormcdf = 1 - w for x > 0, w
// otherwise, so its derivative is -w'(l) in both halves:
//   -w'(l) = c e^(-l^2/2) k [l q(k) + p k (q(k) + k q'(k))].
template <class D> NT2G_HD float fastnormcdf_grad(float x)
{
    const float p = 0.2316419f;
    const float l = fminf(fabsf(x), 100.0f);
    const float k = grcp(1.0f + p * l);
    // the approximation's coefficients b1..b5 (A&S 26.2.17, as NT2 stores them)
    const float b1 = bits_f(0x3ea385fau), b2 = bits_f(0xbeb68f87u), b3 = bits_f(0x3fe40778u),
                b4 = bits_f(0xbfe91eeau), b5 = bits_f(0x3faa466fu);
    const float q = b1 + k * (b2 + k * (b3 + k * (b4 + k * b5)));
    const float dq = b2 + k * (2.0f * b3 + k * (3.0f * b4 + k * 4.0f * b5));
    const float e = kInvSqrt2Pi * exp<D>(-0.5f * l * l);
    const float r = e * k * (l * q + p * k * (q + k * dq));
    return is_nan(x) ? x : r;
}

// The digamma function psi = Gamma'/Gamma, for the derivatives of gamma
// (Gamma psi) and gammaln (psi).  Reflection psi(x) = psi(1 - x) - pi cot(pi x)
// below 1/2, the recurrence psi(x) = psi(x + 1) - 1/x up to x >= 6, then the
// asymptotic series ln x - 1/(2x) - sum B_2k / (2k x^2k) (Bernoulli numbers
// 1/6, -1/30, 1/42, -1/30: terms 1/12, -1/120, 1/252, -1/240).  NaN at the
// poles (zero and the negative integers).
template <class D> NT2G_HD float digamma(float x)
{
    if (is_nan(x) || (x <= 0.0f && x == floorf(x))) return f_nan();
    if (x == f_inf()) return x;
    float acc = 0.0f;
    if (x < 0.5f) {
        acc = -kPi * cotpi<D>(x);
        x = 1.0f - x;
    }
    while (x < 6.0f) {
        acc -= 1.0f / x;
        x += 1.0f;
    }
    const float r = 1.0f / x, r2 = r * r;
    const float series = r2 * (1.0f / 12.0f - r2 * (1.0f / 120.0f - r2 * (1.0f / 252.0f - r2 * (1.0f / 240.0f))));
    return acc + log<D>(x) - 0.5f * r - series;
}

// d/dx sin(x)/x = (cos x - sinc x)/x, which cancels as x -> 0: below 1/2 in
// magnitude the derivative of the Taylor series 1 - x^2/6 + x^4/120 -
// x^6/5040 + x^8/362880 instead, -x/3 + x^3/30 - x^5/840 + x^7/45360.
// sinc is constant (1) below Eps and 0 at infinity: no gradient there.
template <class D> NT2G_HD float sinc_grad(float x, float y)
{
    const float ax = fabsf(x);
    if (ax < bits_f(0x34000000u) || ax == f_inf()) return 0.0f;
    if (ax < 0.5f) {
        const float x2 = x * x;
        return x * (-1.0f / 3.0f + x2 * (1.0f / 30.0f + x2 * (-1.0f / 840.0f + x2 * (1.0f / 45360.0f))));
    }
    return (cos<D>(x) - y) * grcp(x);
}

// sincpi(x) = sinc(pi x): pi sinc'(pi x), the quotient (cospi x - sincpi x)/x
// from |pi x| = 1/2 on.
template <class D> NT2G_HD float sincpi_grad(float x, float y)
{
    const float ax = fabsf(x);
    if (ax < bits_f(0x34000000u) || ax == f_inf()) return 0.0f;
    const float u = kPi * x;
    if (fabsf(u) < 0.5f) {
        const float u2 = u * u;
        return kPi * u * (-1.0f / 3.0f + u2 * (1.0f / 30.0f + u2 * (-1.0f / 840.0f + u2 * (1.0f / 45360.0f))));
    }
    return (cospi<D>(x) - y) * grcp(x);
}

// d/dx sinh(x)/x = (cosh x - sinhc x)/x; below 1/2 the series
// x/3 + x^3/30 + x^5/840 + x^7/45360.
template <class D> NT2G_HD float sinhc_grad(float x, float y)
{
    if (fabsf(x) < 0.5f) {
        const float x2 = x * x;
        return x * (1.0f / 3.0f + x2 * (1.0f / 30.0f + x2 * (1.0f / 840.0f + x2 * (1.0f / 45360.0f))));
    }
    return (cosh<D>(x) - y) * grcp(x);
}

// d/dx E_n(x) = -E_(n-1)(x) for n >= 1 (Abramowitz & Stegun 5.1.26);
// for n = 0, E_0 = e^-x/x and the derivative is -E_0 (1 + 1/x).
template <class D> NT2G_HD float expni_grad(int32_t n, float x, float y)
{
    if (n == 0) return -y * (1.0f + grcp(x));
    return -expni<D>(n - 1, x);
}

// d/dx P(a, x) = x^(a-1) e^-x / Gamma(a), in double (0 at x = 0 for a > 1).
NT2G_HD float gammainc_dx(float x, float a)
{
    const double xd = x, ad = a;
    if (xd == 0.0) return ad < 1.0 ? f_inf() : ad == 1.0 ? 1.0f : 0.0f;
    return (float)::exp((ad - 1.0) * ::log(xd) - xd - ::lgamma(ad));
}

}  // namespace vjp
}  // namespace nt2g
