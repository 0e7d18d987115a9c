// nt2g_exprs.cuh -- per-element bodies of the named fused expressions, shared
// by the plain kernels, the batched persistent kernel and the pattern-bound
// program path so that all of them round identically.
#pragma once
#include "nt2g_math.cuh"

namespace nt2g {

// ---------------------------------------------------------------------------
// Helpers of the fast Black-Scholes path.  Its operands are a priceable
// option's: S, K, T, sigma positive, finite and normal.  Other inputs give NaN
// call/put (one check on d1/d2 replaces the functors' special-value selects);
// the NT2 policy keeps NT2's full IEEE handling.

// log for a positive normal x: NT2's kernel (f_kernel.hpp:43-75) with FMAs,
// without the zero/negative/inf/NaN/subnormal branches; the exponent becomes
// a float by the 2^23 magic-number add instead of an integer conversion.
__device__ __forceinline__ float log_pos_fast(float z)
{
    uint32_t u = f_bits(z);
    float x = bits_f((u & 0x007fffffu) | 0x3f000000u);
    bool lt = x < bits_f(NT2G_SQRT_2O_2);
    // (2^23 + biased exponent) - 2^23 - 126 [- 1]: the unbiased exponent of frexp
    float fe = Fast::sub(bits_f(0x4B000000u | (u >> 23)), lt ? 8388735.0f : 8388734.0f);
    x = Fast::sub(lt ? Fast::add(x, x) : x, 1.0f);
    float x2 = Fast::mul(x, x);
    float y = horner<Fast>(x, bits_f(0xbda5dff0u), bits_f(0x3e0229f9u), bits_f(0xbe04d6b7u), bits_f(0x3e116e80u),
                           bits_f(0xbe2a6aa0u), bits_f(0x3e4cd0a3u), bits_f(0xbe800064u), bits_f(0x3eaaaaa9u));
    y = Fast::mul(Fast::mul(y, x), x2);
    y = Fast::fma(fe, bits_f(NT2G_LOG_2LO), y);
    y = Fast::fma(-0.5f, x2, y);
    return Fast::fma(bits_f(NT2G_LOG_2HI), fe, Fast::add(x, y));
}

// exp for an argument already known finite; clamped to NT2's [Minlog, Maxlog].
__device__ __forceinline__ float exp_clamped_fast(float a0)
{
    a0 = fminf(fmaxf(a0, bits_f(NT2G_MINLOG)), bits_f(NT2G_MAXLOG));
    float scale;
    float s = exp_fast_parts(a0, scale);
    return Fast::mul(Fast::add(s, 1.0f), scale);
}

// 1/sqrt(t) to about one ulp: rsqrt.approx refined by one Newton step.
__device__ __forceinline__ float rsqrt_fast(float t)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
    float h = Fast::mul(t, y);
    return Fast::fma(Fast::mul(0.5f, y), Fast::fma(-h, y, 1.0f), y);
}

// N(d) and N(-d) from one erfc core, without the NaN select (the caller checks d).
__device__ __forceinline__ void normcdf_pair_fast(float x, float &n_pos, float &n_neg)
{
    float half_tail = Fast::mul(0.5f, erfc_tail_fast<true>(fabsf(x)));
    float other = Fast::sub(1.0f, half_tail);
    bool neg = x < 0.0f;
    n_pos = neg ? half_tail : other;
    n_neg = neg ? other : half_tail;
}

// Shared forward prefix of the fast call/put and its adjoint.
struct BsFwd {
    float sq, rs, d1, d2, ert, e;
};

__device__ __forceinline__ BsFwd bs_prefix_fast(float S, float K, float T, float sig, float inv_sig, float r)
{
    BsFwd f;
    f.rs = rsqrt_fast(T);                       // 1/sqrt(T)
    f.sq = Fast::mul(T, f.rs);                  // sqrt(T)
    float lq = log_pos_fast(Fast::fdiv(S, K));
    float a = Fast::fma(Fast::mul(sig, sig), 0.5f, r);
    f.d1 = Fast::mul(Fast::fma(a, T, lq), Fast::mul(f.rs, inv_sig));  // / (sigma sqrt T)
    f.d2 = Fast::fma(-sig, f.sq, f.d1);
    f.ert = exp_clamped_fast(Fast::mul(-r, T));
    f.e = Fast::mul(K, f.ert);
    return f;
}

// Textbook Black-Scholes call+put, written as the NT2 expression
//   d1 = (log(S/K) + fma(sqr(sig),0.5,r)*T) / (sig*sqrt(T))
//   d2 = fnms(sig, sqrt(T), d1)
//   e  = K*exp(-r*T)
//   call = fnms(e, normcdf(d2), S*normcdf(d1))
//   put  = fnms(S, normcdf(-d1), e*normcdf(-d2))
// Nt2 policy: exactly that operation sequence.  Fast policy: the same graph
// with FMAs, rsqrt-based sqrt(T) and 1/(sig sqrt T), approximate-reciprocal
// S/K, and one erfc core shared by N(d) and N(-d).  inv_sig is 1/sig (the
// caller hoists it when sigma is a scalar); the Nt2 policy ignores it.
template <class P>
__device__ __forceinline__ void bs_option(float S, float K, float T, float sig, float inv_sig, float r, float &call,
                                          float &put)
{
    if (P::exact) {
        float sq = P::sqrt(T);
        float lq = log<P>(P::div(S, K));
        float a = P::fma(P::mul(sig, sig), 0.5f, r);
        float d1 = P::div(P::add(lq, P::mul(a, T)), P::mul(sig, sq));
        float d2 = P::sub(d1, P::mul(sig, sq));
        float e = P::mul(K, exp<P>(P::mul(-r, T)));
        float n1, m1, n2, m2;
        normcdf_pair<P>(d1, n1, m1);
        normcdf_pair<P>(d2, n2, m2);
        call = P::sub(P::mul(S, n1), P::mul(e, n2));
        put = P::sub(P::mul(e, m2), P::mul(S, m1));
        return;
    }
    BsFwd f = bs_prefix_fast(S, K, T, sig, inv_sig, r);
    float n1, m1, n2, m2;
    normcdf_pair_fast(f.d1, n1, m1);
    normcdf_pair_fast(f.d2, n2, m2);
    call = Fast::fma(-f.e, n2, Fast::mul(S, n1));
    put = Fast::fma(-S, m1, Fast::mul(f.e, m2));
    if (is_nan(f.d1) || is_nan(f.d2)) { call = f.d1 + f.d2; put = call; }
}

// 1/sigma per option when sigma is a table (rcp.approx + one Newton step).
__device__ __forceinline__ float inv_fast(float x)
{
    float r = Fast::rcp(x);
    return Fast::fma(r, Fast::fma(-x, r, 1.0f), r);
}

// NT2 demo (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59): call only,
// fastnormcdf, d1 = log(S/X) + (fma(sqr(v),0.5,r)*T)/(v*sqrt(T)).
template <class P>
__device__ __forceinline__ float bs_demo_option(float S, float X, float T, float r, float v)
{
    float da = P::sqrt(T);
    float d1 = P::add(log<P>(P::fdiv(S, X)), P::fdiv(P::mul(P::fma(P::mul(v, v), 0.5f, r), T), P::mul(v, da)));
    float d2 = P::exact ? P::sub(d1, P::mul(v, da)) : P::fma(-v, da, d1);
    float a = P::mul(S, fastnormcdf<P>(d1));
    float b = P::mul(X, exp<P>(P::mul(-r, T)));
    return P::exact ? P::sub(a, P::mul(b, fastnormcdf<P>(d2))) : P::fma(-b, fastnormcdf<P>(d2), a);
}

// exp(-sqr(x))*sqrt(abs(y)) + log1p(abs(z))
template <class P>
__device__ __forceinline__ float expr3_elem(float x, float y, float z)
{
    return P::add(P::mul(exp_neg_sqr<P>(x), P::sqrt(fabsf(y))), log1p<P>(fabsf(z)));
}

// Y = alpha*X + Y, two roundings as NT2 (demo/saxpy/nt2/saxpy_nt2.cpp:41)
__device__ __forceinline__ float saxpy_elem(float a, float x, float y) { return __fadd_rn(__fmul_rn(a, x), y); }

// rgb2yuv (demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:30-32).
// Nt2: left to right, unfused, u and v from the rounded y (NT2's result,
// whose b - y / r - y cancellation amplifies y's rounding).
// Fast: y = 0.299r + 0.587g + 0.114b held as yh + yl (each product split
// exactly by FMA, the sum by TwoSum); b - y is formed as TwoSum(b, -yh) minus
// yl, and u = fma(0.492, dh, 0.492*dl) rounds once, so u and v are within
// about half an ulp of their own value even when b or r nearly equals y.
// Memory-bound, so the extra flops are free.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <class P>
__device__ __forceinline__ void yuv_px(float r, float g, float b, float &y, float &u, float &v)
{
    if (P::exact) {
        y = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
        u = __fmul_rn(0.492f, __fsub_rn(b, y));
        v = __fmul_rn(0.877f, __fsub_rn(r, y));
        return;
    }
    float p1 = __fmul_rn(0.299f, r), e1 = __fmaf_rn(0.299f, r, -p1);
    float p2 = __fmul_rn(0.587f, g), e2 = __fmaf_rn(0.587f, g, -p2);
    float p3 = __fmul_rn(0.114f, b), e3 = __fmaf_rn(0.114f, b, -p3);
    float s1, t1, yh, t2;
    two_sum(p1, p2, s1, t1);
    two_sum(s1, p3, yh, t2);
    float yl = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), __fadd_rn(e1, e2)), e3);
    y = __fadd_rn(yh, yl);
    float dh, dl;
    two_sum(b, -yh, dh, dl);
    u = __fmaf_rn(0.492f, dh, __fmul_rn(0.492f, __fsub_rn(dl, yl)));
    two_sum(r, -yh, dh, dl);
    v = __fmaf_rn(0.877f, dh, __fmul_rn(0.877f, __fsub_rn(dl, yl)));
}

// Sigma-delta step on four uint8 pixels packed in a word
// (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:38-57): selinc/seldec of bkg toward
// the frame, d = max - min, m = adds(adds(d,d),d), var toward m where d != 0,
// label = if_zero_else_one(d < var).  Byte-wise SIMD, bit-exact.
__device__ __forceinline__ void sd_word(uint32_t f, uint32_t &b, uint32_t &v, uint32_t &lab)
{
    const uint32_t one = 0x01010101u;
    uint32_t lt = __vcmpltu4(b, f), gt = __vcmpgtu4(b, f);
    b = __vsub4(__vadd4(b, lt & one), gt & one);
    uint32_t d = __vabsdiffu4(b, f);
    uint32_t m = __vaddus4(__vaddus4(d, d), d);
    uint32_t nz = __vcmpne4(d, 0u);
    uint32_t vlt = __vcmpltu4(v, m) & nz, vgt = __vcmpgtu4(v, m) & nz;
    v = __vsub4(__vadd4(v, vlt & one), vgt & one);
    lab = ~__vcmpltu4(d, v) & one;
}

}  // namespace nt2g
