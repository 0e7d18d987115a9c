// nt2g_exprs.cuh -- per-element bodies of the named fused expressions, shared
// by the plain kernels, the batched persistent kernel and the pattern-bound
// program path so that all of them round identically.
#pragma once
#include "nt2g_math.cuh"

namespace nt2g {

// ---------------------------------------------------------------------------
// Helpers of the fast Black-Scholes path.  Its operands are a priceable
// option's: S, K, T, sigma positive, finite and normal.  Other inputs give NaN
// call/put: d1 - d1 (0 for a finite d1, NaN for a NaN or infinite one) is
// added to both outputs in place of the functors' special-value selects; the
// NT2 policy keeps NT2's full IEEE handling.

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

// 1/sqrt(t) to about one ulp: rsqrt.approx refined by one Newton step.
__device__ __forceinline__ float rsqrt_fast(float t)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
    float h = Fast::mul(t, y);
    return Fast::fma(Fast::mul(0.5f, y), Fast::fma(-h, y, 1.0f), y);
}

// 2^x from the special-function unit (ex2.approx.ftz.f32, about 2 ulp).
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// exp(-a^2/2) = (1 + eL) * scale for 0 <= a < 13.26.  The exponent
// t = a^2 log2(e)/2 is carried as th + tl: a^2 split exactly by FMA
// (hi + lo), log2(e)/2 as the float pair LH + LL, and the rounding of
// th = hi*LH recovered by FMA.  t = k + f with k = rint(th) (1.5*2^23
// shifter), f = (th - k) + tl (th - k exact), |f| <= 1/2; 2^-f comes from the
// SFU and scale = 2^-k is built in the exponent field.  Past 13.2 the
// callers zero the tail (k would leave the normal range).
__device__ __forceinline__ float bs_exp_half_sq(float a, float &scale)
{
    const float LH = 0x1.715476p-1f, LL = 0x1.4ae0c0p-27f, shifter = 12582912.0f;
    const float hi = Fast::mul(a, a), lo = Fast::fma(a, a, -hi);
    const float th = Fast::mul(hi, LH);
    float tl = Fast::fma(hi, LH, -th);
    tl = Fast::fma(hi, LL, tl);
    tl = Fast::fma(lo, LH, tl);
    const float kf = Fast::add(th, shifter);
    const float f = Fast::add(Fast::sub(th, Fast::sub(kf, shifter)), tl);
    scale = bits_f((127u - (f_bits(kf) - 0x4B400000u)) << 23);
    return Fast::sub(ex2_approx(-f), 1.0f);
}

// w = 1/(1 + q a) refined once, and its residual r = 1 - den*w against the
// rounded den = 1 + q a, formed from the negated nd = RN(-q a - 1) = -den.
// The multiplier w (1 + r) is exact to first order up to den's own rounding
// (2^-24 relative); the polynomial takes the refined w.
__device__ __forceinline__ void bs_tail_recip(float a, float &w, float &r)
{
    const float q = 0.353553390593273762f;  // 1/(2 sqrt 2)
    const float nd = Fast::fma(-q, a, -1.0f);
    w = Fast::rcp(-nd);
    w = Fast::fma(w, Fast::fma(nd, w, 1.0f), w);
    r = Fast::fma(nd, w, 1.0f);
}

// The four normal CDF values of a Black-Scholes option, N(+-d1) and N(+-d2),
// from the tail form of erfc_tail_fast<true> (2 N(-a) = exp(-a^2/2) w R(w),
// w = 1/(1 + a/(2 sqrt 2)), a = |d|) with ONE exponential.  The model fixes
//   d2^2/2 = d1^2/2 - log(S/K) - rT,  i.e.  exp(-d2^2/2) = exp(-d1^2/2) S / e,
// e = K exp(-rT).  Since d1 - d2 = sigma sqrt T > 0, |d1| <= |d2| exactly
// when S <= e: the exponential is evaluated at the smaller |d| (x) and the
// other one (y) follows by the factor min(S,e)/max(S,e) <= 1, applied to the
// unassembled (1 + eL) 2^k so it cannot overflow.  Besides saving an
// exponential, this keeps S phi(d1) = e phi(d2) consistent in rounding: deep
// in the tails, where call or put is the small difference of two such terms,
// their errors cancel instead of adding (on the standard test mixes, max error
// of call/put relative to the larger term drops from ~90 ulp to ~10).
// g1 (optional) receives exp(-d1^2/2) for the adjoint.
__device__ __forceinline__ void bs_normcdfs_fast(float d1, float d2, float S, float e, float &n1, float &m1,
                                                 float &n2, float &m2, float *g1 = nullptr)
{
    const float amax = 13.2f;  // exp(-a^2/2) leaves the normal range past this
    const float a1 = fabsf(d1), a2 = fabsf(d2);
    const bool c = S <= e;     // |d1| <= |d2|
    const float ax = c ? a1 : a2, ay = c ? a2 : a1;
    float wx, rx, wy, ry;
    bs_tail_recip(ax, wx, rx);
    bs_tail_recip(ay, wy, ry);
    float sc;
    const float el = bs_exp_half_sq(ax, sc);
    // x: (1 + eL)(1 + rx) - 1 = eL + rx + rx eL folded into one term
    const float ex = Fast::add(el, Fast::fma(rx, el, rx));
    const float wrx = Fast::mul(wx, erfc_tail_poly(wx));
    const float tx = (ax < amax) ? Fast::mul(Fast::fma(ex, wrx, wrx), sc) : 0.0f;
    // y: exp(-ay^2/2) = (1 + eL) * ratio * 2^k
    const float ratio = Fast::fdiv(fminf(S, e), fmaxf(S, e));
    const float Ey = Fast::mul(Fast::fma(el, ratio, ratio), sc);
    const float wry = Fast::mul(wy, erfc_tail_poly(wy));
    const float u = Fast::mul(Ey, wry);
    const float ty = (ay < amax) ? Fast::fma(u, ry, u) : 0.0f;
    const float t1 = c ? tx : ty, t2 = c ? ty : tx;
    if (g1) *g1 = (a1 < amax) ? (c ? Fast::mul(Fast::add(el, 1.0f), sc) : Ey) : 0.0f;
    // normcdf(-|d|) = tail/2; the other side 1 - tail/2
    const float h1 = Fast::mul(0.5f, t1), o1 = Fast::sub(1.0f, h1);
    const float h2 = Fast::mul(0.5f, t2), o2 = Fast::sub(1.0f, h2);
    n1 = d1 < 0.0f ? h1 : o1;
    m1 = d1 < 0.0f ? o1 : h1;
    n2 = d2 < 0.0f ? h2 : o2;
    m2 = d2 < 0.0f ? o2 : h2;
}

// -r log2(e), the factor of T in the exponent of e^-rT = 2^(-r log2(e) T).
__device__ __forceinline__ float bs_neg_rate_log2e(float r) { return Fast::mul(-r, 0x1.715476p+0f); }

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
    f.ert = ex2_approx(Fast::mul(bs_neg_rate_log2e(r), T));  // e^-rT = 2^(-r log2(e) T)
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
// S/K, e^-rT and exp(-d^2/2) from the SFU's 2^x, and one erfc core shared by
// N(d) and N(-d).  inv_sig is 1/sig (the
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
    bs_normcdfs_fast(f.d1, f.d2, S, f.e, n1, m1, n2, m2);
    call = Fast::fma(-f.e, n2, Fast::mul(S, n1));
    put = Fast::fma(-S, m1, Fast::mul(f.e, m2));
    const bool bad = !(fabsf(f.d1) < f_inf());  // NaN unless d1 is finite (d2 follows d1)
    call = bad ? f_nan() : call;
    put = bad ? f_nan() : put;
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
