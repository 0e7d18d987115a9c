// nt2g_exprs.cuh -- per-element bodies of the named fused expressions, shared
// by the plain kernels, the batched persistent kernel and the pattern-bound
// program path so that all of them round identically.
#pragma once
#include "nt2g_math.cuh"

namespace nt2g {

// Textbook Black-Scholes call+put, written as the NT2 expression
//   d1 = (log(S/K) + fma(sqr(sig),0.5,r)*T) / (sig*sqrt(T))
//   d2 = fnms(sig, sqrt(T), d1)
//   e  = K*exp(-r*T)
//   call = fnms(e, normcdf(d2), S*normcdf(d1))
//   put  = fnms(S, normcdf(-d1), e*normcdf(-d2))
// Nt2 policy: exactly that operation sequence.  Fast policy: the same graph
// with FMAs, approximate-reciprocal divisions (operands are positive normal
// for any priceable option) and one erfc core shared by N(d) and N(-d).
template <class P>
__device__ __forceinline__ void bs_option(float S, float K, float T, float sig, float r, float &call, float &put)
{
    float sq = P::sqrt(T);
    float lq = log<P>(P::fdiv(S, K));
    float a = P::fma(P::mul(sig, sig), 0.5f, r);
    float d1, d2;
    if (P::exact) {
        d1 = P::div(P::add(lq, P::mul(a, T)), P::mul(sig, sq));
        d2 = P::sub(d1, P::mul(sig, sq));
    } else {
        d1 = P::fdiv(P::fma(a, T, lq), P::mul(sig, sq));
        d2 = P::fma(-sig, sq, d1);
    }
    float e = P::mul(K, exp<P>(P::mul(-r, T)));
    float n1, m1, n2, m2;
    normcdf_pair<P>(d1, n1, m1);
    normcdf_pair<P>(d2, n2, m2);
    if (P::exact) {
        call = P::sub(P::mul(S, n1), P::mul(e, n2));
        put = P::sub(P::mul(e, m2), P::mul(S, m1));
    } else {
        call = P::fma(-e, n2, P::mul(S, n1));
        put = P::fma(-S, m1, P::mul(e, m2));
    }
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
// Fast: y = 0.299r + 0.587g + 0.114b held exactly enough as yh + yl (each
// product split exactly by FMA, the sum by TwoSum), so u = 0.492((b-yh)-yl)
// and v = 0.877((r-yh)-yl) are within about one ulp of their own value even
// when b or r nearly equals y; memory-bound, so the extra flops are free.
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
    u = __fmul_rn(0.492f, __fsub_rn(__fsub_rn(b, yh), yl));
    v = __fmul_rn(0.877f, __fsub_rn(__fsub_rn(r, yh), yl));
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
