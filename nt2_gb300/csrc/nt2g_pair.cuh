// nt2g_pair.cuh -- two FP32 lanes per instruction (sm_100-family packed
// add/sub/mul/fma.rn.f32x2) for the issue-bound fast Black-Scholes path.
//
// Each function here performs, lane by lane, exactly the IEEE operations of
// its scalar counterpart in nt2g_exprs.cuh / nt2g_math.cuh (same operands,
// same order, round-to-nearest, no flush), so a pair of options priced here is
// bit-identical to the same two options priced one at a time.  Where the
// scalar code negates an operand inside an FMA (free in the scalar
// instruction), the pair form either folds the sign into a constant or uses an
// exactly negated value (x * -1); RN is symmetric, so RN(-p + c) is computed
// without changing a bit.  Integer/bit manipulation, compares, selects and the
// MUFU approximations stay per lane.
#pragma once
#include "nt2g_exprs.cuh"

namespace nt2g {

struct f2 {
    unsigned long long v;
};

__device__ __forceinline__ f2 pk(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk(f2 a, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ f2 dup(float x) { return pk(x, x); }
__device__ __forceinline__ f2 add2(f2 a, f2 b)
{
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b)
{
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b)
{
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c)
{
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}
// -a by flipping both sign bits (integer pipe, exact, no FP32 slot)
__device__ __forceinline__ f2 negx2(f2 a)
{
    f2 r;
    r.v = a.v ^ 0x8000000080000000ull;
    return r;
}
__device__ __forceinline__ f2 neg2(f2 a) { return negx2(a); }
template <class F> __device__ __forceinline__ f2 lanes(f2 a, F f)
{
    float x, y;
    upk(a, x, y);
    return pk(f(x), f(y));
}
template <class F> __device__ __forceinline__ f2 lanes(f2 a, f2 b, F f)
{
    float x0, x1, y0, y1;
    upk(a, x0, x1);
    upk(b, y0, y1);
    return pk(f(x0, y0), f(x1, y1));
}

// Horner in NT2's coefficient order, as horner<Fast>.
__device__ __forceinline__ f2 horner2(f2, f2 acc) { return acc; }
template <class... R> __device__ __forceinline__ f2 horner2(f2 x, f2 acc, float c, R... rest)
{
    return horner2(x, fma2(x, acc, dup(c)), rest...);
}

__device__ __forceinline__ float rcp_approx(float b)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float t)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
    return y;
}

// rsqrt_fast: fma(0.5*y, fma(-h, y, 1), y), h = t*y.  With E = fma(h, y, -1)
// = -fma(-h, y, 1) and (-0.5*y)*E = (0.5*y)*fma(-h, y, 1) exactly.
__device__ __forceinline__ f2 rsqrt_fast2(f2 t)
{
    f2 y = lanes(t, rsqrt_approx);
    f2 h = mul2(t, y);
    return fma2(mul2(dup(-0.5f), y), fma2(h, y, dup(-1.0f)), y);
}

// Fast::fdiv(a, b) given nb = -b.
__device__ __forceinline__ f2 fdiv2(f2 a, f2 b, f2 nb)
{
    f2 r = lanes(b, rcp_approx);
    f2 q = mul2(a, r);
    f2 e = fma2(q, nb, a);
    return fma2(e, r, q);
}

// log_pos_fast, lane for lane.
__device__ __forceinline__ f2 log_pos_fast2(f2 z)
{
    float z0, z1;
    upk(z, z0, z1);
    const uint32_t u0 = f_bits(z0), u1 = f_bits(z1);
    const float m0 = bits_f((u0 & 0x007fffffu) | 0x3f000000u), m1 = bits_f((u1 & 0x007fffffu) | 0x3f000000u);
    const bool l0 = m0 < bits_f(NT2G_SQRT_2O_2), l1 = m1 < bits_f(NT2G_SQRT_2O_2);
    f2 fe = sub2(pk(bits_f(0x4B000000u | (uint32_t)((int32_t)u0 >> 23)),
                    bits_f(0x4B000000u | (uint32_t)((int32_t)u1 >> 23))),
                 pk(l0 ? 8388735.0f : 8388734.0f, l1 ? 8388735.0f : 8388734.0f));
    f2 m = pk(m0, m1);
    f2 mm = add2(m, m);
    float mm0, mm1;
    upk(mm, mm0, mm1);
    f2 x = sub2(pk(l0 ? mm0 : m0, l1 ? mm1 : m1), dup(1.0f));
    f2 x2 = mul2(x, x);
    f2 y = horner2(x, dup(bits_f(0xbda5dff0u)), bits_f(0x3e0229f9u), bits_f(0xbe04d6b7u), bits_f(0x3e116e80u),
                   bits_f(0xbe2a6aa0u), bits_f(0x3e4cd0a3u), bits_f(0xbe800064u), bits_f(0x3eaaaaa9u));
    y = mul2(mul2(y, x), x2);
    y = fma2(fe, dup(bits_f(NT2G_LOG_2LO)), y);
    y = fma2(dup(-0.5f), x2, y);
    return fma2(dup(bits_f(NT2G_LOG_2HI)), fe, add2(x, y));
}

__device__ __forceinline__ f2 erfc_tail_poly2(f2 w)
{
    f2 d = sub2(w, dup(0.5f));
    return horner2(d, dup(0x1.5af3d4p-5f), -0x1.38d8fcp-6f, -0x1.382c16p-4f, 0x1.c51560p-5f, 0x1.908f48p-4f,
                   -0x1.a94032p-4f, -0x1.604ccep-3f, 0x1.2a8c2ep-3f, 0x1.1e2dc2p-1f, 0x1.5fd384p-1f, 0x1.058672p-1f);
}

// bs_exp_half_sq, lane for lane (-x as a sign flip, exact).
__device__ __forceinline__ f2 bs_exp_half_sq2(f2 a, f2 &scale)
{
    const float LH = 0x1.715476p-1f, LL = 0x1.4ae0c0p-27f, shifter = 12582912.0f;
    const f2 hi = mul2(a, a), lo = fma2(a, a, negx2(hi));
    const f2 th = mul2(hi, dup(LH));
    f2 tl = fma2(hi, dup(LH), negx2(th));
    tl = fma2(hi, dup(LL), tl);
    tl = fma2(lo, dup(LH), tl);
    const f2 kf = add2(th, dup(shifter));
    const f2 f = add2(sub2(th, sub2(kf, dup(shifter))), tl);
    float f0, f1, k0, k1;
    upk(f, f0, f1);
    upk(kf, k0, k1);
    scale = pk(bits_f((127u - (f_bits(k0) - 0x4B400000u)) << 23), bits_f((127u - (f_bits(k1) - 0x4B400000u)) << 23));
    return sub2(pk(ex2_approx(-f0), ex2_approx(-f1)), dup(1.0f));
}

// bs_tail_recip, lane for lane.
__device__ __forceinline__ void bs_tail_recip2(f2 a, f2 &w, f2 &r)
{
    const float q = 0.353553390593273762f;
    const f2 nd = fma2(dup(-q), a, dup(-1.0f));
    w = lanes(nd, [](float v) { return rcp_approx(-v); });
    w = fma2(w, fma2(nd, w, dup(1.0f)), w);
    r = fma2(nd, w, dup(1.0f));
}

// bs_normcdfs_fast for two options (lane for lane; without g1).
__device__ __forceinline__ void bs_normcdfs_fast2(f2 d1, f2 d2, f2 S, f2 e, f2 &n1, f2 &m1, f2 &n2, f2 &m2)
{
    const float amax = 13.2f;
    float d10, d11, d20, d21, S0, S1, e0, e1;
    upk(d1, d10, d11);
    upk(d2, d20, d21);
    upk(S, S0, S1);
    upk(e, e0, e1);
    const float a10 = fabsf(d10), a11 = fabsf(d11), a20 = fabsf(d20), a21 = fabsf(d21);
    const bool c0 = S0 <= e0, c1 = S1 <= e1;
    const f2 ax = pk(c0 ? a10 : a20, c1 ? a11 : a21), ay = pk(c0 ? a20 : a10, c1 ? a21 : a11);
    f2 wx, rx, wy, ry;
    bs_tail_recip2(ax, wx, rx);
    bs_tail_recip2(ay, wy, ry);
    f2 sc;
    const f2 el = bs_exp_half_sq2(ax, sc);
    const f2 ex = add2(el, fma2(rx, el, rx));
    const f2 wrx = mul2(wx, erfc_tail_poly2(wx));
    const f2 txv = mul2(fma2(ex, wrx, wrx), sc);
    const f2 ratio = fdiv2(pk(fminf(S0, e0), fminf(S1, e1)), pk(fmaxf(S0, e0), fmaxf(S1, e1)),
                           pk(-fmaxf(S0, e0), -fmaxf(S1, e1)));
    const f2 Ey = mul2(fma2(el, ratio, ratio), sc);
    const f2 wry = mul2(wy, erfc_tail_poly2(wy));
    const f2 u = mul2(Ey, wry);
    const f2 tyv = fma2(u, ry, u);
    float ax0, ax1, ay0, ay1, tx0, tx1, ty0, ty1;
    upk(ax, ax0, ax1);
    upk(ay, ay0, ay1);
    upk(txv, tx0, tx1);
    upk(tyv, ty0, ty1);
    tx0 = (ax0 < amax) ? tx0 : 0.0f;
    tx1 = (ax1 < amax) ? tx1 : 0.0f;
    ty0 = (ay0 < amax) ? ty0 : 0.0f;
    ty1 = (ay1 < amax) ? ty1 : 0.0f;
    const f2 t1 = pk(c0 ? tx0 : ty0, c1 ? tx1 : ty1), t2 = pk(c0 ? ty0 : tx0, c1 ? ty1 : tx1);
    const f2 h1 = mul2(dup(0.5f), t1), o1 = sub2(dup(1.0f), h1);
    const f2 h2 = mul2(dup(0.5f), t2), o2 = sub2(dup(1.0f), h2);
    float hh0, hh1, oo0, oo1, hk0, hk1, ok0, ok1;
    upk(h1, hh0, hh1);
    upk(o1, oo0, oo1);
    upk(h2, hk0, hk1);
    upk(o2, ok0, ok1);
    n1 = pk(d10 < 0.0f ? hh0 : oo0, d11 < 0.0f ? hh1 : oo1);
    m1 = pk(d10 < 0.0f ? oo0 : hh0, d11 < 0.0f ? oo1 : hh1);
    n2 = pk(d20 < 0.0f ? hk0 : ok0, d21 < 0.0f ? hk1 : ok1);
    m2 = pk(d20 < 0.0f ? ok0 : hk0, d21 < 0.0f ? ok1 : hk1);
}

// inv_fast(x) given nx = -x.
__device__ __forceinline__ f2 inv_fast2(f2 x, f2 nx)
{
    f2 r = lanes(x, rcp_approx);
    return fma2(r, fma2(nx, r, dup(1.0f)), r);
}

// bs_option<Fast> for two options (sig, inv_sig, r shared or per lane).
__device__ __forceinline__ void bs_option_fast2(f2 S, f2 K, f2 T, f2 sig, f2 inv_sig, float r, f2 &call, f2 &put)
{
    f2 nK = neg2(K);
    f2 rs = rsqrt_fast2(T);
    f2 sq = mul2(T, rs);
    f2 lq = log_pos_fast2(fdiv2(S, K, nK));
    f2 a = fma2(mul2(sig, sig), dup(0.5f), dup(r));
    f2 d1 = mul2(fma2(a, T, lq), mul2(rs, inv_sig));
    f2 d2 = fma2(neg2(sig), sq, d1);
    f2 ert = lanes(mul2(dup(bs_neg_rate_log2e(r)), T), ex2_approx);
    f2 e = mul2(K, ert);
    f2 n1, m1, n2, m2;
    bs_normcdfs_fast2(d1, d2, S, e, n1, m1, n2, m2);
    call = fma2(negx2(e), n2, mul2(S, n1));  // -(K e^-rT) exactly, on the integer pipe
    put = fma2(negx2(S), m1, mul2(e, m2));
    // NaN unless d1 is finite (d2 follows d1): a test and a select per lane
    // on the integer pipe rather than FP32 work
    float d10, d11, c0, c1, p0, p1;
    upk(d1, d10, d11);
    upk(call, c0, c1);
    upk(put, p0, p1);
    const bool bad0 = !(fabsf(d10) < f_inf()), bad1 = !(fabsf(d11) < f_inf());
    call = pk(bad0 ? f_nan() : c0, bad1 ? f_nan() : c1);
    put = pk(bad0 ? f_nan() : p0, bad1 ? f_nan() : p1);
}

// Four options (one float4 of each table) as two pairs, sigma and 1/sigma
// given per option (v, iv).  Bit-identical to bs_option<Fast> per option.
__device__ __forceinline__ void bs_vec4_fast(const float4 &s, const float4 &k, const float4 &t, const float4 &v,
                                             const float4 &iv, float r, float4 &c, float4 &p)
{
    f2 c2, p2;
    bs_option_fast2(pk(s.x, s.y), pk(k.x, k.y), pk(t.x, t.y), pk(v.x, v.y), pk(iv.x, iv.y), r, c2, p2);
    upk(c2, c.x, c.y);
    upk(p2, p.x, p.y);
    bs_option_fast2(pk(s.z, s.w), pk(k.z, k.w), pk(t.z, t.w), pk(v.z, v.w), pk(iv.z, iv.w), r, c2, p2);
    upk(c2, c.z, c.w);
    upk(p2, p.z, p.w);
}

// fastnormcdf (STAT/generic/fastnormcdf.hpp:33-55) for two lanes under the
// fast policy: k = 1/(1 + 0.2316419 l), l = |x| (the SFU reciprocal and one
// Newton step), w = k H(k) phi(l) with H NT2's degree-4 polynomial and
// phi(l) = e^(-l^2/2)/sqrt(2 pi) from the exactly split exponent and the
// SFU's 2^x (bs_exp_half_sq2); 1 - w above 0.  From |x| = 13 on, phi is below
// 1e-37: the result is 1 or 0 there (the scalar form's w is a subnormal).
__device__ __forceinline__ f2 fastnormcdf_fast2(f2 x)
{
    float x0, x1;
    upk(x, x0, x1);
    const f2 l = pk(fminf(fabsf(x0), 13.0f), fminf(fabsf(x1), 13.0f));
    const f2 k = inv_fast2(fma2(dup(0.2316419f), l, dup(1.0f)), fma2(dup(-0.2316419f), l, dup(-1.0f)));
    const f2 h = horner2(k, dup(bits_f(0x3faa466fu)), bits_f(0xbfe91eeau), bits_f(0x3fe40778u), bits_f(0xbeb68f87u),
                         bits_f(0x3ea385fau));
    f2 sc;
    const f2 el = bs_exp_half_sq2(l, sc);
    const f2 w = mul2(mul2(h, k), mul2(fma2(el, sc, sc), dup(bits_f(NT2G_INVSQRT_2PI))));
    float w0, w1;
    upk(w, w0, w1);
    float r0 = x0 > 0.0f ? 1.0f - w0 : w0, r1 = x1 > 0.0f ? 1.0f - w1 : w1;
    r0 = fabsf(x0) >= 13.0f ? (x0 > 0.0f ? 1.0f : 0.0f) : r0;
    r1 = fabsf(x1) >= 13.0f ? (x1 > 0.0f ? 1.0f : 0.0f) : r1;
    return pk(is_nan(x0) ? x0 : r0, is_nan(x1) ? x1 : r1);
}

// NT2's demo Black-Scholes (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59)
// for two options under the fast policy: call only, fastnormcdf,
// d1 = log(S/X) + fma(v^2, 1/2, r) T / (v sqrt(T)), d2 = d1 - v sqrt(T),
// R = S N(d1) - X e^(-rT) N(d2); sqrt(T) as T rsqrt(T), e^(-rT) from the
// SFU's 2^x, the log on the split mantissa (log_pos_fast2).
__device__ __forceinline__ f2 bs_demo_fast2(f2 S, f2 X, f2 T, f2 r, f2 v)
{
    const f2 da = mul2(T, rsqrt_fast2(T));
    const f2 lq = log_pos_fast2(fdiv2(S, X, neg2(X)));
    const f2 num = mul2(fma2(mul2(v, v), dup(0.5f), r), T);
    const f2 vda = mul2(v, da);
    const f2 d1 = add2(lq, fdiv2(num, vda, neg2(vda)));
    const f2 d2 = fma2(neg2(v), da, d1);
    const f2 ert = lanes(mul2(mul2(r, dup(-0x1.715476p+0f)), T), ex2_approx);
    const f2 a = mul2(S, fastnormcdf_fast2(d1));
    return fma2(neg2(mul2(X, ert)), fastnormcdf_fast2(d2), a);
}

// ------------------------------------------------------------ NT2 policy --
// The bit-exact policy two options at a time.  NT2's arithmetic is unfused
// (its fma is a rounded product and a rounded sum), and add/sub.rn.f32x2
// round each lane exactly as the scalar __fadd_rn / __fsub_rn do.  A packed
// product is different: the code generator merges a mul.rn.f32x2 into the
// add.rn.f32x2 that consumes it (one rounding instead of NT2's two), even
// with the explicit rounding mode and with contraction disabled.  So every
// product here is fma.rn.f32x2(a, b, z) with z = -0 in both lanes, loaded from
// memory where the code generator cannot see its value: RN(a*b + -0) is
// RN(a*b) bit for bit (a zero product keeps its own sign), and an FMA whose
// addend is unknown has nothing to merge with.  IEEE division and square
// root, rint, the conversions and all bit manipulation stay per lane.  These
// functions reproduce Nt2's scalar results bit for bit.

static __device__ unsigned long long g_pair_negzero = 0x8000000080000000ull;

// -0 in both lanes, through a load the code generator cannot fold
__device__ __forceinline__ f2 pair_negzero()
{
    f2 z;
    asm volatile("ld.b64 %0, [%1];" : "=l"(z.v) : "l"(&g_pair_negzero));
    return z;
}
// RN(a*b) in each lane, never merged with a following add
__device__ __forceinline__ f2 nmul2(f2 a, f2 b, f2 nz) { return fma2(a, b, nz); }
__device__ __forceinline__ f2 nt2_fma2(f2 a, f2 b, f2 c, f2 nz) { return add2(nmul2(a, b, nz), c); }
__device__ __forceinline__ f2 nt2_horner2(f2, f2, f2 acc) { return acc; }
template <class... R> __device__ __forceinline__ f2 nt2_horner2(f2 nz, f2 x, f2 acc, uint32_t c, R... rest)
{
    return nt2_horner2(nz, x, add2(nmul2(x, acc, nz), dup(bits_f(c))), rest...);
}

__device__ __forceinline__ f2 div_rn2(f2 a, f2 b)
{
    return lanes(a, b, [](float x, float y) { return __fdiv_rn(x, y); });
}
__device__ __forceinline__ f2 sqrt_rn2(f2 a) { return lanes(a, [](float x) { return __fsqrt_rn(x); }); }
__device__ __forceinline__ f2 abs2(f2 a)
{
    f2 r;
    r.v = a.v & 0x7fffffff7fffffffull;
    return r;
}
// per-lane select: c0 ? a.lo : b.lo, c1 ? a.hi : b.hi
__device__ __forceinline__ f2 sel2(bool c0, bool c1, f2 a, f2 b)
{
    float a0, a1, b0, b1;
    upk(a, a0, a1);
    upk(b, b0, b1);
    return pk(c0 ? a0 : b0, c1 ? a1 : b1);
}

// exp<Nt2>, lane for lane.
__device__ __forceinline__ f2 exp_nt2_2(f2 a0, f2 nz)
{
    const f2 kf = lanes(nmul2(dup(bits_f(NT2G_INVLOG_2)), a0, nz), [](float v) { return rintf(v); });
    f2 x = sub2(a0, nmul2(kf, dup(bits_f(NT2G_LOG_2HI)), nz));
    x = sub2(x, nmul2(kf, dup(bits_f(NT2G_LOG_2LO)), nz));
    const f2 y = nt2_horner2(nz, x, dup(bits_f(0x3ab778cfu)), 0x3c098d8bu, 0x3d2aa957u, 0x3e2aa9a5u, 0x3f000000u);
    const f2 c = add2(nt2_fma2(y, nmul2(x, x, nz), x, nz), dup(1.0f));
    float k0, k1, a, b;
    upk(kf, k0, k1);
    upk(a0, a, b);
    const f2 r = nmul2(c, pk(bits_f((uint32_t)((int32_t)k0 + 127) << 23), bits_f((uint32_t)((int32_t)k1 + 127) << 23)),
                       nz);
    // the special values (+inf from Maxlog, 0 from Minlog, NaN) only when a
    // lane leaves (Minlog, Maxlog): one range test per lane on the common path
    const bool in0 = a > bits_f(NT2G_MINLOG) && a < bits_f(NT2G_MAXLOG);
    const bool in1 = b > bits_f(NT2G_MINLOG) && b < bits_f(NT2G_MAXLOG);
    if (in0 && in1) return r;
    float r0, r1;
    upk(r, r0, r1);
    auto fix = [](float a0s, float v) {
        return (a0s >= bits_f(NT2G_MAXLOG)) ? f_inf() : (a0s <= bits_f(NT2G_MINLOG)) ? 0.0f : is_nan(a0s) ? a0s : v;
    };
    return pk(fix(a, r0), fix(b, r1));
}

// log<Nt2>, lane for lane (log_reduce with NT2's log constants).
__device__ __forceinline__ f2 log_nt2_2(f2 a0, f2 nz)
{
    float z0, z1;
    upk(a0, z0, z1);
    const bool den0 = fabsf(z0) < bits_f(NT2G_SMALLESTPOS), den1 = fabsf(z1) < bits_f(NT2G_SMALLESTPOS);
    const f2 zs = nmul2(a0, dup(bits_f(NT2G_TWOTONMB)), nz);
    float s0, s1;
    upk(zs, s0, s1);
    const float w0 = den0 ? s0 : z0, w1 = den1 ? s1 : z1;
    const f2 t = pk(den0 ? bits_f(NT2G_MLOGTWO2NMB) : 0.0f, den1 ? bits_f(NT2G_MLOGTWO2NMB) : 0.0f);
    const uint32_t u0 = f_bits(w0), u1 = f_bits(w1);
    const int32_t e0 = (int32_t)((u0 & 0x7f800000u) >> 23) - 126, e1 = (int32_t)((u1 & 0x7f800000u) >> 23) - 126;
    const float x0 = bits_f((u0 & ~0x7f800000u) | 0x3f000000u), x1 = bits_f((u1 & ~0x7f800000u) | 0x3f000000u);
    const bool lt0 = x0 < bits_f(NT2G_SQRT_2O_2), lt1 = x1 < bits_f(NT2G_SQRT_2O_2);
    const f2 ef = pk((float)e0, (float)e1);
    const f2 fe = sel2(lt0, lt1, add2(ef, dup(-1.0f)), ef);
    const f2 xm = pk(x0, x1);
    const f2 x = sub2(sel2(lt0, lt1, add2(xm, xm), xm), dup(1.0f));
    const f2 x2 = nmul2(x, x, nz);
    f2 y = nt2_horner2(nz, x, dup(bits_f(0xbda5dff0u)), 0x3e0229f9u, 0xbe04d6b7u, 0x3e116e80u, 0xbe2a6aa0u, 0x3e4cd0a3u,
                       0xbe800064u, 0x3eaaaaa9u);
    y = nmul2(nmul2(y, x, nz), x2, nz);
    y = nt2_fma2(fe, dup(bits_f(NT2G_LOG_2LO)), y, nz);
    y = nt2_fma2(dup(-0.5f), x2, y, nz);
    const f2 r = nt2_fma2(dup(bits_f(NT2G_LOG_2HI)), fe, add2(add2(x, y), t), nz);
    // +inf, 0, negative and NaN arguments only when a lane is outside (0, +inf)
    if (z0 > 0.0f && z0 < f_inf() && z1 > 0.0f && z1 < f_inf()) return r;
    float r0, r1;
    upk(r, r0, r1);
    auto fix = [](float a, float v) {
        return (a == f_inf()) ? a : (a == 0.0f) ? -f_inf() : (is_nan(a) || a < 0.0f) ? f_nan() : v;
    };
    return pk(fix(z0, r0), fix(z1, r1));
}

// erfc_core_nt2 for x >= 0, lane for lane.  The scalar code branches on
// x < 2/3; a warp holding both kinds issues both paths anyway, so here both
// polynomials are evaluated (two lanes per instruction) and each lane keeps
// its own.
__device__ __forceinline__ f2 erfc_core_nt2_2(f2 x, f2 nz)
{
    const f2 z = div_rn2(x, add2(x, dup(1.0f)));
    const f2 b1 = nmul2(sub2(dup(1.0f), z),
                       nt2_horner2(nz, z, dup(bits_f(0x41aa8e55u)), 0x401b5680u, 0xc010d956u, 0x3f2cff3bu, 0xc016c985u,
                                   0xbffc9284u, 0xbfa11698u, 0xbe036d7eu, 0x3f7ffffeu), nz);
    const f2 zz = sub2(z, dup(0.4f));
    const f2 b2 = nmul2(exp_nt2_2(negx2(nmul2(x, x, nz)), nz),
                       nt2_horner2(nz, zz, dup(bits_f(0xc0283611u)), 0x40d67e3bu, 0xc0cd1a85u, 0x4050b063u, 0xbfaea865u,
                                   0x3e2006f0u, 0x3e1175c7u, 0x3ec4ca6eu, 0x3e243828u, 0xbf918a62u, 0x3f0a0e8bu), nz);
    float x0, x1, p0, p1, q0, q1;
    upk(x, x0, x1);
    upk(b1, p0, p1);
    upk(b2, q0, q1);
    const float two3 = bits_f(NT2G_TWOTHIRD);
    return pk(x0 < two3 ? p0 : (x0 == f_inf() ? 0.0f : q0), x1 < two3 ? p1 : (x1 == f_inf() ? 0.0f : q1));
}

// normcdf_pair<Nt2>, lane for lane.
__device__ __forceinline__ void normcdf_pair_nt2_2(f2 x, f2 &n_pos, f2 &n_neg, f2 nz)
{
    const f2 t = nmul2(dup(-bits_f(NT2G_SQRT_2O_2)), x, nz);
    const f2 r1 = erfc_core_nt2_2(abs2(t), nz);
    const f2 r2 = sub2(dup(2.0f), r1);
    float t0, t1;
    upk(t, t0, t1);
    n_pos = nmul2(dup(0.5f), sel2(t0 < 0.0f, t1 < 0.0f, r2, r1), nz);
    n_neg = nmul2(dup(0.5f), sel2(-t0 < 0.0f, -t1 < 0.0f, r2, r1), nz);
}

// bs_option<Nt2> for two options; a = fma(sig^2, 1/2, r) given per lane.
__device__ __forceinline__ void bs_option_nt2_2(f2 S, f2 K, f2 T, f2 sig, f2 a, float r, f2 &call, f2 &put,
                                                f2 nz)
{
    const f2 sq = sqrt_rn2(T);
    const f2 lq = log_nt2_2(div_rn2(S, K), nz);
    const f2 ssq = nmul2(sig, sq, nz);
    const f2 d1 = div_rn2(add2(lq, nmul2(a, T, nz)), ssq);
    const f2 d2 = sub2(d1, ssq);
    const f2 e = nmul2(K, exp_nt2_2(nmul2(dup(-r), T, nz), nz), nz);
    f2 n1, m1, n2, m2;
    normcdf_pair_nt2_2(d1, n1, m1, nz);
    normcdf_pair_nt2_2(d2, n2, m2, nz);
    call = sub2(nmul2(S, n1, nz), nmul2(e, n2, nz));
    put = sub2(nmul2(e, m2, nz), nmul2(S, m1, nz));
}

// fastnormcdf<Nt2>, lane for lane: k = 1/(0.2316419 l + 1), NT2's unfused
// Horner, w *= (k / sqrt(2 pi)) exp(-(l*l) * 1/2), 1 - w above 0.
__device__ __forceinline__ f2 fastnormcdf_nt2_2(f2 x, f2 nz)
{
    const f2 l = abs2(x);
    const f2 k = div_rn2(dup(1.0f), add2(nmul2(dup(0.2316419f), l, nz), dup(1.0f)));
    f2 w = nt2_horner2(nz, k, dup(bits_f(0x3faa466fu)), 0xbfe91eeau, 0x3fe40778u, 0xbeb68f87u, 0x3ea385fau);
    const f2 e = exp_nt2_2(nmul2(negx2(nmul2(l, l, nz)), dup(0.5f), nz), nz);
    w = nmul2(w, nmul2(nmul2(k, dup(bits_f(NT2G_INVSQRT_2PI)), nz), e, nz), nz);
    const f2 o = sub2(dup(1.0f), w);
    float x0, x1;
    upk(x, x0, x1);
    return sel2(x0 > 0.0f, x1 > 0.0f, o, w);
}

// bs_demo_option<Nt2> for two options, lane for lane.
__device__ __forceinline__ f2 bs_demo_nt2_2(f2 S, f2 X, f2 T, f2 r, f2 v, f2 nz)
{
    const f2 da = sqrt_rn2(T);
    const f2 a = add2(nmul2(nmul2(v, v, nz), dup(0.5f), nz), r);  // fma(sqr(v), 0.5, r), unfused
    const f2 vda = nmul2(v, da, nz);
    const f2 d1 = add2(log_nt2_2(div_rn2(S, X), nz), div_rn2(nmul2(a, T, nz), vda));
    const f2 d2 = sub2(d1, vda);
    const f2 p = nmul2(S, fastnormcdf_nt2_2(d1, nz), nz);
    const f2 b = nmul2(X, exp_nt2_2(nmul2(negx2(r), T, nz), nz), nz);
    return sub2(p, nmul2(b, fastnormcdf_nt2_2(d2, nz), nz));
}

// Four options as two pairs under the NT2 policy; sigma per option.
__device__ __forceinline__ void bs_vec4_nt2(const float4 &s, const float4 &k, const float4 &t, const float4 &v, float r,
                                            float4 &c, float4 &p)
{
    const f2 nz = pair_negzero();
    const f2 v01 = pk(v.x, v.y), v23 = pk(v.z, v.w);
    // fma(sig*sig, 0.5, r) unfused
    const f2 a01 = add2(nmul2(nmul2(v01, v01, nz), dup(0.5f), nz), dup(r)), a23 = add2(nmul2(nmul2(v23, v23, nz), dup(0.5f), nz), dup(r));
    f2 c2, p2;
    bs_option_nt2_2(pk(s.x, s.y), pk(k.x, k.y), pk(t.x, t.y), v01, a01, r, c2, p2, nz);
    upk(c2, c.x, c.y);
    upk(p2, p.x, p.y);
    bs_option_nt2_2(pk(s.z, s.w), pk(k.z, k.w), pk(t.z, t.w), v23, a23, r, c2, p2, nz);
    upk(c2, c.z, c.w);
    upk(p2, p.z, p.w);
}

}  // namespace nt2g
