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
__device__ __forceinline__ f2 neg2(f2 a) { return mul2(a, dup(-1.0f)); }  // exact
// -a by flipping both sign bits (integer pipe, exact, no FP32 slot)
__device__ __forceinline__ f2 negx2(f2 a)
{
    f2 r;
    r.v = a.v ^ 0x8000000080000000ull;
    return r;
}
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
    f2 ne = mul2(nK, ert);
    f2 n1, m1, n2, m2;
    bs_normcdfs_fast2(d1, d2, S, e, n1, m1, n2, m2);
    call = fma2(ne, n2, mul2(S, n1));
    put = fma2(neg2(S), m1, mul2(e, m2));
    const f2 z = sub2(d1, d1);  // NaN unless d1 is finite
    call = add2(call, z);
    put = add2(put, z);
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

}  // namespace nt2g
