// nt2g_bs.cu -- fused Black-Scholes kernels: call+put forward (both
// arithmetic policies), the NT2 demo's call-only form, and the fused
// forward + reverse-mode (vector-Jacobian) kernel.
//
// One pass over the option tables: 128-bit loads/stores of 4 options per
// thread, every intermediate in registers.  The fast policy prices the 4
// options as two pairs with packed f32x2 arithmetic (nt2g_pair.cuh), with
// e^-rT and exp(-d^2/2) from the SFU's 2^x: ~95 instructions per option for
// 20 bytes of HBM traffic, so the kernel sits at the FP32-pipe / HBM ridge.
// 5 blocks of 256 threads per SM (48 registers).
#include "nt2g_async.cuh"
#include "nt2g_common.cuh"
#include "nt2g_exprs.cuh"
#include "nt2g_pair.cuh"
#include "nt2g_internal.h"

namespace nt2g {

// Four options already in registers (sigma per option when SIG_TAB).
template <class P, bool SIG_TAB>
__device__ __forceinline__ void bs_compute4(const float4 &s, const float4 &k, const float4 &t, const float4 &v,
                                            float inv_sig_s, float r, float4 &c, float4 &p)
{
    if constexpr (!P::exact) {
        // two options per packed instruction, bit-identical to bs_option<Fast>
        float4 iv = make_float4(inv_sig_s, inv_sig_s, inv_sig_s, inv_sig_s);
        if (SIG_TAB) {
            f2 a = inv_fast2(pk(v.x, v.y), neg2(pk(v.x, v.y))), b = inv_fast2(pk(v.z, v.w), neg2(pk(v.z, v.w)));
            upk(a, iv.x, iv.y);
            upk(b, iv.z, iv.w);
        }
        bs_vec4_fast(s, k, t, v, iv, r, c, p);
    } else {
        // NT2's unfused arithmetic two options per packed instruction,
        // bit-identical to bs_option<Nt2>
        bs_vec4_nt2(s, k, t, v, r, c, p);
    }
}

template <class P, bool SIG_TAB>
__device__ __forceinline__ void bs_float4(const float *__restrict__ S, const float *__restrict__ K,
                                          const float *__restrict__ T, const float *__restrict__ sig, float sig_s,
                                          float inv_sig_s, float r, float *__restrict__ call,
                                          float *__restrict__ put, int64_t i)
{
    float4 s = ld_stream((const float4 *)S + i), k = ld_stream((const float4 *)K + i),
           t = ld_stream((const float4 *)T + i);
    float4 v = SIG_TAB ? ld_stream((const float4 *)sig + i) : make_float4(sig_s, sig_s, sig_s, sig_s);
    float4 c, p;
    bs_compute4<P, SIG_TAB>(s, k, t, v, inv_sig_s, r, c, p);
    st_stream((float4 *)call + i, c);
    st_stream((float4 *)put + i, p);
}

// Waits of this file's kernels that gave up (nt2g_wait_timeouts).
__device__ unsigned long long g_bs_wait_timeouts = 0;

// Pipelined form for aligned tables: a persistent grid walks tiles of 1024
// options (one float4 per thread of a 256-thread block).  Thread 0 keeps the
// block's next STAGES - 1 tiles of S, K, T (and sigma) in flight as bulk
// copies into shared memory, each stage completing on its mbarrier, so the
// loads of later tiles overlap the pricing of the current one and no warp
// waits on HBM latency once the pipeline is primed.  Results go straight to
// global memory (streaming float4 stores).  One block barrier per tile: after
// it every thread has read the previous stage, which thread 0 then refills.
// The options past the last whole tile (fewer than 1024) are priced by block
// 0 with plain loads.
template <class P, bool SIG_TAB, int STAGES>
__global__ void __launch_bounds__(256, SIG_TAB ? 4 : 5) k_bs_pipe(const float *__restrict__ S, const float *__restrict__ K,
                                                 const float *__restrict__ T, const float *__restrict__ sig,
                                                 float sig_s, float r, float *__restrict__ call,
                                                 float *__restrict__ put, int64_t n)
{
    constexpr int NT = SIG_TAB ? 4 : 3;  // tables per tile
    constexpr int TILE = 1024;           // options per tile
    constexpr uint32_t TILE_BYTES = TILE * 4;
    extern __shared__ __align__(128) float4 stage_buf[];  // [STAGES][NT][256]
    uint64_t *full = reinterpret_cast<uint64_t *>(stage_buf + STAGES * NT * 256);
    const int tid = threadIdx.x;
    const int64_t ntiles = n / TILE, G = gridDim.x;
    const float inv_sig_s = P::exact || SIG_TAB ? 0.0f : inv_fast(sig_s);
    auto issue = [&](int s, int64_t t) {
        mbar_arrive_expect_tx(&full[s], NT * TILE_BYTES);
        bulk_copy_g2s(stage_buf + (s * NT + 0) * 256, S + t * TILE, TILE_BYTES, &full[s]);
        bulk_copy_g2s(stage_buf + (s * NT + 1) * 256, K + t * TILE, TILE_BYTES, &full[s]);
        bulk_copy_g2s(stage_buf + (s * NT + 2) * 256, T + t * TILE, TILE_BYTES, &full[s]);
        if (SIG_TAB) bulk_copy_g2s(stage_buf + (s * NT + 3) * 256, sig + t * TILE, TILE_BYTES, &full[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
        mbar_init_fence();
        for (int s = 0; s < STAGES; ++s)
            if (blockIdx.x + s * G < ntiles) issue(s, blockIdx.x + s * G);
    }
    __syncthreads();
    int64_t it = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += G, ++it) {
        const int s = (int)(it % STAGES);
        const bool ok = mbar_wait_bounded(&full[s], (uint32_t)((it / STAGES) & 1));
        if (__syncthreads_or(!ok)) {
            // gave up: count it, let this block's copies still in flight land
            // (tiles it .. it + STAGES - 2 were issued), then leave
            if (tid == 0) {
                atomicAdd(&g_bs_wait_timeouts, 1ull);
                for (int64_t k = it; k < it + STAGES - 1 && blockIdx.x + k * G < ntiles; ++k)
                    mbar_wait_bounded(&full[k % STAGES], (uint32_t)((k / STAGES) & 1));
            }
            return;
        }
        // every thread has read the previous stage: refill it with the tile
        // STAGES - 1 ahead of this one
        if (tid == 0 && it > 0 && t + (STAGES - 1) * G < ntiles) {
            fence_proxy_async_smem();
            issue((int)((it - 1) % STAGES), t + (STAGES - 1) * G);
        }
        const float4 sv = stage_buf[(s * NT + 0) * 256 + tid], kv = stage_buf[(s * NT + 1) * 256 + tid],
                     tv = stage_buf[(s * NT + 2) * 256 + tid];
        const float4 vv = SIG_TAB ? stage_buf[(s * NT + 3) * 256 + tid] : make_float4(sig_s, sig_s, sig_s, sig_s);
        float4 c, p;
        bs_compute4<P, SIG_TAB>(sv, kv, tv, vv, inv_sig_s, r, c, p);
        const int64_t o = t * 256 + tid;
        st_stream((float4 *)call + o, c);
        st_stream((float4 *)put + o, p);
    }
    if (blockIdx.x == 0) {
        const int64_t nv = n >> 2;
        for (int64_t i = ntiles * 256 + tid; i < nv; i += blockDim.x)
            bs_float4<P, SIG_TAB>(S, K, T, sig, sig_s, inv_sig_s, r, call, put, i);
        if (tid < (n & 3)) {
            const int64_t i = (nv << 2) + tid;
            const float sj = SIG_TAB ? sig[i] : sig_s;
            bs_option<P>(S[i], K[i], T[i], sj, SIG_TAB ? inv_fast(sj) : inv_sig_s, r, call[i], put[i]);
        }
    }
}

// VEC: the tables are 16-byte aligned and the grid has one thread per float4
// (n/4 of them, rounded up to whole blocks): each thread prices its four
// options and exits, so a block retires as soon as its options are written
// and the next launch's blocks take its place (no sweep tail inside a launch).
// The 0-3 trailing options go to the first threads.  Otherwise (a misaligned
// view) a persistent grid strides over single options.
template <class P, bool SIG_TAB, bool VEC>
__global__ void __launch_bounds__(256, SIG_TAB ? 4 : 5) k_bs(const float *__restrict__ S, const float *__restrict__ K,
                                            const float *__restrict__ T, const float *__restrict__ sig,
                                            float sig_s, float r, float *__restrict__ call,
                                            float *__restrict__ put, int64_t n)
{
    const float inv_sig_s = P::exact ? 0.0f : inv_fast(sig_s);
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (VEC) {
        const int64_t nv = n >> 2;
        if (tid < nv) bs_float4<P, SIG_TAB>(S, K, T, sig, sig_s, inv_sig_s, r, call, put, tid);
        if (tid < (n & 3)) {
            const int64_t i = (nv << 2) + tid;
            const float sj = SIG_TAB ? sig[i] : sig_s;
            bs_option<P>(S[i], K[i], T[i], sj, SIG_TAB ? inv_fast(sj) : inv_sig_s, r, call[i], put[i]);
        }
    } else {
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (int64_t i = tid; i < n; i += stride) {
            float cj, pj;
            const float sj = SIG_TAB ? sig[i] : sig_s;
            bs_option<P>(S[i], K[i], T[i], sj, SIG_TAB ? inv_fast(sj) : inv_sig_s, r, cj, pj);
            call[i] = cj;
            put[i] = pj;
        }
    }
}

template <class P, bool RT, bool VT>
__global__ void __launch_bounds__(256) k_bs_demo(const float *__restrict__ S, const float *__restrict__ X,
                                                 const float *__restrict__ T, const float *__restrict__ rt,
                                                 float r, const float *__restrict__ vt, float v,
                                                 float *__restrict__ R, int64_t n, int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        for (int64_t i = tid; i < nv; i += stride) {
            float4 s = ld_stream((const float4 *)S + i), x = ld_stream((const float4 *)X + i),
                   t = ld_stream((const float4 *)T + i);
            float4 rr = RT ? ld_stream((const float4 *)rt + i) : make_float4(r, r, r, r);
            float4 vv = VT ? ld_stream((const float4 *)vt + i) : make_float4(v, v, v, v);
            float4 o;
            if constexpr (!P::exact) {  // two options per packed instruction
                f2 c2 = bs_demo_fast2(pk(s.x, s.y), pk(x.x, x.y), pk(t.x, t.y), pk(rr.x, rr.y), pk(vv.x, vv.y));
                upk(c2, o.x, o.y);
                c2 = bs_demo_fast2(pk(s.z, s.w), pk(x.z, x.w), pk(t.z, t.w), pk(rr.z, rr.w), pk(vv.z, vv.w));
                upk(c2, o.z, o.w);
            } else {  // NT2's unfused arithmetic two options per packed instruction, bit for bit
                const f2 nz = pair_negzero();
                f2 c2 = bs_demo_nt2_2(pk(s.x, s.y), pk(x.x, x.y), pk(t.x, t.y), pk(rr.x, rr.y), pk(vv.x, vv.y), nz);
                upk(c2, o.x, o.y);
                c2 = bs_demo_nt2_2(pk(s.z, s.w), pk(x.z, x.w), pk(t.z, t.w), pk(rr.z, rr.w), pk(vv.z, vv.w), nz);
                upk(c2, o.z, o.w);
            }
            st_stream((float4 *)R + i, o);
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride)
        R[i] = bs_demo_option<P>(S[i], X[i], T[i], RT ? rt[i] : r, VT ? vt[i] : v);
}

// ------------------------------------------------------------ adjoint ----
// s + e = a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ float two_sum_err(float a, float b, float s)
{
    const float bb = Fast::sub(s, a);
    return Fast::add(Fast::sub(a, Fast::sub(s, bb)), Fast::sub(b, bb));
}

// log_pos_fast(z) (returned, bit for bit) and the rounding error of its two
// final additions, so that hi + lo carries log(z) to about 2^-30 relative.
__device__ __forceinline__ float log_pos_fast_ff(float z, float &lo)
{
    const uint32_t u = f_bits(z);
    float x = bits_f((u & 0x007fffffu) | 0x3f000000u);
    const bool lt = x < bits_f(NT2G_SQRT_2O_2);
    const float fe = Fast::sub(bits_f(0x4B000000u | (u >> 23)), lt ? 8388735.0f : 8388734.0f);
    x = Fast::sub(lt ? Fast::add(x, x) : x, 1.0f);
    const float x2 = Fast::mul(x, x);
    float y = horner<Fast>(x, bits_f(0xbda5dff0u), bits_f(0x3e0229f9u), bits_f(0xbe04d6b7u), bits_f(0x3e116e80u),
                           bits_f(0xbe2a6aa0u), bits_f(0x3e4cd0a3u), bits_f(0xbe800064u), bits_f(0x3eaaaaa9u));
    y = Fast::mul(Fast::mul(y, x), x2);
    y = Fast::fma(fe, bits_f(NT2G_LOG_2LO), y);
    y = Fast::fma(-0.5f, x2, y);
    const float s1 = Fast::add(x, y);
    const float p = Fast::mul(bits_f(NT2G_LOG_2HI), fe);  // exact: LOG_2HI has 9 significant bits
    const float hi = Fast::add(p, s1);                   // = fma(LOG_2HI, fe, s1)
    lo = Fast::add(two_sum_err(x, y, s1), two_sum_err(p, s1, hi));
    return hi;
}

// d1 and d2 of the fast forward are each within a few ulps, but the
// gradients' N(d) and phi(d) amplify an absolute error in d by phi/N (up to
// |d| in the tails) and by 1/(sigma sqrt T) through log(S/K) (40x for
// sigma = 0.05, T = 0.25).  This recovers dd1 = d1* - d1 and dd2 = d2* - d2,
// the exact values' distance from the rounded ones, to first order: the
// quotient S/K's residual, the log's rounding, (r + sigma^2/2) T + log(S/K)
// as a float pair, sqrt(T) refined once, sigma sqrt(T) as a float pair, and
// the residual of d1 * sigma sqrt(T) against that numerator.
__device__ __forceinline__ void bs_d_residuals(float S, float K, float T, float sig, float r, const BsFwd &f,
                                               float &dd1, float &dd2)
{
    const float q = Fast::fdiv(S, K);
    float lq_lo;
    const float lq = log_pos_fast_ff(q, lq_lo);
    lq_lo = Fast::fma(Fast::fma(-q, K, S), Fast::rcp(S), lq_lo);  // log(S/K) - log(q) ~ (S - qK)/S
    // a = r + sigma^2/2 as a + a_lo
    const float ss = Fast::mul(sig, sig), ss_lo = Fast::fma(sig, sig, -ss);
    const float h = Fast::mul(0.5f, ss);
    const float a = Fast::fma(ss, 0.5f, r);
    const float a_lo = Fast::fma(0.5f, ss_lo, two_sum_err(h, r, a));
    // numerator N = fma(a, T, lq) and its error against a* T + log(S/K)
    const float N = Fast::fma(a, T, lq);
    const float p = Fast::mul(a, T), pe = Fast::fma(a, T, -p);
    const float s = Fast::add(p, lq), se = two_sum_err(p, lq, s);
    const float N_lo = Fast::fma(a_lo, T, Fast::add(Fast::add(Fast::sub(s, N), se), Fast::add(pe, lq_lo)));
    // sigma sqrt(T) = vh + vl
    const float sq_lo = Fast::mul(Fast::fma(-f.sq, f.sq, T), Fast::mul(0.5f, f.rs));
    const float vh = Fast::mul(sig, f.sq);
    const float vl = Fast::fma(sig, sq_lo, Fast::fma(sig, f.sq, -vh));
    // d1* - d1 = (N + N_lo - d1 (vh + vl)) / (sigma sqrt T)
    const float res = Fast::fma(-f.d1, vl, Fast::add(Fast::fma(-f.d1, vh, N), N_lo));
    dd1 = Fast::mul(res, Fast::mul(f.rs, inv_fast(sig)));
    // d2 = RN(d1 - sigma sq): d2* - d2 = (t - d2) + t_lo + dd1 - vl, t + t_lo = d1 - vh
    const float t = Fast::sub(f.d1, vh), t_lo = two_sum_err(f.d1, -vh, t);
    dd2 = Fast::add(Fast::add(Fast::sub(t, f.d2), t_lo), Fast::sub(dd1, vl));
}

// Hand-derived reverse sweep of the forward graph
//   sq = sqrt(T), vs = sig*sq, d1 = (log(S/K) + (r + sig^2/2) T)/vs, d2 = d1 - vs,
//   e = K exp(-rT), C = S N(d1) - e N(d2), P = e N(-d2) - S N(-d1)
// with seeds gc, gp and every intermediate recomputed in registers.
// The adjoint reaching d1 through N(d1), N(-d1) is  S phi(d1) (gc+gp)  and
// through d2 = d1 - vs it is  -e phi(d2) (gc+gp); since S phi(d1) =
// K e^{-rT} phi(d2) holds exactly for the model, their sum is identically
// zero and the sweep drops it symbolically instead of computing two nearly
// equal FP32 products (whose rounding noise, divided by vs, would dominate
// every gradient for short-dated low-volatility options).  What survives:
//   vs-bar = S phi(d1) (gc+gp)               (from d2 = d1 - vs)
//   S-bar  = gc N(d1) - gp N(-d1)
//   e-bar  = gp N(-d2) - gc N(d2)  ->  K-bar = e-bar e^{-rT}
//   sig-bar = vs-bar sq;  T-bar = vs-bar sig/(2 sq) - r e-bar e
//   r-bar   = -T e-bar e
__device__ __forceinline__ void bs_vjp_option(float S, float K, float T, float sig, float r, float gc,
                                              float gp, float &C, float &P_, float &dS, float &dK,
                                              float &dT, float &dsig, float &dr)
{
    // forward (the fast forward kernel's arithmetic, bit for bit)
    BsFwd f = bs_prefix_fast(S, K, T, sig, inv_fast(sig), r);
    float n1, m1, n2, m2, g1;  // g1 = exp(-d1^2/2)
    bs_normcdfs_fast(f.d1, f.d2, S, f.e, n1, m1, n2, m2, &g1);
    const float sq = f.sq, ert = f.ert, e = f.e;
    C = Fast::fma(-e, n2, Fast::mul(S, n1));
    P_ = Fast::fma(-S, m1, Fast::mul(e, m2));
    const bool bad = !(fabsf(f.d1) < f_inf());  // as the forward kernel: NaN unless d1 is finite
    C = bad ? f_nan() : C;
    P_ = bad ? f_nan() : P_;
    // the gradients take N(d) and phi(d) at the exact d: first-order
    // corrections N(d + dd) = N(d) + phi(d) dd, phi(d + dd) = phi(d)(1 - d dd)
    const float inv_sqrt_2pi = 0.398942280401432678f;
    float dd1, dd2;
    bs_d_residuals(S, K, T, sig, r, f, dd1, dd2);
    const float phi1 = Fast::mul(inv_sqrt_2pi, g1);
    const float phi2 = Fast::mul(phi1, Fast::mul(S, Fast::rcp(e)));  // S phi(d1) = e phi(d2)
    const float c1 = Fast::mul(phi1, dd1), c2 = Fast::mul(phi2, dd2);
    n1 = Fast::add(n1, c1);
    m1 = Fast::sub(m1, c1);
    n2 = Fast::add(n2, c2);
    m2 = Fast::sub(m2, c2);
    g1 = Fast::fma(Fast::mul(-f.d1, dd1), g1, g1);
    // reverse
    float gs = Fast::add(gc, gp);
    float bvs = Fast::mul(Fast::mul(Fast::mul(inv_sqrt_2pi, g1), S), gs);
    float be = Fast::fma(gp, m2, -Fast::mul(gc, n2));
    float bee = Fast::mul(be, e);
    dS = Fast::fma(gc, n1, -Fast::mul(gp, m1));
    dK = Fast::mul(be, ert);
    dsig = Fast::mul(bvs, sq);
    dT = Fast::fma(Fast::mul(bvs, sig), Fast::mul(0.5f, f.rs), -Fast::mul(r, bee));
    dr = -Fast::mul(T, bee);
}

__global__ void __launch_bounds__(256) k_bs_vjp(const float *__restrict__ S, const float *__restrict__ K,
                                                const float *__restrict__ T, const float *__restrict__ sig,
                                                float r, const float *__restrict__ gc,
                                                const float *__restrict__ gp, float *__restrict__ C,
                                                float *__restrict__ P, float *__restrict__ dS,
                                                float *__restrict__ dK, float *__restrict__ dT,
                                                float *__restrict__ dsig, float *__restrict__ dr,
                                                int64_t n, int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        for (int64_t i = tid; i < nv; i += stride) {
            float4 s = ld_stream((const float4 *)S + i), k = ld_stream((const float4 *)K + i),
                   t = ld_stream((const float4 *)T + i), v = ld_stream((const float4 *)sig + i),
                   a = ld_stream((const float4 *)gc + i), b = ld_stream((const float4 *)gp + i);
            float4 c, p, o0, o1, o2, o3, o4;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float cj, pj, x0, x1, x2, x3, x4;
                bs_vjp_option(get(s, j), get(k, j), get(t, j), get(v, j), r, get(a, j), get(b, j), cj, pj,
                              x0, x1, x2, x3, x4);
                set(c, j, cj); set(p, j, pj);
                set(o0, j, x0); set(o1, j, x1); set(o2, j, x2); set(o3, j, x3); set(o4, j, x4);
            }
            st_stream((float4 *)C + i, c);
            st_stream((float4 *)P + i, p);
            st_stream((float4 *)dS + i, o0);
            st_stream((float4 *)dK + i, o1);
            st_stream((float4 *)dT + i, o2);
            st_stream((float4 *)dsig + i, o3);
            st_stream((float4 *)dr + i, o4);
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride)
        bs_vjp_option(S[i], K[i], T[i], sig[i], r, gc[i], gp[i], C[i], P[i], dS[i], dK[i], dT[i], dsig[i],
                      dr[i]);
}

// ---------------------------------------------------------- launchers ----
template <class KERN>
static int grid_for(KERN k, int64_t n)
{
    return persistent_blocks(k, 256, 0, 256 * 4, n);
}

// The pipelined kernel takes aligned batches from 2^22 options on: it keeps
// bulk copies of three tiles per block in flight, which matches the
// one-float4-per-thread kernel's throughput there (both are issue-bound at
// ~98 instructions per option) while reading HBM through the copy engine;
// below it the persistent grid's ramp costs more than it saves.
constexpr int64_t kBsPipeMin = 1ll << 22;
constexpr int kBsPipeStages = 3;

template <class P, bool SIG_TAB, int STAGES>
static nt2g_status launch_bs_pipe_n(const float *S, const float *K, const float *T, const float *sig, float sig_s,
                                    float r, float *call, float *put, int64_t n, cudaStream_t st)
{
    const size_t smem = (size_t)STAGES * (SIG_TAB ? 4 : 3) * 256 * sizeof(float4) + STAGES * sizeof(uint64_t);
    static const cudaError_t attr = cudaFuncSetAttribute(k_bs_pipe<P, SIG_TAB, STAGES>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess) return cuda_status(attr, "blackscholes pipeline: shared memory");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bs_pipe<P, SIG_TAB, STAGES>, 256, smem) !=
            cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t tiles = n / 1024, full = (int64_t)device_sm_count() * per_sm;
    const int grid = (int)(tiles < full ? tiles : full);
    k_bs_pipe<P, SIG_TAB, STAGES><<<grid, 256, smem, st>>>(S, K, T, sig, sig_s, r, call, put, n);
    NT2G_LAUNCH_CHECK("blackscholes pipeline launch");
    return NT2G_OK;
}

nt2g_status launch_bs(const float *S, const float *K, const float *T, const float *sig, float sig_s, float r,
                      float *call, float *put, int64_t n, int precision, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(S) && aligned16(K) && aligned16(T) && aligned16(call) && aligned16(put) &&
              (!sig || aligned16(sig));
    // vec: one thread per float4 (at least one block, for the trailing options)
    const int64_t exact_grid = ((n >> 2) + 255) / 256 > 0 ? ((n >> 2) + 255) / 256 : 1;
#define NT2G_BS(PP, TAB)                                                                                       \
    do {                                                                                                       \
        if (vec) k_bs<PP, TAB, true><<<(int)exact_grid, 256, 0, st>>>(S, K, T, sig, sig_s, r, call, put, n);   \
        else k_bs<PP, TAB, false><<<grid_for(k_bs<PP, TAB, false>, n), 256, 0, st>>>(S, K, T, sig, sig_s, r,   \
                                                                                      call, put, n);           \
    } while (0)
    if (vec && n >= kBsPipeMin) {
        constexpr int ST = kBsPipeStages;
        if (precision == NT2G_PREC_NT2)
            return sig ? launch_bs_pipe_n<Nt2, true, ST>(S, K, T, sig, sig_s, r, call, put, n, st)
                       : launch_bs_pipe_n<Nt2, false, ST>(S, K, T, sig, sig_s, r, call, put, n, st);
        return sig ? launch_bs_pipe_n<Fast, true, ST>(S, K, T, sig, sig_s, r, call, put, n, st)
                   : launch_bs_pipe_n<Fast, false, ST>(S, K, T, sig, sig_s, r, call, put, n, st);
    }
    if (precision == NT2G_PREC_NT2) {
        if (sig) NT2G_BS(Nt2, true);
        else NT2G_BS(Nt2, false);
    } else {
        if (sig) NT2G_BS(Fast, true);
        else NT2G_BS(Fast, false);
    }
#undef NT2G_BS
    NT2G_LAUNCH_CHECK("blackscholes launch");
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_wait_timeouts(uint64_t *count)
{
    NT2G_CHECK_ARG(count != nullptr, "nt2g_wait_timeouts: count is NULL");
    unsigned long long v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_bs_wait_timeouts, sizeof v);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_wait_timeouts");
    *count = v;
    return NT2G_OK;
}

nt2g_status launch_bs_demo(const float *S, const float *X, const float *T, const float *rt, float r, const float *vt,
                           float v, float *R, int64_t n, int precision, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(S) && aligned16(X) && aligned16(T) && aligned16(R) && (!rt || aligned16(rt)) &&
              (!vt || aligned16(vt));
#define NT2G_DEMO(PP, A, B)                                                                                   \
    k_bs_demo<PP, A, B><<<grid_for(k_bs_demo<PP, A, B>, n), 256, 0, st>>>(S, X, T, rt, r, vt, v, R, n, vec)
    if (precision == NT2G_PREC_NT2) {
        if (rt && vt) NT2G_DEMO(Nt2, true, true);
        else if (rt) NT2G_DEMO(Nt2, true, false);
        else if (vt) NT2G_DEMO(Nt2, false, true);
        else NT2G_DEMO(Nt2, false, false);
    } else {
        if (rt && vt) NT2G_DEMO(Fast, true, true);
        else if (rt) NT2G_DEMO(Fast, true, false);
        else if (vt) NT2G_DEMO(Fast, false, true);
        else NT2G_DEMO(Fast, false, false);
    }
#undef NT2G_DEMO
    NT2G_LAUNCH_CHECK("blackscholes demo launch");
    return NT2G_OK;
}

nt2g_status launch_bs_vjp(const float *S, const float *K, const float *T, const float *sig, float r, const float *gc,
                          const float *gp, float *C, float *P, float *dS, float *dK, float *dT, float *dsig,
                          float *dr, int64_t n, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    const void *ps[] = {S, K, T, sig, gc, gp, C, P, dS, dK, dT, dsig, dr};
    int vec = 1;
    for (const void *p : ps) vec &= aligned16(p);
    k_bs_vjp<<<grid_for(k_bs_vjp, n), 256, 0, st>>>(S, K, T, sig, r, gc, gp, C, P, dS, dK, dT, dsig, dr, n, vec);
    NT2G_LAUNCH_CHECK("blackscholes vjp launch");
    return NT2G_OK;
}

}  // namespace nt2g
