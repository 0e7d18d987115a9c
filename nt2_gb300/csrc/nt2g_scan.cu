// nt2g_scan.cu -- cumulative sums, products, maxima and minima along one
// dimension (cumsum, cumprod, cummax, cummin) of a table viewed as
// [lo, inner, hi] (column-major): out[l + lo*(k + inner*h)] = the scan over
// k' <= k of x[l + lo*(k' + inner*h)].
//
// NT2 reshapes a cumulative function like a reduction and scans each segment
// in order from the neutral element: summary = bop(summary, x); out = summary
// (core/swar/include/nt2/dsl/functions/cumulative/run.hpp:26-67,
// core/swar/include/nt2/core/functions/details/scan_step.hpp:27-43; the
// functors cumsum = (plus, Zero), cumprod = (multiplies, One), cummax =
// (max, Minf), cummin = (min, Inf) in boost/simd/swar/functions/cum*.hpp).
//
// NT2 policy: one thread per segment in that order with NT2's unfused float
// operations: bit-identical wherever NT2 spreads segments over threads.
//
// Fast policy, three phases with no block waiting on another:
//   1. each chunk of each segment reduces to an aggregate,
//   2. per segment, the chunk aggregates are scanned in order (exclusive),
//   3. each chunk is scanned again, starting from its prefix.
// Contiguous segments (lo = 1) run one warp per chunk in tiles of 512
// elements (16 consecutive ones per lane, an in-order warp scan of the lane
// totals);
// phase 1 of cumsum/cumprod is a plain reduction (order does not matter to a
// commutative aggregate).  Strided segments run one thread per segment (four
// with float4) over chunks of the scan range, 8 rows of loads at a time.  cumsum carries compensated sums (s + c; chunk prefixes in
// FP64), so each output is within about an ulp of the exact prefix; cumprod
// carries FP64 products; cummax/cummin are exact: NT2's (s > x) ? s : x is
// not associative once a NaN appears (a NaN summary is replaced by the next
// element), so each element is a pair (value, starts-a-segment) with NaN
// elements starting segments, which makes the in-order combine associative
// and reproduces NT2's sequential result, NaNs included.  When a segment fits
// one chunk, phase 3 alone runs.
#include "nt2g_accum.cuh"
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

constexpr int kScanThreads = 256;
constexpr int64_t kScanChunk = 16384;  // multiple of the 512-element tile
constexpr int64_t kScanTarget = 152 * 1024;

// ------------------------------------------------------------- elements --
// MAX/MIN (the primary template): (value, flags) pairs.  flags bit 0: the
// stretch starts at a NaN element (a segment head); bit 1: the stretch is
// empty (the identity: the neutral value folded with nothing).
template <int OP> struct SE {
    float v;
    int h;
    __device__ static SE id() { return SE{OP == NT2G_SCAN_MAX ? -INFINITY : INFINITY, 2}; }
    __device__ static SE of(float x) { return SE{x, x != x ? 1 : 0}; }
    __device__ static float op(float s, float x)
    {
        return OP == NT2G_SCAN_MAX ? ((s > x) ? s : x) : ((s < x) ? s : x);
    }
    __device__ static SE combine(const SE &a, const SE &b)  // a precedes b
    {
        if (b.h & 2) return a;
        if (a.h & 2) return SE{op(a.v, b.v), b.h};  // the neutral value meets the first element
        return (b.h & 1) ? b : SE{op(a.v, b.v), a.h};
    }
    __device__ float out() const { return v; }
    __device__ SE shfl_up(int off) const
    {
        return SE{__shfl_up_sync(0xffffffffu, v, off), __shfl_up_sync(0xffffffffu, h, off)};
    }
    __device__ SE shfl(int lane) const { return SE{__shfl_sync(0xffffffffu, v, lane), __shfl_sync(0xffffffffu, h, lane)}; }
};
// SUM: compensated pair
template <> struct SE<NT2G_SCAN_SUM> {
    CSum v;
    __device__ static SE id() { return SE{CSum{0.0f, 0.0f}}; }
    __device__ static SE of(float x) { return SE{CSum{x, 0.0f}}; }
    __device__ static SE combine(const SE &a, const SE &b)  // a precedes b
    {
        SE r = a;
        csum_merge(r.v, b.v);
        return r;
    }
    __device__ float out() const { return __fadd_rn(v.s, v.c); }
    __device__ double agg() const { return (double)v.s + (double)v.c; }
    __device__ static SE from(double p)
    {
        const float hi = (float)p;
        return SE{CSum{hi, (float)(p - (double)hi)}};
    }
    __device__ SE shfl_up(int off) const
    {
        return SE{CSum{__shfl_up_sync(0xffffffffu, v.s, off), __shfl_up_sync(0xffffffffu, v.c, off)}};
    }
    __device__ SE shfl(int lane) const
    {
        return SE{CSum{__shfl_sync(0xffffffffu, v.s, lane), __shfl_sync(0xffffffffu, v.c, lane)}};
    }
};
// PROD: double
template <> struct SE<NT2G_SCAN_PROD> {
    double v;
    __device__ static SE id() { return SE{1.0}; }
    __device__ static SE of(float x) { return SE{(double)x}; }
    __device__ static SE combine(const SE &a, const SE &b) { return SE{a.v * b.v}; }
    __device__ float out() const { return (float)v; }
    __device__ double agg() const { return v; }
    __device__ static SE from(double p) { return SE{p}; }
    __device__ SE shfl_up(int off) const { return SE{__shfl_up_sync(0xffffffffu, v, off)}; }
    __device__ SE shfl(int lane) const { return SE{__shfl_sync(0xffffffffu, v, lane)}; }
};

// 16-byte chunk record in the workspace: an aggregate, later its prefix
struct ScanRec {
    double d;  // SUM, PROD
    float v;   // MAX, MIN
    int h;
};
template <int OP> __device__ __forceinline__ ScanRec to_rec(const SE<OP> &e)
{
    ScanRec r{0.0, 0.0f, 0};
    if constexpr (OP == NT2G_SCAN_SUM || OP == NT2G_SCAN_PROD) r.d = e.agg();
    else { r.v = e.v; r.h = e.h; }
    return r;
}
template <int OP> __device__ __forceinline__ SE<OP> from_rec(const ScanRec &r)
{
    if constexpr (OP == NT2G_SCAN_SUM || OP == NT2G_SCAN_PROD) return SE<OP>::from(r.d);
    else return SE<OP>{r.v, r.h};
}

// In-order inclusive warp scan of one value per lane.
template <int OP> __device__ __forceinline__ SE<OP> warp_scan(SE<OP> x, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        SE<OP> o = x.shfl_up(off);
        if (lane >= off) x = SE<OP>::combine(o, x);
    }
    return x;
}

// ----------------------------------------- contiguous segments (lo == 1) --
// One warp per (segment, chunk): tiles of 512 elements, lane l owning
// elements 16l..16l+15 of the tile.  PHASE 1 keeps the running carry and stores
// the chunk aggregate; PHASE 3 starts from the chunk's prefix (or the
// identity when there is one chunk) and writes every inclusive value.
template <int OP, int PHASE>
__global__ void __launch_bounds__(kScanThreads) k_scan_inner(const float *x, int64_t inner, int64_t hi,
                                                             int64_t chunk, int64_t q, int vec,
                                                             ScanRec *__restrict__ rec, float *out)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t item = warp; item < hi * q; item += nwarps) {
        const int64_t seg = item / q, c = item - seg * q;
        const int64_t k0 = c * chunk, k1 = (k0 + chunk < inner) ? k0 + chunk : inner;
        const float *p = x + seg * inner;
        float *o = out + seg * inner;
        if constexpr (PHASE == 1 && (OP == NT2G_SCAN_SUM || OP == NT2G_SCAN_PROD)) {
            // the chunk aggregate of a commutative operation needs no scan: each
            // lane folds its float4s (8 in flight), then the lanes combine in order
            CSum acc{0.0f, 0.0f};
            double prod = 1.0;
            for (int64_t t0 = k0; t0 < k1; t0 += 1024) {
                float f[8][4];
                int nn[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int64_t e = t0 + 128 * u + 4 * lane;
                    nn[u] = (int)(k1 - e < 4 ? (k1 - e > 0 ? k1 - e : 0) : 4);
                    if (vec && nn[u] == 4) {
                        const float4 v = ld_stream((const float4 *)(p + e));
                        f[u][0] = v.x; f[u][1] = v.y; f[u][2] = v.z; f[u][3] = v.w;
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j) f[u][j] = j < nn[u] ? p[e + j] : 0.0f;
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (OP == NT2G_SCAN_SUM) csum_add(acc, f[u][j]);
                        else if (j < nn[u]) prod *= (double)f[u][j];
                    }
            }
            if (OP == NT2G_SCAN_SUM) {
                acc = warp_csum(acc);
                if (lane == 0) rec[item] = ScanRec{(double)acc.s + (double)acc.c, 0.0f, 0};
            } else {
#pragma unroll
                for (int off = 16; off; off >>= 1) prod *= __shfl_down_sync(0xffffffffu, prod, off);
                if (lane == 0) rec[item] = ScanRec{prod, 0.0f, 0};
            }
            continue;
        }
        SE<OP> carry = (PHASE == 3 && q > 1) ? from_rec<OP>(rec[item]) : SE<OP>::id();
        // tiles of 512 elements, 16 consecutive ones per lane: the lane folds its
        // run, one in-order warp scan of the lane totals gives every lane its
        // prefix, and the lane's outputs follow in order from that prefix
        for (int64_t t0 = k0; t0 < k1; t0 += 512) {
            const int64_t e0 = t0 + 16 * lane;
            const int cnt = (int)(k1 - e0 < 16 ? (k1 - e0 > 0 ? k1 - e0 : 0) : 16);
            float f[16];
            if (vec && cnt == 16) {
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float4 w = ld_stream((const float4 *)(p + e0) + v);
                    f[4 * v] = w.x; f[4 * v + 1] = w.y; f[4 * v + 2] = w.z; f[4 * v + 3] = w.w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) f[j] = j < cnt ? p[e0 + j] : 0.0f;
            }
            SE<OP> agg = SE<OP>::id();
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (j < cnt) agg = SE<OP>::combine(agg, SE<OP>::of(f[j]));
            const SE<OP> inc = warp_scan<OP>(agg, lane);
            SE<OP> ex = inc.shfl_up(1);
            if (lane == 0) ex = SE<OP>::id();
            if (PHASE == 3) {
                SE<OP> run = SE<OP>::combine(carry, ex);
                float r[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    run = SE<OP>::combine(run, SE<OP>::of(f[j]));
                    r[j] = run.out();
                }
                if (vec && cnt == 16) {
#pragma unroll
                    for (int v = 0; v < 4; ++v)
                        st_stream((float4 *)(o + e0) + v, make_float4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]));
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (j < cnt) o[e0 + j] = r[j];
                }
            }
            carry = SE<OP>::combine(carry, inc.shfl(31));
        }
        if (PHASE == 1 && lane == 0) rec[item] = to_rec<OP>(carry);
    }
}

// ---------------------------------------------- strided scans (lo > 1) --
// Thread per segment (VEC: four neighbouring segments via float4) over the
// chunk [c*ck, min((c+1)*ck, inner)) of the scan range; grid.y = chunk.
template <int OP, int VEC, int PHASE>
__global__ void __launch_bounds__(kScanThreads) k_scan_outer(const float *x, int64_t lo, int64_t inner,
                                                             int64_t hi, int64_t ck, int64_t q,
                                                             ScanRec *__restrict__ rec, float *out)
{
    const int64_t lv = lo / VEC;
    const int64_t c = blockIdx.y;
    const int64_t k0 = c * ck, k1 = (k0 + ck < inner) ? k0 + ck : inner;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < lv * hi; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = t / lv, l = (t - h * lv) * VEC;
        const int64_t base = l + lo * inner * h;
        SE<OP> carry[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const int64_t seg = l + v + lo * h;
            carry[v] = (PHASE == 3 && q > 1) ? from_rec<OP>(rec[c * lo * hi + seg]) : SE<OP>::id();
        }
        // groups of kGroup rows: all loads of a group are issued before its scan
        constexpr int kGroup = (OP == NT2G_SCAN_PROD && VEC == 4) ? 4 : 8;  // FP64 products: fewer registers free
        auto step = [&](int64_t k, const float (&e)[VEC]) {
            float r[VEC];
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                carry[v] = SE<OP>::combine(carry[v], SE<OP>::of(e[v]));
                r[v] = carry[v].out();
            }
            if (PHASE == 3) {
                if constexpr (VEC == 4) st_stream((float4 *)(out + base + lo * k), make_float4(r[0], r[1], r[2], r[3]));
                else out[base + lo * k] = r[0];
            }
        };
        auto fetch = [&](int64_t k, float (&e)[VEC]) {
            if constexpr (VEC == 4) {
                const float4 f = ld_stream((const float4 *)(x + base + lo * k));
                e[0] = f.x; e[1] = f.y; e[2] = f.z; e[3] = f.w;
            } else {
                e[0] = ld_stream(x + base + lo * k);
            }
        };
        int64_t k = k0;
        for (; k + kGroup <= k1; k += kGroup) {
            float e[kGroup][VEC];
#pragma unroll
            for (int g = 0; g < kGroup; ++g) fetch(k + g, e[g]);
#pragma unroll
            for (int g = 0; g < kGroup; ++g) step(k + g, e[g]);
        }
        for (; k < k1; ++k) {
            float e[VEC];
            fetch(k, e);
            step(k, e);
        }
        if (PHASE == 1) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) rec[c * lo * hi + (l + v + lo * h)] = to_rec<OP>(carry[v]);
        }
    }
}

// Chunk records combine in FP64 (sum, prod) or by the pair rule (max, min).
template <int OP> __device__ __forceinline__ ScanRec rec_id()
{
    if constexpr (OP == NT2G_SCAN_SUM) return ScanRec{0.0, 0.0f, 0};
    else if constexpr (OP == NT2G_SCAN_PROD) return ScanRec{1.0, 0.0f, 0};
    else return to_rec<OP>(SE<OP>::id());
}
template <int OP> __device__ __forceinline__ ScanRec rec_combine(const ScanRec &a, const ScanRec &b)
{
    if constexpr (OP == NT2G_SCAN_SUM) return ScanRec{a.d + b.d, 0.0f, 0};
    else if constexpr (OP == NT2G_SCAN_PROD) return ScanRec{a.d * b.d, 0.0f, 0};
    else return to_rec<OP>(SE<OP>::combine(from_rec<OP>(a), from_rec<OP>(b)));
}

// Phase 2: per segment, replace the chunk aggregates by their exclusive
// prefixes in order (few chunks: one thread per segment).
template <int OP>
__global__ void __launch_bounds__(kScanThreads) k_scan_prefix(ScanRec *__restrict__ rec, int64_t n_seg, int64_t q,
                                                              int64_t cs)
{
    // record c of segment s at rec[s * ss + c * cs]: ss = q, cs = 1 for contiguous
    // scans; ss = 1, cs = n_seg (chunk-major, coalesced over segments) for strided ones
    const int64_t ss = cs == 1 ? q : 1;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += (int64_t)gridDim.x * blockDim.x) {
        ScanRec *r = rec + s * ss;
        ScanRec acc = rec_id<OP>();
        int64_t c = 0;
        for (; c + 8 <= q; c += 8) {  // eight independent loads in flight
            ScanRec a[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = r[(c + u) * cs];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                r[(c + u) * cs] = acc;
                acc = rec_combine<OP>(acc, a[u]);
            }
        }
        for (; c < q; ++c) {
            const ScanRec a = r[c * cs];
            r[c * cs] = acc;
            acc = rec_combine<OP>(acc, a);
        }
    }
}

// Phase 2 for many chunks: one block per segment (below).  The combine order
// is fixed for a given q.
template <int OP> __device__ __forceinline__ ScanRec rec_shfl_up(const ScanRec &a, int off)
{
    return ScanRec{__shfl_up_sync(0xffffffffu, a.d, off), __shfl_up_sync(0xffffffffu, a.v, off),
                    __shfl_up_sync(0xffffffffu, a.h, off)};
}

template <int OP>
__global__ void __launch_bounds__(kScanThreads) k_scan_prefix_block(ScanRec *__restrict__ rec, int64_t n_seg,
                                                                    int64_t q, int64_t cs)
{
    // tiles of kScanThreads x 8 consecutive records: each thread loads its 8
    // (independent loads), the thread totals are scanned in order across the
    // block (warp shuffles, then the warp totals), and a carry runs over the tiles
    constexpr int kPer = 8, kWarps = kScanThreads / 32;
    __shared__ ScanRec wtot[kWarps];
    __shared__ ScanRec carry_s;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int64_t s = blockIdx.x; s < n_seg; s += gridDim.x) {
        ScanRec *r = rec + s * (cs == 1 ? q : 1);
        ScanRec carry = rec_id<OP>();
        for (int64_t t0 = 0; t0 < q; t0 += (int64_t)kScanThreads * kPer) {
            const int64_t c0 = t0 + (int64_t)tid * kPer;
            ScanRec a[kPer];
#pragma unroll
            for (int u = 0; u < kPer; ++u) a[u] = c0 + u < q ? r[(c0 + u) * cs] : rec_id<OP>();
            ScanRec tot = rec_id<OP>();
#pragma unroll
            for (int u = 0; u < kPer; ++u) tot = rec_combine<OP>(tot, a[u]);
            ScanRec inc = tot;  // in-order inclusive scan of the thread totals in the warp
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const ScanRec o = rec_shfl_up<OP>(inc, off);
                if (lane >= off) inc = rec_combine<OP>(o, inc);
            }
            if (lane == 31) wtot[wid] = inc;
            __syncthreads();
            if (tid == 0) {  // the warp totals in order, and the next tile's carry
                ScanRec run = carry;
                for (int w = 0; w < kWarps; ++w) {
                    const ScanRec x = wtot[w];
                    wtot[w] = run;
                    run = rec_combine<OP>(run, x);
                }
                carry_s = run;
            }
            __syncthreads();
            ScanRec ex = rec_shfl_up<OP>(inc, 1);
            if (lane == 0) ex = rec_id<OP>();
            ScanRec pre = rec_combine<OP>(wtot[wid], ex);
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                if (c0 + u < q) r[(c0 + u) * cs] = pre;
                pre = rec_combine<OP>(pre, a[u]);
            }
            carry = carry_s;
            __syncthreads();
        }
    }
}

// NT2 policy: the segment in order, NT2's operations.
template <int OP>
__global__ void __launch_bounds__(kScanThreads) k_scan_nt2(const float *x, int64_t lo, int64_t inner,
                                                           int64_t hi, float *out)
{
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < lo * hi; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = s / lo, l = s - h * lo;
        const int64_t base = l + lo * inner * h;
        float acc = OP == NT2G_SCAN_PROD ? 1.0f : OP == NT2G_SCAN_MAX ? -INFINITY : OP == NT2G_SCAN_MIN ? INFINITY : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = x[base + lo * k];
            if (OP == NT2G_SCAN_SUM) acc = __fadd_rn(acc, v);
            else if (OP == NT2G_SCAN_PROD) acc = __fmul_rn(acc, v);
            else if (OP == NT2G_SCAN_MAX) acc = (acc > v) ? acc : v;
            else acc = (acc < v) ? acc : v;
            out[base + lo * k] = acc;
        }
    }
}

// ---------------------------------------------------------------- plans --
struct ScanPlan {
    int kind = 1;  // 1 contiguous, 2 strided
    int vec = 0;
    int64_t chunk = 0, q = 1;
};

static ScanPlan plan_scan(int64_t lo, int64_t inner, int64_t hi, bool aligned)
{
    ScanPlan p;
    if (lo == 1) {
        p.kind = 1;
        p.vec = aligned && inner % 4 == 0;
        const int64_t want = 152 * 8 * 4;
        int64_t chunk = kScanChunk;
        if (hi * ((inner + chunk - 1) / chunk) < want) {
            const int64_t per = (want + hi - 1) / hi;
            chunk = (inner + per - 1) / per;
            if (chunk < 1024) chunk = 1024;
        }
        chunk = (chunk + 511) / 512 * 512;
        p.chunk = chunk;
        p.q = inner > 0 ? (inner + chunk - 1) / chunk : 1;
        return p;
    }
    p.kind = 2;
    p.vec = aligned && lo % 4 == 0 ? 4 : 1;
    const int64_t threads = lo * hi / p.vec;
    int64_t q = 1;
    if (threads < kScanTarget) {
        q = (kScanTarget + threads - 1) / threads;
        const int64_t qmax = inner / 16 > 0 ? inner / 16 : 1;
        if (q > qmax) q = qmax;
        if (q > 65535) q = 65535;
    }
    p.chunk = inner > 0 ? (inner + q - 1) / q : 1;
    p.q = inner > 0 ? (inner + p.chunk - 1) / p.chunk : 1;
    return p;
}

nt2g_status scan_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    const ScanPlan a = plan_scan(lo, inner, hi, true), b = plan_scan(lo, inner, hi, false);
    const int64_t q = a.q > b.q ? a.q : b.q;
    *bytes = q > 1 ? (size_t)(lo * hi) * (size_t)q * sizeof(ScanRec) : 0;
    return NT2G_OK;
}

template <int OP> static void launch_prefix(ScanRec *rec, int64_t n_seg, int64_t q, int64_t cs, cudaStream_t st)
{
    auto cap = [](int64_t g) { return (int)(g < 152 * 32 ? (g > 0 ? g : 1) : 152 * 32); };
    if (q >= 512) k_scan_prefix_block<OP><<<cap(n_seg), kScanThreads, 0, st>>>(rec, n_seg, q, cs);
    else k_scan_prefix<OP><<<cap((n_seg + kScanThreads - 1) / kScanThreads), kScanThreads, 0, st>>>(rec, n_seg, q, cs);
}

template <int OP>
static nt2g_status launch_scan_op(const float *x, int64_t lo, int64_t inner, int64_t hi, int precision, void *ws,
                                  size_t ws_bytes, float *out, cudaStream_t st)
{
    const int64_t n_seg = lo * hi;
    auto cap = [](int64_t g) { return (int)(g < 152 * 32 ? (g > 0 ? g : 1) : 152 * 32); };
    if (precision == NT2G_PREC_NT2) {
        k_scan_nt2<OP><<<cap((n_seg + kScanThreads - 1) / kScanThreads), kScanThreads, 0, st>>>(x, lo, inner, hi, out);
        NT2G_LAUNCH_CHECK("scan launch");
        return NT2G_OK;
    }
    const ScanPlan p = plan_scan(lo, inner, hi, aligned16(x) && aligned16(out));
    if (p.q > 1 && (size_t)(n_seg * p.q) * sizeof(ScanRec) > ws_bytes) {
        set_error("nt2g_scan_f32: workspace of %zu bytes, %zu needed", ws_bytes, (size_t)(n_seg * p.q) * sizeof(ScanRec));
        return NT2G_ERR_INVALID;
    }
    ScanRec *rec = (ScanRec *)ws;
    if (p.kind == 1) {
        const int grid = cap((hi * p.q + 7) / 8);
        if (p.q > 1) {
            k_scan_inner<OP, 1><<<grid, kScanThreads, 0, st>>>(x, inner, hi, p.chunk, p.q, p.vec, rec, out);
            launch_prefix<OP>(rec, n_seg, p.q, 1, st);
        }
        k_scan_inner<OP, 3><<<grid, kScanThreads, 0, st>>>(x, inner, hi, p.chunk, p.q, p.vec, rec, out);
    } else {
        dim3 grid(cap((n_seg / p.vec + kScanThreads - 1) / kScanThreads), (unsigned)p.q);
        if (p.vec == 4) {
            if (p.q > 1) {
                k_scan_outer<OP, 4, 1><<<grid, kScanThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, rec, out);
                launch_prefix<OP>(rec, n_seg, p.q, n_seg, st);
            }
            k_scan_outer<OP, 4, 3><<<grid, kScanThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, rec, out);
        } else {
            if (p.q > 1) {
                k_scan_outer<OP, 1, 1><<<grid, kScanThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, rec, out);
                launch_prefix<OP>(rec, n_seg, p.q, n_seg, st);
            }
            k_scan_outer<OP, 1, 3><<<grid, kScanThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, rec, out);
        }
    }
    NT2G_LAUNCH_CHECK("scan launch");
    return NT2G_OK;
}

nt2g_status launch_scan(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws,
                        size_t ws_bytes, float *out, cudaStream_t st)
{
    if (lo * inner * hi == 0) return NT2G_OK;
    switch (op) {
    case NT2G_SCAN_SUM: return launch_scan_op<NT2G_SCAN_SUM>(x, lo, inner, hi, precision, ws, ws_bytes, out, st);
    case NT2G_SCAN_PROD: return launch_scan_op<NT2G_SCAN_PROD>(x, lo, inner, hi, precision, ws, ws_bytes, out, st);
    case NT2G_SCAN_MAX: return launch_scan_op<NT2G_SCAN_MAX>(x, lo, inner, hi, precision, ws, ws_bytes, out, st);
    default: return launch_scan_op<NT2G_SCAN_MIN>(x, lo, inner, hi, precision, ws, ws_bytes, out, st);
    }
}

}  // namespace nt2g
