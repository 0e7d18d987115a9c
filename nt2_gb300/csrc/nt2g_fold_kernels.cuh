// nt2g_fold_kernels.cuh -- device side of the reductions along one dimension
// (sum, prod, max, min, mean, asum1, asum2, norm2, var, stdev, nbtrue,
// all/any/none, nansum, nanmean) of values viewed as [lo, inner, hi]
// (column-major), folding over `inner`: out[l + lo*h] = fold_k x(l + lo*(k + inner*h)).
//
// The element values come from a source type Src with
//   float  at(int64_t pos)   the element at linear position pos
//   float4 at4(int64_t pos)  the four elements pos .. pos+3 (pos a multiple of 4;
//                            only called when the source is 16-byte addressable)
// The library instantiates the bodies over a table (nt2g_fold.cu); the
// run-time compiler instantiates them over a compiled expression, so a fold of
// an expression (sum(exp(x)*y), sum(abs(x - y), 1), ...) evaluates every
// element in registers inside the fold: one pass, no temporary table.  This
// header is also compiled by NVRTC, so it includes nothing under
// __CUDACC_RTC__ (the run-time source puts nt2g_math.cuh and nt2g_accum.cuh
// ahead of it).
//
// NT2 reshapes every reduction this way before folding
// (core/reduction/include/nt2/dsl/functions/reduction/run.hpp:51-89): a fold
// over the first non-singleton dimension is an inner_fold over contiguous
// segments (lo = 1), a fold over a later dimension an outer_fold over strided
// ones (lo > 1).  The global forms (globalsum, globalmax, ...) fold the
// flattened table: lo = hi = 1.
//
// NT2 policy: one thread per output folds its elements in index order from
// the neutral element with NT2's unfused float operations, the order of NT2's
// per-segment fold (shared_memory/worker/inner_fold.hpp:47-80,
// worker/outer_fold.hpp, details/fold_step.hpp:31-43): bit-identical to NT2
// wherever NT2 spreads the outputs over threads.  mean = rec(float(n)) * sum
// (core/functions/expr/mean.hpp:22-33), asum1 = sum(abs), asum2 = sum(sqr_abs),
// norm2 = sqrt(asum2) (expr/asum1.hpp, expr/asum2.hpp, expr/norm2.hpp),
// var = f * asum2(a - mean(a)) with f = rec(n - 1) (rec(n) for var(a, 1); 1
// when n <= 1) and stdev = sqrt(var) (expr/var.hpp, expr/stdev.hpp): a mean
// pass, then the centred sum of squares.
//
// Fast policy: sums are compensated FP32 (TwoSum; squares carry their FMA
// product error) per chunk, chunks combined in FP64 in index order; var/stdev
// centre on the float mean and correct for its rounding error
// (sum (x - m)^2 - n (mu - m)^2, mu the FP64 mean); prod in FP64; max/min are
// exact.  Contiguous segments are cut into chunks, one warp per chunk with
// 128-bit loads; strided folds run one thread per output (four with 128-bit
// loads) over chunks of the fold range.  With more than one chunk per output,
// partials go to the caller's workspace and a second kernel combines them in
// order, so results are deterministic for a given shape.
#pragma once
#if !defined(__CUDACC_RTC__)
#include <stdint.h>
#include "nt2g_accum.cuh"
#define NT2G_FOLD_INF __builtin_huge_valf()
#else
#define NT2G_FOLD_INF __int_as_float(0x7f800000)
#endif

namespace nt2g {
namespace fold {

// fold operations (the values of nt2g_fold_op, repeated here because the
// run-time compiled source cannot include the C header)
enum : int {
    SUM = 0, PROD = 1, MAX = 2, MIN = 3, MEAN = 4, ASUM1 = 5, ASUM2 = 6, NORM2 = 7, VAR = 8, STDEV = 9,
    VAR1 = 10, STDEV1 = 11, NBTRUE = 12, ALL = 13, ANY = 14, NONE = 15, NANSUM = 16, NANMEAN = 17, MEANAD = 18,
    // internal: the mean of each output written with the rounding error of its
    // float value (the centre of a fast-policy variance); the count of non-NaN
    // elements (the divisor of nanmean)
    MEAN_C = 100, NOT_NAN = 101
};

constexpr int kThreads = 256;

__host__ __device__ constexpr bool is_var(int op) { return op == VAR || op == STDEV || op == VAR1 || op == STDEV1; }
// counts of elements: nbtrue and the logical folds all/any/none over x != 0
__host__ __device__ constexpr bool is_count(int op) { return op == NBTRUE || op == ALL || op == ANY || op == NONE; }
// folds of the deviations from each output's mean
__host__ __device__ constexpr bool is_centred(int op) { return is_var(op) || op == MEANAD; }
// folds that need a per-output value from a first pass (the centre, the count)
__host__ __device__ constexpr bool is_two_pass(int op) { return is_centred(op) || op == NANMEAN; }
__host__ __device__ constexpr bool is_sum(int op)
{
    return op == SUM || op == MEAN || op == ASUM1 || op == ASUM2 || op == NORM2 || op == MEAN_C || is_var(op) ||
           is_count(op) || op == NANSUM || op == NANMEAN || op == NOT_NAN || op == MEANAD;
}

// max/min in NT2's order: the fold keeps acc unless x is strictly better, so
// among equal values (== : +0 and -0 included) the LAST wins; the index
// reported is the FIRST element equal to the result (NT2's globalmax(a, i)
// = globalfind(a == max), common/globalmax.hpp:36-48).  NaN: the fast
// policy propagates it (the first NaN wins).
struct Best {
    float v;
    int64_t ilast, ifirst;
};
template <bool MX> __device__ __forceinline__ bool better(float a, float b) { return MX ? a > b : a < b; }
// Symmetric merge of two partial results (ilast < 0: empty).  Strictly
// better wins; among equal values the bits of the later element and the
// index of the earlier one; a NaN beats numbers, the earlier NaN another NaN.
template <bool MX> __device__ __forceinline__ Best best_merge(const Best &a, const Best &b)
{
    if (a.ilast < 0) return b;
    if (b.ilast < 0) return a;
    const bool an = a.v != a.v, bn = b.v != b.v;
    if (an || bn) {
        if (an && bn) return a.ifirst <= b.ifirst ? a : b;
        return an ? a : b;
    }
    if (better<MX>(a.v, b.v)) return a;
    if (better<MX>(b.v, a.v)) return b;
    Best r = a.ilast > b.ilast ? a : b;
    r.ifirst = a.ifirst < b.ifirst ? a.ifirst : b.ifirst;
    return r;
}

// Per-thread running max/min over elements visited in increasing position,
// positions relative to the thread's chunk start (32-bit), branch-free:
// x replaces v unless v is strictly better (NT2's rule), the first position
// of the current value and the first NaN are kept.  to_best() rebases.
template <bool MX, bool FIRST = true> struct Run {
    float v = MX ? -NT2G_FOLD_INF : NT2G_FOLD_INF;
    int32_t ifirst = -1, ilast = -1, inan = -1;
    __device__ __forceinline__ void add(float x, int32_t k)
    {
        const bool isn = x != x;
        const bool gt = MX ? x > v : x < v;
        const bool eq = x == v;
        inan = (isn && inan < 0) ? k : inan;
        if (FIRST) ifirst = (gt || (eq && ifirst < 0)) ? k : ifirst;  // only for a requested index
        ilast = (gt || eq) ? k : ilast;
        v = (gt || eq) ? x : v;
    }
    __device__ __forceinline__ Best to_best(int64_t base) const
    {
        if (inan >= 0) return Best{__int_as_float(0x7fffffff), base + inan, base + inan};
        if (ilast < 0) return Best{0.0f, -1, -1};
        return Best{v, base + ilast, base + ifirst};
    }
};

// per-op element contribution to a compensated sum
template <int OP> __device__ __forceinline__ void sum_elem(CSum &a, float x)
{
    if (OP == ASUM1) {
        csum_add(a, fabsf(x));
    } else if (OP == ASUM2 || OP == NORM2) {
        const float p = __fmul_rn(x, x);
        csum_add(a, p);
        a.c = __fadd_rn(a.c, __fmaf_rn(x, x, -p));  // exact product error
    } else if (is_count(OP)) {
        csum_add(a, x != 0.0f ? 1.0f : 0.0f);  // NaN counts: NT2's is_nez(NaN) is true
    } else if (OP == NOT_NAN) {
        csum_add(a, x == x ? 1.0f : 0.0f);
    } else if (OP == NANSUM || OP == NANMEAN) {
        csum_add(a, x == x ? x : 0.0f);
    } else {
        csum_add(a, x);
    }
}

// variance terms: (x - m)^2 with the difference kept exactly as dh + dl
// (TwoSum) and the square's rounding error carried, so the sum of squared
// deviations is compensated like the other sums.  Mean absolute deviation
// terms: |x - mu| with mu = m + md (the float mean and its rounding error),
// as |dh| plus the low part dl - md with the sign of dh (|lo| where dh is 0).
template <int OP> __device__ __forceinline__ void sum_elem_c(CSum &a, float x, float m, float md = 0.0f)
{
    if constexpr (OP == MEANAD) {
        const float dh = __fsub_rn(x, m);
        const float bb = __fsub_rn(dh, x);
        const float dl = __fadd_rn(__fsub_rn(x, __fsub_rn(dh, bb)), __fsub_rn(-m, bb));
        const float lo = __fsub_rn(dl, md);
        csum_add(a, fabsf(dh));
        a.c = __fadd_rn(a.c, dh > 0.0f ? lo : dh < 0.0f ? -lo : fabsf(lo));
    } else if constexpr (is_var(OP)) {
        const float dh = __fsub_rn(x, m);
        const float bb = __fsub_rn(dh, x);
        const float dl = __fadd_rn(__fsub_rn(x, __fsub_rn(dh, bb)), __fsub_rn(-m, bb));
        const float p = __fmul_rn(dh, dh);
        csum_add(a, p);
        a.c = __fadd_rn(a.c, __fmaf_rn(2.0f * dh, dl, __fmaf_rn(dh, dh, -p)));
    } else {
        sum_elem<OP>(a, x);
    }
}

// ---------------------------------------------------------------- partials --
// 32 bytes per (output, chunk): a double (sums, prod) or a Best.
struct Partial {
    double d;
    Best b;
};

// The FP64 value of a sum-type (or product) fold before it is rounded to the
// float output: mean = t/n, norm2 = sqrt(t), a count or a sum as is.
template <int OP> __device__ __forceinline__ double finish_double(double t, int64_t inner)
{
    if (OP == MEAN || OP == MEANAD) return t / (double)inner;
    if (OP == NORM2) return sqrt(t);
    return t;
}

// Writes output o of a sum-type (or product) fold from its FP64 total (and,
// when out64 is given, that total's FP64 result: the mean, the norm, the
// variance, ... before rounding to float).
// Variance: the sum of squares about the float centre m, corrected to the
// exact mean mu = m + delta (sum (x - m)^2 = sum (x - mu)^2 + n delta^2),
// divided by n - 1 (by n for VAR1/STDEV1; 1 when n <= 1).
template <int OP>
__device__ __forceinline__ void fold_put(float *out, double *out64, int64_t o, int64_t n_out, double t, int64_t inner,
                                         const float *cen)
{
    double r = 0.0;
    if constexpr (OP == MEAN_C) {
        const double mu = t / (double)inner;
        const float m = (float)mu;
        out[o] = m;
        out[n_out + o] = (float)(mu - (double)m);
        return;
    } else if constexpr (is_count(OP)) {
        const bool all = t == (double)inner, none = t == 0.0;
        r = OP == NBTRUE ? t : OP == ALL ? (all ? 1.0 : 0.0) : OP == ANY ? (none ? 0.0 : 1.0) : (none ? 1.0 : 0.0);
    } else if constexpr (OP == NANMEAN) {  // nansum / max(count, 1)
        const double c = (double)cen[o];
        r = t / (c > 1.0 ? c : 1.0);
    } else if constexpr (is_var(OP)) {
        const double d = (double)cen[n_out + o];
        const double n = (double)inner;
        double v = t - n * d * d;
        v = v > 0.0 ? v : 0.0;
        const bool by_n = OP == VAR1 || OP == STDEV1;
        if (inner > 1) v /= by_n ? n : n - 1.0;
        r = (OP == STDEV || OP == STDEV1) ? sqrt(v) : v;
    } else {
        r = finish_double<OP>(t, inner);
    }
    out[o] = (float)r;
    if (out64) out64[o] = r;
}

// ------------------------------------------- warp-shuffle merges (fast) --
__device__ __forceinline__ double warp_prod(double a)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) a *= __shfl_down_sync(0xffffffffu, a, off);
    return a;
}
template <bool MX> __device__ __forceinline__ Best warp_best(Best a)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        Best b{__shfl_down_sync(0xffffffffu, a.v, off), __shfl_down_sync(0xffffffffu, a.ilast, off),
               __shfl_down_sync(0xffffffffu, a.ifirst, off)};
        a = best_merge<MX>(a, b);  // symmetric: lanes hold interleaved elements
    }
    return a;
}

// ----------------------------------------- contiguous segments (lo == 1) --
// One warp per (segment, chunk) work item.  FINAL: one chunk per segment, the
// warp writes the output directly.  vec: segment starts and chunk bounds are
// multiples of 4 and the source is 16-byte addressable.
template <class Src, int OP, bool FINAL, bool IDX>
__device__ __forceinline__ void inner_body(const Src &src, int64_t inner, int64_t hi, int64_t chunk, int64_t q,
                                           int vec, Partial *__restrict__ part, float *__restrict__ out,
                                           int64_t *__restrict__ index, const float *__restrict__ cen,
                                           double *__restrict__ out64)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t item = warp; item < hi * q; item += nwarps) {
        const int64_t seg = item / q, c = item - seg * q;
        const int64_t k0 = c * chunk, k1 = (k0 + chunk < inner) ? k0 + chunk : inner;
        const int64_t base = seg * inner;
        CSum acc{0.0f, 0.0f};
        double prod = 1.0;
        const float m = is_centred(OP) ? cen[seg] : 0.0f;
        const float md = OP == MEANAD ? cen[hi + seg] : 0.0f;
        Run<OP == MAX, IDX> run[4];  // one per float4 component: four independent chains
        auto take = [&](int cc, float v, int32_t k) {  // k: position relative to k0
            if (is_sum(OP)) sum_elem_c<OP>(acc, v, m, md);
            else if (OP == PROD) prod *= (double)v;
            else run[cc].add(v, k);
        };
        int64_t k = k0;
        if (vec) {
            const int64_t v1 = k1 >> 2;
#pragma unroll 8
            for (int64_t j = (k0 >> 2) + lane; j < v1; j += 32) {
                const float4 f = src.at4(base + 4 * j);
                const int32_t r0 = (int32_t)(4 * j - k0);
                take(0, f.x, r0); take(1, f.y, r0 + 1); take(2, f.z, r0 + 2); take(3, f.w, r0 + 3);
            }
            k = v1 << 2;
        }
        for (int64_t j = k + lane; j < k1; j += 32) take(0, src.at(base + j), (int32_t)(j - k0));
        Partial r;
        if (is_sum(OP)) {
            acc = warp_csum(acc);
            r.d = (double)acc.s + (double)acc.c;
        } else if (OP == PROD) {
            r.d = warp_prod(prod);
        } else {
            constexpr bool MX = OP == MAX;
            Best b = best_merge<MX>(best_merge<MX>(run[0].to_best(k0), run[1].to_best(k0)),
                                    best_merge<MX>(run[2].to_best(k0), run[3].to_best(k0)));
            r.b = warp_best<MX>(b);
        }
        if (lane == 0) {
            if (FINAL) {
                if (is_sum(OP) || OP == PROD) fold_put<OP>(out, out64, seg, hi, r.d, inner, cen);
                else { out[seg] = r.b.v; if (index) index[seg] = r.b.ifirst; }
            } else {
                part[item] = r;
            }
        }
    }
}

// Short contiguous segments: one thread per segment, in order.
template <class Src, int OP>
__device__ __forceinline__ void short_body(const Src &src, int64_t inner, int64_t hi, float *__restrict__ out,
                                           int64_t *__restrict__ index, const float *__restrict__ cen,
                                           double *__restrict__ out64)
{
    for (int64_t seg = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; seg < hi;
         seg += (int64_t)gridDim.x * blockDim.x) {
        const int64_t base = seg * inner;
        CSum acc{0.0f, 0.0f};
        double prod = 1.0;
        Run<OP == MAX> run;
        const float m = is_centred(OP) ? cen[seg] : 0.0f;
        const float md = OP == MEANAD ? cen[hi + seg] : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = src.at(base + k);
            if (is_sum(OP)) sum_elem_c<OP>(acc, v, m, md);
            else if (OP == PROD) prod *= (double)v;
            else run.add(v, (int32_t)k);
        }
        if (is_sum(OP)) fold_put<OP>(out, out64, seg, hi, (double)acc.s + (double)acc.c, inner, cen);
        else if (OP == PROD) { out[seg] = (float)prod; if (out64) out64[seg] = prod; }
        else {
            const Best b = run.to_best(0);
            out[seg] = b.v;
            if (index) index[seg] = b.ifirst;
        }
    }
}

// ---------------------------------------------- strided folds (lo > 1) --
// Thread per output (VEC: four consecutive outputs via float4), over the
// chunk [c*ck, min((c+1)*ck, inner)) of the fold range; grid.y = chunk.
template <class Src, int OP, int VEC, bool FINAL>
__device__ __forceinline__ void outer_body(const Src &src, int64_t lo, int64_t inner, int64_t hi, int64_t ck,
                                           int64_t q, Partial *__restrict__ part, float *__restrict__ out,
                                           int64_t *__restrict__ index, const float *__restrict__ cen,
                                           double *__restrict__ out64)
{
    const int64_t lv = lo / VEC;  // thread columns per h
    const int64_t c = blockIdx.y;
    const int64_t k0 = c * ck, k1 = (k0 + ck < inner) ? k0 + ck : inner;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < lv * hi; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = t / lv, l = (t - h * lv) * VEC;
        const int64_t base = l + lo * inner * h;
        CSum acc[VEC];
        double prod[VEC];
        Run<OP == MAX> run[VEC];
        float m[VEC], md[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            acc[v] = CSum{0.0f, 0.0f};
            prod[v] = 1.0;
            m[v] = is_centred(OP) ? cen[l + v + lo * h] : 0.0f;
            md[v] = OP == MEANAD ? cen[lo * hi + l + v + lo * h] : 0.0f;
        }
        for (int64_t k = k0; k < k1; ++k) {
            float e[VEC];
            if constexpr (VEC == 4) {
                const float4 f = src.at4(base + lo * k);
                e[0] = f.x; e[1] = f.y; e[2] = f.z; e[3] = f.w;
            } else {
                e[0] = src.at(base + lo * k);
            }
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                if (is_sum(OP)) sum_elem_c<OP>(acc[v], e[v], m[v], md[v]);
                else if (OP == PROD) prod[v] *= (double)e[v];
                else run[v].add(e[v], (int32_t)(k - k0));
            }
        }
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const int64_t o = l + v + lo * h;
            Partial r;
            if (is_sum(OP)) r.d = (double)acc[v].s + (double)acc[v].c;
            else if (OP == PROD) r.d = prod[v];
            else r.b = run[v].to_best(k0);
            if (FINAL) {
                if (is_sum(OP)) fold_put<OP>(out, out64, o, lo * hi, r.d, inner, cen);
                else if (OP == PROD) { out[o] = (float)r.d; if (out64) out64[o] = r.d; }
                else { out[o] = r.b.v; if (index) index[o] = r.b.ifirst; }
            } else {
                part[o * q + c] = r;
            }
        }
    }
}

// ------------------------------------------------ NT2 policy: in order --
template <class Src, int OP>
__device__ __forceinline__ void nt2_body(const Src &src, int64_t lo, int64_t inner, int64_t hi,
                                         float *__restrict__ out, int64_t *__restrict__ index,
                                         const float *__restrict__ cen)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < lo * hi; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = o / lo, l = o - h * lo;
        const int64_t base = l + lo * inner * h;
        float acc = OP == PROD ? 1.0f
                  : OP == MAX  ? -__int_as_float(0x7f800000)
                  : OP == MIN  ? __int_as_float(0x7f800000)
                               : 0.0f;
        const float m = is_two_pass(OP) ? cen[o] : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = src.at(base + lo * k);
            if constexpr (is_var(OP)) {  // asum2(center(a)): (x - mean(a))^2 in order
                const float d = __fsub_rn(v, m);
                acc = __fadd_rn(acc, __fmul_rn(d, d));
                continue;
            }
            if constexpr (OP == MEANAD) {  // sum(abs(center(a))) in order
                acc = __fadd_rn(acc, fabsf(__fsub_rn(v, m)));
                continue;
            }
            if constexpr (is_count(OP)) {  // nbtrue: the sum of is_nez(x)
                acc = __fadd_rn(acc, v != 0.0f ? 1.0f : 0.0f);
                continue;
            }
            if constexpr (OP == NOT_NAN) {
                acc = __fadd_rn(acc, v == v ? 1.0f : 0.0f);
                continue;
            }
            if constexpr (OP == NANSUM || OP == NANMEAN) {  // sum(if_zero_else(is_nan(x), x))
                acc = __fadd_rn(acc, v == v ? v : 0.0f);
                continue;
            }
            switch (OP) {
            case PROD: acc = __fmul_rn(acc, v); break;
            case MAX: acc = (acc > v) ? acc : v; break;
            case MIN: acc = (acc < v) ? acc : v; break;
            case ASUM1: acc = __fadd_rn(acc, fabsf(v)); break;
            case ASUM2: case NORM2: acc = __fadd_rn(acc, __fmul_rn(v, v)); break;
            default: acc = __fadd_rn(acc, v); break;
            }
        }
        if (OP == MEAN || OP == MEANAD) acc = __fmul_rn(__fdiv_rn(1.0f, (float)inner), acc);  // mean: rec(n) * sum
        if (OP == NORM2) acc = __fsqrt_rn(acc);
        if constexpr (is_count(OP)) {
            const float n = (float)inner;
            acc = OP == NBTRUE ? acc
                : OP == ALL    ? (acc == n ? 1.0f : 0.0f)
                : OP == ANY    ? (acc != 0.0f ? 1.0f : 0.0f)
                               : (acc == 0.0f ? 1.0f : 0.0f);
        }
        if constexpr (OP == NANMEAN)  // rec(max(nbtrue(is_not_nan(a)), 1)) * nansum(a)
            acc = __fmul_rn(__fdiv_rn(1.0f, m > 1.0f ? m : 1.0f), acc);
        if constexpr (is_var(OP)) {  // var = f * asum2, f = n <= 1 ? 1 : rec(n - 1) (rec(n) for w = 1)
            const float n = (float)inner;
            const bool by_n = OP == VAR1 || OP == STDEV1;
            const float f = (n <= 1.0f) ? 1.0f : __fdiv_rn(1.0f, by_n ? n : __fsub_rn(n, 1.0f));
            acc = __fmul_rn(f, acc);
            if (OP == STDEV || OP == STDEV1) acc = __fsqrt_rn(acc);
        }
        out[o] = acc;
        if ((OP == MAX || OP == MIN) && index) {
            int64_t f = -1;
            for (int64_t k = 0; k < inner && f < 0; ++k)
                if (src.at(base + lo * k) == acc) f = k;
            index[o] = f;
        }
    }
}

}  // namespace fold
}  // namespace nt2g
