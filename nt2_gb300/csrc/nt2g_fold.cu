// nt2g_fold.cu -- reductions along one dimension: sum, prod, max, min, mean,
// asum1, asum2, norm2, var, stdev of a table viewed as [lo, inner, hi] (column-major),
// folding over `inner`.  out[l + lo*h] = fold_k x[l + lo*(k + inner*h)].
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
// (sum (x - m)^2 - n (mu - m)^2, mu the FP64 mean); prod in
// FP64; max/min are exact.  Contiguous segments are cut into chunks, one warp
// per chunk with 128-bit loads; strided folds run one thread per output (four
// with 128-bit loads) over chunks of the fold range.  With more than one
// chunk per output, partials go to the caller's workspace and a second kernel
// combines them in order, so results are deterministic for a given shape.
#include "nt2g_accum.cuh"
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

constexpr int kFoldThreads = 256;
constexpr int64_t kChunk = 16384;        // elements per warp work item (contiguous folds)
constexpr int64_t kSmallSeg = 64;        // segments up to this length: one thread each
constexpr int64_t kTargetThreads = 152 * 1024;

// Internal: the mean of each output written with the rounding error of its
// float value (the centre of a fast-policy variance); the count of non-NaN
// elements (the divisor of nanmean).
constexpr int kFoldMeanC = 100;
constexpr int kFoldNotNan = 101;

__host__ __device__ constexpr bool fold_is_var(int op)
{
    return op == NT2G_FOLD_VAR || op == NT2G_FOLD_STDEV || op == NT2G_FOLD_VAR1 || op == NT2G_FOLD_STDEV1;
}
// counts of elements: nbtrue and the logical folds all/any/none over x != 0
__host__ __device__ constexpr bool fold_is_count(int op)
{
    return op == NT2G_FOLD_NBTRUE || op == NT2G_FOLD_ALL || op == NT2G_FOLD_ANY || op == NT2G_FOLD_NONE;
}
// folds that need a per-output value from a first pass (the centre, the count)
__host__ __device__ constexpr bool fold_is_two_pass(int op) { return fold_is_var(op) || op == NT2G_FOLD_NANMEAN; }
__host__ __device__ constexpr bool fold_is_sum(int op)
{
    return op == NT2G_FOLD_SUM || op == NT2G_FOLD_MEAN || op == NT2G_FOLD_ASUM1 || op == NT2G_FOLD_ASUM2 ||
           op == NT2G_FOLD_NORM2 || op == kFoldMeanC || fold_is_var(op) || fold_is_count(op) ||
           op == NT2G_FOLD_NANSUM || op == NT2G_FOLD_NANMEAN || op == kFoldNotNan;
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
template <bool MAX> __device__ __forceinline__ bool better(float a, float b) { return MAX ? a > b : a < b; }
// Symmetric merge of two partial results (ilast < 0: empty).  Strictly
// better wins; among equal values the bits of the later element and the
// index of the earlier one; a NaN beats numbers, the earlier NaN another NaN.
template <bool MAX> __device__ __forceinline__ Best best_merge(const Best &a, const Best &b)
{
    if (a.ilast < 0) return b;
    if (b.ilast < 0) return a;
    const bool an = a.v != a.v, bn = b.v != b.v;
    if (an || bn) {
        if (an && bn) return a.ifirst <= b.ifirst ? a : b;
        return an ? a : b;
    }
    if (better<MAX>(a.v, b.v)) return a;
    if (better<MAX>(b.v, a.v)) return b;
    Best r = a.ilast > b.ilast ? a : b;
    r.ifirst = a.ifirst < b.ifirst ? a.ifirst : b.ifirst;
    return r;
}

// Per-thread running max/min over elements visited in increasing position,
// positions relative to the thread's chunk start (32-bit), branch-free:
// x replaces v unless v is strictly better (NT2's rule), the first position
// of the current value and the first NaN are kept.  to_best() rebases.
template <bool MAX, bool FIRST = true> struct Run {
    float v = MAX ? -INFINITY : INFINITY;
    int32_t ifirst = -1, ilast = -1, inan = -1;
    __device__ __forceinline__ void add(float x, int32_t k)
    {
        const bool isn = x != x;
        const bool gt = MAX ? x > v : x < v;
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
    if (OP == NT2G_FOLD_ASUM1) {
        csum_add(a, fabsf(x));
    } else if (OP == NT2G_FOLD_ASUM2 || OP == NT2G_FOLD_NORM2) {
        const float p = __fmul_rn(x, x);
        csum_add(a, p);
        a.c = __fadd_rn(a.c, __fmaf_rn(x, x, -p));  // exact product error
    } else if (fold_is_count(OP)) {
        csum_add(a, x != 0.0f ? 1.0f : 0.0f);  // NaN counts: NT2's is_nez(NaN) is true
    } else if (OP == kFoldNotNan) {
        csum_add(a, x == x ? 1.0f : 0.0f);
    } else if (OP == NT2G_FOLD_NANSUM || OP == NT2G_FOLD_NANMEAN) {
        csum_add(a, x == x ? x : 0.0f);
    } else {
        csum_add(a, x);
    }
}

// variance terms: (x - m)^2 with the difference kept exactly as dh + dl
// (TwoSum) and the square's rounding error carried, so the sum of squared
// deviations is compensated like the other sums
template <int OP> __device__ __forceinline__ void sum_elem_c(CSum &a, float x, float m)
{
    if constexpr (fold_is_var(OP)) {
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

template <int OP> __device__ __forceinline__ float finish_double(double t, int64_t inner)
{
    if (OP == NT2G_FOLD_MEAN) return (float)(t / (double)inner);
    if (OP == NT2G_FOLD_NORM2) return (float)sqrt(t);
    return (float)t;
}

// Writes output o of a sum-type (or product) fold from its FP64 total.
// Variance: the sum of squares about the float centre m, corrected to the
// exact mean mu = m + delta (sum (x - m)^2 = sum (x - mu)^2 + n delta^2),
// divided by n - 1 (by n for VAR1/STDEV1; 1 when n <= 1).
template <int OP>
__device__ __forceinline__ void fold_put(float *out, int64_t o, int64_t n_out, double t, int64_t inner, const float *cen)
{
    if constexpr (OP == kFoldMeanC) {
        const double mu = t / (double)inner;
        const float m = (float)mu;
        out[o] = m;
        out[n_out + o] = (float)(mu - (double)m);
    } else if constexpr (fold_is_count(OP)) {
        const bool all = t == (double)inner, none = t == 0.0;
        out[o] = OP == NT2G_FOLD_NBTRUE ? (float)t
               : OP == NT2G_FOLD_ALL    ? (all ? 1.0f : 0.0f)
               : OP == NT2G_FOLD_ANY    ? (none ? 0.0f : 1.0f)
                                        : (none ? 1.0f : 0.0f);
    } else if constexpr (OP == NT2G_FOLD_NANMEAN) {  // nansum / max(count, 1)
        const double c = (double)cen[o];
        out[o] = (float)(t / (c > 1.0 ? c : 1.0));
    } else if constexpr (fold_is_var(OP)) {
        const double d = (double)cen[n_out + o];
        const double n = (double)inner;
        double v = t - n * d * d;
        v = v > 0.0 ? v : 0.0;
        const bool by_n = OP == NT2G_FOLD_VAR1 || OP == NT2G_FOLD_STDEV1;
        if (inner > 1) v /= by_n ? n : n - 1.0;
        out[o] = (OP == NT2G_FOLD_STDEV || OP == NT2G_FOLD_STDEV1) ? (float)sqrt(v) : (float)v;
    } else {
        out[o] = finish_double<OP>(t, inner);
    }
}

// ------------------------------------------- warp-shuffle merges (fast) --
__device__ __forceinline__ double warp_prod(double a)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) a *= __shfl_down_sync(0xffffffffu, a, off);
    return a;
}
template <bool MAX> __device__ __forceinline__ Best warp_best(Best a)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        Best b{__shfl_down_sync(0xffffffffu, a.v, off), __shfl_down_sync(0xffffffffu, a.ilast, off),
               __shfl_down_sync(0xffffffffu, a.ifirst, off)};
        a = best_merge<MAX>(a, b);  // symmetric: lanes hold interleaved elements
    }
    return a;
}

// ----------------------------------------- contiguous segments (lo == 1) --
// One warp per (segment, chunk) work item.  FINAL: one chunk per segment, the
// warp writes the output directly.
template <int OP, bool FINAL, bool IDX>
__global__ void __launch_bounds__(kFoldThreads) k_fold_inner(const float *__restrict__ x, int64_t inner, int64_t hi,
                                                             int64_t chunk, int64_t q, int vec,
                                                             Partial *__restrict__ part, float *__restrict__ out,
                                                             int64_t *__restrict__ index, const float *__restrict__ cen)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t item = warp; item < hi * q; item += nwarps) {
        const int64_t seg = item / q, c = item - seg * q;
        const int64_t k0 = c * chunk, k1 = (k0 + chunk < inner) ? k0 + chunk : inner;
        const float *p = x + seg * inner;
        CSum acc{0.0f, 0.0f};
        double prod = 1.0;
        const float m = fold_is_var(OP) ? cen[seg] : 0.0f;
        Run<OP == NT2G_FOLD_MAX, IDX> run[4];  // one per float4 component: four independent chains
        auto take = [&](int c, float v, int32_t k) {  // k: position relative to k0
            if (fold_is_sum(OP)) sum_elem_c<OP>(acc, v, m);
            else if (OP == NT2G_FOLD_PROD) prod *= (double)v;
            else run[c].add(v, k);
        };
        int64_t k = k0;
        if (vec) {  // segment starts and chunk bounds are 16-byte aligned: float4 per lane
            const int64_t v1 = k1 >> 2;
#pragma unroll 8
            for (int64_t j = (k0 >> 2) + lane; j < v1; j += 32) {
                const float4 f = ld_stream((const float4 *)p + j);
                const int32_t r0 = (int32_t)(4 * j - k0);
                take(0, f.x, r0); take(1, f.y, r0 + 1); take(2, f.z, r0 + 2); take(3, f.w, r0 + 3);
            }
            k = v1 << 2;
        }
        for (int64_t j = k + lane; j < k1; j += 32) take(0, ld_stream(p + j), (int32_t)(j - k0));
        Partial r;
        if (fold_is_sum(OP)) {
            acc = warp_csum(acc);
            r.d = (double)acc.s + (double)acc.c;
        } else if (OP == NT2G_FOLD_PROD) {
            r.d = warp_prod(prod);
        } else {
            constexpr bool MX = OP == NT2G_FOLD_MAX;
            Best b = best_merge<MX>(best_merge<MX>(run[0].to_best(k0), run[1].to_best(k0)),
                                    best_merge<MX>(run[2].to_best(k0), run[3].to_best(k0)));
            r.b = warp_best<MX>(b);
        }
        if (lane == 0) {
            if (FINAL) {
                if (fold_is_sum(OP) || OP == NT2G_FOLD_PROD) fold_put<OP>(out, seg, hi, r.d, inner, cen);
                else { out[seg] = r.b.v; if (index) index[seg] = r.b.ifirst; }
            } else {
                part[item] = r;
            }
        }
    }
}

// Short contiguous segments: one thread per segment, in order.
template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_short(const float *__restrict__ x, int64_t inner, int64_t hi,
                                                             float *__restrict__ out, int64_t *__restrict__ index,
                                                             const float *__restrict__ cen)
{
    for (int64_t seg = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; seg < hi;
         seg += (int64_t)gridDim.x * blockDim.x) {
        const float *p = x + seg * inner;
        CSum acc{0.0f, 0.0f};
        double prod = 1.0;
        Run<OP == NT2G_FOLD_MAX> run;
        const float m = fold_is_var(OP) ? cen[seg] : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = p[k];
            if (fold_is_sum(OP)) sum_elem_c<OP>(acc, v, m);
            else if (OP == NT2G_FOLD_PROD) prod *= (double)v;
            else run.add(v, (int32_t)k);
        }
        if (fold_is_sum(OP)) fold_put<OP>(out, seg, hi, (double)acc.s + (double)acc.c, inner, cen);
        else if (OP == NT2G_FOLD_PROD) out[seg] = (float)prod;
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
template <int OP, int VEC, bool FINAL>
__global__ void __launch_bounds__(kFoldThreads) k_fold_outer(const float *__restrict__ x, int64_t lo, int64_t inner,
                                                             int64_t hi, int64_t ck, int64_t q,
                                                             Partial *__restrict__ part, float *__restrict__ out,
                                                             int64_t *__restrict__ index, const float *__restrict__ cen)
{
    const int64_t lv = lo / VEC;  // thread columns per h
    const int64_t c = blockIdx.y;
    const int64_t k0 = c * ck, k1 = (k0 + ck < inner) ? k0 + ck : inner;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < lv * hi; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = t / lv, l = (t - h * lv) * VEC;
        const float *p = x + l + lo * inner * h;
        CSum acc[VEC];
        double prod[VEC];
        Run<OP == NT2G_FOLD_MAX> run[VEC];
        float m[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            acc[v] = CSum{0.0f, 0.0f};
            prod[v] = 1.0;
            m[v] = fold_is_var(OP) ? cen[l + v + lo * h] : 0.0f;
        }
        for (int64_t k = k0; k < k1; ++k) {
            float e[VEC];
            if constexpr (VEC == 4) {
                const float4 f = ld_stream((const float4 *)(p + lo * k));
                e[0] = f.x; e[1] = f.y; e[2] = f.z; e[3] = f.w;
            } else {
                e[0] = ld_stream(p + lo * k);
            }
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                if (fold_is_sum(OP)) sum_elem_c<OP>(acc[v], e[v], m[v]);
                else if (OP == NT2G_FOLD_PROD) prod[v] *= (double)e[v];
                else run[v].add(e[v], (int32_t)(k - k0));
            }
        }
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const int64_t o = l + v + lo * h;
            Partial r;
            if (fold_is_sum(OP)) r.d = (double)acc[v].s + (double)acc[v].c;
            else if (OP == NT2G_FOLD_PROD) r.d = prod[v];
            else r.b = run[v].to_best(k0);
            if (FINAL) {
                if (fold_is_sum(OP) || OP == NT2G_FOLD_PROD) fold_put<OP>(out, o, lo * hi, r.d, inner, cen);
                else { out[o] = r.b.v; if (index) index[o] = r.b.ifirst; }
            } else {
                part[o * q + c] = r;
            }
        }
    }
}

// Combine the q partials of each output in order.
template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_finish(const Partial *__restrict__ part, int64_t n_out,
                                                              int64_t q, int64_t inner, float *__restrict__ out,
                                                              int64_t *__restrict__ index, const float *__restrict__ cen)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += (int64_t)gridDim.x * blockDim.x) {
        const Partial *p = part + o * q;
        if (fold_is_sum(OP) || OP == NT2G_FOLD_PROD) {
            double t = OP == NT2G_FOLD_PROD ? 1.0 : 0.0;
            for (int64_t c = 0; c < q; ++c) t = OP == NT2G_FOLD_PROD ? t * p[c].d : t + p[c].d;
            fold_put<OP>(out, o, n_out, t, inner, cen);
        } else {
            Best b{0.0f, -1, -1};
            for (int64_t c = 0; c < q; ++c)
                if (p[c].b.ilast >= 0) b = b.ilast < 0 ? p[c].b : best_merge<OP == NT2G_FOLD_MAX>(b, p[c].b);
            out[o] = b.v;
            if (index) index[o] = b.ifirst;
        }
    }
}

// Many partials per output (global folds): one block per output, thread t
// combining partials t, t+T, t+2T, ... in that order, then a fixed
// shared-memory tree over the threads' results.  Deterministic for a given q.
template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_finish_block(const Partial *__restrict__ part, int64_t n_out,
                                                                    int64_t q, int64_t inner, float *__restrict__ out,
                                                                    int64_t *__restrict__ index, const float *__restrict__ cen)
{
    constexpr bool DBL = fold_is_sum(OP) || OP == NT2G_FOLD_PROD;
    __shared__ double sd[kFoldThreads];
    __shared__ Best sb[kFoldThreads];
    for (int64_t o = blockIdx.x; o < n_out; o += gridDim.x) {
        const Partial *p = part + o * q;
        if (DBL) {
            double t = OP == NT2G_FOLD_PROD ? 1.0 : 0.0;
#pragma unroll 4
            for (int64_t c = threadIdx.x; c < q; c += blockDim.x) t = OP == NT2G_FOLD_PROD ? t * p[c].d : t + p[c].d;
            sd[threadIdx.x] = t;
        } else {
            Best b{0.0f, -1, -1};
#pragma unroll 4
            for (int64_t c = threadIdx.x; c < q; c += blockDim.x) b = best_merge<OP == NT2G_FOLD_MAX>(b, p[c].b);
            sb[threadIdx.x] = b;
        }
        __syncthreads();
        for (int w = kFoldThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                if (DBL) sd[threadIdx.x] = OP == NT2G_FOLD_PROD ? sd[threadIdx.x] * sd[threadIdx.x + w]
                                                                : sd[threadIdx.x] + sd[threadIdx.x + w];
                else sb[threadIdx.x] = best_merge<OP == NT2G_FOLD_MAX>(sb[threadIdx.x], sb[threadIdx.x + w]);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (DBL) {
                fold_put<OP>(out, o, n_out, sd[0], inner, cen);
            } else {
                out[o] = sb[0].v;
                if (index) index[o] = sb[0].ifirst;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------ NT2 policy: in order --
template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_nt2(const float *__restrict__ x, int64_t lo, int64_t inner,
                                                           int64_t hi, float *__restrict__ out,
                                                           int64_t *__restrict__ index, const float *__restrict__ cen)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < lo * hi; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = o / lo, l = o - h * lo;
        const float *p = x + l + lo * inner * h;
        float acc = OP == NT2G_FOLD_PROD ? 1.0f
                  : OP == NT2G_FOLD_MAX  ? -__int_as_float(0x7f800000)
                  : OP == NT2G_FOLD_MIN  ? __int_as_float(0x7f800000)
                                         : 0.0f;
        const float m = fold_is_two_pass(OP) ? cen[o] : 0.0f;
        for (int64_t k = 0; k < inner; ++k) {
            const float v = p[lo * k];
            if constexpr (fold_is_var(OP)) {  // asum2(center(a)): (x - mean(a))^2 in order
                const float d = __fsub_rn(v, m);
                acc = __fadd_rn(acc, __fmul_rn(d, d));
                continue;
            }
            if constexpr (fold_is_count(OP)) {  // nbtrue: the sum of is_nez(x)
                acc = __fadd_rn(acc, v != 0.0f ? 1.0f : 0.0f);
                continue;
            }
            if constexpr (OP == kFoldNotNan) {
                acc = __fadd_rn(acc, v == v ? 1.0f : 0.0f);
                continue;
            }
            if constexpr (OP == NT2G_FOLD_NANSUM || OP == NT2G_FOLD_NANMEAN) {  // sum(if_zero_else(is_nan(x), x))
                acc = __fadd_rn(acc, v == v ? v : 0.0f);
                continue;
            }
            switch (OP) {
            case NT2G_FOLD_PROD: acc = __fmul_rn(acc, v); break;
            case NT2G_FOLD_MAX: acc = (acc > v) ? acc : v; break;
            case NT2G_FOLD_MIN: acc = (acc < v) ? acc : v; break;
            case NT2G_FOLD_ASUM1: acc = __fadd_rn(acc, fabsf(v)); break;
            case NT2G_FOLD_ASUM2: case NT2G_FOLD_NORM2: acc = __fadd_rn(acc, __fmul_rn(v, v)); break;
            default: acc = __fadd_rn(acc, v); break;
            }
        }
        if (OP == NT2G_FOLD_MEAN) acc = __fmul_rn(__fdiv_rn(1.0f, (float)inner), acc);
        if (OP == NT2G_FOLD_NORM2) acc = __fsqrt_rn(acc);
        if constexpr (fold_is_count(OP)) {
            const float n = (float)inner;
            acc = OP == NT2G_FOLD_NBTRUE ? acc
                : OP == NT2G_FOLD_ALL    ? (acc == n ? 1.0f : 0.0f)
                : OP == NT2G_FOLD_ANY    ? (acc != 0.0f ? 1.0f : 0.0f)
                                         : (acc == 0.0f ? 1.0f : 0.0f);
        }
        if constexpr (OP == NT2G_FOLD_NANMEAN)  // rec(max(nbtrue(is_not_nan(a)), 1)) * nansum(a)
            acc = __fmul_rn(__fdiv_rn(1.0f, m > 1.0f ? m : 1.0f), acc);
        if constexpr (fold_is_var(OP)) {  // var = f * asum2, f = n <= 1 ? 1 : rec(n - 1) (rec(n) for w = 1)
            const float n = (float)inner;
            const bool by_n = OP == NT2G_FOLD_VAR1 || OP == NT2G_FOLD_STDEV1;
            const float f = (n <= 1.0f) ? 1.0f : __fdiv_rn(1.0f, by_n ? n : __fsub_rn(n, 1.0f));
            acc = __fmul_rn(f, acc);
            if (OP == NT2G_FOLD_STDEV || OP == NT2G_FOLD_STDEV1) acc = __fsqrt_rn(acc);
        }
        out[o] = acc;
        if ((OP == NT2G_FOLD_MAX || OP == NT2G_FOLD_MIN) && index) {
            int64_t f = -1;
            for (int64_t k = 0; k < inner && f < 0; ++k)
                if (p[lo * k] == acc) f = k;
            index[o] = f;
        }
    }
}

// --------------------------------------------------------------- plans --
struct FoldPlan {
    int kind = 0;       // 0 short segments, 1 warp chunks (lo == 1), 2 strided
    int64_t chunk = 0;  // elements per chunk along the fold
    int64_t q = 1;      // chunks per output
    int vec = 0;
};

static FoldPlan plan_fold(int64_t lo, int64_t inner, int64_t hi, bool aligned)
{
    FoldPlan p;
    if (lo == 1) {
        if (inner <= kSmallSeg && hi >= 1024) { p.kind = 0; return p; }
        p.kind = 1;
        p.vec = aligned && (inner % 4 == 0);
        // enough warp items to fill the GPU: 8 warps per SM at least 4 times over
        const int64_t want = 152 * 8 * 4;
        int64_t chunk = kChunk;
        if (hi * ((inner + chunk - 1) / chunk) < want) {
            int64_t per = (want + hi - 1) / hi;
            chunk = (inner + per - 1) / per;
            if (chunk < 1024) chunk = 1024;
        }
        chunk = (chunk + 127) / 128 * 128;
        p.chunk = chunk;
        p.q = (inner + chunk - 1) / chunk;
        return p;
    }
    p.kind = 2;
    p.vec = aligned && (lo % 4 == 0) ? 4 : 1;
    const int64_t threads = lo * hi / p.vec;
    int64_t q = 1;
    if (threads < kTargetThreads) {
        q = (kTargetThreads + threads - 1) / threads;
        const int64_t qmax = inner / 16 > 0 ? inner / 16 : 1;
        if (q > qmax) q = qmax;
        if (q > 65535) q = 65535;  // grid.y
    }
    if ((inner + q - 1) / q > (1 << 30)) q = (inner + (1 << 30) - 1) >> 30;  // 32-bit positions in a chunk
    p.chunk = (inner + q - 1) / q;
    p.q = (inner + p.chunk - 1) / p.chunk;
    return p;
}

// Workspace: the partials of the chunked plans, then (for var/stdev) each
// output's centre and its rounding error, 16-byte aligned.
static size_t fold_partial_bytes(int64_t lo, int64_t inner, int64_t hi)
{
    FoldPlan p = plan_fold(lo, inner, hi, true);
    FoldPlan u = plan_fold(lo, inner, hi, false);
    int64_t q = p.q > u.q ? p.q : u.q;
    return q > 1 ? (size_t)(lo * hi) * (size_t)q * sizeof(Partial) : 0;
}
static size_t fold_centre_offset(int64_t lo, int64_t inner, int64_t hi)
{
    return (fold_partial_bytes(lo, inner, hi) + 15) / 16 * 16;
}

nt2g_status fold_partials_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    *bytes = fold_partial_bytes(lo, inner, hi);
    return NT2G_OK;
}

nt2g_status fold_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    *bytes = fold_centre_offset(lo, inner, hi) + (size_t)(lo * hi) * 2 * sizeof(float);
    return NT2G_OK;
}

template <int OP>
static nt2g_status launch_fold_op(const float *x, int64_t lo, int64_t inner, int64_t hi, int precision, void *ws,
                                  size_t ws_bytes, float *out, int64_t *index, cudaStream_t st,
                                  const float *cen = nullptr)
{
    const int64_t n_out = lo * hi;
    if constexpr (fold_is_two_pass(OP)) {
        if (!cen) {  // first the centre of every output: NT2's float mean, or (fast) the mean and its rounding
                     // error; for nanmean the count of non-NaN elements
            const size_t off = fold_centre_offset(lo, inner, hi);
            if (!ws || off + (size_t)n_out * 2 * sizeof(float) > ws_bytes) {
                set_error("nt2g_fold_f32: workspace of %zu bytes, %zu needed", ws_bytes,
                          off + (size_t)n_out * 2 * sizeof(float));
                return NT2G_ERR_INVALID;
            }
            float *c = (float *)((char *)ws + off);
            nt2g_status s;
            if constexpr (OP == NT2G_FOLD_NANMEAN)
                s = launch_fold_op<kFoldNotNan>(x, lo, inner, hi, precision, ws, off, c, nullptr, st);
            else if (precision == NT2G_PREC_NT2 || inner == 0)
                s = launch_fold_op<NT2G_FOLD_MEAN>(x, lo, inner, hi, precision, ws, off, c, nullptr, st);
            else
                s = launch_fold_op<kFoldMeanC>(x, lo, inner, hi, precision, ws, off, c, nullptr, st);
            if (s != NT2G_OK) return s;
            return launch_fold_op<OP>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st, c);
        }
    }
    auto cap = [](int64_t g) { return (int)(g < 152 * 32 ? (g > 0 ? g : 1) : 152 * 32); };
    if (precision == NT2G_PREC_NT2 || inner == 0) {  // (an empty fold yields the neutral element)
        k_fold_nt2<OP><<<cap((n_out + kFoldThreads - 1) / kFoldThreads), kFoldThreads, 0, st>>>(x, lo, inner, hi, out,
                                                                                               index, cen);
        NT2G_LAUNCH_CHECK("fold launch");
        return NT2G_OK;
    }
    const bool aligned = aligned16(x);
    FoldPlan p = plan_fold(lo, inner, hi, aligned);
    if (p.q > 1 && (size_t)(n_out * p.q) * sizeof(Partial) > ws_bytes) {
        set_error("nt2g_fold_f32: workspace of %zu bytes, %zu needed", ws_bytes, (size_t)(n_out * p.q) * sizeof(Partial));
        return NT2G_ERR_INVALID;
    }
    Partial *part = (Partial *)ws;
    if (p.kind == 0) {
        k_fold_short<OP><<<cap((hi + kFoldThreads - 1) / kFoldThreads), kFoldThreads, 0, st>>>(x, inner, hi, out, index,
                                                                                                cen);
    } else if (p.kind == 1) {
        const int64_t items = hi * p.q;
        const int grid = cap((items + 7) / 8);
        const bool idx = index != nullptr && (OP == NT2G_FOLD_MAX || OP == NT2G_FOLD_MIN);
        if (p.q == 1) {
            if (idx) k_fold_inner<OP, true, true><<<grid, kFoldThreads, 0, st>>>(x, inner, hi, p.chunk, 1, p.vec, part, out, index, cen);
            else k_fold_inner<OP, true, false><<<grid, kFoldThreads, 0, st>>>(x, inner, hi, p.chunk, 1, p.vec, part, out, index, cen);
        } else {
            if (idx) k_fold_inner<OP, false, true><<<grid, kFoldThreads, 0, st>>>(x, inner, hi, p.chunk, p.q, p.vec, part, out, index, cen);
            else k_fold_inner<OP, false, false><<<grid, kFoldThreads, 0, st>>>(x, inner, hi, p.chunk, p.q, p.vec, part, out, index, cen);
        }
    } else {
        const int64_t threads = n_out / p.vec;
        dim3 grid(cap((threads + kFoldThreads - 1) / kFoldThreads), (unsigned)p.q);
        if (p.vec == 4) {
            if (p.q == 1) k_fold_outer<OP, 4, true><<<grid, kFoldThreads, 0, st>>>(x, lo, inner, hi, p.chunk, 1, part, out, index, cen);
            else k_fold_outer<OP, 4, false><<<grid, kFoldThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, part, out, index, cen);
        } else {
            if (p.q == 1) k_fold_outer<OP, 1, true><<<grid, kFoldThreads, 0, st>>>(x, lo, inner, hi, p.chunk, 1, part, out, index, cen);
            else k_fold_outer<OP, 1, false><<<grid, kFoldThreads, 0, st>>>(x, lo, inner, hi, p.chunk, p.q, part, out, index, cen);
        }
    }
    NT2G_LAUNCH_CHECK("fold launch");
    if (p.q > 1 && p.kind != 0) {
        if (p.q >= 512)
            k_fold_finish_block<OP><<<cap(n_out), kFoldThreads, 0, st>>>(part, n_out, p.q, inner, out, index, cen);
        else
            k_fold_finish<OP><<<cap((n_out + kFoldThreads - 1) / kFoldThreads), kFoldThreads, 0, st>>>(
                part, n_out, p.q, inner, out, index, cen);
        NT2G_LAUNCH_CHECK("fold combine launch");
    }
    return NT2G_OK;
}

nt2g_status launch_fold(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws,
                        size_t ws_bytes, float *out, int64_t *index, cudaStream_t st)
{
    if (lo * hi == 0) return NT2G_OK;
    switch (op) {
    case NT2G_FOLD_SUM: return launch_fold_op<NT2G_FOLD_SUM>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_PROD: return launch_fold_op<NT2G_FOLD_PROD>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_MAX: return launch_fold_op<NT2G_FOLD_MAX>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_MIN: return launch_fold_op<NT2G_FOLD_MIN>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_MEAN: return launch_fold_op<NT2G_FOLD_MEAN>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_ASUM1: return launch_fold_op<NT2G_FOLD_ASUM1>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_ASUM2: return launch_fold_op<NT2G_FOLD_ASUM2>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_NORM2: return launch_fold_op<NT2G_FOLD_NORM2>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_VAR: return launch_fold_op<NT2G_FOLD_VAR>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_STDEV: return launch_fold_op<NT2G_FOLD_STDEV>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_VAR1: return launch_fold_op<NT2G_FOLD_VAR1>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_STDEV1: return launch_fold_op<NT2G_FOLD_STDEV1>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_NBTRUE: return launch_fold_op<NT2G_FOLD_NBTRUE>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_ALL: return launch_fold_op<NT2G_FOLD_ALL>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_ANY: return launch_fold_op<NT2G_FOLD_ANY>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_NONE: return launch_fold_op<NT2G_FOLD_NONE>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    case NT2G_FOLD_NANSUM: return launch_fold_op<NT2G_FOLD_NANSUM>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    default: return launch_fold_op<NT2G_FOLD_NANMEAN>(x, lo, inner, hi, precision, ws, ws_bytes, out, index, st);
    }
}

}  // namespace nt2g
