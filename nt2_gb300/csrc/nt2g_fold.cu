// nt2g_fold.cu -- reductions along one dimension of a table or of an
// expression: the host side (plans, workspace, launches) and the kernels over
// a table.  The folding itself is nt2g_fold_kernels.cuh, shared with the
// run-time compiled kernels that fold an expression (nt2g_jit.cu).
#include "nt2g_fold_kernels.cuh"
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

using namespace fold;
static_assert((int)SUM == (int)NT2G_FOLD_SUM &&
              (int)PROD == (int)NT2G_FOLD_PROD &&
              (int)MAX == (int)NT2G_FOLD_MAX &&
              (int)MIN == (int)NT2G_FOLD_MIN &&
              (int)MEAN == (int)NT2G_FOLD_MEAN &&
              (int)ASUM1 == (int)NT2G_FOLD_ASUM1 &&
              (int)ASUM2 == (int)NT2G_FOLD_ASUM2 &&
              (int)NORM2 == (int)NT2G_FOLD_NORM2 &&
              (int)VAR == (int)NT2G_FOLD_VAR &&
              (int)STDEV == (int)NT2G_FOLD_STDEV &&
              (int)VAR1 == (int)NT2G_FOLD_VAR1 &&
              (int)STDEV1 == (int)NT2G_FOLD_STDEV1 &&
              (int)NBTRUE == (int)NT2G_FOLD_NBTRUE &&
              (int)ALL == (int)NT2G_FOLD_ALL &&
              (int)ANY == (int)NT2G_FOLD_ANY &&
              (int)NONE == (int)NT2G_FOLD_NONE &&
              (int)NANSUM == (int)NT2G_FOLD_NANSUM &&
              (int)NANMEAN == (int)NT2G_FOLD_NANMEAN &&
              (int)MEANAD == (int)NT2G_FOLD_MEANAD,
              "fold op numbering");

constexpr int kFoldThreads = kThreads;
constexpr int64_t kChunk = 16384;        // elements per warp work item (contiguous folds)
constexpr int64_t kSmallSeg = 64;        // segments up to this length: one thread each
constexpr int64_t kTargetThreads = 152 * 1024;

// A table as a fold source: streaming loads.
struct RawSrc {
    const float *x;
    __device__ __forceinline__ float at(int64_t pos) const { return ld_stream(x + pos); }
    __device__ __forceinline__ float4 at4(int64_t pos) const { return ld_stream((const float4 *)(x + pos)); }
};

template <int OP, bool FINAL, bool IDX>
__global__ void __launch_bounds__(kFoldThreads) k_fold_inner(RawSrc src, int64_t inner, int64_t hi, int64_t chunk,
                                                             int64_t q, int vec, Partial *__restrict__ part,
                                                             float *__restrict__ out, int64_t *__restrict__ index,
                                                             const float *__restrict__ cen, double *__restrict__ out64)
{
    inner_body<RawSrc, OP, FINAL, IDX>(src, inner, hi, chunk, q, vec, part, out, index, cen, out64);
}

template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_short(RawSrc src, int64_t inner, int64_t hi,
                                                             float *__restrict__ out, int64_t *__restrict__ index,
                                                             const float *__restrict__ cen, double *__restrict__ out64)
{
    short_body<RawSrc, OP>(src, inner, hi, out, index, cen, out64);
}

template <int OP, int VEC, bool FINAL>
__global__ void __launch_bounds__(kFoldThreads) k_fold_outer(RawSrc src, int64_t lo, int64_t inner, int64_t hi,
                                                             int64_t ck, int64_t q, Partial *__restrict__ part,
                                                             float *__restrict__ out, int64_t *__restrict__ index,
                                                             const float *__restrict__ cen, double *__restrict__ out64)
{
    outer_body<RawSrc, OP, VEC, FINAL>(src, lo, inner, hi, ck, q, part, out, index, cen, out64);
}

template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_nt2(RawSrc src, int64_t lo, int64_t inner, int64_t hi,
                                                           float *__restrict__ out, int64_t *__restrict__ index,
                                                           const float *__restrict__ cen)
{
    nt2_body<RawSrc, OP>(src, lo, inner, hi, out, index, cen);
}

// Combine the q partials of each output in order.
template <int OP>
__global__ void __launch_bounds__(kFoldThreads) k_fold_finish(const Partial *__restrict__ part, int64_t n_out,
                                                              int64_t q, int64_t inner, float *__restrict__ out,
                                                              int64_t *__restrict__ index, const float *__restrict__ cen,
                                                              double *__restrict__ out64)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += (int64_t)gridDim.x * blockDim.x) {
        const Partial *p = part + o * q;
        if (is_sum(OP) || OP == PROD) {
            double t = OP == PROD ? 1.0 : 0.0;
            for (int64_t c = 0; c < q; ++c) t = OP == PROD ? t * p[c].d : t + p[c].d;
            fold_put<OP>(out, out64, o, n_out, t, inner, cen);
        } else {
            Best b{0.0f, -1, -1};
            for (int64_t c = 0; c < q; ++c)
                if (p[c].b.ilast >= 0) b = b.ilast < 0 ? p[c].b : best_merge<OP == MAX>(b, p[c].b);
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
                                                                    int64_t *__restrict__ index,
                                                                    const float *__restrict__ cen,
                                                                    double *__restrict__ out64)
{
    constexpr bool DBL = is_sum(OP) || OP == PROD;
    __shared__ double sd[kFoldThreads];
    __shared__ Best sb[kFoldThreads];
    for (int64_t o = blockIdx.x; o < n_out; o += gridDim.x) {
        const Partial *p = part + o * q;
        if (DBL) {
            double t = OP == PROD ? 1.0 : 0.0;
#pragma unroll 4
            for (int64_t c = threadIdx.x; c < q; c += blockDim.x) t = OP == PROD ? t * p[c].d : t + p[c].d;
            sd[threadIdx.x] = t;
        } else {
            Best b{0.0f, -1, -1};
#pragma unroll 4
            for (int64_t c = threadIdx.x; c < q; c += blockDim.x) b = best_merge<OP == MAX>(b, p[c].b);
            sb[threadIdx.x] = b;
        }
        __syncthreads();
        for (int w = kFoldThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) {
                if (DBL) sd[threadIdx.x] = OP == PROD ? sd[threadIdx.x] * sd[threadIdx.x + w]
                                                      : sd[threadIdx.x] + sd[threadIdx.x + w];
                else sb[threadIdx.x] = best_merge<OP == MAX>(sb[threadIdx.x], sb[threadIdx.x + w]);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (DBL) {
                fold_put<OP>(out, out64, o, n_out, sd[0], inner, cen);
            } else {
                out[o] = sb[0].v;
                if (index) index[o] = sb[0].ifirst;
            }
        }
        __syncthreads();
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

// Where a fold's elements come from: a table, or the FOLD value of a program
// whose element function is compiled at run time.
struct FoldInput {
    bool expr = false;  // the elements are an expression's (else the table x)
    const float *x = nullptr;
    const std::vector<nt2g_op> *ops = nullptr;
    const std::vector<uint8_t> *logical = nullptr;
    const DArgs *args = nullptr;
    int precision = 0;       // the fold: NT2's index order or the compensated one
    int elem_precision = 0;  // an expression's arithmetic (nt2g_precision, NT2_ELEMENTS included)
    bool aligned = false;    // 128-bit reads allowed at multiples of 4
};

static cudaError_t launch_by_handle(cudaKernel_t k, dim3 grid, void **params, cudaStream_t st)
{
    return cudaLaunchKernel((const void *)k, grid, dim3(kFoldThreads), params, 0, st);
}

template <int OP>
static nt2g_status launch_fold_op(const FoldInput &in, int64_t lo, int64_t inner, int64_t hi, void *ws,
                                  size_t ws_bytes, float *out, int64_t *index, double *out64, cudaStream_t st,
                                  const float *cen = nullptr)
{
    const int precision = in.precision;
    const int64_t n_out = lo * hi;
    if constexpr (is_two_pass(OP)) {
        if (!cen) {  // first the centre of every output: NT2's float mean, or (fast) the mean and its rounding
                     // error; for nanmean the count of non-NaN elements
            const size_t off = fold_centre_offset(lo, inner, hi);
            if (!ws || off + (size_t)n_out * 2 * sizeof(float) > ws_bytes) {
                set_error("fold: workspace of %zu bytes, %zu needed", ws_bytes, off + (size_t)n_out * 2 * sizeof(float));
                return NT2G_ERR_INVALID;
            }
            float *c = (float *)((char *)ws + off);
            nt2g_status s;
            if constexpr (OP == NANMEAN)
                s = launch_fold_op<NOT_NAN>(in, lo, inner, hi, ws, off, c, nullptr, nullptr, st);
            else if (precision == NT2G_PREC_NT2 || inner == 0)
                s = launch_fold_op<MEAN>(in, lo, inner, hi, ws, off, c, nullptr, nullptr, st);
            else
                s = launch_fold_op<MEAN_C>(in, lo, inner, hi, ws, off, c, nullptr, nullptr, st);
            if (s != NT2G_OK) return s;
            return launch_fold_op<OP>(in, lo, inner, hi, ws, ws_bytes, out, index, out64, st, c);
        }
    }
    const JitFoldKernels *jk = nullptr;
    if (in.expr) {
        std::string why;
        jk = jit_fold_kernels(*in.ops, *in.logical, in.elem_precision, OP, &why);
        if (!jk) {
            set_error("fold of an expression: no run-time compiled kernel (%s)", why.c_str());
            return NT2G_ERR_UNSUPPORTED;
        }
    }
    const RawSrc src{in.x};
    const DArgs *jargs = in.args;
    auto cap = [](int64_t g) { return (int)(g < 152 * 32 ? (g > 0 ? g : 1) : 152 * 32); };
    cudaError_t ce = cudaSuccess;
    if (precision == NT2G_PREC_NT2 || inner == 0) {  // (an empty fold yields the neutral element)
        const dim3 g(cap((n_out + kFoldThreads - 1) / kFoldThreads));
        if (!in.expr) {
            k_fold_nt2<OP><<<g, kFoldThreads, 0, st>>>(src, lo, inner, hi, out, index, cen);
            ce = cudaGetLastError();
        } else {
            void *pr[] = {(void *)jargs, &lo, &inner, &hi, &out, &index, &cen};
            ce = launch_by_handle(jk->nt2, g, pr, st);
        }
        if (ce != cudaSuccess) return cuda_status(ce, "fold launch");
        return NT2G_OK;
    }
    FoldPlan p = plan_fold(lo, inner, hi, in.aligned);
    if (p.q > 1 && (size_t)(n_out * p.q) * sizeof(Partial) > ws_bytes) {
        set_error("fold: workspace of %zu bytes, %zu needed", ws_bytes, (size_t)(n_out * p.q) * sizeof(Partial));
        return NT2G_ERR_INVALID;
    }
    Partial *part = (Partial *)ws;
    if (p.kind == 0) {
        const dim3 g(cap((hi + kFoldThreads - 1) / kFoldThreads));
        if (!in.expr) {
            k_fold_short<OP><<<g, kFoldThreads, 0, st>>>(src, inner, hi, out, index, cen, out64);
            ce = cudaGetLastError();
        } else {
            void *pr[] = {(void *)jargs, &inner, &hi, &out, &index, &cen, &out64};
            ce = launch_by_handle(jk->shrt, g, pr, st);
        }
    } else if (p.kind == 1) {
        const int64_t items = hi * p.q;
        const dim3 g(cap((items + 7) / 8));
        const bool idx = index != nullptr && (OP == MAX || OP == MIN);
        const bool fin = p.q == 1;
        int64_t chunk = p.chunk, q = p.q;
        int vec = p.vec;
        if (!in.expr) {
#define NT2G_INNER(F, I) k_fold_inner<OP, F, I><<<g, kFoldThreads, 0, st>>>(src, inner, hi, chunk, q, vec, part, out, \
                                                                            index, cen, out64)
            if (fin) { if (idx) NT2G_INNER(true, true); else NT2G_INNER(true, false); }
            else { if (idx) NT2G_INNER(false, true); else NT2G_INNER(false, false); }
#undef NT2G_INNER
            ce = cudaGetLastError();
        } else {
            void *pr[] = {(void *)jargs, &inner, &hi, &chunk, &q, &vec, &part, &out, &index, &cen, &out64};
            ce = launch_by_handle(jk->inner[fin][idx], g, pr, st);
        }
    } else {
        const int64_t threads = n_out / p.vec;
        const dim3 g(cap((threads + kFoldThreads - 1) / kFoldThreads), (unsigned)p.q);
        const bool fin = p.q == 1;
        int64_t chunk = p.chunk, q = p.q;
        if (!in.expr) {
#define NT2G_OUTER(V, F) k_fold_outer<OP, V, F><<<g, kFoldThreads, 0, st>>>(src, lo, inner, hi, chunk, q, part, out, \
                                                                            index, cen, out64)
            if (p.vec == 4) { if (fin) NT2G_OUTER(4, true); else NT2G_OUTER(4, false); }
            else { if (fin) NT2G_OUTER(1, true); else NT2G_OUTER(1, false); }
#undef NT2G_OUTER
            ce = cudaGetLastError();
        } else {
            void *pr[] = {(void *)jargs, &lo, &inner, &hi, &chunk, &q, &part, &out, &index, &cen, &out64};
            ce = launch_by_handle(jk->outer[p.vec == 4][fin], g, pr, st);
        }
    }
    if (ce != cudaSuccess) return cuda_status(ce, "fold launch");
    if (p.q > 1 && p.kind != 0) {
        if (p.q >= 512)
            k_fold_finish_block<OP><<<cap(n_out), kFoldThreads, 0, st>>>(part, n_out, p.q, inner, out, index, cen, out64);
        else
            k_fold_finish<OP><<<cap((n_out + kFoldThreads - 1) / kFoldThreads), kFoldThreads, 0, st>>>(
                part, n_out, p.q, inner, out, index, cen, out64);
        NT2G_LAUNCH_CHECK("fold combine launch");
    }
    return NT2G_OK;
}

static nt2g_status fold_dispatch(const FoldInput &in, int64_t lo, int64_t inner, int64_t hi, int op, void *ws,
                                 size_t ws_bytes, float *out, int64_t *index, double *out64, cudaStream_t st)
{
    if (lo * hi == 0) return NT2G_OK;
#define NT2G_OP_CASE(O) \
    case O: return launch_fold_op<O>(in, lo, inner, hi, ws, ws_bytes, out, index, out64, st);
    switch (op) {
    NT2G_OP_CASE(SUM) NT2G_OP_CASE(PROD) NT2G_OP_CASE(MAX) NT2G_OP_CASE(MIN) NT2G_OP_CASE(MEAN)
    NT2G_OP_CASE(ASUM1) NT2G_OP_CASE(ASUM2) NT2G_OP_CASE(NORM2) NT2G_OP_CASE(VAR) NT2G_OP_CASE(STDEV)
    NT2G_OP_CASE(VAR1) NT2G_OP_CASE(STDEV1) NT2G_OP_CASE(NBTRUE) NT2G_OP_CASE(ALL) NT2G_OP_CASE(ANY)
    NT2G_OP_CASE(NONE) NT2G_OP_CASE(NANSUM) NT2G_OP_CASE(MEANAD)
    default: return launch_fold_op<NANMEAN>(in, lo, inner, hi, ws, ws_bytes, out, index, out64, st);
    }
#undef NT2G_OP_CASE
}

nt2g_status launch_fold(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws,
                        size_t ws_bytes, float *out, int64_t *index, cudaStream_t st)
{
    FoldInput in;
    in.x = x;
    in.precision = precision;
    in.aligned = aligned16(x);
    return fold_dispatch(in, lo, inner, hi, op, ws, ws_bytes, out, index, nullptr, st);
}

// trapz(y, dim) (core/functions/expr/trapz.hpp:24-50): NT2 folds adjfun(plus,
// y, dim) -- the n - 1 float sums y_k + y_(k+1) of neighbours along the
// dimension -- and halves the sum.  NT2 policy: one thread per output, those
// sums folded in index order from 0, times 1/2.  Fast policy: the
// compensated fold of y (FP64 combine) less half of the two ends,
// sum(y) - (y_0 + y_(n-1))/2, NT2's value in exact arithmetic, rounded once;
// a non-finite sum is kept as it is (an infinity at an end is NT2's result).
__global__ void __launch_bounds__(kFoldThreads) k_trapz_nt2(const float *__restrict__ x, int64_t lo, int64_t n,
                                                             int64_t hi, float *__restrict__ out)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < lo * hi;
         o += (int64_t)gridDim.x * blockDim.x) {
        const float *b = x + o % lo + lo * n * (o / lo);
        float s = 0.0f;
        for (int64_t k = 0; k + 1 < n; ++k) s = __fadd_rn(s, __fadd_rn(b[lo * k], b[lo * (k + 1)]));
        out[o] = __fmul_rn(0.5f, s);
    }
}

__global__ void __launch_bounds__(kFoldThreads) k_trapz_finish(const float *__restrict__ x, int64_t lo, int64_t n,
                                                                int64_t hi, const double *__restrict__ s64,
                                                                float *__restrict__ out)
{
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < lo * hi;
         o += (int64_t)gridDim.x * blockDim.x) {
        const float *b = x + o % lo + lo * n * (o / lo);
        const double s = s64[o];
        out[o] = n < 2 ? 0.0f
                       : (s - s == 0.0 ? (float)(s - 0.5 * ((double)b[0] + (double)b[lo * (n - 1)])) : (float)s);
    }
}

nt2g_status trapz_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    *bytes = (fold_partial_bytes(lo, inner, hi) + 15) / 16 * 16 + (size_t)(lo * hi) * sizeof(double);
    return NT2G_OK;
}

nt2g_status launch_trapz(const float *x, int64_t lo, int64_t inner, int64_t hi, int precision, void *ws,
                         size_t ws_bytes, float *out, cudaStream_t st)
{
    const int64_t n_out = lo * hi;
    if (n_out == 0) return NT2G_OK;
    const int g = (int)((n_out + kFoldThreads - 1) / kFoldThreads < 152 * 32 ? (n_out + kFoldThreads - 1) / kFoldThreads
                                                                              : 152 * 32);
    if (precision == NT2G_PREC_NT2 || inner < 2) {
        k_trapz_nt2<<<g, kFoldThreads, 0, st>>>(x, lo, inner, hi, out);
        NT2G_LAUNCH_CHECK("trapz launch");
        return NT2G_OK;
    }
    const size_t off = (fold_partial_bytes(lo, inner, hi) + 15) / 16 * 16;
    double *s64 = (double *)((char *)ws + off);
    FoldInput in;
    in.x = x;
    in.precision = NT2G_PREC_FAST;
    in.aligned = aligned16(x);
    nt2g_status s = fold_dispatch(in, lo, inner, hi, SUM, ws, off, out, nullptr, s64, st);
    if (s != NT2G_OK) return s;
    k_trapz_finish<<<g, kFoldThreads, 0, st>>>(x, lo, inner, hi, s64, out);
    NT2G_LAUNCH_CHECK("trapz launch");
    return NT2G_OK;
}

nt2g_status launch_fold_expr(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                             int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws, size_t ws_bytes,
                             float *out, int64_t *index, double *out64, cudaStream_t st)
{
    FoldInput in;
    in.expr = true;
    in.ops = &ops;
    in.logical = &logical;
    in.args = &args;
    in.precision = precision == NT2G_PREC_NT2 ? NT2G_PREC_NT2 : NT2G_PREC_FAST;  // the fold's order
    in.elem_precision = precision;
    // whole-vector element reads need every float table 16-byte and every uint8 table 4-byte aligned
    bool al = true;
    for (int s = 0; s < kMaxSlots; ++s)
        if (args.ptr[s]) al &= ((uintptr_t)args.ptr[s] & (args.dtype[s] == NT2G_F32 ? 15u : 3u)) == 0;
    in.aligned = al;
    return fold_dispatch(in, lo, inner, hi, op, ws, ws_bytes, out, index, out64, st);
}

}  // namespace nt2g
