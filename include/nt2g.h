/*
 * nt2g.h -- C ABI of libnt2gpu, the sm_103a evaluator for NT2's fused
 * elementwise expressions over nt2::table and its sum/dot reductions.
 *
 * Plain pointers, sizes and status codes: no C++ or torch types cross this
 * boundary.  Every call returns an nt2g_status; no call exits, throws or
 * prints.  nt2g_last_error() holds the text of the last failure on the
 * calling thread.  Device pointers are caller-owned; the calls are
 * stream-ordered and asynchronous (a cudaStream_t is passed as void*).
 *
 * What each entry point replaces in NT2 (paths inside the NT2 source tree):
 *   CSDK  = modules/core/sdk/include/nt2
 *   TABLE = modules/core/container/table/include/nt2
 *   SHM   = modules/arch/shared_memory/include/nt2
 *   RED   = modules/core/reduction/include/nt2
 *   CUDA  = modules/arch/cuda/include/nt2
 */
#ifndef NT2G_H
#define NT2G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NT2G_ABI_VERSION 2

typedef enum nt2g_status {
    NT2G_OK = 0,
    NT2G_ERR_INVALID = 1,     /* bad pointer, size, alignment, opcode or slot */
    NT2G_ERR_UNSUPPORTED = 2, /* valid request this build cannot run */
    NT2G_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    NT2G_ERR_DEVICE_FLAG = 4, /* a kernel reported an error through its flag */
    NT2G_ERR_NOMEM = 5        /* host or device allocation failed */
} nt2g_status;

/* Arithmetic policy of the float math.
 * NT2G_PREC_FAST: fused multiply-add, approximate-reciprocal division with a
 *   Newton step where the operands are known normal, erfc/normcdf on an exact
 *   split of x^2; every functor within 4 ulp of FP64 (gammaln excepted: NT2's
 *   form, 6.3 ulp near Gamma's minimum), away from the poles and zeros where
 *   a function's own conditioning decides.
 * NT2G_PREC_NT2: NT2's own scalar algorithms and operation order (unfused
 *   fma/Horner, IEEE division and sqrt); bit-identical to NT2's CPU result. */
typedef enum nt2g_precision {
    NT2G_PREC_FAST = 0,
    NT2G_PREC_NT2 = 1,
    /* folds of an expression only (nt2g_eval_fold): NT2's element arithmetic,
       folded by the compensated fast-policy fold (what sum(), dot() and
       globalsum() do with NT2 elements) */
    NT2G_PREC_NT2_ELEMENTS = 2
} nt2g_precision;

typedef enum nt2g_dtype { NT2G_F32 = 0, NT2G_U8 = 1 } nt2g_dtype;

const char *nt2g_last_error(void);
int nt2g_abi_version(void);

/* ------------------------------------------------------------------ */
/* Fused expression programs: the lowered form of an nt2 expression.  */
/* Replaces the transform_ overload on the shared_memory site         */
/* (SHM/core/functions/shared_memory/transform.hpp:27-51) and the      */
/* intended external_kernel code generator                             */
/* (tools/external_kernel/backend.cpp:32-52) for site cuda_.           */
/* ------------------------------------------------------------------ */

/* Opcodes.  Values are numbered in program order (SSA): operand fields a,b,c
 * name earlier instructions; LOAD/SCALAR/STORE name argument slots.  The
 * result dtype of each instruction is op.dtype. */
typedef enum nt2g_opcode {
    NT2G_OP_LOAD = 1,      /* a = slot of a device table                     */
    NT2G_OP_SCALAR = 2,    /* a = slot of a scalar argument (broadcast)      */
    NT2G_OP_CONST = 3,     /* imm                                            */
    NT2G_OP_STORE = 4,     /* a = value, b = slot of the output table        */
    NT2G_OP_INDEX = 5,     /* the element's linear position p (offset + i) in
                              the op's dtype: NT2's enumerate<T>(p), the leaf of
                              colon / linspace / logspace (uint8: p mod 256)    */
    NT2G_OP_FOLD = 6,      /* a = the float value nt2g_eval_fold folds (a
                              comparison folds as 0/1); a program has at most
                              one FOLD and then no STORE                       */
    NT2G_OP_ADD = 10, NT2G_OP_SUB, NT2G_OP_MUL, NT2G_OP_DIV, NT2G_OP_NEG, NT2G_OP_ABS,
    NT2G_OP_SQR, NT2G_OP_SQRT, NT2G_OP_REC, NT2G_OP_MIN, NT2G_OP_MAX,
    NT2G_OP_FMA = 30,      /* a*b + c (unfused under NT2G_PREC_NT2)          */
    NT2G_OP_FNMS,          /* c - a*b                                        */
    NT2G_OP_EXP = 40, NT2G_OP_LOG, NT2G_OP_LOG1P, NT2G_OP_ERFC, NT2G_OP_NORMCDF,
    NT2G_OP_FASTNORMCDF,
    NT2G_OP_EXP2 = 46, NT2G_OP_EXP10, NT2G_OP_EXPM1, NT2G_OP_LOG2, NT2G_OP_LOG10,
    NT2G_OP_SIN = 51, NT2G_OP_COS, NT2G_OP_TAN, NT2G_OP_SINPI, NT2G_OP_COSPI,
    NT2G_OP_POW = 56,      /* a^b (float)                                    */
    NT2G_OP_SINH = 57, NT2G_OP_COSH, NT2G_OP_TANH,
    NT2G_OP_LT = 60, NT2G_OP_GT, NT2G_OP_LE, NT2G_OP_GE, NT2G_OP_EQ, NT2G_OP_NE, /* -> logical */
    NT2G_OP_IF_ELSE = 70,  /* a ? b : c                                      */
    NT2G_OP_SELINC,        /* a ? b+1 : b                                    */
    NT2G_OP_SELDEC,        /* a ? b-1 : b                                    */
    NT2G_OP_IF_ZERO_ELSE_ONE, /* a ? 0 : 1                                   */
    NT2G_OP_ADDS,          /* saturating add (uint8)                         */
    NT2G_OP_ASIN = 90, NT2G_OP_ACOS, NT2G_OP_ATAN,
    NT2G_OP_ATAN2,         /* atan2(a, b) (float)                            */
    NT2G_OP_ASINH = 94, NT2G_OP_ACOSH, NT2G_OP_ATANH,
    NT2G_OP_CBRT = 97,
    NT2G_OP_HYPOT = 98,    /* hypot(a, b) (float)                            */
    NT2G_OP_COT = 100, NT2G_OP_SEC, NT2G_OP_CSC, NT2G_OP_SIND, NT2G_OP_COSD, NT2G_OP_TAND,
    NT2G_OP_TANPI = 106, NT2G_OP_COTPI, NT2G_OP_COTD, NT2G_OP_SECPI, NT2G_OP_CSCPI, NT2G_OP_SECD, NT2G_OP_CSCD,
    NT2G_OP_SINC = 113, NT2G_OP_SINCPI, NT2G_OP_ACOTD, NT2G_OP_ASEC, NT2G_OP_COTH, NT2G_OP_SINHC,
    NT2G_OP_ACSC = 119, NT2G_OP_ASECH, NT2G_OP_ACOTH, NT2G_OP_ACSCH,
    NT2G_OP_ERF = 123, NT2G_OP_ERFCX, NT2G_OP_EXPX2, NT2G_OP_GAMMA, NT2G_OP_GAMMALN, NT2G_OP_EXPRECNEG,
    NT2G_OP_EXPRECNEGC, NT2G_OP_SQRT1PM1, NT2G_OP_ERFINV, NT2G_OP_ERFCINV,
    NT2G_OP_FLOOR = 133, NT2G_OP_CEIL, NT2G_OP_TRUNC, NT2G_OP_ROUND, NT2G_OP_ROUND2EVEN, NT2G_OP_FRAC, NT2G_OP_SIGN,
    NT2G_OP_SIGNNZ,
    NT2G_OP_COPYSIGN = 141, /* copysign(a, b) (float)                   */
    /* predicates of a float -> logical (boost/simd predicates: is_nan, is_inf, is_finite = x - x == 0,
       is_eqz, is_nez, is_ltz, is_gtz) */
    NT2G_OP_IS_NAN = 142, NT2G_OP_IS_INF, NT2G_OP_IS_FINITE, NT2G_OP_IS_EQZ, NT2G_OP_IS_NEZ, NT2G_OP_IS_LTZ,
    NT2G_OP_IS_GTZ,
    NT2G_OP_SIGNGAM = 149, /* sign of Gamma (NaN at the poles)             */
    NT2G_OP_DIGAMMA = 150, /* psi = Gamma'/Gamma, NT2's double algorithm    */
    NT2G_OP_DAWSON = 151,  /* Dawson's integral                            */
    /* integer operands (n) ride in a float, truncated toward zero (NaN -> 0) */
    NT2G_OP_NTHROOT = 152, /* nthroot(a, n = b): real n-th root           */
    NT2G_OP_EXPNI = 153,   /* expni(n = a, b): exponential integral E_n(b) */
    NT2G_OP_GAMMAINC = 154, /* gammainc(a, b): regularised lower incomplete
                              gamma P(b, a), evaluated in double          */
    NT2G_OP_SPENCE = 155,  /* spence(a): dilogarithm (Cephes' spence)     */
    NT2G_OP_GAMMAINCINV = 156, /* gammaincinv(a, b): the x with P(b, x) = a,
                                  evaluated in double                     */
    NT2G_OP_STIRLING = 157, /* stirling(a): NT2's Stirling approximation of
                               Gamma                                      */
    NT2G_OP_PROPER_TANPI = 158, /* proper_tanpi(a): tan(pi a) on [-1/2, 1/2],
                                   NaN outside, +-inf at +-1/2            */
    NT2G_OP_MOD = 159, /* mod(a, b): a - floor(a/b) b (a where b == 0)      */
    NT2G_OP_REM = 160, /* rem(a, b): a - b trunc(a/b), the quotient through
                          a saturating int32 (a where b == 0)              */
    NT2G_OP_POW2 = 161 /* pow2(a, b): a * 2^n, n = b truncated to int32, by
                          NT2's fast_ldexp: (n + 127) << 23 in wrapping int32
                          arithmetic as the scale's bits (n outside
                          [-127, 128] gives that bit pattern)              */
} nt2g_opcode;

typedef struct nt2g_op {
    int16_t code;  /* nt2g_opcode */
    int16_t dtype; /* nt2g_dtype of the result (logical results: the dtype compared) */
    int32_t a, b, c;
    float imm;
} nt2g_op;

typedef struct nt2g_arg {
    void *ptr;     /* device table (LOAD / STORE slots) */
    double scalar; /* value of a SCALAR slot */
    int32_t dtype; /* nt2g_dtype */
    int32_t kind;  /* 0 = table, 1 = scalar */
} nt2g_arg;

typedef struct nt2g_program nt2g_program;

typedef struct nt2g_program_info {
    int32_t kernel;       /* 0 = generic interpreter, >0 = fused kernel id */
    int32_t n_ops;        /* after common-subexpression and dead-code removal */
    int32_t n_regs;       /* interpreter registers after allocation */
    int32_t n_slots;
    char kernel_name[48];
} nt2g_program_info;

/* Validate, canonicalise (CSE + DCE), register-allocate and bind a program.
 * When the program is one of the fused kernels' expressions (Black-Scholes
 * call+put, the NT2 demo Black-Scholes, saxpy, expr3, rgb2yuv, sigma-delta)
 * it is bound to that kernel; otherwise to the generic interpreter. */
nt2g_status nt2g_program_create(const nt2g_op *ops, int32_t n_ops, int32_t n_slots,
                                nt2g_program **out);
nt2g_status nt2g_program_info_get(const nt2g_program *p, nt2g_program_info *info);
void nt2g_program_destroy(nt2g_program *p);

/* transform(out, expr, range): evaluate elements [offset, offset+count) of
 * every table slot (TABLE/core/functions/expr/transform.hpp:40-60 range
 * semantics).  Kernel choice:
 *   force_generic = 0: the bound fused kernel; otherwise the program's
 *                      run-time compiled kernel; otherwise the interpreter;
 *   force_generic = 1: the run-time compiled kernel, else the interpreter;
 *   force_generic = 2: the interpreter.
 * The compiled kernel and the interpreter give bit-identical results.  The
 * compiled kernel is built by NVRTC (loaded with dlopen) on first use per
 * device, precision and program; NT2G_JIT=0 in the environment disables it. */
nt2g_status nt2g_eval(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t offset,
                      int64_t count, int32_t precision, int32_t force_generic, void *stream);

/* The CUDA source of the program's run-time compiled kernel (no GPU needed).
 * *len receives the size including the terminating NUL; cap = 0 only queries
 * it.  NT2's planned per-expression CUDA generator:
 * tools/external_kernel/backend.cpp:32-52 with tools/kernel_gen/kernel_gen.cpp:8-113. */
nt2g_status nt2g_program_jit_source(const nt2g_program *p, int32_t precision, char *buf, size_t cap,
                                    size_t *len);

/* Compile and load the program's kernel now (before a stream capture, or to
 * keep compilation out of a timed region).  NT2G_ERR_UNSUPPORTED, with the
 * reason in nt2g_last_error(), when NVRTC is unavailable or rejects it. */
nt2g_status nt2g_program_jit_prepare(const nt2g_program *p, int32_t precision);

/* ------------------------------------------------------------------ */
/* Reductions along one dimension (sum(a, dim), max(a, [], dim), ...)  */
/* ------------------------------------------------------------------ */
/* The table is viewed as [lo, inner, hi] (column-major) and folded over
 * inner: out[l + lo*h] = fold_k x[l + lo*(k + inner*h)], lo*hi outputs.
 * This is NT2's reshape before inner_fold / outer_fold
 * (core/reduction/include/nt2/dsl/functions/reduction/run.hpp:51-89):
 *   2-D m x n table, dim 1 (per column): lo = 1, inner = m, hi = n;
 *   dim 2 (per row): lo = m, inner = n, hi = 1;  global*: lo = hi = 1.
 * Ops follow NT2's definitions: MEAN = rec(n) * sum (expr/mean.hpp),
 * ASUM1 = sum(abs), ASUM2 = sum(sqr_abs), NORM2 = sqrt(asum2); MAX/MIN fold
 * with (acc > x) ? acc : x, and index (optional, 0-based along the fold,
 * -1 if none) receives the first position equal to the result, as NT2's
 * globalmax(a, i) = globalfind(a == max).
 * precision NT2G_PREC_NT2: each output folded in index order with NT2's
 * unfused float operations (NT2's own order when it spreads outputs over
 * threads), one thread per output.  NT2G_PREC_FAST: compensated FP32 sums
 * combined in FP64, FP64 products, exact max/min (equal to the NT2 order on
 * NaN-free data; a NaN propagates); deterministic for a given shape.
 * workspace: nt2g_fold_workspace_size bytes (enough for every op; var and
 * stdev keep each output's centre there, so they need it under either
 * policy, the others only under NT2G_PREC_FAST and only for chunked shapes). */
typedef enum nt2g_fold_op {
    NT2G_FOLD_SUM = 0,
    NT2G_FOLD_PROD = 1,
    NT2G_FOLD_MAX = 2,
    NT2G_FOLD_MIN = 3,
    NT2G_FOLD_MEAN = 4,
    NT2G_FOLD_ASUM1 = 5,
    NT2G_FOLD_ASUM2 = 6,
    NT2G_FOLD_NORM2 = 7,
    NT2G_FOLD_VAR = 8,     /* asum2(a - mean(a)) / (n - 1)  (NT2's var(a))     */
    NT2G_FOLD_STDEV = 9,   /* sqrt(var)                                       */
    NT2G_FOLD_VAR1 = 10,   /* asum2(a - mean(a)) / n        (NT2's var(a, 1))  */
    NT2G_FOLD_STDEV1 = 11, /* sqrt(var1)                                      */
    NT2G_FOLD_NBTRUE = 12, /* number of nonzero elements (NaN counts)         */
    NT2G_FOLD_ALL = 13,    /* 1 if every element is nonzero, else 0           */
    NT2G_FOLD_ANY = 14,    /* 1 if some element is nonzero                    */
    NT2G_FOLD_NONE = 15,   /* 1 if no element is nonzero                      */
    NT2G_FOLD_NANSUM = 16, /* sum of the non-NaN elements                     */
    NT2G_FOLD_NANMEAN = 17, /* nansum / max(number of non-NaN elements, 1)    */
    NT2G_FOLD_MEANAD = 18   /* mean(abs(a - mean(a))) (NT2's meanad)          */
} nt2g_fold_op;

nt2g_status nt2g_fold_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);

/* trapz(a, dim): the trapezoidal integral with unit spacing over the same
 * [lo, inner, hi] view (core/functions/expr/trapz.hpp:24-50: half the sum of
 * adjfun(plus, a, dim), the n - 1 sums of neighbours).  NT2G_PREC_NT2: those
 * float sums folded in index order, halved, bit-identical to NT2;
 * NT2G_PREC_FAST: sum(a) by the compensated fold less half of the two ends,
 * rounded once.  inner < 2 gives 0.  workspace: nt2g_trapz_workspace_size
 * bytes (none needed under NT2G_PREC_NT2). */
nt2g_status nt2g_trapz_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status nt2g_trapz_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t precision,
                           void *workspace, size_t workspace_bytes, float *out, void *stream);

/* median(a, dim) and medianad(a, dim) = median(abs(a - median(a, dim)), dim)
 * over the same [lo, inner, hi] view
 * (core/reduction/include/nt2/core/functions/expr/median.hpp:37-50,
 *  expr/medianad.hpp:38-54; globalmedian / globalmedianad: lo = hi = 1).
 * NT2 sorts each slice and takes the middle element (odd inner) or meanof of
 * the two middle ones (even inner); the result is an order statistic, the
 * same under either arithmetic policy, found here by radix selection.  A
 * slice holding a NaN gives NaN (NT2's sort leaves that case unspecified);
 * an empty slice (inner = 0) gives NaN.  workspace: 0 bytes for
 * inner <= 40960 (each slice in one block's shared memory), else
 * nt2g_median_workspace_size bytes (slice histograms). */
typedef enum nt2g_median_op { NT2G_MEDIAN = 0, NT2G_MEDIANAD = 1 } nt2g_median_op;
nt2g_status nt2g_median_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status nt2g_median_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op, void *workspace,
                            size_t workspace_bytes, float *out, void *stream);
nt2g_status nt2g_fold_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op, int32_t precision,
                          void *workspace, size_t workspace_bytes, float *out, int64_t *index, void *stream);

/* The same fold over an expression: x at linear position p is the value of
 * the program's FOLD instruction for element p of its tables (every table
 * slot holds lo*inner*hi elements in the same column-major layout; INDEX
 * leaves read p).  NT2's folds take the expression itself
 * (RED/core/functions/scalar/inner_fold.hpp:23-49 with fold_step over the
 * AST, RED/core/functions/simd/global.hpp:27-69): here every element is
 * evaluated in registers inside the fold kernels -- sum(exp(x)*y),
 * globalsum(a*b+c), sum(abs(x-y), 1) read their input tables once and write
 * no temporary.  Results equal nt2g_fold_f32 of the expression evaluated into
 * an aligned table by nt2g_eval's run-time compiled kernel (same policy,
 * force_generic = 1), bit for bit.  out64 (optional, may be
 * NULL; not under NT2G_PREC_NT2) receives the FP64 result of each output of a
 * sum-type fold (sum, mean, asum1/2, norm2, var, stdev, counts, nansum,
 * nanmean) or of prod, before rounding to float.  The kernels are compiled at
 * run time (NVRTC) on first use per device, policy, op and program: make that
 * first call outside any stream capture.  NT2G_ERR_UNSUPPORTED when NVRTC is
 * unavailable.  precision: NT2G_PREC_FAST, NT2G_PREC_NT2 (NT2's elements folded
 * in NT2's index order), or NT2G_PREC_NT2_ELEMENTS (NT2's elements, compensated
 * fold).  workspace: nt2g_fold_workspace_size bytes. */
nt2g_status nt2g_eval_fold(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t lo, int64_t inner,
                           int64_t hi, int32_t op, int32_t precision, void *workspace, size_t workspace_bytes,
                           float *out, int64_t *index, double *out64, void *stream);

/* Reverse mode of a program: the vector-Jacobian product over elements
 * [0, count).  All three arrays are indexed by slot (n_args entries):
 *   cotangents[s]  device table of the cotangent of the value the program
 *                  stores into float output slot s (NULL: zero);
 *   table_grads[s] device table receiving, for a float table slot s the
 *                  program reads, the gradient with respect to that input
 *                  (NULL: not wanted; zeros when no output depends on it);
 *   scalar_grads   device array of n_args doubles, or NULL: entry s receives
 *                  the gradient with respect to float scalar slot s summed
 *                  over the elements (the same bits on every run); the other
 *                  entries are left alone.
 * Forward values are recomputed, not stored, exactly as nt2g_eval with
 * force_generic = 1 computes them under `precision`; the derivative
 * arithmetic is the fast policy's, in FP32.  Gradient tables may be the
 * program's input or cotangent tables (each element's inputs are read before
 * its gradients are written).  workspace: nt2g_program_vjp_workspace_size
 * bytes (8-byte aligned) when scalar_grads is given, else unused.  Needs the
 * run-time compiler (NVRTC): NT2G_ERR_UNSUPPORTED without it.  Programs that
 * fold (FOLD) are refused.  No counterpart in the reference (NT2 has no
 * reverse mode); NT2G_OP_* rules are the derivatives of the functions as
 * this library evaluates them (fastnormcdf: of NT2's approximation). */
nt2g_status nt2g_program_vjp(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t count,
                             const float *const *cotangents, float *const *table_grads, double *scalar_grads,
                             int32_t precision, void *workspace, size_t workspace_bytes, void *stream);
nt2g_status nt2g_program_vjp_workspace_size(const nt2g_program *p, int64_t count, size_t *bytes);
/* The CUDA source of the program's reverse-mode kernel (no GPU needed; *len
 * receives the size including the terminating NUL, cap = 0 only queries it). */
nt2g_status nt2g_program_vjp_source(const nt2g_program *p, int32_t precision, char *buf, size_t cap, size_t *len);

/* The CUDA source nt2g_eval_fold compiles for a program and fold op (no GPU
 * needed; *len receives the size including the terminating NUL, cap = 0 only
 * queries it).  No counterpart in the reference: it exposes the generated
 * code for inspection and for compile checks. */
nt2g_status nt2g_program_fold_source(const nt2g_program *p, int32_t precision, int32_t op, char *buf, size_t cap,
                                     size_t *len);

/* ------------------------------------------------------------------ */
/* Cumulative functions along one dimension (cumsum, cumprod, ...)     */
/* ------------------------------------------------------------------ */
/* Same [lo, inner, hi] view as the folds; out has the shape of x (out may be
 * x): out[l + lo*(k + inner*h)] = scan over k' <= k (NT2's run_assign of a
 * cumulative node, core/swar/include/nt2/dsl/functions/cumulative/run.hpp:26-67;
 * summary = bop(summary, x) in order from the neutral element,
 * core/swar/include/nt2/core/functions/details/scan_step.hpp:27-43).
 * NT2G_PREC_NT2: that order with NT2's unfused float operations, one thread
 * per segment.  NT2G_PREC_FAST: compensated cumsum (within about an ulp of the
 * exact prefix), FP64 cumprod, exact cummax/cummin equal to NT2's order (NaN
 * included); deterministic for a given shape. */
typedef enum nt2g_scan_op {
    NT2G_SCAN_SUM = 0,
    NT2G_SCAN_PROD = 1,
    NT2G_SCAN_MAX = 2,
    NT2G_SCAN_MIN = 3
} nt2g_scan_op;

nt2g_status nt2g_scan_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status nt2g_scan_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op, int32_t precision,
                          void *workspace, size_t workspace_bytes, float *out, void *stream);

/* Host tables.  Every entry point accepts host pointers for its tables and
 * workspaces where the current device can reach the memory: pinned or
 * registered host memory (cudaMallocHost, cudaHostRegister) on any system,
 * and any host memory, malloc'd included, on systems with pageable memory
 * access (Grace-Blackwell over NVLink-C2C, or HMM).  The kernels then read
 * and write the host tables in place over the host link: no staging copy and
 * no device allocation (NT2's cuda copy path, CUDA/memory/functions/cuda/
 * copy.hpp:24-100, stages every host table through a device buffer).  A host
 * pointer the device cannot reach is rejected with NT2G_ERR_INVALID before
 * any launch.  *pageable receives 1 when the current device has pageable
 * memory access. */
nt2g_status nt2g_host_access(int32_t *pageable);

/* ------------------------------------------------------------------ */
/* Fused kernels for the named expressions (also reached through      */
/* nt2g_eval).  All tables have n elements.                           */
/* ------------------------------------------------------------------ */

/* Textbook Black-Scholes call+put (normcdf = Half*erfc(-Sqrt_2o_2*x),
 * modules/core/statistics/include/nt2/statistics/functions/generic/normcdf.hpp:34).
 * sigma == NULL selects the scalar sigma_s; r is a scalar. */
nt2g_status nt2g_blackscholes_f32(const float *S, const float *K, const float *T, const float *sigma,
                                  float sigma_s, float r, float *call, float *put, int64_t n,
                                  int32_t precision, void *stream);

/* NT2 demo form, call only, fastnormcdf
 * (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59).  r_t / v_t NULL
 * select the scalars r / v. */
nt2g_status nt2g_blackscholes_demo_f32(const float *S, const float *X, const float *T, const float *r_t,
                                       float r, const float *v_t, float v, float *R, int64_t n,
                                       int32_t precision, void *stream);

/* Fused forward + reverse-mode (vector-Jacobian) Black-Scholes: given
 * upstream gradients gc, gp it writes call, put and the per-option
 * gradients of gc*call + gp*put w.r.t. S, K, T, sigma and r.  Intermediates
 * are recomputed, not stored.  No NT2 counterpart (NT2 has no adjoint). */
nt2g_status nt2g_blackscholes_vjp_f32(const float *S, const float *K, const float *T,
                                      const float *sigma, float r, const float *gc, const float *gp,
                                      float *call, float *put, float *dS, float *dK, float *dT,
                                      float *dsigma, float *dr, int64_t n, void *stream);

/* Y = alpha*X + Y (demo/saxpy/nt2/saxpy_nt2.cpp:41), two roundings. */
nt2g_status nt2g_saxpy_f32(float alpha, const float *X, float *Y, int64_t n, void *stream);

/* out = exp(-sqr(x))*sqrt(abs(y)) + log1p(abs(z)). */
nt2g_status nt2g_expr3_f32(const float *x, const float *y, const float *z, float *out, int64_t n,
                           int32_t precision, void *stream);

/* y/u/v planes (demo/rgb2yuv/nt2/rgb2yuv_nt2.cpp:30-32).  NT2G_PREC_NT2:
 * NT2's unfused left-to-right evaluation (bit-identical); NT2G_PREC_FAST: y
 * carried as a double-float so u and v keep ~1 ulp under b-y cancellation. */
nt2g_status nt2g_rgb2yuv_f32(const float *r, const float *g, const float *b, float *y, float *u,
                             float *v, int64_t n, int32_t precision, void *stream);

/* One sigma-delta step on uint8 pixels, bkg/var updated in place, label
 * written (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:38-57).  Bit-exact. */
nt2g_status nt2g_sigmadelta_u8(const uint8_t *frame, uint8_t *bkg, uint8_t *var, uint8_t *label,
                               int64_t n, void *stream);

/* n_frames consecutive steps in one pass (frames and labels are n_frames
 * planes of n pixels); bkg/var stay in registers between frames. */
nt2g_status nt2g_sigmadelta_frames_u8(const uint8_t *frames, uint8_t *bkg, uint8_t *var,
                                      uint8_t *labels, int64_t n, int32_t n_frames, void *stream);

/* Element functions y = f(x) for the accuracy tests and simple maps.
 * fn: 0 exp, 1 log, 2 log1p, 3 erfc, 4 normcdf, 5 fastnormcdf, 6 sqrt,
 * 7 normcdf(-x) through the shared pair core, 8 exp2, 9 exp10, 10 expm1, 11 log2, 12 log10,
 * 13 sin, 14 cos, 15 tan, 16 sinpi, 17 cospi, 18 sinh, 19 cosh, 20 tanh, 21 asin,
 * 22 acos, 23 atan, 24 asinh, 25 acosh, 26 atanh, 27 cbrt, 28 cot, 29 sec, 30 csc, 31 sind,
 * 32 cosd, 33 tand, 34 tanpi, 35 cotpi, 36 cotd, 37 secpi, 38 cscpi, 39 secd, 40 cscd, 41 sinc,
 * 42 sincpi, 43 acotd, 44 asec, 45 coth, 46 sinhc, 47 acsc, 48 asech, 49 acoth, 50 acsch, 64 erf, 65 erfcx, 66 expx2, 67 gamma, 68 gammaln,
 * 69 erfinv, 70 erfcinv,
 * 71 digamma, 72 signgam, 73 dawson, 74 spence, 75 stirling, 80 exprecneg, 81 exprecnegc, 82 sqrt1pm1. */
nt2g_status nt2g_map_f32(int32_t fn, const float *x, float *y, int64_t n, int32_t precision,
                         void *stream);

/* ------------------------------------------------------------------ */
/* Reductions: sum(x), dot(x,y) = sum(x*y), globalsum                  */
/* (RED/reduction/functions/expr/dot.hpp:22-42,                       */
/*  SHM/core/functions/shared_memory/inner_fold.hpp:25-64,            */
/*  RED/core/functions/globalsum.hpp:43-45).                          */
/* Compensated FP32 (TwoSum) per thread, warp and block; FP64 only in */
/* the cross-block combine.  Deterministic for a given n and device.  */
/* ------------------------------------------------------------------ */

/* Device workspace bytes the reductions need for n elements. */
nt2g_status nt2g_reduce_workspace_size(int64_t n, size_t *bytes);

/* out64 (device, 1 double): the FP64-combined result; out32 (device, 1
 * float, may be NULL): the same rounded to float, which is what NT2's
 * sum(table<float>) returns.  y == NULL -> sum(x). */
nt2g_status nt2g_reduce_f32(const float *x, const float *y, int64_t n, void *workspace,
                            size_t workspace_bytes, double *out64, float *out32, void *stream);

/* The same reduction for callers that cannot allocate device memory: hosts
 * whose runtime owns every device allocation through its own pool, code that
 * must not risk cudaMalloc/cudaFree synchronizing the device, thin wrappers
 * with nowhere to keep a workspace.  Its scratch (a block ticket and one
 * FP64 partial per block, at most 4864 blocks: 39,168 bytes) is a static
 * device array inside the library, held by every GPU that loads it until the
 * process exits; it never calls cudaMalloc or cudaFree.  The first call on a
 * device looks up that array's device address (with the device current);
 * make that first call before any stream capture.  The address is cached per
 * device and context: after cudaDeviceReset the next call looks it up again
 * in the new context (make that call before a capture too).  All calls share the one
 * array, so calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller.  A launch that would need more block
 * partials than the array holds is rejected with NT2G_ERR_UNSUPPORTED.
 * No counterpart in the reference (NT2 allocates its reduction temporaries
 * on the host). */
nt2g_status nt2g_reduce_f32_noalloc(const float *x, const float *y, int64_t n, double *out64,
                                    float *out32, void *stream);

/* ------------------------------------------------------------------ */
/* Batched uneven tables: one persistent launch over many tables, each */
/* with its own expression.                                             */
/* ------------------------------------------------------------------ */
/* Items name one of the three library expressions, or carry a compiled
 * program (NT2G_BATCH_PROGRAM) with its arguments -- NT2's one generated
 * kernel per expression (tools/kernel_gen/kernel_gen.cpp:64-76), here every
 * distinct program of the batch linked into one run-time compiled kernel
 * that dispatches on the program block-uniformly, one tile at a time.  A run
 * is one persistent launch for the library expressions and one for the
 * programs (either absent when it has no items).  Program items evaluate
 * exactly as nt2g_eval with force_generic = 1 does. */

typedef enum nt2g_batch_expr {
    NT2G_BATCH_BLACKSCHOLES = 0, /* in0=S in1=K in2=T, out0=call out1=put, s0=sigma s1=r */
    NT2G_BATCH_SAXPY = 1,        /* in0=X, out0=Y (in place), s0=alpha */
    NT2G_BATCH_EXPR3 = 2,        /* in0=x in1=y in2=z, out0 */
    NT2G_BATCH_PROGRAM = 3       /* program over args: any compiled elementwise program without FOLD */
} nt2g_batch_expr;

typedef struct nt2g_batch_item {
    int32_t expr;                /* nt2g_batch_expr */
    int32_t n_args;              /* NT2G_BATCH_PROGRAM: entries of args */
    int64_t n;                   /* elements of the table */
    const float *in[3];
    float *out[2];
    float s[2];
    const nt2g_program *program; /* NT2G_BATCH_PROGRAM: the element program (outlives the batch) */
    const nt2g_arg *args;        /* NT2G_BATCH_PROGRAM: its slots, read by nt2g_batch_create */
} nt2g_batch_item;

typedef struct nt2g_batch_tune {
    int32_t block_threads;     /* 128..1024, multiple of 32 */
    int32_t blocks_per_sm;     /* resident blocks per SM of the persistent grid */
    int32_t tile_vectors;      /* float4 vectors per tile per thread */
    int32_t precision;         /* nt2g_precision */
    int32_t vector_width;      /* float4 vectors a thread has in flight per step: 1 or 2 (0 = 1) */
    int32_t reserved;
} nt2g_batch_tune;

typedef struct nt2g_batch nt2g_batch;

/* Upload the item table and its tile prefix sums (allocates device memory
 * once, here; runs allocate nothing). */
nt2g_status nt2g_batch_create(const nt2g_batch_item *items, int32_t n_items,
                              const nt2g_batch_tune *tune, nt2g_batch **out);
void nt2g_batch_destroy(nt2g_batch *b);
/* One persistent launch over every tile of every table. */
nt2g_status nt2g_batch_run(nt2g_batch *b, void *stream);
/* The comparison path: one plain launch per table, same kernels. */
nt2g_status nt2g_batch_run_per_table(nt2g_batch *b, void *stream);
/* Capture nt2g_batch_run into a CUDA graph on `stream` once; later calls
 * replay it. */
nt2g_status nt2g_batch_run_graph(nt2g_batch *b, void *stream);
/* Autotuner: times nt2g_batch_run for each candidate tune (NULL: a built-in
 * grid over block size, float4 vectors per thread per tile and resident
 * blocks per SM / static striding) and returns the fastest, with its time per
 * run.  Plans are built per candidate (device memory allocated at tuning
 * time); in-place expressions are applied once per timed run. */
nt2g_status nt2g_batch_autotune(const nt2g_batch_item *items, int32_t n_items,
                                const nt2g_batch_tune *candidates, int32_t n_candidates, int32_t reps,
                                int32_t precision, void *stream, nt2g_batch_tune *best, float *best_ms);
/* Total elements and algorithmic bytes of the batch. */
nt2g_status nt2g_batch_stats(const nt2g_batch *b, int64_t *elements, int64_t *bytes);
/* The CUDA source nt2g_batch_create compiles for a batch whose distinct
 * programs are programs[0..n_programs) (no GPU needed; *len receives the size
 * including the terminating NUL, cap = 0 only queries it).  Exposes the
 * generated code for inspection and compile checks; no counterpart in the
 * reference. */
nt2g_status nt2g_batch_source(const nt2g_program *const *programs, int32_t n_programs, int32_t precision,
                              int32_t block_threads, char *buf, size_t cap, size_t *len);

/* Bounded waits that gave up so far, process-wide (kernels that wait on an
 * mbarrier -- the pipelined Black-Scholes -- poll a limited number of times,
 * count a timeout here and return; nothing ever spins forever).  0 on a
 * healthy device.  Synchronises with the device. */
nt2g_status nt2g_wait_timeouts(uint64_t *count);

/* ------------------------------------------------------------------ */
/* Device memory for the table layer: nt2::table<T, device_> storage   */
/* (CUDA/sdk/memory/cuda/allocator.hpp:59-74, copies                   */
/* CUDA/memory/functions/cuda/copy.hpp:52-86).                         */
/* ------------------------------------------------------------------ */
nt2g_status nt2g_device_alloc(size_t bytes, void **ptr);
nt2g_status nt2g_device_free(void *ptr);
/* kind: 1 host->device, 2 device->host, 3 device->device */
nt2g_status nt2g_memcpy(void *dst, const void *src, size_t bytes, int32_t kind, void *stream);
nt2g_status nt2g_stream_synchronize(void *stream);
/* The calling thread's current device (the table layer keys its per-thread
 * reduction scratch on it; NT2 keeps its device in CUDA/sdk/cuda/settings). */
nt2g_status nt2g_device_current(int32_t *device);
/* A non-blocking stream for the table layer's evaluation options (callers
 * that do not link the CUDA runtime themselves). */
nt2g_status nt2g_stream_create(void **stream);
nt2g_status nt2g_stream_destroy(void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NT2G_H */
