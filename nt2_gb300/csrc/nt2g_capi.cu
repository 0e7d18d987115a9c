// nt2g_capi.cu -- the C ABI of libnt2gpu: argument validation, status codes,
// the expression-program compiler, and the dispatch from a compiled program
// to a fused kernel or to the generic interpreter.
//
// The program compiler takes the lowered form of an nt2 expression (SSA op
// list, see nt2g.h), and
//   1. validates opcodes, operand order, dtypes and slot use;
//   2. forwards stores to later loads of the same table (the element-
//      synchronous semantics of NT2's tie(), TABLE/core/functions/expr/
//      tie.hpp:40-121: a child may read a table an earlier child wrote);
//   3. removes common subexpressions and dead code;
//   4. allocates interpreter registers (linear scan);
//   5. binds the program to a fused kernel when it is structurally one of
//      the named expressions (same DAG modulo slot numbering), recording which
//      argument slot plays which role.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <map>
#include <new>
#include <tuple>
#include <vector>
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

// ------------------------------------------------------------------ errors --
static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

nt2g_status cuda_status(cudaError_t e, const char *what)
{
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    cudaGetLastError();  // clear a non-sticky error so the context stays usable
    return NT2G_ERR_CUDA;
}

int device_sm_count()
{
    static thread_local int cache_dev = -1, cache_sms = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != cache_dev) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
        cache_dev = dev;
        cache_sms = sms;
    }
    return cache_sms;
}

// ------------------------------------------------------------ host tables --
// Tables may live in host memory the device can reach: pinned or registered
// host memory everywhere, any host memory where the device has pageable
// memory access (Grace-Blackwell's NVLink-C2C with ATS, or HMM).  The kernels
// then read and write them in place over the host link.  A host pointer the
// device cannot reach is rejected before a launch instead of faulting.
static bool pageable_access()
{
    static thread_local int cache_dev = -1, cache_val = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return false; }
    if (dev != cache_dev) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) { cudaGetLastError(); v = 0; }
        cache_dev = dev;
        cache_val = v;
    }
    return cache_val != 0;
}

bool reachable(const void *p)
{
    if (!p || pageable_access()) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type != cudaMemoryTypeUnregistered;
}

// ---------------------------------------------------------------- patterns --
// P_NEG matches -x: a NEG node over its child, or -- when the child is a
// scalar role -- a constant or scalar argument holding the negated value
// (what C++ produces for -r*T with a float r: the negation happens before
// the expression is built).
// P_FOLD matches fma(sqr(x), c, y) -- or, when x and y are scalars, the
// float constant C++ computes for it before building the expression (NT2's
// scalar fma/sqr run on the host: x*x, *c, +y, each rounded); the constant is
// checked against the bound x and y once the whole match is known.
enum PKind { P_OP, P_TABLE, P_SCALAR, P_TABSCAL, P_CVAL, P_NEG, P_FOLD };

struct PNode {
    PKind kind;
    int code, dtype;
    int ch[3];
    int role;
    float cval;
};

struct Pattern {
    FusedKernel kernel;
    const char *name;
    std::vector<PNode> nodes;
    std::vector<std::pair<int, int>> outs;  // (node, output role)
    int n_roles;
};

struct PB {
    Pattern p;
    int add(PNode n) { p.nodes.push_back(n); return (int)p.nodes.size() - 1; }
    int op(int code, int a, int b = -1, int c = -1, int dt = NT2G_F32)
    {
        return add(PNode{P_OP, code, dt, {a, b, c}, -1, 0.f});
    }
    int table(int role, int dt = NT2G_F32) { return add(PNode{P_TABLE, 0, dt, {-1, -1, -1}, role, 0.f}); }
    int scalar(int role) { return add(PNode{P_SCALAR, 0, NT2G_F32, {-1, -1, -1}, role, 0.f}); }
    int tabscal(int role) { return add(PNode{P_TABSCAL, 0, NT2G_F32, {-1, -1, -1}, role, 0.f}); }
    int cval(float v, int dt = NT2G_F32) { return add(PNode{P_CVAL, 0, dt, {-1, -1, -1}, -1, v}); }
    int neg(int a) { return add(PNode{P_NEG, NT2G_OP_NEG, NT2G_F32, {a, -1, -1}, -1, 0.f}); }
    int fold_fma_sqr(int x, float c, int y)
    {
        int full = op(NT2G_OP_FMA, op(NT2G_OP_SQR, x), cval(c), y);
        return add(PNode{P_FOLD, 0, NT2G_F32, {full, x, y}, -1, c});
    }
    void out(int node, int role) { p.outs.push_back({node, role}); }
};

static std::vector<Pattern> build_patterns()
{
    std::vector<Pattern> v;
    {  // textbook Black-Scholes; roles S0 K1 T2 SIG3 R4 | CALL5 PUT6
        PB b;
        b.p.kernel = kBlackScholes; b.p.name = "blackscholes"; b.p.n_roles = 7;
        int S = b.table(0), K = b.table(1), T = b.table(2), sig = b.tabscal(3), r = b.scalar(4);
        int sq = b.op(NT2G_OP_SQRT, T);
        int lq = b.op(NT2G_OP_LOG, b.op(NT2G_OP_DIV, S, K));
        int a = b.fold_fma_sqr(sig, 0.5f, r);
        int d1 = b.op(NT2G_OP_DIV, b.op(NT2G_OP_ADD, lq, b.op(NT2G_OP_MUL, a, T)), b.op(NT2G_OP_MUL, sig, sq));
        int d2 = b.op(NT2G_OP_FNMS, sig, sq, d1);
        int e = b.op(NT2G_OP_MUL, K, b.op(NT2G_OP_EXP, b.op(NT2G_OP_MUL, b.neg(r), T)));
        int call = b.op(NT2G_OP_FNMS, e, b.op(NT2G_OP_NORMCDF, d2), b.op(NT2G_OP_MUL, S, b.op(NT2G_OP_NORMCDF, d1)));
        int put = b.op(NT2G_OP_FNMS, S, b.op(NT2G_OP_NORMCDF, b.neg(d1)),
                       b.op(NT2G_OP_MUL, e, b.op(NT2G_OP_NORMCDF, b.neg(d2))));
        b.out(call, 5);
        b.out(put, 6);
        v.push_back(b.p);
    }
    {  // NT2 demo Black-Scholes; roles S0 X1 T2 R3 V4 | OUT5
        PB b;
        b.p.kernel = kBlackScholesDemo; b.p.name = "blackscholes_demo"; b.p.n_roles = 6;
        int S = b.table(0), X = b.table(1), T = b.table(2), r = b.tabscal(3), va = b.tabscal(4);
        int da = b.op(NT2G_OP_SQRT, T);
        int d1 = b.op(NT2G_OP_ADD, b.op(NT2G_OP_LOG, b.op(NT2G_OP_DIV, S, X)),
                      b.op(NT2G_OP_DIV, b.op(NT2G_OP_MUL, b.fold_fma_sqr(va, 0.5f, r), T),
                           b.op(NT2G_OP_MUL, va, da)));
        int d2 = b.op(NT2G_OP_FNMS, va, da, d1);
        int R = b.op(NT2G_OP_FNMS, b.op(NT2G_OP_MUL, X, b.op(NT2G_OP_EXP, b.op(NT2G_OP_MUL, b.neg(r), T))),
                     b.op(NT2G_OP_FASTNORMCDF, d2), b.op(NT2G_OP_MUL, S, b.op(NT2G_OP_FASTNORMCDF, d1)));
        b.out(R, 5);
        v.push_back(b.p);
    }
    {  // saxpy; roles A0 X1 Y2 | OUT3
        PB b;
        b.p.kernel = kSaxpy; b.p.name = "saxpy"; b.p.n_roles = 4;
        int A = b.scalar(0), X = b.table(1), Y = b.table(2);
        b.out(b.op(NT2G_OP_ADD, b.op(NT2G_OP_MUL, A, X), Y), 3);
        v.push_back(b.p);
    }
    {  // expr3; roles x0 y1 z2 | OUT3
        PB b;
        b.p.kernel = kExpr3; b.p.name = "expr3"; b.p.n_roles = 4;
        int x = b.table(0), y = b.table(1), z = b.table(2);
        int t = b.op(NT2G_OP_MUL, b.op(NT2G_OP_EXP, b.op(NT2G_OP_NEG, b.op(NT2G_OP_SQR, x))),
                     b.op(NT2G_OP_SQRT, b.op(NT2G_OP_ABS, y)));
        b.out(b.op(NT2G_OP_ADD, t, b.op(NT2G_OP_LOG1P, b.op(NT2G_OP_ABS, z))), 3);
        v.push_back(b.p);
    }
    {  // rgb2yuv; roles r0 g1 b2 | Y3 U4 V5
        PB b;
        b.p.kernel = kRgb2Yuv; b.p.name = "rgb2yuv"; b.p.n_roles = 6;
        int r = b.table(0), g = b.table(1), bl = b.table(2);
        int y = b.op(NT2G_OP_ADD, b.op(NT2G_OP_ADD, b.op(NT2G_OP_MUL, b.cval(0.299f), r), b.op(NT2G_OP_MUL, b.cval(0.587f), g)),
                     b.op(NT2G_OP_MUL, b.cval(0.114f), bl));
        b.out(y, 3);
        b.out(b.op(NT2G_OP_MUL, b.cval(0.492f), b.op(NT2G_OP_SUB, bl, y)), 4);
        b.out(b.op(NT2G_OP_MUL, b.cval(0.877f), b.op(NT2G_OP_SUB, r, y)), 5);
        v.push_back(b.p);
    }
    {  // sigma-delta; roles frame0 bkg1 var2 | BKG3 VAR4 LABEL5
        PB b;
        const int U = NT2G_U8;
        b.p.kernel = kSigmaDelta; b.p.name = "sigmadelta"; b.p.n_roles = 6;
        int f = b.table(0, U), bk = b.table(1, U), va = b.table(2, U);
        int nb = b.op(NT2G_OP_SELINC, b.op(NT2G_OP_LT, bk, f, -1, U), b.op(NT2G_OP_SELDEC, b.op(NT2G_OP_GT, bk, f, -1, U), bk, -1, U), -1, U);
        int d = b.op(NT2G_OP_SUB, b.op(NT2G_OP_MAX, nb, f, -1, U), b.op(NT2G_OP_MIN, nb, f, -1, U), -1, U);
        int m = b.op(NT2G_OP_ADDS, b.op(NT2G_OP_ADDS, d, d, -1, U), d, -1, U);
        int nv = b.op(NT2G_OP_IF_ELSE, b.op(NT2G_OP_NE, d, b.cval(0.f, U), -1, U),
                      b.op(NT2G_OP_SELINC, b.op(NT2G_OP_LT, va, m, -1, U), b.op(NT2G_OP_SELDEC, b.op(NT2G_OP_GT, va, m, -1, U), va, -1, U), -1, U),
                      va, U);
        int lab = b.op(NT2G_OP_IF_ZERO_ELSE_ONE, b.op(NT2G_OP_LT, d, nv, -1, U), -1, -1, U);
        b.out(nb, 3);
        b.out(nv, 4);
        b.out(lab, 5);
        v.push_back(b.p);
    }
    return v;
}

static const std::vector<Pattern> &patterns()
{
    static const std::vector<Pattern> p = build_patterns();
    return p;
}

// A role resolves to a table slot, a constant, or a scalar slot (possibly
// holding the negated value).
struct RoleBind {
    int kind = -1;  // 0 table slot, 1 const, 2 scalar slot, 3 negated scalar slot
    int slot = -1;
    float value = 0.f;
};

struct DeferredConst {
    int slot;
    float value;
};

// A folded fma(sqr(x), c, y) constant to verify against the roles x, y.
struct DeferredFold {
    float value, c;
    int x_role, y_role;
};

// NT2's scalar fma(sqr(x), c, y) in float: three separately rounded steps
// (volatile keeps the host compiler from contracting them).
static float nt2_fold(float x, float c, float y)
{
    volatile float sq = x * x;
    volatile float m = sq * c;
    volatile float r = m + y;
    return r;
}

}  // namespace nt2g

using namespace nt2g;

struct nt2g_program {
    std::vector<nt2g_op> ops;  // canonical SSA
    std::vector<uint8_t> logical;
    int n_slots = 0;
    std::vector<int> slot_use;    // bit 1 load, 2 store, 4 scalar
    std::vector<int> slot_dtype;
    DProgram dprog{};
    int kernel = kGeneric;
    const char *kernel_name = "generic";
    std::vector<RoleBind> roles;
    std::vector<DeferredConst> deferred;
    bool folds = false;  // the program's value is folded (nt2g_eval_fold), it stores nothing
};

namespace nt2g {

static bool is_value_op(int code) { return code != NT2G_OP_STORE && code != NT2G_OP_FOLD; }

static int n_operands(int code)
{
    switch (code) {
    case NT2G_OP_LOAD: case NT2G_OP_SCALAR: case NT2G_OP_CONST: case NT2G_OP_INDEX: return 0;
    case NT2G_OP_STORE: case NT2G_OP_FOLD: return 1;
    case NT2G_OP_NEG: case NT2G_OP_ABS: case NT2G_OP_SQR: case NT2G_OP_SQRT: case NT2G_OP_REC:
    case NT2G_OP_EXP: case NT2G_OP_LOG: case NT2G_OP_LOG1P: case NT2G_OP_ERFC: case NT2G_OP_NORMCDF:
    case NT2G_OP_FASTNORMCDF: case NT2G_OP_IF_ZERO_ELSE_ONE: case NT2G_OP_EXP2: case NT2G_OP_EXP10:
    case NT2G_OP_EXPM1: case NT2G_OP_LOG2: case NT2G_OP_LOG10: case NT2G_OP_SIN: case NT2G_OP_COS:
    case NT2G_OP_TAN: case NT2G_OP_SINPI: case NT2G_OP_COSPI: case NT2G_OP_SINH: case NT2G_OP_COSH:
    case NT2G_OP_TANH: case NT2G_OP_ASIN: case NT2G_OP_ACOS: case NT2G_OP_ATAN: case NT2G_OP_ASINH:
    case NT2G_OP_ACOSH: case NT2G_OP_ATANH: case NT2G_OP_CBRT: case NT2G_OP_COT: case NT2G_OP_SEC:
    case NT2G_OP_CSC: case NT2G_OP_SIND: case NT2G_OP_COSD: case NT2G_OP_TAND:
    case NT2G_OP_TANPI: case NT2G_OP_PROPER_TANPI: case NT2G_OP_COTPI: case NT2G_OP_COTD: case NT2G_OP_SECPI:
    case NT2G_OP_CSCPI:
    case NT2G_OP_SECD: case NT2G_OP_CSCD: case NT2G_OP_SINC: case NT2G_OP_SINCPI: case NT2G_OP_ACOTD:
    case NT2G_OP_ASEC: case NT2G_OP_COTH: case NT2G_OP_SINHC:
    case NT2G_OP_ACSC: case NT2G_OP_ASECH: case NT2G_OP_ACOTH: case NT2G_OP_ACSCH:
    case NT2G_OP_ERF: case NT2G_OP_ERFCX: case NT2G_OP_EXPX2: case NT2G_OP_GAMMA: case NT2G_OP_GAMMALN:
    case NT2G_OP_EXPRECNEG: case NT2G_OP_EXPRECNEGC: case NT2G_OP_SQRT1PM1: case NT2G_OP_ERFINV:
    case NT2G_OP_ERFCINV: case NT2G_OP_SIGNGAM: case NT2G_OP_DIGAMMA: case NT2G_OP_DAWSON: case NT2G_OP_SPENCE: case NT2G_OP_STIRLING:
    case NT2G_OP_FLOOR: case NT2G_OP_CEIL: case NT2G_OP_TRUNC: case NT2G_OP_ROUND: case NT2G_OP_ROUND2EVEN:
    case NT2G_OP_FRAC: case NT2G_OP_SIGN: case NT2G_OP_SIGNNZ:
    case NT2G_OP_IS_NAN: case NT2G_OP_IS_INF: case NT2G_OP_IS_FINITE: case NT2G_OP_IS_EQZ: case NT2G_OP_IS_NEZ:
    case NT2G_OP_IS_LTZ: case NT2G_OP_IS_GTZ: return 1;
    case NT2G_OP_ADD: case NT2G_OP_SUB: case NT2G_OP_MUL: case NT2G_OP_DIV: case NT2G_OP_MIN: case NT2G_OP_MAX:
    case NT2G_OP_LT: case NT2G_OP_GT: case NT2G_OP_LE: case NT2G_OP_GE: case NT2G_OP_EQ: case NT2G_OP_NE:
    case NT2G_OP_SELINC: case NT2G_OP_SELDEC: case NT2G_OP_ADDS: case NT2G_OP_POW:
    case NT2G_OP_ATAN2: case NT2G_OP_HYPOT: case NT2G_OP_COPYSIGN: case NT2G_OP_NTHROOT: case NT2G_OP_EXPNI:
    case NT2G_OP_GAMMAINC: case NT2G_OP_GAMMAINCINV: case NT2G_OP_MOD: case NT2G_OP_REM:
    case NT2G_OP_POW2: return 2;
    case NT2G_OP_FMA: case NT2G_OP_FNMS: case NT2G_OP_IF_ELSE: return 3;
    default: return -1;
    }
}

static bool float_only(int code)
{
    switch (code) {
    case NT2G_OP_DIV: case NT2G_OP_SQRT: case NT2G_OP_REC: case NT2G_OP_FMA: case NT2G_OP_FNMS:
    case NT2G_OP_EXP: case NT2G_OP_LOG: case NT2G_OP_LOG1P: case NT2G_OP_ERFC: case NT2G_OP_NORMCDF:
    case NT2G_OP_FASTNORMCDF: case NT2G_OP_EXP2: case NT2G_OP_EXP10: case NT2G_OP_EXPM1:
    case NT2G_OP_LOG2: case NT2G_OP_LOG10: case NT2G_OP_SIN: case NT2G_OP_COS: case NT2G_OP_TAN:
    case NT2G_OP_SINPI: case NT2G_OP_COSPI: case NT2G_OP_POW: case NT2G_OP_SINH: case NT2G_OP_COSH:
    case NT2G_OP_TANH: case NT2G_OP_ASIN: case NT2G_OP_ACOS: case NT2G_OP_ATAN: case NT2G_OP_ATAN2:
    case NT2G_OP_ASINH: case NT2G_OP_ACOSH: case NT2G_OP_ATANH: case NT2G_OP_CBRT: case NT2G_OP_HYPOT:
    case NT2G_OP_COT: case NT2G_OP_SEC: case NT2G_OP_CSC: case NT2G_OP_SIND: case NT2G_OP_COSD: case NT2G_OP_TAND:
    case NT2G_OP_TANPI: case NT2G_OP_PROPER_TANPI: case NT2G_OP_COTPI: case NT2G_OP_COTD: case NT2G_OP_SECPI:
    case NT2G_OP_CSCPI:
    case NT2G_OP_SECD: case NT2G_OP_CSCD: case NT2G_OP_SINC: case NT2G_OP_SINCPI: case NT2G_OP_ACOTD:
    case NT2G_OP_ASEC: case NT2G_OP_COTH: case NT2G_OP_SINHC:
    case NT2G_OP_ACSC: case NT2G_OP_ASECH: case NT2G_OP_ACOTH: case NT2G_OP_ACSCH:
    case NT2G_OP_ERF: case NT2G_OP_ERFCX: case NT2G_OP_EXPX2: case NT2G_OP_GAMMA: case NT2G_OP_GAMMALN:
    case NT2G_OP_EXPRECNEG: case NT2G_OP_EXPRECNEGC: case NT2G_OP_SQRT1PM1: case NT2G_OP_ERFINV:
    case NT2G_OP_ERFCINV: case NT2G_OP_SIGNGAM: case NT2G_OP_DIGAMMA: case NT2G_OP_DAWSON: case NT2G_OP_SPENCE: case NT2G_OP_STIRLING:
    case NT2G_OP_NTHROOT: case NT2G_OP_EXPNI: case NT2G_OP_GAMMAINC: case NT2G_OP_GAMMAINCINV:
    case NT2G_OP_FLOOR: case NT2G_OP_CEIL: case NT2G_OP_TRUNC: case NT2G_OP_ROUND: case NT2G_OP_ROUND2EVEN:
    case NT2G_OP_FRAC: case NT2G_OP_SIGN: case NT2G_OP_SIGNNZ: case NT2G_OP_COPYSIGN: case NT2G_OP_MOD:
    case NT2G_OP_REM: case NT2G_OP_POW2:
    case NT2G_OP_IS_NAN: case NT2G_OP_IS_INF: case NT2G_OP_IS_FINITE: case NT2G_OP_IS_EQZ: case NT2G_OP_IS_NEZ:
    case NT2G_OP_IS_LTZ: case NT2G_OP_IS_GTZ:
        return true;
    default: return false;
    }
}

static bool is_compare(int code)
{
    return (code >= NT2G_OP_LT && code <= NT2G_OP_NE) || (code >= NT2G_OP_IS_NAN && code <= NT2G_OP_IS_GTZ);
}

// Structural match of program value v against pattern node pn.
struct Matcher {
    const nt2g_program &prog;
    const Pattern &pat;
    std::vector<int> pmap;  // pattern node -> program value
    std::vector<RoleBind> roles;
    std::vector<DeferredConst> deferred;
    std::vector<DeferredFold> folds;

    Matcher(const nt2g_program &p, const Pattern &q)
        : prog(p), pat(q), pmap(q.nodes.size(), -1), roles(q.n_roles) {}

    bool bind_role(int role, RoleBind rb)
    {
        RoleBind &r = roles[role];
        if (r.kind < 0) { r = rb; return true; }
        return r.kind == rb.kind && r.slot == rb.slot && (r.kind != 1 || r.value == rb.value);
    }

    bool match(int v, int pn)
    {
        if (pmap[pn] >= 0) return pmap[pn] == v;
        const PNode &n = pat.nodes[pn];
        const nt2g_op &o = prog.ops[v];
        bool ok = false;
        switch (n.kind) {
        case P_TABLE:
            ok = o.code == NT2G_OP_LOAD && o.dtype == n.dtype && bind_role(n.role, RoleBind{0, o.a, 0.f});
            break;
        case P_SCALAR:
            ok = (o.code == NT2G_OP_CONST && o.dtype == NT2G_F32 && bind_role(n.role, RoleBind{1, -1, o.imm})) ||
                 (o.code == NT2G_OP_SCALAR && o.dtype == NT2G_F32 && bind_role(n.role, RoleBind{2, o.a, 0.f}));
            break;
        case P_TABSCAL:
            ok = (o.code == NT2G_OP_LOAD && o.dtype == NT2G_F32 && bind_role(n.role, RoleBind{0, o.a, 0.f})) ||
                 (o.code == NT2G_OP_CONST && o.dtype == NT2G_F32 && bind_role(n.role, RoleBind{1, -1, o.imm})) ||
                 (o.code == NT2G_OP_SCALAR && o.dtype == NT2G_F32 && bind_role(n.role, RoleBind{2, o.a, 0.f}));
            break;
        case P_CVAL:
            if (o.code == NT2G_OP_CONST && o.dtype == n.dtype) ok = o.imm == n.cval;
            else if (o.code == NT2G_OP_SCALAR && o.dtype == n.dtype) {
                deferred.push_back(DeferredConst{o.a, n.cval});
                ok = true;
            }
            break;
        case P_NEG: {
            const PNode &c = pat.nodes[n.ch[0]];
            const bool scalar_role = c.kind == P_SCALAR || c.kind == P_TABSCAL;
            if (o.code == NT2G_OP_NEG && o.dtype == NT2G_F32) ok = match(o.a, n.ch[0]);
            else if (scalar_role && o.code == NT2G_OP_CONST && o.dtype == NT2G_F32)
                ok = bind_role(c.role, RoleBind{1, -1, -o.imm});
            else if (scalar_role && o.code == NT2G_OP_SCALAR && o.dtype == NT2G_F32)
                ok = bind_role(c.role, RoleBind{3, o.a, 0.f});
            break;
        }
        case P_FOLD: {
            if (o.code == NT2G_OP_CONST && o.dtype == NT2G_F32) {
                folds.push_back(DeferredFold{o.imm, n.cval, pat.nodes[n.ch[1]].role, pat.nodes[n.ch[2]].role});
                ok = true;
            } else {
                ok = match(v, n.ch[0]);
            }
            break;
        }
        case P_OP:
            if (o.code != n.code || o.dtype != n.dtype) break;
            ok = true;
            for (int k = 0; k < n_operands(n.code) && ok; ++k) {
                int pv = k == 0 ? o.a : k == 1 ? o.b : o.c;
                ok = match(pv, n.ch[k]);
            }
            break;
        }
        if (ok) pmap[pn] = v;
        return ok;
    }
};

static bool try_bind(nt2g_program &p, const Pattern &pat)
{
    // stores of the program, in order
    std::vector<int> stores;
    for (int i = 0; i < (int)p.ops.size(); ++i)
        if (p.ops[i].code == NT2G_OP_STORE) stores.push_back(i);
    if (stores.size() != pat.outs.size()) return false;
    Matcher m(p, pat);
    for (size_t k = 0; k < stores.size(); ++k) {
        const nt2g_op &s = p.ops[stores[k]];
        if (!m.bind_role(pat.outs[k].second, RoleBind{0, s.b, 0.f})) return false;
        if (!m.match(s.a, pat.outs[k].first)) return false;
    }
    for (const RoleBind &r : m.roles)
        if (r.kind < 0) return false;
    for (const DeferredFold &f : m.folds) {
        const RoleBind &x = m.roles[f.x_role], &y = m.roles[f.y_role];
        if (x.kind != 1 || y.kind != 1 || nt2_fold(x.value, f.c, y.value) != f.value) return false;
    }
    p.kernel = pat.kernel;
    p.kernel_name = pat.name;
    p.roles = m.roles;
    p.deferred = m.deferred;
    return true;
}

}  // namespace nt2g

// ------------------------------------------------------------------ C ABI --
extern "C" const char *nt2g_last_error(void) { return g_err; }
extern "C" int nt2g_abi_version(void) { return NT2G_ABI_VERSION; }

extern "C" nt2g_status nt2g_program_create(const nt2g_op *ops, int32_t n_ops, int32_t n_slots, nt2g_program **out)
{
    NT2G_CHECK_ARG(out != nullptr, "nt2g_program_create: out is NULL");
    *out = nullptr;
    NT2G_CHECK_ARG(ops != nullptr && n_ops > 0, "nt2g_program_create: empty program");
    NT2G_CHECK_ARG(n_slots > 0 && n_slots <= kMaxSlots, "nt2g_program_create: n_slots %d outside [1,%d]", n_slots,
                   kMaxSlots);
    std::vector<int> slot_use(n_slots, 0), slot_dtype(n_slots, -1);
    std::vector<uint8_t> logical(n_ops, 0);
    int n_fold = 0;
    // 1. validation
    for (int i = 0; i < n_ops; ++i) {
        const nt2g_op &o = ops[i];
        int na = n_operands(o.code);
        NT2G_CHECK_ARG(na >= 0, "op %d: unknown opcode %d", i, o.code);
        NT2G_CHECK_ARG(o.dtype == NT2G_F32 || o.dtype == NT2G_U8, "op %d: unknown dtype %d", i, o.dtype);
        if (o.dtype == NT2G_U8 && float_only(o.code)) {
            set_error("op %d: opcode %d is defined for float tables only", i, o.code);
            return NT2G_ERR_UNSUPPORTED;
        }
        if (o.code == NT2G_OP_ADDS && o.dtype != NT2G_U8) {
            set_error("op %d: saturating add is defined for uint8 tables only", i);
            return NT2G_ERR_UNSUPPORTED;
        }
        const int32_t opnd[3] = {o.a, o.b, o.c};
        if (o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR) {
            NT2G_CHECK_ARG(o.a >= 0 && o.a < n_slots, "op %d: slot %d outside [0,%d)", i, o.a, n_slots);
            int use = o.code == NT2G_OP_LOAD ? 1 : 4;
            NT2G_CHECK_ARG(!((slot_use[o.a] | use) & 4) || (slot_use[o.a] | use) == 4,
                           "op %d: slot %d used both as a table and as a scalar", i, o.a);
            NT2G_CHECK_ARG(slot_dtype[o.a] < 0 || slot_dtype[o.a] == o.dtype, "op %d: slot %d dtype mismatch", i, o.a);
            slot_use[o.a] |= use;
            slot_dtype[o.a] = o.dtype;
            continue;
        }
        if (o.code == NT2G_OP_STORE) {
            NT2G_CHECK_ARG(o.a >= 0 && o.a < i && is_value_op(ops[o.a].code), "op %d: store of invalid value %d", i, o.a);
            NT2G_CHECK_ARG(o.b >= 0 && o.b < n_slots, "op %d: slot %d outside [0,%d)", i, o.b, n_slots);
            NT2G_CHECK_ARG(!(slot_use[o.b] & 4), "op %d: store into scalar slot %d", i, o.b);
            NT2G_CHECK_ARG(slot_dtype[o.b] < 0 || slot_dtype[o.b] == o.dtype, "op %d: slot %d dtype mismatch", i, o.b);
            NT2G_CHECK_ARG(logical[o.a] || ops[o.a].dtype == o.dtype, "op %d: stored value dtype %d into dtype %d", i,
                           ops[o.a].dtype, o.dtype);
            slot_use[o.b] |= 2;
            slot_dtype[o.b] = o.dtype;
            continue;
        }
        if (o.code == NT2G_OP_FOLD) {
            NT2G_CHECK_ARG(o.a >= 0 && o.a < i && is_value_op(ops[o.a].code), "op %d: fold of invalid value %d", i, o.a);
            NT2G_CHECK_ARG(logical[o.a] || ops[o.a].dtype == NT2G_F32, "op %d: the folded value is not a float", i);
            NT2G_CHECK_ARG(++n_fold == 1, "op %d: a program folds one value", i);
            continue;
        }
        for (int k = 0; k < na; ++k) {
            NT2G_CHECK_ARG(opnd[k] >= 0 && opnd[k] < i && is_value_op(ops[opnd[k]].code),
                           "op %d: operand %d refers to %d", i, k, opnd[k]);
        }
        bool cond_first = o.code == NT2G_OP_IF_ELSE || o.code == NT2G_OP_SELINC || o.code == NT2G_OP_SELDEC ||
                          o.code == NT2G_OP_IF_ZERO_ELSE_ONE;
        if (cond_first) NT2G_CHECK_ARG(logical[o.a], "op %d: condition operand is not a comparison result", i);
        for (int k = cond_first ? 1 : 0; k < na; ++k)
            NT2G_CHECK_ARG(!logical[opnd[k]] || o.code == NT2G_OP_IF_ELSE,
                           "op %d: logical operand %d used as a number", i, k);
        for (int k = cond_first ? 1 : 0; k < na; ++k)
            NT2G_CHECK_ARG(logical[opnd[k]] || ops[opnd[k]].dtype == o.dtype, "op %d: operand %d dtype mismatch", i, k);
        if (is_compare(o.code)) logical[i] = 1;
        if (o.code == NT2G_OP_IF_ELSE) {
            NT2G_CHECK_ARG(logical[o.b] == logical[o.c], "op %d: if_else branches of different kinds", i);
            logical[i] = logical[o.b];
        }
    }
    // 2-3. forwarding, CSE, then DCE
    std::vector<int> remap(n_ops, -1), last_store(n_slots, -1);
    std::vector<nt2g_op> cse;
    std::vector<uint8_t> cse_logical;
    std::map<std::tuple<int, int, int, int, int, uint32_t>, int> seen;
    for (int i = 0; i < n_ops; ++i) {
        nt2g_op o = ops[i];
        if (o.code == NT2G_OP_LOAD && last_store[o.a] >= 0) {  // forward the stored value
            remap[i] = last_store[o.a];
            continue;
        }
        int na = n_operands(o.code);
        if (o.code == NT2G_OP_STORE) {
            o.a = remap[o.a];
            last_store[o.b] = o.a;
            cse.push_back(o);
            cse_logical.push_back(logical[i]);
            continue;
        }
        if (o.code == NT2G_OP_FOLD) {
            o.a = remap[o.a];
            o.b = o.c = -1;
            cse.push_back(o);
            cse_logical.push_back(0);
            continue;
        }
        if (na >= 1 && o.code != NT2G_OP_LOAD && o.code != NT2G_OP_SCALAR) o.a = remap[o.a];
        if (na >= 2) o.b = remap[o.b];
        if (na >= 3) o.c = remap[o.c];
        if (na < 1 && (o.code == NT2G_OP_CONST || o.code == NT2G_OP_INDEX)) o.a = -1;
        if (na < 2) o.b = -1;
        if (na < 3) o.c = -1;
        uint32_t immbits = 0;
        if (o.code == NT2G_OP_CONST) memcpy(&immbits, &o.imm, 4);
        else o.imm = 0.f;
        auto key = std::make_tuple((int)o.code, (int)o.dtype, o.a, o.b, o.c, immbits);
        auto it = seen.find(key);
        if (it != seen.end()) { remap[i] = it->second; continue; }
        remap[i] = (int)cse.size();
        seen[key] = remap[i];
        cse.push_back(o);
        cse_logical.push_back(logical[i]);
    }
    // keep only the last store to each slot; mark live values
    std::vector<uint8_t> live(cse.size(), 0);
    std::vector<int> final_store(n_slots, -1);
    for (int i = 0; i < (int)cse.size(); ++i)
        if (cse[i].code == NT2G_OP_STORE) final_store[cse[i].b] = i;
    for (int i = (int)cse.size() - 1; i >= 0; --i) {
        const nt2g_op &o = cse[i];
        if (o.code == NT2G_OP_STORE) {
            if (final_store[o.b] != i) continue;
            live[i] = 1;
            live[o.a] = 1;
            continue;
        }
        if (o.code == NT2G_OP_FOLD) {
            live[i] = 1;
            live[o.a] = 1;
            continue;
        }
        if (!live[i]) continue;
        int na = n_operands(o.code);
        if (o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR || o.code == NT2G_OP_CONST) continue;
        if (na >= 1) live[o.a] = 1;
        if (na >= 2) live[o.b] = 1;
        if (na >= 3) live[o.c] = 1;
    }
    nt2g_program *p = new (std::nothrow) nt2g_program();
    if (!p) { set_error("nt2g_program_create: out of host memory"); return NT2G_ERR_NOMEM; }
    std::vector<int> idx(cse.size(), -1);
    for (int i = 0; i < (int)cse.size(); ++i) {
        if (!live[i]) continue;
        nt2g_op o = cse[i];
        int na = n_operands(o.code);
        bool slot_op = o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR;
        if (!slot_op && o.code != NT2G_OP_CONST) {
            if (na >= 1) o.a = idx[o.a];
            if (o.code != NT2G_OP_STORE && na >= 2) o.b = idx[o.b];
            if (na >= 3) o.c = idx[o.c];
        }
        idx[i] = (int)p->ops.size();
        p->ops.push_back(o);
        p->logical.push_back(cse_logical[i]);
    }
    p->n_slots = n_slots;
    p->slot_use = slot_use;
    p->slot_dtype = slot_dtype;
    bool has_store = false, has_fold = false;
    for (const nt2g_op &o : p->ops) {
        has_store |= o.code == NT2G_OP_STORE;
        has_fold |= o.code == NT2G_OP_FOLD;
    }
    if (has_store == has_fold) {
        delete p;
        set_error(has_fold ? "nt2g_program_create: a program either folds one value or stores"
                           : "nt2g_program_create: the program stores nothing");
        return NT2G_ERR_INVALID;
    }
    p->folds = has_fold;
    // 4. register allocation for the interpreter
    const int n = (int)p->ops.size();
    if (n > kMaxInstr) {
        delete p;
        set_error("nt2g_program_create: %d instructions after simplification exceed %d", n, kMaxInstr);
        return NT2G_ERR_UNSUPPORTED;
    }
    std::vector<int> last_use(n, -1), reg(n, -1);
    for (int i = 0; i < n; ++i) {
        const nt2g_op &o = p->ops[i];
        if (o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR || o.code == NT2G_OP_CONST) continue;
        int na = n_operands(o.code);
        if (na >= 1) last_use[o.a] = i;
        if (na >= 2 && o.code != NT2G_OP_STORE) last_use[o.b] = i;
        if (na >= 3) last_use[o.c] = i;
    }
    std::vector<int> free_regs;
    int n_regs = 0;
    DProgram &dp = p->dprog;
    dp.n = n;
    for (int i = 0; i < n; ++i) {
        const nt2g_op &o = p->ops[i];
        DInstr &d = dp.ins[i];
        d = DInstr{};
        d.op = (uint8_t)o.code;
        d.dt = (uint8_t)o.dtype;
        d.imm = o.imm;
        int na = n_operands(o.code);
        bool slot_op = o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR;
        if (slot_op) d.a = (uint8_t)o.a;
        else if (o.code == NT2G_OP_STORE) {
            d.a = (uint8_t)reg[o.a];
            d.b = (uint8_t)o.b;
            d.logical = p->logical[o.a];
        } else if (o.code != NT2G_OP_CONST) {
            if (na >= 1) d.a = (uint8_t)reg[o.a];
            if (na >= 2) d.b = (uint8_t)reg[o.b];
            if (na >= 3) d.c = (uint8_t)reg[o.c];
            // comparisons carry the compared dtype; conditions are the logical operand
        }
        // release operands whose last use is here (an operand register may be
        // reused as the destination: the interpreter reads element j of every
        // operand before writing element j of the result)
        if (!slot_op && o.code != NT2G_OP_CONST) {
            int opv[3] = {o.a, o.code == NT2G_OP_STORE ? -1 : o.b, o.c};
            for (int k = 0; k < (na < 3 ? na : 3); ++k) {
                int v = opv[k];
                if (v >= 0 && last_use[v] == i) {
                    bool dup = false;
                    for (int q = 0; q < k; ++q) dup |= opv[q] == v;
                    if (!dup) free_regs.push_back(reg[v]);
                }
            }
        }
        if (o.code != NT2G_OP_STORE) {
            if (last_use[i] < 0) { reg[i] = 0; d.dst = 0; continue; }  // unused value (cannot happen after DCE)
            int r;
            if (!free_regs.empty()) {
                // lowest free register keeps the file compact
                size_t best = 0;
                for (size_t q = 1; q < free_regs.size(); ++q)
                    if (free_regs[q] < free_regs[best]) best = q;
                r = free_regs[best];
                free_regs.erase(free_regs.begin() + best);
            } else {
                r = n_regs++;
            }
            reg[i] = r;
            d.dst = (uint8_t)r;
        }
    }
    dp.n_regs = n_regs;
    if (n_regs > kMaxRegs) {
        delete p;
        set_error("nt2g_program_create: %d live values exceed the %d interpreter registers", n_regs, kMaxRegs);
        return NT2G_ERR_UNSUPPORTED;
    }
    // 5. fused-kernel binding (transforms only)
    if (!p->folds)
        for (const Pattern &pat : patterns())
            if (try_bind(*p, pat)) break;
    *out = p;
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_program_info_get(const nt2g_program *p, nt2g_program_info *info)
{
    NT2G_CHECK_ARG(p && info, "nt2g_program_info_get: NULL argument");
    memset(info, 0, sizeof *info);
    info->kernel = p->kernel;
    info->n_ops = (int32_t)p->ops.size();
    info->n_regs = p->dprog.n_regs;
    info->n_slots = p->n_slots;
    snprintf(info->kernel_name, sizeof info->kernel_name, "%s", p->kernel_name);
    return NT2G_OK;
}

extern "C" void nt2g_program_destroy(nt2g_program *p) { delete p; }

static size_t dtype_size(int dt) { return dt == NT2G_U8 ? 1 : 4; }

// The device arguments of a program over elements [offset, offset + count):
// scalars converted, table pointers advanced to element `offset`, and (for a
// non-empty range) every table checked reachable from the device.
static nt2g_status bind_args(const nt2g_program *p, const nt2g_arg *args, int64_t offset, int64_t count,
                             const char *who, DArgs &da)
{
    da = DArgs{};
    da.pos0 = offset;
    for (int s = 0; s < p->n_slots; ++s) {
        const int use = p->slot_use[s];
        if (!use) continue;
        const nt2g_arg &a = args[s];
        if (use & 4) {
            NT2G_CHECK_ARG(a.kind == 1, "%s: slot %d must be a scalar", who, s);
            da.scal[s] = (float)a.scalar;
            double u = a.scalar;
            da.scal_u8[s] = (uint32_t)(u < 0 ? 0 : u > 255 ? 255 : u);
            da.dtype[s] = p->slot_dtype[s];
        } else {
            NT2G_CHECK_ARG(a.kind == 0, "%s: slot %d must be a table", who, s);
            NT2G_CHECK_ARG(a.dtype == p->slot_dtype[s], "%s: slot %d has dtype %d, program expects %d", who, s,
                           a.dtype, p->slot_dtype[s]);
            NT2G_CHECK_ARG(a.ptr != nullptr || count == 0, "%s: slot %d table pointer is NULL", who, s);
            da.ptr[s] = a.ptr ? (char *)a.ptr + offset * dtype_size(a.dtype) : nullptr;
            da.dtype[s] = a.dtype;
        }
    }
    if (count == 0) return NT2G_OK;
    for (int s = 0; s < p->n_slots; ++s)
        NT2G_CHECK_ARG(!(p->slot_use[s] & 3) || reachable(da.ptr[s]),
                       "%s: slot %d is host memory the device cannot access (pin or register it)", who, s);
    return NT2G_OK;
}

namespace nt2g {

const std::vector<nt2g_op> &program_ops(const nt2g_program *p) { return p->ops; }
const std::vector<uint8_t> &program_logical(const nt2g_program *p) { return p->logical; }
bool program_folds(const nt2g_program *p) { return p->folds; }

nt2g_status program_bind(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t count, const char *who,
                         DArgs &da)
{
    NT2G_CHECK_ARG(n_args >= p->n_slots && (args != nullptr || p->n_slots == 0), "%s: %d arguments for %d slots", who,
                   n_args, p->n_slots);
    return bind_args(p, args, 0, count, who, da);
}

int64_t program_bytes_per_element(const nt2g_program *p)
{
    int64_t b = 0;
    for (int s = 0; s < p->n_slots; ++s) {
        const int use = p->slot_use[s];
        if (use & 4) continue;
        b += (int64_t)(((use & 1) ? 1 : 0) + ((use & 2) ? 1 : 0)) * (int64_t)dtype_size(p->slot_dtype[s]);
    }
    return b;
}

nt2g_status program_eval(const nt2g_program *p, const DArgs &da, int64_t count, int precision, cudaStream_t st)
{
    if (count == 0) return NT2G_OK;
    nt2g_status js = launch_jit(p->ops, p->logical, da, count, precision, st);
    if (js != NT2G_ERR_UNSUPPORTED) return js;
    return launch_interp(p->dprog, da, count, precision, st);
}

}  // namespace nt2g

extern "C" nt2g_status nt2g_eval(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t offset,
                                 int64_t count, int32_t precision, int32_t force_generic, void *stream)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_eval: NULL program");
    NT2G_CHECK_ARG(n_args >= p->n_slots && (args != nullptr || p->n_slots == 0),
                   "nt2g_eval: %d arguments for %d slots", n_args, p->n_slots);
    NT2G_CHECK_ARG(offset >= 0 && count >= 0, "nt2g_eval: negative range (%lld, %lld)", (long long)offset,
                   (long long)count);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_eval: precision %d", precision);
    NT2G_CHECK_ARG(!p->folds, "nt2g_eval: the program folds its value (nt2g_eval_fold)");
    cudaStream_t st = (cudaStream_t)stream;
    DArgs da{};
    nt2g_status bs = bind_args(p, args, offset, count, "nt2g_eval", da);
    if (bs != NT2G_OK) return bs;
    if (count == 0) return NT2G_OK;
    int kernel = force_generic ? kGeneric : p->kernel;
    for (const DeferredConst &dc : p->deferred)
        if ((float)args[dc.slot].scalar != dc.value) kernel = kGeneric;
    if (kernel != kGeneric) {
        auto T = [&](int role) -> float * { return (float *)da.ptr[p->roles[role].slot]; };
        auto U8 = [&](int role) -> uint8_t * { return (uint8_t *)da.ptr[p->roles[role].slot]; };
        auto V = [&](int role) -> float {
            const RoleBind &r = p->roles[role];
            return r.kind == 1 ? r.value : r.kind == 3 ? -da.scal[r.slot] : da.scal[r.slot];
        };
        auto TV = [&](int role) -> float * { return p->roles[role].kind == 0 ? T(role) : nullptr; };
        switch (kernel) {
        case kBlackScholes:
            return launch_bs(T(0), T(1), T(2), TV(3), TV(3) ? 0.f : V(3), V(4), T(5), T(6), count, precision, st);
        case kBlackScholesDemo:
            return launch_bs_demo(T(0), T(1), T(2), TV(3), TV(3) ? 0.f : V(3), TV(4), TV(4) ? 0.f : V(4), T(5), count,
                                  precision, st);
        case kSaxpy: return launch_saxpy(V(0), T(1), T(2), T(3), count, st);
        case kExpr3: return launch_expr3(T(0), T(1), T(2), T(3), count, precision, st);
        case kRgb2Yuv: return launch_rgb2yuv(T(0), T(1), T(2), T(3), T(4), T(5), count, precision, st);
        case kSigmaDelta: {
            // the fused kernel updates bkg/var in place: it needs the output
            // roles to be the same tables as the inputs
            if (p->roles[3].slot == p->roles[1].slot && p->roles[4].slot == p->roles[2].slot)
                return launch_sigmadelta(U8(0), U8(1), U8(2), U8(5), count, st);
            break;
        }
        default: break;
        }
    }
    if (force_generic != 2) {
        nt2g_status js = launch_jit(p->ops, p->logical, da, count, precision, st);
        if (js != NT2G_ERR_UNSUPPORTED) return js;
    }
    return launch_interp(p->dprog, da, count, precision, st);
}

extern "C" nt2g_status nt2g_eval_fold(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t lo,
                                      int64_t inner, int64_t hi, int32_t op, int32_t precision, void *workspace,
                                      size_t workspace_bytes, float *out, int64_t *index, double *out64, void *stream)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_eval_fold: NULL program");
    NT2G_CHECK_ARG(p->folds, "nt2g_eval_fold: the program has no FOLD instruction");
    NT2G_CHECK_ARG(n_args >= p->n_slots && (args != nullptr || p->n_slots == 0),
                   "nt2g_eval_fold: %d arguments for %d slots", n_args, p->n_slots);
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_eval_fold: negative extent (%lld, %lld, %lld)",
                   (long long)lo, (long long)inner, (long long)hi);
    NT2G_CHECK_ARG(op >= NT2G_FOLD_SUM && op <= NT2G_FOLD_MEANAD, "nt2g_eval_fold: op %d", op);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2 || precision == NT2G_PREC_NT2_ELEMENTS,
                   "nt2g_eval_fold: precision %d", precision);
    NT2G_CHECK_ARG(index == nullptr || op == NT2G_FOLD_MAX || op == NT2G_FOLD_MIN,
                   "nt2g_eval_fold: an index is defined for max and min only");
    NT2G_CHECK_ARG(out64 == nullptr || (precision != NT2G_PREC_NT2 && op != NT2G_FOLD_MAX && op != NT2G_FOLD_MIN),
                   "nt2g_eval_fold: FP64 results are given for sum-type and product folds of the compensated fold");
    const int64_t n_out = lo * hi;
    DArgs da{};
    nt2g_status bs = bind_args(p, args, 0, n_out * inner, "nt2g_eval_fold", da);
    if (bs != NT2G_OK) return bs;
    if (n_out == 0) return NT2G_OK;
    NT2G_CHECK_ARG(out != nullptr, "nt2g_eval_fold: out is NULL");
    size_t need = 0;
    const bool centred = (op >= NT2G_FOLD_VAR && op <= NT2G_FOLD_STDEV1) || op == NT2G_FOLD_NANMEAN ||
                         op == NT2G_FOLD_MEANAD;
    if (centred) fold_workspace_bytes(lo, inner, hi, &need);
    else fold_partials_bytes(lo, inner, hi, &need);
    NT2G_CHECK_ARG((precision == NT2G_PREC_NT2 && !centred) || need == 0 ||
                       (workspace != nullptr && workspace_bytes >= need),
                   "nt2g_eval_fold: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_eval_fold: workspace not 16-byte aligned");
    NT2G_CHECK_ARG(reachable(out) && reachable(index) && reachable(out64) && reachable(workspace),
                   "nt2g_eval_fold: an output or the workspace is host memory the device cannot access");
    return launch_fold_expr(p->ops, p->logical, da, lo, inner, hi, op, precision, workspace, workspace_bytes, out,
                            index, out64, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_program_vjp(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t count,
                                        const float *const *cotangents, float *const *table_grads,
                                        double *scalar_grads, int32_t precision, void *workspace,
                                        size_t workspace_bytes, void *stream)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_program_vjp: NULL program");
    NT2G_CHECK_ARG(!p->folds, "nt2g_program_vjp: the program folds its value");
    NT2G_CHECK_ARG(n_args >= p->n_slots && (args != nullptr || p->n_slots == 0),
                   "nt2g_program_vjp: %d arguments for %d slots", n_args, p->n_slots);
    NT2G_CHECK_ARG(count >= 0, "nt2g_program_vjp: negative count %lld", (long long)count);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_program_vjp: precision %d",
                   precision);
    DArgs da{};
    nt2g_status bs = bind_args(p, args, 0, count, "nt2g_program_vjp", da);
    if (bs != NT2G_OK) return bs;
    const float *ct[kMaxSlots] = {};
    float *gr[kMaxSlots] = {};
    std::vector<int> float_scalars;
    for (int s = 0; s < p->n_slots; ++s) {
        const int use = p->slot_use[s];
        const bool f32 = p->slot_dtype[s] == NT2G_F32;
        if ((use & 4) && f32) float_scalars.push_back(s);
        if (cotangents && cotangents[s]) {
            NT2G_CHECK_ARG((use & 2) && f32, "nt2g_program_vjp: slot %d is not a float output, it takes no cotangent",
                           s);
            NT2G_CHECK_ARG(count == 0 || reachable(cotangents[s]),
                           "nt2g_program_vjp: cotangent %d is host memory the device cannot access", s);
            ct[s] = cotangents[s];
        }
        if (table_grads && table_grads[s]) {
            NT2G_CHECK_ARG((use & 1) && !(use & 4) && f32,
                           "nt2g_program_vjp: slot %d is not a float table the program reads", s);
            NT2G_CHECK_ARG(count == 0 || reachable(table_grads[s]),
                           "nt2g_program_vjp: gradient %d is host memory the device cannot access", s);
            gr[s] = table_grads[s];
        }
    }
    NT2G_CHECK_ARG(reachable(scalar_grads), "nt2g_program_vjp: scalar_grads is host memory the device cannot access");
    return launch_vjp(p->ops, p->logical, da, ct, gr, scalar_grads, float_scalars, count, precision, workspace,
                      workspace_bytes, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_program_vjp_workspace_size(const nt2g_program *p, int64_t count, size_t *bytes)
{
    NT2G_CHECK_ARG(p != nullptr && bytes != nullptr, "nt2g_program_vjp_workspace_size: NULL argument");
    NT2G_CHECK_ARG(count >= 0, "nt2g_program_vjp_workspace_size: negative count");
    *bytes = vjp_workspace_bytes(p->ops, p->logical, count);
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_program_vjp_source(const nt2g_program *p, int32_t precision, char *buf, size_t cap,
                                               size_t *len)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_program_vjp_source: NULL program");
    NT2G_CHECK_ARG(!p->folds, "nt2g_program_vjp_source: the program folds its value");
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_program_vjp_source: precision %d",
                   precision);
    NT2G_CHECK_ARG(buf != nullptr || cap == 0, "nt2g_program_vjp_source: NULL buffer");
    std::string why;
    std::string src = jit_vjp_source(p->ops, p->logical, precision, &why);
    if (src.empty()) {
        set_error("nt2g_program_vjp_source: %s", why.c_str());
        return NT2G_ERR_UNSUPPORTED;
    }
    if (len) *len = src.size() + 1;
    if (cap == 0) return NT2G_OK;
    NT2G_CHECK_ARG(cap > src.size(), "nt2g_program_vjp_source: %zu-byte buffer, %zu needed", cap, src.size() + 1);
    memcpy(buf, src.c_str(), src.size() + 1);
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_program_jit_source(const nt2g_program *p, int32_t precision, char *buf, size_t cap,
                                               size_t *len)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_program_jit_source: NULL program");
    NT2G_CHECK_ARG(!p->folds, "nt2g_program_jit_source: the program folds its value (nt2g_program_fold_source)");
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_program_jit_source: precision %d",
                   precision);
    NT2G_CHECK_ARG(buf != nullptr || cap == 0, "nt2g_program_jit_source: NULL buffer");
    std::string src = jit_source(p->ops, p->logical, precision);
    if (len) *len = src.size() + 1;
    if (cap == 0) return NT2G_OK;
    NT2G_CHECK_ARG(cap > src.size(), "nt2g_program_jit_source: %zu-byte buffer, %zu needed", cap, src.size() + 1);
    memcpy(buf, src.c_str(), src.size() + 1);
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_program_fold_source(const nt2g_program *p, int32_t precision, int32_t op, char *buf,
                                                size_t cap, size_t *len)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_program_fold_source: NULL program");
    NT2G_CHECK_ARG(p->folds, "nt2g_program_fold_source: the program has no FOLD instruction");
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2 || precision == NT2G_PREC_NT2_ELEMENTS,
                   "nt2g_program_fold_source: precision %d", precision);
    NT2G_CHECK_ARG(op >= NT2G_FOLD_SUM && op <= NT2G_FOLD_MEANAD, "nt2g_program_fold_source: op %d", op);
    NT2G_CHECK_ARG(buf != nullptr || cap == 0, "nt2g_program_fold_source: NULL buffer");
    std::string src = jit_fold_source(p->ops, p->logical, precision, op);
    if (len) *len = src.size() + 1;
    if (cap == 0) return NT2G_OK;
    NT2G_CHECK_ARG(cap > src.size(), "nt2g_program_fold_source: %zu-byte buffer, %zu needed", cap, src.size() + 1);
    memcpy(buf, src.c_str(), src.size() + 1);
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_program_jit_prepare(const nt2g_program *p, int32_t precision)
{
    NT2G_CHECK_ARG(p != nullptr, "nt2g_program_jit_prepare: NULL program");
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2,
                   "nt2g_program_jit_prepare: precision %d", precision);
    return jit_prepare(p->ops, p->logical, precision);
}

// ------------------------------------------------------- direct kernels ----
#define NT2G_REQ(ptr) NT2G_CHECK_ARG((ptr) != nullptr || n == 0, "%s: " #ptr " is NULL", __func__)
// after the other checks, for a non-empty call: every table the kernel touches is reachable
#define NT2G_REACH(ptr)                                                                                        \
    NT2G_CHECK_ARG(n == 0 || reachable(ptr), "%s: " #ptr " is host memory the device cannot access (pin or "   \
                   "register it)", __func__)
// for what a kernel writes even when n == 0 (a reduction's result and workspace)
#define NT2G_REACH_ALWAYS(ptr)                                                                                 \
    NT2G_CHECK_ARG(reachable(ptr), "%s: " #ptr " is host memory the device cannot access (pin or register it)", \
                   __func__)
#define NT2G_REQ_N() NT2G_CHECK_ARG(n >= 0, "%s: negative size %lld", __func__, (long long)n)
#define NT2G_REQ_PREC()                                                                                        \
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "%s: precision %d", __func__,     \
                   precision)

extern "C" nt2g_status nt2g_blackscholes_f32(const float *S, const float *K, const float *T, const float *sigma,
                                             float sigma_s, float r, float *call, float *put, int64_t n,
                                             int32_t precision, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(S); NT2G_REQ(K); NT2G_REQ(T); NT2G_REQ(call); NT2G_REQ(put); NT2G_REQ_PREC();
    NT2G_REACH(S); NT2G_REACH(K); NT2G_REACH(T); NT2G_REACH(sigma); NT2G_REACH(call); NT2G_REACH(put);
    return launch_bs(S, K, T, sigma, sigma_s, r, call, put, n, precision, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_blackscholes_demo_f32(const float *S, const float *X, const float *T, const float *r_t,
                                                  float r, const float *v_t, float v, float *R, int64_t n,
                                                  int32_t precision, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(S); NT2G_REQ(X); NT2G_REQ(T); NT2G_REQ(R); NT2G_REQ_PREC();
    NT2G_REACH(S); NT2G_REACH(X); NT2G_REACH(T); NT2G_REACH(r_t); NT2G_REACH(v_t); NT2G_REACH(R);
    return launch_bs_demo(S, X, T, r_t, r, v_t, v, R, n, precision, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_blackscholes_vjp_f32(const float *S, const float *K, const float *T, const float *sigma,
                                                 float r, const float *gc, const float *gp, float *call, float *put,
                                                 float *dS, float *dK, float *dT, float *dsigma, float *dr, int64_t n,
                                                 void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(S); NT2G_REQ(K); NT2G_REQ(T); NT2G_REQ(sigma); NT2G_REQ(gc); NT2G_REQ(gp);
    NT2G_REQ(call); NT2G_REQ(put); NT2G_REQ(dS); NT2G_REQ(dK); NT2G_REQ(dT); NT2G_REQ(dsigma); NT2G_REQ(dr);
    NT2G_REACH(S); NT2G_REACH(K); NT2G_REACH(T); NT2G_REACH(sigma); NT2G_REACH(gc); NT2G_REACH(gp);
    NT2G_REACH(call); NT2G_REACH(put); NT2G_REACH(dS); NT2G_REACH(dK); NT2G_REACH(dT); NT2G_REACH(dsigma);
    NT2G_REACH(dr);
    return launch_bs_vjp(S, K, T, sigma, r, gc, gp, call, put, dS, dK, dT, dsigma, dr, n, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_saxpy_f32(float alpha, const float *X, float *Y, int64_t n, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(X); NT2G_REQ(Y);
    NT2G_REACH(X); NT2G_REACH(Y);
    return launch_saxpy(alpha, X, Y, Y, n, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_expr3_f32(const float *x, const float *y, const float *z, float *out, int64_t n,
                                      int32_t precision, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(x); NT2G_REQ(y); NT2G_REQ(z); NT2G_REQ(out); NT2G_REQ_PREC();
    NT2G_REACH(x); NT2G_REACH(y); NT2G_REACH(z); NT2G_REACH(out);
    return launch_expr3(x, y, z, out, n, precision, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_rgb2yuv_f32(const float *r, const float *g, const float *b, float *y, float *u, float *v,
                                        int64_t n, int32_t precision, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(r); NT2G_REQ(g); NT2G_REQ(b); NT2G_REQ(y); NT2G_REQ(u); NT2G_REQ(v); NT2G_REQ_PREC();
    NT2G_REACH(r); NT2G_REACH(g); NT2G_REACH(b); NT2G_REACH(y); NT2G_REACH(u); NT2G_REACH(v);
    return launch_rgb2yuv(r, g, b, y, u, v, n, precision, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_sigmadelta_u8(const uint8_t *frame, uint8_t *bkg, uint8_t *var, uint8_t *label, int64_t n,
                                          void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(frame); NT2G_REQ(bkg); NT2G_REQ(var); NT2G_REQ(label);
    NT2G_REACH(frame); NT2G_REACH(bkg); NT2G_REACH(var); NT2G_REACH(label);
    return launch_sigmadelta(frame, bkg, var, label, n, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_sigmadelta_frames_u8(const uint8_t *frames, uint8_t *bkg, uint8_t *var, uint8_t *labels,
                                                 int64_t n, int32_t n_frames, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(frames); NT2G_REQ(bkg); NT2G_REQ(var); NT2G_REQ(labels);
    NT2G_REACH(frames); NT2G_REACH(bkg); NT2G_REACH(var); NT2G_REACH(labels);
    NT2G_CHECK_ARG(n_frames >= 0, "nt2g_sigmadelta_frames_u8: negative frame count %d", n_frames);
    return launch_sigmadelta_frames(frames, bkg, var, labels, n, n_frames, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_map_f32(int32_t fn, const float *x, float *y, int64_t n, int32_t precision, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(x); NT2G_REQ(y); NT2G_REQ_PREC();
    NT2G_REACH(x); NT2G_REACH(y);
    NT2G_CHECK_ARG((fn >= 0 && fn <= 50) || (fn >= 64 && fn <= 75) || (fn >= 80 && fn <= 82), "nt2g_map_f32: unknown function %d", fn);
    return launch_map(fn, x, y, n, precision, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_reduce_workspace_size(int64_t n, size_t *bytes)
{
    NT2G_CHECK_ARG(bytes != nullptr, "nt2g_reduce_workspace_size: bytes is NULL");
    NT2G_REQ_N();
    return reduce_workspace_bytes(bytes);
}

extern "C" nt2g_status nt2g_reduce_f32(const float *x, const float *y, int64_t n, void *workspace,
                                       size_t workspace_bytes, double *out64, float *out32, void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(x);
    NT2G_CHECK_ARG(out64 != nullptr, "nt2g_reduce_f32: out64 is NULL");
    size_t need = 0;
    reduce_workspace_bytes(&need);
    NT2G_CHECK_ARG(workspace != nullptr && workspace_bytes >= need,
                   "nt2g_reduce_f32: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_reduce_f32: workspace not 16-byte aligned");
    NT2G_REACH(x); NT2G_REACH(y);
    NT2G_REACH_ALWAYS(workspace); NT2G_REACH_ALWAYS(out64); NT2G_REACH_ALWAYS(out32);
    return launch_reduce(x, y, n, workspace, out64, out32, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_reduce_f32_noalloc(const float *x, const float *y, int64_t n, double *out64, float *out32,
                                               void *stream)
{
    NT2G_REQ_N(); NT2G_REQ(x);
    NT2G_CHECK_ARG(out64 != nullptr, "nt2g_reduce_f32_noalloc: out64 is NULL");
    NT2G_REACH(x); NT2G_REACH(y); NT2G_REACH_ALWAYS(out64); NT2G_REACH_ALWAYS(out32);
    return launch_reduce_noalloc(x, y, n, out64, out32, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_fold_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    NT2G_CHECK_ARG(bytes != nullptr, "nt2g_fold_workspace_size: bytes is NULL");
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_fold_workspace_size: negative extent");
    return fold_workspace_bytes(lo, inner, hi, bytes);
}

extern "C" nt2g_status nt2g_fold_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op,
                                     int32_t precision, void *workspace, size_t workspace_bytes, float *out,
                                     int64_t *index, void *stream)
{
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_fold_f32: negative extent (%lld, %lld, %lld)",
                   (long long)lo, (long long)inner, (long long)hi);
    NT2G_CHECK_ARG(op >= NT2G_FOLD_SUM && op <= NT2G_FOLD_MEANAD, "nt2g_fold_f32: op %d", op);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_fold_f32: precision %d",
                   precision);
    NT2G_CHECK_ARG(index == nullptr || op == NT2G_FOLD_MAX || op == NT2G_FOLD_MIN,
                   "nt2g_fold_f32: an index is defined for max and min only");
    const int64_t n = lo * hi;
    if (n == 0) return NT2G_OK;
    NT2G_CHECK_ARG(out != nullptr, "nt2g_fold_f32: out is NULL");
    NT2G_CHECK_ARG(x != nullptr || inner == 0, "nt2g_fold_f32: x is NULL");
    size_t need = 0;
    // var/stdev keep each output's centre in the workspace, nanmean its count
    const bool centred = (op >= NT2G_FOLD_VAR && op <= NT2G_FOLD_STDEV1) || op == NT2G_FOLD_NANMEAN ||
                         op == NT2G_FOLD_MEANAD;
    if (centred) fold_workspace_bytes(lo, inner, hi, &need);
    else fold_partials_bytes(lo, inner, hi, &need);
    NT2G_CHECK_ARG((precision == NT2G_PREC_NT2 && !centred) || need == 0 ||
                       (workspace != nullptr && workspace_bytes >= need),
                   "nt2g_fold_f32: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_fold_f32: workspace not 16-byte aligned");
    NT2G_REACH(x); NT2G_REACH(out); NT2G_REACH(index); NT2G_REACH(workspace);
    return launch_fold(x, lo, inner, hi, op, precision, workspace, workspace_bytes, out, index,
                       (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_trapz_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    NT2G_CHECK_ARG(bytes != nullptr, "nt2g_trapz_workspace_size: bytes is NULL");
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_trapz_workspace_size: negative extent");
    return trapz_workspace_bytes(lo, inner, hi, bytes);
}

extern "C" nt2g_status nt2g_trapz_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t precision,
                                      void *workspace, size_t workspace_bytes, float *out, void *stream)
{
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_trapz_f32: negative extent (%lld, %lld, %lld)",
                   (long long)lo, (long long)inner, (long long)hi);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_trapz_f32: precision %d",
                   precision);
    const int64_t n = lo * hi;
    if (n == 0) return NT2G_OK;
    NT2G_CHECK_ARG(out != nullptr, "nt2g_trapz_f32: out is NULL");
    NT2G_CHECK_ARG(x != nullptr || inner == 0, "nt2g_trapz_f32: x is NULL");
    size_t need = 0;
    trapz_workspace_bytes(lo, inner, hi, &need);
    NT2G_CHECK_ARG(precision == NT2G_PREC_NT2 || inner < 2 || (workspace != nullptr && workspace_bytes >= need),
                   "nt2g_trapz_f32: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_trapz_f32: workspace not 16-byte aligned");
    NT2G_REACH(x); NT2G_REACH(out); NT2G_REACH(workspace);
    return launch_trapz(x, lo, inner, hi, precision, workspace, workspace_bytes, out, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_median_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    NT2G_CHECK_ARG(bytes != nullptr, "nt2g_median_workspace_size: bytes is NULL");
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_median_workspace_size: negative extent");
    *bytes = median_workspace_bytes(lo, inner, hi);
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_median_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op,
                                       void *workspace, size_t workspace_bytes, float *out, void *stream)
{
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_median_f32: negative extent (%lld, %lld, %lld)",
                   (long long)lo, (long long)inner, (long long)hi);
    NT2G_CHECK_ARG(op == NT2G_MEDIAN || op == NT2G_MEDIANAD, "nt2g_median_f32: op %d", op);
    const int64_t S = lo * hi;
    if (S == 0) return NT2G_OK;
    NT2G_CHECK_ARG(S < ((int64_t)1 << 31), "nt2g_median_f32: %lld slices (at most 2^31 - 1)", (long long)S);
    NT2G_CHECK_ARG(out != nullptr, "nt2g_median_f32: out is NULL");
    NT2G_CHECK_ARG(x != nullptr || inner == 0, "nt2g_median_f32: x is NULL");
    NT2G_CHECK_ARG(out + S <= x || x + lo * inner * hi <= out || inner == 0, "nt2g_median_f32: out overlaps x");
    const size_t need = median_workspace_bytes(lo, inner, hi);
    NT2G_CHECK_ARG(need == 0 || (workspace != nullptr && workspace_bytes >= need),
                   "nt2g_median_f32: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_median_f32: workspace not 16-byte aligned");
    const int64_t n = S;  // the pointer checks below apply to non-empty calls
    NT2G_REACH(x); NT2G_REACH(out); NT2G_REACH(workspace);
    return launch_median(x, lo, inner, hi, op, workspace, out, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_scan_workspace_size(int64_t lo, int64_t inner, int64_t hi, size_t *bytes)
{
    NT2G_CHECK_ARG(bytes != nullptr, "nt2g_scan_workspace_size: bytes is NULL");
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_scan_workspace_size: negative extent");
    return scan_workspace_bytes(lo, inner, hi, bytes);
}

extern "C" nt2g_status nt2g_scan_f32(const float *x, int64_t lo, int64_t inner, int64_t hi, int32_t op,
                                     int32_t precision, void *workspace, size_t workspace_bytes, float *out,
                                     void *stream)
{
    NT2G_CHECK_ARG(lo >= 0 && inner >= 0 && hi >= 0, "nt2g_scan_f32: negative extent (%lld, %lld, %lld)",
                   (long long)lo, (long long)inner, (long long)hi);
    NT2G_CHECK_ARG(op >= NT2G_SCAN_SUM && op <= NT2G_SCAN_MIN, "nt2g_scan_f32: op %d", op);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_scan_f32: precision %d",
                   precision);
    const int64_t n = lo * inner * hi;
    if (n == 0) return NT2G_OK;
    NT2G_CHECK_ARG(x != nullptr && out != nullptr, "nt2g_scan_f32: NULL table");
    NT2G_CHECK_ARG(out == x || (out + n <= x || x + n <= out), "nt2g_scan_f32: out partially overlaps x");
    size_t need = 0;
    scan_workspace_bytes(lo, inner, hi, &need);
    NT2G_CHECK_ARG(precision == NT2G_PREC_NT2 || need == 0 || (workspace != nullptr && workspace_bytes >= need),
                   "nt2g_scan_f32: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    NT2G_CHECK_ARG(((uintptr_t)workspace & 15u) == 0, "nt2g_scan_f32: workspace not 16-byte aligned");
    NT2G_REACH(x); NT2G_REACH(out); NT2G_REACH(workspace);
    return launch_scan(x, lo, inner, hi, op, precision, workspace, workspace_bytes, out, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_host_access(int32_t *pageable)
{
    NT2G_CHECK_ARG(pageable != nullptr, "nt2g_host_access: pageable is NULL");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_host_access");
    *pageable = pageable_access() ? 1 : 0;
    return NT2G_OK;
}

// ------------------------------------------------------------- memory ----
extern "C" nt2g_status nt2g_device_alloc(size_t bytes, void **ptr)
{
    NT2G_CHECK_ARG(ptr != nullptr, "nt2g_device_alloc: ptr is NULL");
    *ptr = nullptr;
    if (bytes == 0) return NT2G_OK;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        set_error("nt2g_device_alloc: %zu bytes: out of device memory", bytes);
        return NT2G_ERR_NOMEM;
    }
    return e == cudaSuccess ? NT2G_OK : cuda_status(e, "nt2g_device_alloc");
}

extern "C" nt2g_status nt2g_device_free(void *ptr)
{
    if (!ptr) return NT2G_OK;
    cudaError_t e = cudaFree(ptr);
    return e == cudaSuccess ? NT2G_OK : cuda_status(e, "nt2g_device_free");
}

extern "C" nt2g_status nt2g_memcpy(void *dst, const void *src, size_t bytes, int32_t kind, void *stream)
{
    NT2G_CHECK_ARG(kind >= 1 && kind <= 3, "nt2g_memcpy: kind %d", kind);
    if (bytes == 0) return NT2G_OK;
    NT2G_CHECK_ARG(dst && src, "nt2g_memcpy: NULL pointer");
    cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice : kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream);
    return e == cudaSuccess ? NT2G_OK : cuda_status(e, "nt2g_memcpy");
}

extern "C" nt2g_status nt2g_device_current(int32_t *device)
{
    NT2G_CHECK_ARG(device != nullptr, "nt2g_device_current: device is NULL");
    int d = 0;
    cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_device_current");
    *device = d;
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_stream_create(void **stream)
{
    NT2G_CHECK_ARG(stream != nullptr, "nt2g_stream_create: stream is NULL");
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_stream_create");
    *stream = st;
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_stream_destroy(void *stream)
{
    NT2G_CHECK_ARG(stream != nullptr, "nt2g_stream_destroy: NULL stream");
    cudaError_t e = cudaStreamDestroy((cudaStream_t)stream);
    return e == cudaSuccess ? NT2G_OK : cuda_status(e, "nt2g_stream_destroy");
}

extern "C" nt2g_status nt2g_stream_synchronize(void *stream)
{
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? NT2G_OK : cuda_status(e, "nt2g_stream_synchronize");
}
