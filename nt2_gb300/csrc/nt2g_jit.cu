// nt2g_jit.cu -- one fused kernel per generic expression, compiled at run time.
//
// NT2 planned GPU kernels as code generated per expression: its
// external_kernel tool collects the expression symbols of a program and a
// back-end writes a CUDA file that kernel_gen compiles with nvcc
// (tools/external_kernel/backend.cpp:32-52, tools/kernel_gen/kernel_gen.cpp:8-113;
// the CUDA back-end itself never shipped).  Here the library does it in
// process: an expression program that binds none of the hand-written fused
// kernels is turned into a straight-line CUDA kernel -- one statement per SSA
// instruction, every value in a register, the same device math header as the
// rest of the library -- compiled by NVRTC for sm_103a, loaded through the
// runtime's library API and cached per device, policy and program text.
//
// Each statement computes exactly what the interpreter computes for the same
// instruction, so both give bit-identical results; the JIT kernel just has no
// dispatch and no register file in memory.  NVRTC is opened with dlopen: when
// it is not installed the generic path stays on the interpreter.
#include <dlfcn.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "nt2g_common.cuh"
#include "nt2g_internal.h"
#include "nt2g_math_src.h"   // kNt2gMathSrc: nt2g_math.cuh as a string (generated at build)
#include "nt2g_accum_src.h"  // kNt2gAccumSrc: nt2g_accum.cuh
#include "nt2g_fold_src.h"   // kNt2gFoldSrc: nt2g_fold_kernels.cuh
#include "nt2g_vjp_src.h"    // kNt2gVjpSrc: nt2g_vjp.cuh

namespace nt2g {

// ------------------------------------------------------------ nvrtc, dlopen --
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram *nvrtcProgram_t;
struct Nvrtc {
    void *h = nullptr;
    nvrtcResult_t (*create)(nvrtcProgram_t *, const char *, const char *, int, const char *const *,
                            const char *const *) = nullptr;
    nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char *const *) = nullptr;
    nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t *) = nullptr;
    nvrtcResult_t (*cubin)(nvrtcProgram_t, char *) = nullptr;
    nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t *) = nullptr;
    nvrtcResult_t (*log)(nvrtcProgram_t, char *) = nullptr;
    nvrtcResult_t (*destroy)(nvrtcProgram_t *) = nullptr;
    std::string error;
};

static Nvrtc &nvrtc()
{
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *env = getenv("NT2G_NVRTC");
        std::vector<std::string> names;
        if (env) names.push_back(env);
        names.push_back("libnvrtc.so.13");
        names.push_back("libnvrtc.so");
        const char *home = getenv("CUDA_HOME");
        names.push_back(std::string(home ? home : "/usr/local/cuda") + "/lib64/libnvrtc.so.13");
        for (const std::string &nm : names)
            if ((n.h = dlopen(nm.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
        if (!n.h) { n.error = "NVRTC not found (libnvrtc.so.13)"; return; }
        n.create = (decltype(n.create))dlsym(n.h, "nvrtcCreateProgram");
        n.compile = (decltype(n.compile))dlsym(n.h, "nvrtcCompileProgram");
        n.cubin_size = (decltype(n.cubin_size))dlsym(n.h, "nvrtcGetCUBINSize");
        n.cubin = (decltype(n.cubin))dlsym(n.h, "nvrtcGetCUBIN");
        n.log_size = (decltype(n.log_size))dlsym(n.h, "nvrtcGetProgramLogSize");
        n.log = (decltype(n.log))dlsym(n.h, "nvrtcGetProgramLog");
        n.destroy = (decltype(n.destroy))dlsym(n.h, "nvrtcDestroyProgram");
        if (!(n.create && n.compile && n.cubin_size && n.cubin && n.log_size && n.log && n.destroy)) {
            n.error = "NVRTC is missing entry points";
            n.h = nullptr;
        }
    });
    return n;
}

// ----------------------------------------------------------------- codegen --
// The kernel processes 4 consecutive elements per thread (one float4 per f32
// table when every table is aligned, one 32-bit word per uint8 table), so a
// value is a 4-lane array that the compiler keeps in registers.
static const char kJitPrelude[] = R"NT2G_SRC(
struct JitArgs { void *ptr[16]; float scal[16]; unsigned scal_u8[16]; int dtype[16]; long long pos0; };
#define NT2G_L _Pragma("unroll") for (int j = 0; j < 4; ++j)
#define NT2G_LL _Pragma("unroll") for (int j = 0; j < L; ++j)
template <bool FULL> __device__ __forceinline__ void jit_ldf(float (&d)[4], const void *p, long long i, int cnt)
{
    const float *q = (const float *)p + i;
    if (FULL) { float4 t = __ldcs((const float4 *)q); d[0] = t.x; d[1] = t.y; d[2] = t.z; d[3] = t.w; }
    else { NT2G_L d[j] = j < cnt ? q[j] : 0.0f; }
}
template <bool FULL> __device__ __forceinline__ void jit_ldb(unsigned (&d)[4], const void *p, long long i, int cnt)
{
    const unsigned char *q = (const unsigned char *)p + i;
    if (FULL) { unsigned w = *(const unsigned *)q; NT2G_L d[j] = (w >> (8 * j)) & 255u; }
    else { NT2G_L d[j] = j < cnt ? (unsigned)q[j] : 0u; }
}
template <bool FULL> __device__ __forceinline__ void jit_stf(void *p, long long i, int cnt, const float (&v)[4])
{
    float *q = (float *)p + i;
    if (FULL) __stcs((float4 *)q, make_float4(v[0], v[1], v[2], v[3]));
    else { NT2G_L if (j < cnt) q[j] = v[j]; }
}
template <bool FULL> __device__ __forceinline__ void jit_stb(void *p, long long i, int cnt, const unsigned (&v)[4])
{
    unsigned char *q = (unsigned char *)p + i;
    if (FULL) *(unsigned *)q = (v[0] & 255u) | (v[1] & 255u) << 8 | (v[2] & 255u) << 16 | (v[3] & 255u) << 24;
    else { NT2G_L if (j < cnt) q[j] = (unsigned char)v[j]; }
}
// Two vectors per thread (batched tiles): lanes 0-3 at element i, lanes 4-7 a
// block-width of vectors further (i + 4 blockDim.x), so a warp's accesses stay
// contiguous; only whole, aligned pairs take this form.
template <int L> __device__ __forceinline__ long long jit_pos(long long i, int j)
{
    return L <= 4 ? i + j : i + (j & 3) + (long long)(j >> 2) * blockDim.x * 4;
}
template <bool FULL> __device__ __forceinline__ void jit_ldf(float (&d)[8], const void *p, long long i, int)
{
    const float *q = (const float *)p + i;
    const float4 t = __ldcs((const float4 *)q), u = __ldcs((const float4 *)(q + (long long)blockDim.x * 4));
    d[0] = t.x; d[1] = t.y; d[2] = t.z; d[3] = t.w; d[4] = u.x; d[5] = u.y; d[6] = u.z; d[7] = u.w;
}
template <bool FULL> __device__ __forceinline__ void jit_ldb(unsigned (&d)[8], const void *p, long long i, int)
{
    const unsigned char *q = (const unsigned char *)p + i;
    const unsigned w0 = *(const unsigned *)q, w1 = *(const unsigned *)(q + (long long)blockDim.x * 4);
    NT2G_L { d[j] = (w0 >> (8 * j)) & 255u; d[j + 4] = (w1 >> (8 * j)) & 255u; }
}
template <bool FULL> __device__ __forceinline__ void jit_stf(void *p, long long i, int, const float (&v)[8])
{
    float *q = (float *)p + i;
    __stcs((float4 *)q, make_float4(v[0], v[1], v[2], v[3]));
    __stcs((float4 *)(q + (long long)blockDim.x * 4), make_float4(v[4], v[5], v[6], v[7]));
}
template <bool FULL> __device__ __forceinline__ void jit_stb(void *p, long long i, int, const unsigned (&v)[8])
{
    unsigned char *q = (unsigned char *)p + i;
    *(unsigned *)q = (v[0] & 255u) | (v[1] & 255u) << 8 | (v[2] & 255u) << 16 | (v[3] & 255u) << 24;
    *(unsigned *)(q + (long long)blockDim.x * 4) =
        (v[4] & 255u) | (v[5] & 255u) << 8 | (v[6] & 255u) << 16 | (v[7] & 255u) << 24;
}
)NT2G_SRC";

static std::string fconst(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    char b[40];
    snprintf(b, sizeof b, "__uint_as_float(0x%08xu)", u);
    return b;
}

// The statements of a program over L lanes (4 consecutive elements per call
// in a transform; 1 or 4 in a fold's element function).  STORE writes the
// output tables; FOLD (fold programs) hands the folded value to out[].
static void emit_body(std::string &s, const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical,
                      bool stores = true)
{
    auto v = [](int x) { return "v" + std::to_string(x) + "[j]"; };
    // every table load first, so a tile's memory requests are in flight while its
    // arithmetic runs (a load never follows a store to its table: the compiler
    // forwards stored values)
    for (size_t k = 0; k < ops.size(); ++k) {
        const nt2g_op &o = ops[k];
        if (o.code != NT2G_OP_LOAD) continue;
        const bool f32 = o.dtype == NT2G_F32;
        s += (f32 ? "    float v" : "    unsigned v") + std::to_string(k) + "[A]; " +
             (f32 ? "jit_ldf<FULL>(v" : "jit_ldb<FULL>(v") + std::to_string(k) + ", a.ptr[" + std::to_string(o.a) +
             "], i, cnt);\n";
    }
    // normcdf(y) and normcdf(-y) in one program share one erfc core
    // (normcdf_pair: bit-identical to the two calls in both policies, as
    // |-c y| == |c y| and only the final select differs); the pair is emitted
    // at the first of the two, the second is skipped
    std::vector<int> partner(ops.size(), -1);
    {
        std::vector<int> ncdf_of(ops.size(), -1);  // argument value -> normcdf value
        for (size_t k = 0; k < ops.size(); ++k)
            if (ops[k].code == NT2G_OP_NORMCDF && ncdf_of[ops[k].a] < 0) ncdf_of[ops[k].a] = (int)k;
        for (size_t k = 0; k < ops.size(); ++k) {
            if (ops[k].code != NT2G_OP_NORMCDF || partner[k] >= 0) continue;
            const nt2g_op &arg = ops[ops[k].a];
            if (arg.code != NT2G_OP_NEG || arg.dtype != NT2G_F32) continue;
            const int j = ncdf_of[arg.a];
            if (j >= 0 && partner[j] < 0 && j != (int)k) {
                partner[j] = (int)k;
                partner[k] = j;
            }
        }
    }
    for (size_t k = 0; k < ops.size(); ++k) {
        const nt2g_op &o = ops[k];
        const bool f32 = o.dtype == NT2G_F32;
        const bool u = logical[k] || !f32;  // uint32 lanes: uint8 data and logicals
        if (partner[k] >= 0) {
            const int p = partner[k];
            if (p < (int)k) continue;  // emitted with its partner
            // the positive side is the one whose argument is y itself
            const bool k_is_neg = ops[o.a].code == NT2G_OP_NEG && ops[o.a].a == ops[p].a;
            const int pos = k_is_neg ? p : (int)k, neg = k_is_neg ? (int)k : p;
            s += "    float v" + std::to_string(k) + "[A], v" + std::to_string(p) + "[A]; NT2G_LL nt2g::normcdf_pair<P>(" +
                 v(ops[pos].a) + ", " + v(pos) + ", " + v(neg) + ");\n";
            continue;
        }
        const std::string A = o.a >= 0 ? v(o.a) : "", B = o.b >= 0 ? v(o.b) : "", C = o.c >= 0 ? v(o.c) : "";
        const std::string slot = std::to_string(o.a);
        std::string e;
        switch (o.code) {
        case NT2G_OP_LOAD: continue;  // emitted above
        case NT2G_OP_FOLD:  // a comparison result folds as 0.0f / 1.0f
            if (stores) s += "    NT2G_LL out[j] = (float)v" + std::to_string(o.a) + "[j];\n";
            continue;
        case NT2G_OP_STORE: {
            if (!stores) continue;  // the reverse sweep recomputes values, it stores none
            const std::string src = "v" + std::to_string(o.a);
            const std::string dst = std::to_string(o.b);
            if (f32 && logical[o.a])  // a comparison result stored as 0.0f / 1.0f
                s += "    { float t[A]; NT2G_LL t[j] = (float)" + src + "[j]; jit_stf<FULL>(a.ptr[" + dst + "], i, cnt, t); }\n";
            else
                s += std::string(f32 ? "    jit_stf<FULL>(a.ptr[" : "    jit_stb<FULL>(a.ptr[") + dst + "], i, cnt, " +
                     src + ");\n";
            continue;
        }
        case NT2G_OP_SCALAR: e = f32 ? "a.scal[" + slot + "]" : "a.scal_u8[" + slot + "]"; break;
        case NT2G_OP_CONST: e = f32 ? fconst(o.imm) : std::to_string((uint32_t)o.imm & 255u) + "u"; break;
        case NT2G_OP_INDEX:
            e = f32 ? "nt2g::pos_to_float(a.pos0 + jit_pos<L>(i, j))" : "(unsigned)((a.pos0 + jit_pos<L>(i, j)) & 255)";
            break;
        case NT2G_OP_ADD: e = f32 ? "P::add(" + A + ", " + B + ")" : "(" + A + " + " + B + ") & 255u"; break;
        case NT2G_OP_SUB: e = f32 ? "P::sub(" + A + ", " + B + ")" : "(" + A + " - " + B + ") & 255u"; break;
        case NT2G_OP_MUL: e = f32 ? "P::mul(" + A + ", " + B + ")" : "(" + A + " * " + B + ") & 255u"; break;
        case NT2G_OP_DIV: e = "P::div(" + A + ", " + B + ")"; break;
        case NT2G_OP_MIN: e = "(" + A + " < " + B + " ? " + A + " : " + B + ")"; break;  // NT2: a < b ? a : b
        case NT2G_OP_MAX: e = "(" + A + " > " + B + " ? " + A + " : " + B + ")"; break;  // NT2: a > b ? a : b
        case NT2G_OP_ADDS: e = "((" + A + " + " + B + ") > 255u ? 255u : (" + A + " + " + B + "))"; break;
        case NT2G_OP_FMA: e = "P::fma(" + A + ", " + B + ", " + C + ")"; break;
        case NT2G_OP_POW: e = "nt2g::pow<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_ATAN2: e = "nt2g::atan2<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_HYPOT: e = "nt2g::hypot<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_MOD: e = "nt2g::mod_<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_REM: e = "nt2g::rem_<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_POW2: e = "nt2g::pow2_<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_CBRT: e = "nt2g::cbrt<P>(" + A + ")"; break;
        case NT2G_OP_COT: e = "nt2g::cot<P>(" + A + ")"; break;
        case NT2G_OP_SEC: e = "nt2g::sec<P>(" + A + ")"; break;
        case NT2G_OP_CSC: e = "nt2g::csc<P>(" + A + ")"; break;
        case NT2G_OP_SIND: e = "nt2g::sind<P>(" + A + ")"; break;
        case NT2G_OP_COSD: e = "nt2g::cosd<P>(" + A + ")"; break;
        case NT2G_OP_TAND: e = "nt2g::tand<P>(" + A + ")"; break;
        case NT2G_OP_TANPI: e = "nt2g::tanpi<P>(" + A + ")"; break;
        case NT2G_OP_PROPER_TANPI: e = "nt2g::proper_tanpi<P>(" + A + ")"; break;
        case NT2G_OP_COTPI: e = "nt2g::cotpi<P>(" + A + ")"; break;
        case NT2G_OP_COTD: e = "nt2g::cotd<P>(" + A + ")"; break;
        case NT2G_OP_SECPI: e = "nt2g::secpi<P>(" + A + ")"; break;
        case NT2G_OP_CSCPI: e = "nt2g::cscpi<P>(" + A + ")"; break;
        case NT2G_OP_SECD: e = "nt2g::secd<P>(" + A + ")"; break;
        case NT2G_OP_CSCD: e = "nt2g::cscd<P>(" + A + ")"; break;
        case NT2G_OP_SINC: e = "nt2g::sinc<P>(" + A + ")"; break;
        case NT2G_OP_SINCPI: e = "nt2g::sincpi<P>(" + A + ")"; break;
        case NT2G_OP_ACOTD: e = "nt2g::acotd<P>(" + A + ")"; break;
        case NT2G_OP_ASEC: e = "nt2g::asec<P>(" + A + ")"; break;
        case NT2G_OP_COTH: e = "nt2g::coth<P>(" + A + ")"; break;
        case NT2G_OP_SINHC: e = "nt2g::sinhc<P>(" + A + ")"; break;
        case NT2G_OP_ACSC: e = "nt2g::acsc<P>(" + A + ")"; break;
        case NT2G_OP_ASECH: e = "nt2g::asech<P>(" + A + ")"; break;
        case NT2G_OP_ACOTH: e = "nt2g::acoth<P>(" + A + ")"; break;
        case NT2G_OP_ACSCH: e = "nt2g::acsch<P>(" + A + ")"; break;
        case NT2G_OP_ERF: e = "nt2g::erf<P>(" + A + ")"; break;
        case NT2G_OP_ERFCX: e = "nt2g::erfcx<P>(" + A + ")"; break;
        case NT2G_OP_EXPX2: e = "nt2g::expx2<P>(" + A + ")"; break;
        case NT2G_OP_GAMMA: e = "nt2g::gamma<P>(" + A + ")"; break;
        case NT2G_OP_GAMMALN: e = "nt2g::gammaln<P>(" + A + ")"; break;
        case NT2G_OP_SIGNGAM: e = "nt2g::signgam(" + A + ")"; break;
        case NT2G_OP_DIGAMMA: e = "nt2g::digamma<P>(" + A + ")"; break;
        case NT2G_OP_DAWSON: e = "nt2g::dawson<P>(" + A + ")"; break;
        case NT2G_OP_SPENCE: e = "nt2g::spence<P>(" + A + ")"; break;
        case NT2G_OP_STIRLING: e = "nt2g::stirling<P>(" + A + ")"; break;
        case NT2G_OP_GAMMAINCINV: e = "nt2g::gammaincinv<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_NTHROOT: e = "nt2g::nthroot<P>(" + A + ", nt2g::int_operand(" + B + "))"; break;
        case NT2G_OP_EXPNI: e = "nt2g::expni<P>(nt2g::int_operand(" + A + "), " + B + ")"; break;
        case NT2G_OP_GAMMAINC: e = "nt2g::gammainc<P>(" + A + ", " + B + ")"; break;
        case NT2G_OP_ERFINV: e = "nt2g::erfinv<P>(" + A + ")"; break;
        case NT2G_OP_ERFCINV: e = "nt2g::erfcinv<P>(" + A + ")"; break;
        case NT2G_OP_FLOOR: e = "floorf(" + A + ")"; break;
        case NT2G_OP_CEIL: e = "ceilf(" + A + ")"; break;
        case NT2G_OP_TRUNC: e = "truncf(" + A + ")"; break;
        case NT2G_OP_ROUND: e = "roundf(" + A + ")"; break;
        case NT2G_OP_ROUND2EVEN: e = "nt2g::nt2_round2even(" + A + ")"; break;
        case NT2G_OP_FRAC: e = "nt2g::nt2_frac<P>(" + A + ")"; break;
        case NT2G_OP_SIGN: e = "nt2g::nt2_sign(" + A + ")"; break;
        case NT2G_OP_SIGNNZ: e = "nt2g::nt2_signnz(" + A + ")"; break;
        case NT2G_OP_COPYSIGN: e = "copysignf(" + A + ", " + B + ")"; break;
        case NT2G_OP_IS_NAN: e = "(" + A + " != " + A + ") ? 1u : 0u"; break;
        case NT2G_OP_IS_INF: e = "(fabsf(" + A + ") == __int_as_float(0x7f800000)) ? 1u : 0u"; break;
        case NT2G_OP_IS_FINITE: e = "((" + A + " - " + A + ") == 0.0f) ? 1u : 0u"; break;
        case NT2G_OP_IS_EQZ: e = "(" + A + " == 0.0f) ? 1u : 0u"; break;
        case NT2G_OP_IS_NEZ: e = "(" + A + " != 0.0f) ? 1u : 0u"; break;
        case NT2G_OP_IS_LTZ: e = "(" + A + " < 0.0f) ? 1u : 0u"; break;
        case NT2G_OP_IS_GTZ: e = "(" + A + " > 0.0f) ? 1u : 0u"; break;
        case NT2G_OP_EXPRECNEG: e = "nt2g::exprecneg<P>(" + A + ")"; break;
        case NT2G_OP_EXPRECNEGC: e = "nt2g::exprecnegc<P>(" + A + ")"; break;
        case NT2G_OP_SQRT1PM1: e = "nt2g::sqrt1pm1<P>(" + A + ")"; break;
        case NT2G_OP_FNMS: e = "P::fma(-" + A + ", " + B + ", " + C + ")"; break;
        case NT2G_OP_LT: e = "(" + A + " < " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_GT: e = "(" + A + " > " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_LE: e = "(" + A + " <= " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_GE: e = "(" + A + " >= " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_EQ: e = "(" + A + " == " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_NE: e = "(" + A + " != " + B + ") ? 1u : 0u"; break;
        case NT2G_OP_IF_ELSE: e = A + " ? " + B + " : " + C; break;
        case NT2G_OP_SELINC:
            e = f32 ? A + " ? P::add(" + B + ", 1.0f) : " + B : A + " ? ((" + B + " + 1u) & 255u) : " + B;
            break;
        case NT2G_OP_SELDEC:
            e = f32 ? A + " ? P::add(" + B + ", -1.0f) : " + B : A + " ? ((" + B + " - 1u) & 255u) : " + B;
            break;
        case NT2G_OP_IF_ZERO_ELSE_ONE: e = f32 ? A + " ? 0.0f : 1.0f" : A + " ? 0u : 1u"; break;
        case NT2G_OP_NEG: e = f32 ? "-" + A : "(0u - " + A + ") & 255u"; break;
        case NT2G_OP_ABS: e = f32 ? "fabsf(" + A + ")" : A; break;
        case NT2G_OP_SQR: e = f32 ? "P::mul(" + A + ", " + A + ")" : "(" + A + " * " + A + ") & 255u"; break;
        case NT2G_OP_SQRT: e = "P::sqrt(" + A + ")"; break;
        case NT2G_OP_REC: e = "P::div(1.0f, " + A + ")"; break;
        case NT2G_OP_EXP: e = "nt2g::exp<P>(" + A + ")"; break;
        case NT2G_OP_LOG: e = "nt2g::log<P>(" + A + ")"; break;
        case NT2G_OP_LOG1P: e = "nt2g::log1p<P>(" + A + ")"; break;
        case NT2G_OP_ERFC: e = "nt2g::erfc<P>(" + A + ")"; break;
        case NT2G_OP_NORMCDF: e = "nt2g::normcdf<P>(" + A + ")"; break;
        case NT2G_OP_EXP2: e = "nt2g::exp2<P>(" + A + ")"; break;
        case NT2G_OP_EXP10: e = "nt2g::exp10<P>(" + A + ")"; break;
        case NT2G_OP_EXPM1: e = "nt2g::expm1<P>(" + A + ")"; break;
        case NT2G_OP_LOG2: e = "nt2g::log2<P>(" + A + ")"; break;
        case NT2G_OP_LOG10: e = "nt2g::log10<P>(" + A + ")"; break;
        case NT2G_OP_SIN: e = "nt2g::sin<P>(" + A + ")"; break;
        case NT2G_OP_COS: e = "nt2g::cos<P>(" + A + ")"; break;
        case NT2G_OP_TAN: e = "nt2g::tan<P>(" + A + ")"; break;
        case NT2G_OP_SINPI: e = "nt2g::sinpi<P>(" + A + ")"; break;
        case NT2G_OP_COSPI: e = "nt2g::cospi<P>(" + A + ")"; break;
        case NT2G_OP_SINH: e = "nt2g::sinh<P>(" + A + ")"; break;
        case NT2G_OP_COSH: e = "nt2g::cosh<P>(" + A + ")"; break;
        case NT2G_OP_TANH: e = "nt2g::tanh<P>(" + A + ")"; break;
        case NT2G_OP_ASIN: e = "nt2g::asin<P>(" + A + ")"; break;
        case NT2G_OP_ACOS: e = "nt2g::acos<P>(" + A + ")"; break;
        case NT2G_OP_ATAN: e = "nt2g::atan<P>(" + A + ")"; break;
        case NT2G_OP_ASINH: e = "nt2g::asinh<P>(" + A + ")"; break;
        case NT2G_OP_ACOSH: e = "nt2g::acosh<P>(" + A + ")"; break;
        case NT2G_OP_ATANH: e = "nt2g::atanh<P>(" + A + ")"; break;
        default: e = "nt2g::fastnormcdf<P>(" + A + ")"; break;
        }
        s += std::string(u ? "    unsigned v" : "    float v") + std::to_string(k) + "[A]; NT2G_LL v" +
             std::to_string(k) + "[j] = " + e + ";\n";
    }
}

std::string jit_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision)
{
    std::string s;
    s.reserve(sizeof kJitPrelude + 40000 + ops.size() * 96);
    s += kNt2gMathSrc;
    s += kJitPrelude;
    s += "template <class P, bool FULL>\n__device__ __forceinline__ void jit_tile(const JitArgs &a, long long i, int cnt)\n{\n"
         "    constexpr int L = 4, A = 4;\n";
    emit_body(s, ops, logical);
    s += "}\n\nextern \"C\" __global__ void __launch_bounds__(256) nt2g_jit_kernel(const JitArgs a, long long n, int vec)\n{\n";
    s += precision == NT2G_PREC_NT2 ? "    typedef nt2g::Nt2 P;\n" : "    typedef nt2g::Fast P;\n";
    s += "    const long long stride = (long long)gridDim.x * blockDim.x * 4;\n"
         "    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4; i < n; i += stride) {\n"
         "        const int cnt = n - i < 4 ? (int)(n - i) : 4;\n"
         "        if (vec && cnt == 4) jit_tile<P, true>(a, i, 4);\n"
         "        else jit_tile<P, false>(a, i, cnt);\n"
         "    }\n}\n";
    return s;
}

// A fold of a program's FOLD value: the program becomes the element function
// jit_value (L = 1: one element; L = 4: four consecutive elements, 128-bit
// table reads when FULL), wrapped as the fold source ExprSrc, and the fold
// bodies of nt2g_fold_kernels.cuh are instantiated over it for op.  The NT2
// policy folds in index order (fold_nt2) only; the fast policy and NT2's
// elements under the compensated fold also get the short-segment, contiguous
// (FINAL x IDX) and strided (VEC x FINAL) kernels.
std::string jit_fold_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                            int op)
{
    std::string s;
    s.reserve(sizeof kJitPrelude + sizeof kNt2gAccumSrc + sizeof kNt2gFoldSrc + 40000 + ops.size() * 96);
    s += kNt2gMathSrc;
    s += kJitPrelude;
    s += kNt2gAccumSrc;
    s += kNt2gFoldSrc;
    s += "template <class P, bool FULL, int L>\n__device__ __forceinline__ void jit_value(const JitArgs &a, long long i, "
         "int cnt, float (&out)[4])\n{\n    constexpr int A = 4;\n";
    emit_body(s, ops, logical);
    s += "}\n\n";
    s += precision == NT2G_PREC_FAST ? "typedef nt2g::Fast P;\n" : "typedef nt2g::Nt2 P;\n";
    s += "struct ExprSrc {\n"
         "    JitArgs a;\n"
         "    __device__ __forceinline__ float at(long long pos) const { float o[4]; jit_value<P, false, 1>(a, pos, 1, o); "
         "return o[0]; }\n"
         "    __device__ __forceinline__ float4 at4(long long pos) const { float o[4]; jit_value<P, true, 4>(a, pos, 4, o); "
         "return make_float4(o[0], o[1], o[2], o[3]); }\n"
         "};\n";
    s += "#define NT2G_FOP " + std::to_string(op) + "\n";
    s += "using nt2g::fold::Partial;\n"
         "extern \"C\" __global__ void __launch_bounds__(256) fold_nt2(const JitArgs a, long long lo, long long inner, "
         "long long hi, float *out, long long *index, const float *cen)\n"
         "{ nt2g::fold::nt2_body<ExprSrc, NT2G_FOP>(ExprSrc{a}, lo, inner, hi, out, index, cen); }\n";
    if (precision == NT2G_PREC_NT2) return s;
    s += "extern \"C\" __global__ void __launch_bounds__(256) fold_short(const JitArgs a, long long inner, long long hi, "
         "float *out, long long *index, const float *cen, double *out64)\n"
         "{ nt2g::fold::short_body<ExprSrc, NT2G_FOP>(ExprSrc{a}, inner, hi, out, index, cen, out64); }\n";
    for (int fin = 0; fin < 2; ++fin)
        for (int idx = 0; idx < 2; ++idx) {
            const std::string F = fin ? "true" : "false", I = idx ? "true" : "false";
            s += "extern \"C\" __global__ void __launch_bounds__(256) fold_inner_" + std::to_string(fin) +
                 std::to_string(idx) +
                 "(const JitArgs a, long long inner, long long hi, long long chunk, long long q, int vec, Partial *part, "
                 "float *out, long long *index, const float *cen, double *out64)\n"
                 "{ nt2g::fold::inner_body<ExprSrc, NT2G_FOP, " + F + ", " + I +
                 ">(ExprSrc{a}, inner, hi, chunk, q, vec, part, out, index, cen, out64); }\n";
        }
    for (int v4 = 0; v4 < 2; ++v4)
        for (int fin = 0; fin < 2; ++fin) {
            const std::string V = v4 ? "4" : "1", F = fin ? "true" : "false";
            s += "extern \"C\" __global__ void __launch_bounds__(256) fold_outer_" + std::to_string(v4) +
                 std::to_string(fin) +
                 "(const JitArgs a, long long lo, long long inner, long long hi, long long ck, long long q, "
                 "Partial *part, float *out, long long *index, const float *cen, double *out64)\n"
                 "{ nt2g::fold::outer_body<ExprSrc, NT2G_FOP, " + V + ", " + F +
                 ">(ExprSrc{a}, lo, inner, hi, ck, q, part, out, index, cen, out64); }\n";
        }
    return s;
}

// The programs of a batch linked into one persistent kernel.  Each program
// becomes prog<k>_tile (W float4 vectors per thread: 4 W lanes, the second
// vector a block-width further); the kernel takes tiles of the batch's items
// (a static stride over the grid or an atomic counter) and switches on the
// item's program once per tile, so the dispatch is block-uniform.  A tile is
// run in whole aligned pairs of vectors while they last (W = 2), then one
// vector at a time, the ragged end by element.  The statements are those of
// jit_source, so every element is bit-identical to the program's own kernel.
std::string jit_batch_source(const std::vector<ProgramCode> &progs, int precision, int block_threads)
{
    std::string s;
    s.reserve(sizeof kJitPrelude + 40000 + progs.size() * 4096);
    s += kNt2gMathSrc;
    s += kJitPrelude;
    s += "struct BItem { JitArgs a; long long n; int prog; int vec; };\n";
    for (size_t k = 0; k < progs.size(); ++k) {
        s += "template <class P, bool FULL, int W>\n__device__ __forceinline__ void prog" + std::to_string(k) +
             "_tile(const JitArgs &a, long long i, int cnt)\n{\n    constexpr int L = 4 * W, A = 4 * W;\n";
        emit_body(s, *progs[k].ops, *progs[k].logical);
        s += "}\n";
    }
    s += precision == NT2G_PREC_NT2 ? "typedef nt2g::Nt2 P;\n" : "typedef nt2g::Fast P;\n";
    s += "#define NT2G_RUN(fn) { \\\n"
         "    const long long step = (long long)blockDim.x * 4; \\\n"
         "    long long i = start + (long long)threadIdx.x * 4; \\\n"
         "    if constexpr (W == 2) { \\\n"
         "        if (it.vec) for (; i + step + 4 <= end; i += 2 * step) fn<P, true, 2>(it.a, i, 8); } \\\n"
         "    for (; i < end; i += step) { \\\n"
         "        const int cnt = end - i < 4 ? (int)(end - i) : 4; \\\n"
         "        if (it.vec && cnt == 4) fn<P, true, 1>(it.a, i, 4); else fn<P, false, 1>(it.a, i, cnt); } }\n";
    s += "__device__ __forceinline__ int find_item(const long long *prefix, int n_items, long long t)\n{\n"
         "    int lo = 0, hi = n_items;\n"
         "    while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (__ldg(prefix + mid) <= t) lo = mid; else hi = mid; }\n"
         "    return lo;\n}\n";
    s += "template <bool DYNAMIC, int W>\n__device__ __forceinline__ void batch_body(const BItem *items, "
         "const long long *prefix, int n_items, long long total_tiles, long long tile_elems, "
         "unsigned long long *counter)\n{\n"
         "    __shared__ long long s_tile;\n"
         "    long long t = DYNAMIC ? 0 : blockIdx.x;\n"
         "    while (true) {\n"
         "        if (DYNAMIC) {\n"
         "            if (threadIdx.x == 0) s_tile = (long long)atomicAdd(counter, 1ull);\n"
         "            __syncthreads();\n"
         "            t = s_tile;\n"
         "            __syncthreads();\n"
         "        }\n"
         "        if (t >= total_tiles) return;\n"
         "        const int k = find_item(prefix, n_items, t);\n"
         "        const BItem it = items[k];\n"
         "        const long long start = (t - __ldg(prefix + k)) * tile_elems;\n"
         "        const long long end = start + tile_elems < it.n ? start + tile_elems : it.n;\n"
         "        switch (it.prog) {\n";
    for (size_t k = 0; k < progs.size(); ++k)
        s += "        case " + std::to_string(k) + ": NT2G_RUN(prog" + std::to_string(k) + "_tile); break;\n";
    s += "        default: break;\n"
         "        }\n"
         "        if (!DYNAMIC) t += gridDim.x;\n"
         "    }\n}\n";
    const std::string bt = std::to_string(block_threads);
    for (int dyn = 0; dyn < 2; ++dyn)
        for (int w = 1; w <= 2; ++w)
            s += "extern \"C\" __global__ void __launch_bounds__(" + bt + ") batch_" + std::to_string(dyn) +
                 std::to_string(w) + "(const BItem *items, const long long *prefix, int n_items, long long total_tiles, "
                 "long long tile_elems, unsigned long long *counter)\n{ batch_body<" + (dyn ? "true" : "false") + ", " +
                 std::to_string(w) + ">(items, prefix, n_items, total_tiles, tile_elems, counter); }\n";
    return s;
}

// ------------------------------------------------------------ reverse mode --
// The adjoint rule of one instruction: the statements that add its result's
// adjoint G (g<k>) times the local partial derivatives into the adjoints of
// its active operands.  Forward values are the v<k> registers; D is the fast
// policy, used for the derivative arithmetic.  Empty when the instruction
// passes no gradient (comparisons, rounding, sign, constants); false when the
// opcode has no rule.
static bool adjoint_rule(std::string &s, const std::vector<nt2g_op> &ops, int k, const std::vector<uint8_t> &active,
                         std::vector<uint8_t> &phi_done)
{
    const nt2g_op &o = ops[k];
    auto v = [](int x) { return "v" + std::to_string(x) + "[j]"; };
    auto g = [](int x) { return "g" + std::to_string(x) + "[j]"; };
    const std::string G = g(k), Y = v(k);
    const std::string A = o.a >= 0 ? v(o.a) : "", B = o.b >= 0 ? v(o.b) : "", C = o.c >= 0 ? v(o.c) : "";
    std::vector<std::pair<int, std::string>> add;  // (operand, partial derivative term to add: G * d)
    std::string pre;  // per-lane temporaries the terms share
    auto to = [&](int operand, const std::string &term) {
        if (operand >= 0 && active[operand]) add.emplace_back(operand, term);
    };
    auto act = [&](int operand) { return operand >= 0 && active[operand]; };
    const std::string pi = "nt2g::vjp::kPi", deg = "nt2g::vjp::kDegToRad";
    auto rcp = [](const std::string &x) { return "nt2g::vjp::grcp(" + x + ")"; };
    auto rsq = [](const std::string &x) { return "nt2g::vjp::grsqrt(" + x + ")"; };
    const std::string one_m_a2 = "((1.0f - " + A + ") * (1.0f + " + A + "))";  // exact difference near |a| = 1
    const std::string abs_a2_m1 = "((fabsf(" + A + ") - 1.0f) * (fabsf(" + A + ") + 1.0f))";
    switch (o.code) {
    case NT2G_OP_ADD: to(o.a, G); to(o.b, G); break;
    case NT2G_OP_SUB: to(o.a, G); to(o.b, "-" + G); break;
    case NT2G_OP_MUL: to(o.a, G + " * " + B); to(o.b, G + " * " + A); break;
    case NT2G_OP_DIV:  // a/b: G/b and -G (a/b) / b, one reciprocal
        pre = "const float q = " + G + " * " + rcp(B) + ";";
        to(o.a, "q");
        to(o.b, "-q * " + Y);
        break;
    case NT2G_OP_NEG: to(o.a, "-" + G); break;
    case NT2G_OP_ABS: to(o.a, "(" + A + " > 0.0f ? " + G + " : " + A + " < 0.0f ? -" + G + " : 0.0f)"); break;
    case NT2G_OP_SQR: to(o.a, "2.0f * " + A + " * " + G); break;
    case NT2G_OP_SQRT: to(o.a, "0.5f * " + G + " * " + rcp(Y)); break;
    case NT2G_OP_REC: to(o.a, "-" + G + " * " + Y + " * " + Y); break;
    case NT2G_OP_MIN: to(o.a, "(" + A + " < " + B + " ? " + G + " : 0.0f)"); to(o.b, "(" + A + " < " + B + " ? 0.0f : " + G + ")"); break;
    case NT2G_OP_MAX: to(o.a, "(" + A + " > " + B + " ? " + G + " : 0.0f)"); to(o.b, "(" + A + " > " + B + " ? 0.0f : " + G + ")"); break;
    case NT2G_OP_FMA: to(o.a, G + " * " + B); to(o.b, G + " * " + A); to(o.c, G); break;
    case NT2G_OP_FNMS: to(o.a, "-" + G + " * " + B); to(o.b, "-" + G + " * " + A); to(o.c, G); break;
    case NT2G_OP_EXP: to(o.a, G + " * " + Y); break;
    case NT2G_OP_LOG: to(o.a, G + " * " + rcp(A)); break;
    case NT2G_OP_LOG1P: to(o.a, G + " * " + rcp("1.0f + " + A)); break;
    case NT2G_OP_ERF: to(o.a, G + " * nt2g::vjp::kTwoOverSqrtPi * nt2g::exp<D>(-" + A + " * " + A + ")"); break;
    case NT2G_OP_ERFC: to(o.a, "-" + G + " * nt2g::vjp::kTwoOverSqrtPi * nt2g::exp<D>(-" + A + " * " + A + ")"); break;
    case NT2G_OP_NORMCDF: {
        // phi(y) once for normcdf(y) and normcdf(-y) (the pair of a
        // call/put): the density is even
        const bool neg = ops[o.a].code == NT2G_OP_NEG && ops[o.a].dtype == NT2G_F32;
        const int base = neg ? ops[o.a].a : o.a;
        const std::string phi = "phi" + std::to_string(base);
        if (act(o.a) && !phi_done[base]) {
            phi_done[base] = 1;
            s += "    float " + phi + "[4]; NT2G_L " + phi + "[j] = nt2g::vjp::kInvSqrt2Pi * nt2g::exp<D>(-0.5f * " +
                 v(base) + " * " + v(base) + ");\n";
        }
        to(o.a, G + " * " + phi + "[j]");
        break;
    }
    case NT2G_OP_FASTNORMCDF: to(o.a, G + " * nt2g::vjp::fastnormcdf_grad<D>(" + A + ")"); break;
    case NT2G_OP_EXP2: to(o.a, G + " * " + Y + " * nt2g::vjp::kLn2"); break;
    case NT2G_OP_EXP10: to(o.a, G + " * " + Y + " * nt2g::vjp::kLn10"); break;
    case NT2G_OP_EXPM1: to(o.a, G + " * nt2g::exp<D>(" + A + ")"); break;  // not y + 1: it cancels as y -> -1
    case NT2G_OP_LOG2: to(o.a, G + " * " + rcp(A) + " * nt2g::vjp::kInvLn2"); break;
    case NT2G_OP_LOG10: to(o.a, G + " * " + rcp(A) + " * nt2g::vjp::kInvLn10"); break;
    case NT2G_OP_SIN: to(o.a, G + " * nt2g::cos<D>(" + A + ")"); break;
    case NT2G_OP_COS: to(o.a, "-" + G + " * nt2g::sin<D>(" + A + ")"); break;
    case NT2G_OP_TAN: to(o.a, G + " * (1.0f + " + Y + " * " + Y + ")"); break;
    case NT2G_OP_SINPI: to(o.a, G + " * " + pi + " * nt2g::cospi<D>(" + A + ")"); break;
    case NT2G_OP_COSPI: to(o.a, "-" + G + " * " + pi + " * nt2g::sinpi<D>(" + A + ")"); break;
    case NT2G_OP_TANPI: case NT2G_OP_PROPER_TANPI:
        to(o.a, G + " * " + pi + " * (1.0f + " + Y + " * " + Y + ")");
        break;
    case NT2G_OP_SIND: to(o.a, G + " * " + deg + " * nt2g::cosd<D>(" + A + ")"); break;
    case NT2G_OP_COSD: to(o.a, "-" + G + " * " + deg + " * nt2g::sind<D>(" + A + ")"); break;
    case NT2G_OP_TAND: to(o.a, G + " * " + deg + " * (1.0f + " + Y + " * " + Y + ")"); break;
    case NT2G_OP_COT: to(o.a, "-" + G + " * (1.0f + " + Y + " * " + Y + ")"); break;
    case NT2G_OP_COTPI: to(o.a, "-" + G + " * " + pi + " * (1.0f + " + Y + " * " + Y + ")"); break;
    case NT2G_OP_COTD: to(o.a, "-" + G + " * " + deg + " * (1.0f + " + Y + " * " + Y + ")"); break;
    case NT2G_OP_SEC: to(o.a, G + " * " + Y + " * nt2g::tan<D>(" + A + ")"); break;
    case NT2G_OP_SECPI: to(o.a, G + " * " + pi + " * " + Y + " * nt2g::tanpi<D>(" + A + ")"); break;
    case NT2G_OP_SECD: to(o.a, G + " * " + deg + " * " + Y + " * nt2g::tand<D>(" + A + ")"); break;
    case NT2G_OP_CSC: to(o.a, "-" + G + " * " + Y + " * nt2g::cot<D>(" + A + ")"); break;
    case NT2G_OP_CSCPI: to(o.a, "-" + G + " * " + pi + " * " + Y + " * nt2g::cotpi<D>(" + A + ")"); break;
    case NT2G_OP_CSCD: to(o.a, "-" + G + " * " + deg + " * " + Y + " * nt2g::cotd<D>(" + A + ")"); break;
    case NT2G_OP_SINC: to(o.a, G + " * nt2g::vjp::sinc_grad<D>(" + A + ", " + Y + ")"); break;
    case NT2G_OP_SINCPI: to(o.a, G + " * nt2g::vjp::sincpi_grad<D>(" + A + ", " + Y + ")"); break;
    case NT2G_OP_SINHC: to(o.a, G + " * nt2g::vjp::sinhc_grad<D>(" + A + ", " + Y + ")"); break;
    case NT2G_OP_POW:  // b a^(b-1); a^b ln a (0 where a^b is 0, NaN for a < 0)
        to(o.a, G + " * " + B + " * nt2g::pow<D>(" + A + ", " + B + " - 1.0f)");
        to(o.b, "(" + A + " > 0.0f ? " + G + " * " + Y + " * nt2g::log<D>(" + A + ") : " + Y + " == 0.0f ? 0.0f : __int_as_float(0x7fc00000))");
        break;
    case NT2G_OP_SINH: to(o.a, G + " * nt2g::cosh<D>(" + A + ")"); break;
    case NT2G_OP_COSH: to(o.a, G + " * nt2g::sinh<D>(" + A + ")"); break;
    // 1 - tanh^2 = 1/cosh^2 and 1 - coth^2 = -1/sinh^2: the forms in y would
    // magnify y's rounding where |y| nears 1
    case NT2G_OP_TANH:
        pre = "const float c = nt2g::cosh<D>(" + A + ");";
        to(o.a, G + " * " + rcp("c * c"));
        break;
    case NT2G_OP_COTH:
        pre = "const float c = nt2g::sinh<D>(" + A + ");";
        to(o.a, "-" + G + " * " + rcp("c * c"));
        break;
    // 1 - a^2 as (1 - a)(1 + a), a^2 - 1 as (|a| - 1)(|a| + 1): exact differences near |a| = 1
    case NT2G_OP_ASIN: to(o.a, G + " * " + rsq(one_m_a2)); break;
    case NT2G_OP_ACOS: to(o.a, "-" + G + " * " + rsq(one_m_a2)); break;
    case NT2G_OP_ATAN: to(o.a, G + " * " + rcp("1.0f + " + A + " * " + A)); break;
    case NT2G_OP_ATAN2:  // atan2(a, b): (b, -a) / (a^2 + b^2)
        pre = "const float q = " + G + " * " + rcp(A + " * " + A + " + " + B + " * " + B) + ";";
        to(o.a, "q * " + B);
        to(o.b, "-q * " + A);
        break;
    case NT2G_OP_MOD:  // a - floor(a/b) b: 1 and -floor(a/b) between the jumps (b = 0: 1 and 0)
        to(o.a, G);
        to(o.b, "(" + B + " != 0.0f ? -" + G + " * floorf(" + A + " / " + B + ") : 0.0f)");
        break;
    case NT2G_OP_REM:  // a - b trunc(a/b): 1 and -trunc(a/b) between the jumps
        to(o.a, G);
        to(o.b, "(" + B + " != 0.0f ? -" + G + " * (float)nt2g::toints(" + A + " / " + B + ") : 0.0f)");
        break;
    case NT2G_OP_POW2:  // a 2^n: the scale for a; n is piecewise constant
        to(o.a, G + " * nt2g::pow2_<D>(1.0f, " + B + ")");
        break;
    case NT2G_OP_HYPOT:
        pre = "const float q = " + Y + " == 0.0f ? 0.0f : " + G + " * " + rcp(Y) + ";";
        to(o.a, "q * " + A);
        to(o.b, "q * " + B);
        break;
    case NT2G_OP_ASINH: to(o.a, G + " * " + rsq(A + " * " + A + " + 1.0f")); break;
    case NT2G_OP_ACOSH: to(o.a, G + " * " + rsq(A + " - 1.0f") + " * " + rsq(A + " + 1.0f")); break;
    case NT2G_OP_ATANH: to(o.a, G + " * " + rcp(one_m_a2)); break;
    case NT2G_OP_ACOTD: to(o.a, "-" + G + " * nt2g::vjp::kRadToDeg * " + rcp("1.0f + " + A + " * " + A)); break;
    case NT2G_OP_ASEC: to(o.a, G + " * " + rcp("fabsf(" + A + ")") + " * " + rsq(abs_a2_m1)); break;
    case NT2G_OP_ACSC: to(o.a, "-" + G + " * " + rcp("fabsf(" + A + ")") + " * " + rsq(abs_a2_m1)); break;
    case NT2G_OP_ASECH: to(o.a, "-" + G + " * " + rcp(A) + " * " + rsq(one_m_a2)); break;
    case NT2G_OP_ACOTH: to(o.a, G + " * " + rcp(one_m_a2)); break;
    case NT2G_OP_ACSCH: to(o.a, "-" + G + " * " + rcp("fabsf(" + A + ")") + " * " + rsq("1.0f + " + A + " * " + A)); break;
    case NT2G_OP_CBRT: to(o.a, G + " * " + rcp("3.0f * " + Y + " * " + Y)); break;
    case NT2G_OP_ERFCX: to(o.a, G + " * (2.0f * " + A + " * " + Y + " - nt2g::vjp::kTwoOverSqrtPi)"); break;
    case NT2G_OP_EXPX2: to(o.a, G + " * 2.0f * " + A + " * " + Y); break;
    case NT2G_OP_GAMMA: to(o.a, G + " * " + Y + " * nt2g::vjp::digamma<D>(" + A + ")"); break;
    case NT2G_OP_GAMMALN: to(o.a, G + " * nt2g::vjp::digamma<D>(" + A + ")"); break;
    case NT2G_OP_DAWSON: to(o.a, G + " * (1.0f - 2.0f * " + A + " * " + Y + ")"); break;
    case NT2G_OP_SPENCE:  // -log(x) / (x - 1), -1 at x = 1 (x - 1 exact near 1)
        to(o.a, "(" + A + " == 1.0f ? -" + G + " : -" + G + " * nt2g::log<D>(" + A + ") * " + rcp(A + " - 1.0f") + ")");
        break;
    case NT2G_OP_NTHROOT:  // y / (n x); the integer n passes no gradient
        to(o.a, G + " * " + Y + " * " + rcp("(float)nt2g::int_operand(" + B + ") * " + A));
        break;
    case NT2G_OP_EXPNI:  // dE_n/dx = -E_(n-1)(x); E_0 = e^-x / x: -E_0 (1 + 1/x)
        to(o.b, G + " * nt2g::vjp::expni_grad<D>(nt2g::int_operand(" + A + "), " + B + ", " + Y + ")");
        break;
    case NT2G_OP_GAMMAINCINV:  // dx/dp = 1 / P'(x) at x = y; no rule for a
        if (act(o.b)) return false;
        to(o.a, G + " * " + rcp("nt2g::vjp::gammainc_dx(" + Y + ", " + B + ")"));
        break;
    case NT2G_OP_GAMMAINC:  // dP(a, x)/dx = x^(a-1) e^-x / Gamma(a); no rule for a
        if (act(o.b)) return false;
        to(o.a, G + " * nt2g::vjp::gammainc_dx(" + A + ", " + B + ")");
        break;
    case NT2G_OP_EXPRECNEG: to(o.a, G + " * " + Y + " * " + rcp(A + " * " + A)); break;
    // -e^(-1/x)/x^2 and 1/(2 sqrt(1 + x)) directly: y - 1 and y + 1 would cancel
    case NT2G_OP_EXPRECNEGC: to(o.a, "-" + G + " * nt2g::exprecneg<D>(" + A + ") * " + rcp(A + " * " + A)); break;
    case NT2G_OP_SQRT1PM1: to(o.a, "0.5f * " + G + " * " + rsq("1.0f + " + A)); break;
    case NT2G_OP_ERFINV: to(o.a, G + " * nt2g::vjp::kHalfSqrtPi * nt2g::exp<D>(" + Y + " * " + Y + ")"); break;
    case NT2G_OP_ERFCINV: to(o.a, "-" + G + " * nt2g::vjp::kHalfSqrtPi * nt2g::exp<D>(" + Y + " * " + Y + ")"); break;
    case NT2G_OP_FRAC: to(o.a, G); break;
    case NT2G_OP_COPYSIGN:  // |a| with b's sign: sign(a) sign(b)
        to(o.a, "((__float_as_uint(" + A + ") ^ __float_as_uint(" + B + ")) & 0x80000000u ? -" + G + " : " + G + ")");
        break;
    case NT2G_OP_IF_ELSE: to(o.b, "(" + A + " ? " + G + " : 0.0f)"); to(o.c, "(" + A + " ? 0.0f : " + G + ")"); break;
    case NT2G_OP_SELINC: case NT2G_OP_SELDEC: to(o.b, G); break;
    case NT2G_OP_FLOOR: case NT2G_OP_CEIL: case NT2G_OP_TRUNC: case NT2G_OP_ROUND: case NT2G_OP_ROUND2EVEN:
    case NT2G_OP_SIGN: case NT2G_OP_SIGNNZ: case NT2G_OP_IF_ZERO_ELSE_ONE: case NT2G_OP_SIGNGAM:
        break;  // piecewise constant: no gradient
    default: return false;
    }
    if (add.empty()) return true;
    if (pre.empty()) {
        for (const auto &t : add) s += "    NT2G_L g" + std::to_string(t.first) + "[j] += " + t.second + ";\n";
    } else {
        s += "    NT2G_L { " + pre;
        for (const auto &t : add) s += " g" + std::to_string(t.first) + "[j] += " + t.second + ";";
        s += " }\n";
    }
    return true;
}

// Which values carry an adjoint: float (not logical) values that depend on a
// float table or scalar argument and reach a stored value.
static std::vector<uint8_t> active_values(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical)
{
    const size_t n = ops.size();
    std::vector<uint8_t> dep(n, 0), live(n, 0), act(n, 0);
    auto is_float = [&](size_t k) { return ops[k].dtype == NT2G_F32 && !logical[k]; };
    for (size_t k = 0; k < n; ++k) {
        const nt2g_op &o = ops[k];
        if (o.code == NT2G_OP_STORE || o.code == NT2G_OP_FOLD) continue;
        if (o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR) { dep[k] = is_float(k); continue; }
        if (o.code == NT2G_OP_CONST || o.code == NT2G_OP_INDEX) continue;
        for (int x : {o.a, o.b, o.c})
            if (x >= 0 && dep[x]) dep[k] = 1;
        dep[k] &= is_float(k);
    }
    for (size_t k = n; k-- > 0;) {
        const nt2g_op &o = ops[k];
        if (o.code == NT2G_OP_STORE) { live[o.a] = 1; continue; }
        if (!live[k]) continue;
        for (int x : {o.a, o.b, o.c})
            if (x >= 0 && o.code != NT2G_OP_LOAD && o.code != NT2G_OP_SCALAR && o.code != NT2G_OP_CONST &&
                o.code != NT2G_OP_INDEX)
                live[x] = 1;
    }
    for (size_t k = 0; k < n; ++k) act[k] = dep[k] && live[k];
    return act;
}

// The float scalar slots a program's gradient sums over (in slot order).
std::vector<int> vjp_scalar_slots(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical)
{
    const std::vector<uint8_t> act = active_values(ops, logical);
    std::vector<int> slots;
    for (size_t k = 0; k < ops.size(); ++k)
        if (ops[k].code == NT2G_OP_SCALAR && act[k]) {
            bool seen = false;
            for (int s : slots) seen |= s == ops[k].a;
            if (!seen) slots.push_back(ops[k].a);
        }
    std::sort(slots.begin(), slots.end());
    return slots;
}

// The reverse-mode kernel of a program: each thread recomputes the forward
// values of 4 consecutive elements (the statements of jit_source, so the
// same bits as nt2g_eval), seeds the adjoints of the values stored into each
// output slot with that slot's cotangent table, runs the adjoint rules in
// reverse instruction order, and writes the adjoints of the loaded values to
// the slots' gradient tables.  Adjoints of float scalars are summed per
// thread in FP64, then per block (fixed order) into partials[block][scalar].
std::string jit_vjp_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                           std::string *why)
{
    const std::vector<uint8_t> act = active_values(ops, logical);
    const std::vector<int> sslots = vjp_scalar_slots(ops, logical);
    const int ns = (int)sslots.size();
    std::string s;
    s.reserve(sizeof kJitPrelude + sizeof kNt2gVjpSrc + 40000 + ops.size() * 256);
    s += kNt2gMathSrc;
    s += kNt2gVjpSrc;
    s += kJitPrelude;
    s += "struct VjpArgs { const float *ct[16]; float *grad[16]; };\n";
    s += "#define NT2G_NS " + std::to_string(ns > 0 ? ns : 1) + "\n";
    s += "template <class P, bool FULL>\n__device__ __forceinline__ void vjp_tile(const JitArgs &a, const VjpArgs &g, "
         "long long i, int cnt, double (&sacc)[NT2G_NS])\n{\n    typedef nt2g::Fast D;\n    constexpr int L = 4, A = 4;\n";
    emit_body(s, ops, logical, false);
    for (size_t k = 0; k < ops.size(); ++k)
        if (act[k]) s += "    float g" + std::to_string(k) + "[4] = {0.0f, 0.0f, 0.0f, 0.0f};\n";
    // seeds: the cotangent of each output slot flows into the last value stored there
    std::vector<int> last_store(kMaxSlots, -1);
    for (size_t k = 0; k < ops.size(); ++k)
        if (ops[k].code == NT2G_OP_STORE) last_store[ops[k].b] = (int)k;
    for (int slot = 0; slot < kMaxSlots; ++slot) {
        const int st = last_store[slot];
        if (st < 0 || !act[ops[st].a]) continue;
        const std::string sl = std::to_string(slot), val = std::to_string(ops[st].a);
        s += "    if (g.ct[" + sl + "]) { float t[4]; jit_ldf<FULL>(t, g.ct[" + sl + "], i, cnt); NT2G_L g" + val +
             "[j] += t[j]; }\n";
    }
    std::vector<uint8_t> phi_done(ops.size(), 0);
    for (size_t k = ops.size(); k-- > 0;) {
        const nt2g_op &o = ops[k];
        if (!act[k] || o.code == NT2G_OP_LOAD || o.code == NT2G_OP_SCALAR) continue;
        if (!adjoint_rule(s, ops, (int)k, act, phi_done)) {
            if (why) *why = "opcode " + std::to_string(o.code) + " has no adjoint rule";
            return "";
        }
    }
    // gradients: each loaded float table slot (its loads summed), each scalar slot
    std::vector<std::string> grad_of(kMaxSlots);
    for (size_t k = 0; k < ops.size(); ++k) {
        if (!act[k]) continue;
        const std::string gk = "g" + std::to_string(k) + "[j]";
        if (ops[k].code == NT2G_OP_LOAD) {
            std::string &e = grad_of[ops[k].a];
            e = e.empty() ? gk : e + " + " + gk;
        }
    }
    std::vector<uint8_t> read_f32(kMaxSlots, 0);
    for (size_t k = 0; k < ops.size(); ++k)
        if (ops[k].code == NT2G_OP_LOAD && ops[k].dtype == NT2G_F32) read_f32[ops[k].a] = 1;
    for (int slot = 0; slot < kMaxSlots; ++slot) {
        if (!read_f32[slot]) continue;
        const std::string sl = std::to_string(slot);
        const std::string val = grad_of[slot].empty() ? "0.0f" : grad_of[slot];  // no output depends on it
        s += "    if (g.grad[" + sl + "]) { float t[4]; NT2G_L t[j] = " + val + "; jit_stf<FULL>(g.grad[" + sl +
             "], i, cnt, t); }\n";
    }
    for (int q = 0; q < ns; ++q)
        for (size_t k = 0; k < ops.size(); ++k)
            if (ops[k].code == NT2G_OP_SCALAR && act[k] && ops[k].a == sslots[q])
                s += "    NT2G_L if (j < cnt) sacc[" + std::to_string(q) + "] += (double)g" + std::to_string(k) + "[j];\n";
    s += "}\n\n";
    s += "extern \"C\" __global__ void __launch_bounds__(256) nt2g_vjp_kernel(const JitArgs a, const VjpArgs g, "
         "long long n, int vec, double *partials)\n{\n";
    s += precision == NT2G_PREC_NT2 ? "    typedef nt2g::Nt2 P;\n" : "    typedef nt2g::Fast P;\n";
    s += "    double sacc[NT2G_NS];\n"
         "    for (int q = 0; q < NT2G_NS; ++q) sacc[q] = 0.0;\n"
         "    const long long stride = (long long)gridDim.x * blockDim.x * 4;\n"
         "    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4; i < n; i += stride) {\n"
         "        const int cnt = n - i < 4 ? (int)(n - i) : 4;\n"
         "        if (vec && cnt == 4) vjp_tile<P, true>(a, g, i, 4, sacc);\n"
         "        else vjp_tile<P, false>(a, g, i, cnt, sacc);\n"
         "    }\n";
    if (ns > 0)
        s += "    __shared__ double red[8][NT2G_NS];\n"
             "    for (int q = 0; q < NT2G_NS; ++q) {\n"
             "        double x = sacc[q];\n"
             "        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);\n"
             "        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = x;\n"
             "    }\n"
             "    __syncthreads();\n"
             "    if (partials && threadIdx.x < NT2G_NS) {\n"
             "        double x = 0.0;\n"
             "        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += red[w][threadIdx.x];\n"
             "        partials[(long long)blockIdx.x * NT2G_NS + threadIdx.x] = x;\n"
             "    }\n";
    s += "}\n";
    return s;
}

// ------------------------------------------------------------------- cache --
struct JitEntry {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
    int blocks_per_sm = 0;
    std::string error;
};

static std::mutex g_mu;
static std::map<std::string, JitEntry> g_cache;  // key: device | precision | program text

static std::string compile_cubin(const std::string &src, std::string &err)
{
    Nvrtc &nv = nvrtc();
    if (!nv.h) { err = nv.error; return ""; }
    nvrtcProgram_t prog = nullptr;
    if (nv.create(&prog, src.c_str(), "nt2g_jit.cu", 0, nullptr, nullptr) != 0) {
        err = "nvrtcCreateProgram failed";
        return "";
    }
    // no fast-math flags: the statements must round exactly like the interpreter's
    const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device"};
    int rc = nv.compile(prog, 3, opts);
    std::string cubin;
    if (rc != 0) {
        size_t n = 0;
        nv.log_size(prog, &n);
        std::string log(n, '\0');
        if (n) nv.log(prog, &log[0]);
        err = "NVRTC compile failed: " + log.substr(0, 400);
    } else {
        size_t n = 0;
        nv.cubin_size(prog, &n);
        cubin.assign(n, '\0');
        nv.cubin(prog, &cubin[0]);
    }
    nv.destroy(&prog);
    return cubin;
}

// Compiled kernel for (device, precision, program); nullptr with *why set when
// JIT is unavailable for it.
static JitEntry *jit_get(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                         std::string *why)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::string key = std::to_string(dev) + "|" + std::to_string(precision) + "|";
    key.append((const char *)ops.data(), ops.size() * sizeof(nt2g_op));
    key.append((const char *)logical.data(), logical.size());
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) {
        JitEntry e;
        std::string src = jit_source(ops, logical, precision);
        std::string cubin = compile_cubin(src, e.error);
        if (!cubin.empty()) {
            cudaError_t ce = cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
            if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.kernel, e.lib, "nt2g_jit_kernel");
            if (ce == cudaSuccess)
                ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e.blocks_per_sm, (const void *)e.kernel, 256, 0);
            if (ce != cudaSuccess) {
                e.error = std::string("loading the JIT kernel: ") + cudaGetErrorString(ce);
                cudaGetLastError();
                e.kernel = nullptr;
            }
        }
        it = g_cache.emplace(key, e).first;
    }
    if (!it->second.kernel) {
        if (why) *why = it->second.error;
        return nullptr;
    }
    return &it->second;
}

struct JitFoldEntry {
    cudaLibrary_t lib = nullptr;
    JitFoldKernels k;
    bool ok = false;
    std::string error;
};
static std::map<std::string, JitFoldEntry> g_fold_cache;  // key: device | precision | op | program text

const JitFoldKernels *jit_fold_kernels(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical,
                                       int precision, int op, std::string *why)
{
    if (!jit_enabled()) {
        if (why) *why = "JIT disabled (NT2G_JIT=0)";
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::string key = std::to_string(dev) + "|" + std::to_string(precision) + "|" + std::to_string(op) + "|";
    key.append((const char *)ops.data(), ops.size() * sizeof(nt2g_op));
    key.append((const char *)logical.data(), logical.size());
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_fold_cache.find(key);
    if (it == g_fold_cache.end()) {
        JitFoldEntry e;
        std::string cubin = compile_cubin(jit_fold_source(ops, logical, precision, op), e.error);
        if (!cubin.empty()) {
            cudaError_t ce = cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
            if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.k.nt2, e.lib, "fold_nt2");
            if (precision != NT2G_PREC_NT2) {
                if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.k.shrt, e.lib, "fold_short");
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b) {
                        const std::string ab = std::to_string(a) + std::to_string(b);
                        if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.k.inner[a][b], e.lib, ("fold_inner_" + ab).c_str());
                        if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.k.outer[a][b], e.lib, ("fold_outer_" + ab).c_str());
                    }
            }
            if (ce == cudaSuccess) {
                e.ok = true;
            } else {
                e.error = std::string("loading the JIT fold kernels: ") + cudaGetErrorString(ce);
                cudaGetLastError();
            }
        }
        it = g_fold_cache.emplace(key, e).first;
    }
    if (!it->second.ok) {
        if (why) *why = it->second.error;
        return nullptr;
    }
    return &it->second.k;
}

struct JitBatchEntry {
    cudaLibrary_t lib = nullptr;
    BatchJitKernels k;
    bool ok = false;
    std::string error;
};
static std::map<std::string, JitBatchEntry> g_batch_cache;  // key: device | precision | block | programs

const BatchJitKernels *jit_batch_kernels(const std::vector<ProgramCode> &progs, int precision, int block_threads,
                                         std::string *why)
{
    if (!jit_enabled()) {
        if (why) *why = "JIT disabled (NT2G_JIT=0)";
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::string key = std::to_string(dev) + "|" + std::to_string(precision) + "|" + std::to_string(block_threads);
    for (const ProgramCode &pc : progs) {
        key += "|" + std::to_string(pc.ops->size()) + ":";
        key.append((const char *)pc.ops->data(), pc.ops->size() * sizeof(nt2g_op));
        key.append((const char *)pc.logical->data(), pc.logical->size());
    }
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_batch_cache.find(key);
    if (it == g_batch_cache.end()) {
        JitBatchEntry e;
        std::string cubin = compile_cubin(jit_batch_source(progs, precision, block_threads), e.error);
        if (!cubin.empty()) {
            cudaError_t ce = cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
            for (int d = 0; d < 2; ++d)
                for (int w = 0; w < 2; ++w) {
                    const std::string name = "batch_" + std::to_string(d) + std::to_string(w + 1);
                    if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.k.k[d][w], e.lib, name.c_str());
                    if (ce == cudaSuccess)
                        ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e.k.per_sm[d][w], (const void *)e.k.k[d][w],
                                                                           block_threads, 0);
                }
            if (ce == cudaSuccess) {
                e.ok = true;
            } else {
                e.error = std::string("loading the JIT batch kernels: ") + cudaGetErrorString(ce);
                cudaGetLastError();
            }
        }
        it = g_batch_cache.emplace(key, e).first;
    }
    if (!it->second.ok) {
        if (why) *why = it->second.error;
        return nullptr;
    }
    return &it->second.k;
}

struct JitVjpEntry {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
    int blocks_per_sm = 0;
    std::string error;
};
static std::map<std::string, JitVjpEntry> g_vjp_cache;  // key: device | precision | program text

static JitVjpEntry *jit_vjp_get(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                                std::string *why)
{
    if (!jit_enabled()) {
        if (why) *why = "JIT disabled (NT2G_JIT=0)";
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::string key = std::to_string(dev) + "|" + std::to_string(precision) + "|";
    key.append((const char *)ops.data(), ops.size() * sizeof(nt2g_op));
    key.append((const char *)logical.data(), logical.size());
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_vjp_cache.find(key);
    if (it == g_vjp_cache.end()) {
        JitVjpEntry e;
        std::string src = jit_vjp_source(ops, logical, precision, &e.error);
        std::string cubin = src.empty() ? std::string() : compile_cubin(src, e.error);
        if (!cubin.empty()) {
            cudaError_t ce = cudaLibraryLoadData(&e.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
            if (ce == cudaSuccess) ce = cudaLibraryGetKernel(&e.kernel, e.lib, "nt2g_vjp_kernel");
            if (ce == cudaSuccess)
                ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e.blocks_per_sm, (const void *)e.kernel, 256, 0);
            if (ce != cudaSuccess) {
                e.error = std::string("loading the reverse-mode kernel: ") + cudaGetErrorString(ce);
                cudaGetLastError();
                e.kernel = nullptr;
            }
        }
        it = g_vjp_cache.emplace(key, e).first;
    }
    if (!it->second.kernel) {
        if (why) *why = it->second.error;
        return nullptr;
    }
    return &it->second;
}

// Blocks of the reverse-mode grid: 256 threads x 4 elements each, at most
// 8 resident blocks (2048 threads) per SM.
static int64_t vjp_grid_bound(int64_t count)
{
    const int64_t need = (count + 1023) / 1024;
    const int64_t full = (int64_t)device_sm_count() * 8;
    return need < full ? need : full;
}

size_t vjp_workspace_bytes(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int64_t count)
{
    const size_t ns = vjp_scalar_slots(ops, logical).size();
    return ns == 0 ? 0 : (size_t)vjp_grid_bound(count) * ns * sizeof(double);
}

struct VjpSlotMap {
    int slot[kMaxSlots];  // accumulator q -> scalar slot
    int zero[kMaxSlots];  // float scalar slots no output depends on
    int nzero;
};

// One block per accumulator, summing the blocks' partials in a fixed order
// (thread-strided, then warp shuffles, then warps in index order), so the
// gradient of a scalar is the same bits on every run; one more block writes
// the zero gradients.
__global__ void __launch_bounds__(256) k_vjp_finish(const double *partials, int blocks, int ns, VjpSlotMap map,
                                                    double *out)
{
    __shared__ double red[8];
    const int q = blockIdx.x;
    if (q == ns) {
        if (threadIdx.x < map.nzero) out[map.zero[threadIdx.x]] = 0.0;
        return;
    }
    double x = 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x) x += partials[(long long)b * ns + q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        out[map.slot[q]] = t;
    }
}

nt2g_status launch_vjp(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                       const float *const ct[kMaxSlots], float *const grad[kMaxSlots], double *scalar_grads,
                       const std::vector<int> &float_scalars, int64_t count, int precision, void *ws, size_t ws_bytes,
                       cudaStream_t st)
{
    std::string why;
    JitVjpEntry *e = jit_vjp_get(ops, logical, precision, &why);
    if (!e) {
        set_error("reverse mode needs the run-time compiler: %s", why.c_str());
        return NT2G_ERR_UNSUPPORTED;
    }
    const std::vector<int> sslots = vjp_scalar_slots(ops, logical);
    const int ns = (int)sslots.size();
    const int64_t bound = vjp_grid_bound(count);
    int64_t full = (int64_t)device_sm_count() * (e->blocks_per_sm > 0 ? e->blocks_per_sm : 1);
    const int grid = (int)(bound < full ? bound : full);
    double *partials = nullptr;
    if (scalar_grads && ns > 0) {
        const size_t need = (size_t)grid * ns * sizeof(double);
        if (!ws || ws_bytes < need || ((uintptr_t)ws & 7u)) {
            set_error("nt2g_program_vjp: workspace of %zu bytes, %zu needed (8-byte aligned)", ws_bytes, need);
            return NT2G_ERR_INVALID;
        }
        partials = (double *)ws;
    }
    struct { const float *ct[kMaxSlots]; float *grad[kMaxSlots]; } g;
    int vec = 1;
    for (int s = 0; s < kMaxSlots; ++s) {
        g.ct[s] = ct[s];
        g.grad[s] = grad[s];
        if (args.ptr[s]) vec &= ((uintptr_t)args.ptr[s] & (args.dtype[s] == NT2G_F32 ? 15u : 3u)) == 0;
        if (ct[s]) vec &= ((uintptr_t)ct[s] & 15u) == 0;
        if (grad[s]) vec &= ((uintptr_t)grad[s] & 15u) == 0;
    }
    if (grid > 0) {
        long long n = count;
        void *params[] = {(void *)&args, (void *)&g, (void *)&n, (void *)&vec, (void *)&partials};
        cudaError_t ce = cudaLaunchKernel((const void *)e->kernel, dim3(grid), dim3(256), params, 0, st);
        if (ce != cudaSuccess) return cuda_status(ce, "reverse-mode kernel launch");
    }
    if (scalar_grads && !float_scalars.empty()) {
        VjpSlotMap map{};
        for (int q = 0; q < ns; ++q) map.slot[q] = sslots[q];
        for (int s : float_scalars)
            if (std::find(sslots.begin(), sslots.end(), s) == sslots.end()) map.zero[map.nzero++] = s;
        k_vjp_finish<<<ns + 1, 256, 0, st>>>(partials, grid, ns, map, scalar_grads);
        NT2G_LAUNCH_CHECK("reverse-mode finish");
    }
    return NT2G_OK;
}

bool jit_enabled()
{
    const char *e = getenv("NT2G_JIT");
    return !(e && e[0] == '0');
}

// Compile and load the kernel of a program ahead of its first evaluation
// (compilation takes a fraction of a second; a stream capture must not be the
// first use).
nt2g_status jit_prepare(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision)
{
    if (!jit_enabled()) { set_error("JIT disabled (NT2G_JIT=0)"); return NT2G_ERR_UNSUPPORTED; }
    std::string why;
    if (!jit_get(ops, logical, precision, &why)) { set_error("%s", why.c_str()); return NT2G_ERR_UNSUPPORTED; }
    return NT2G_OK;
}

// Launch the JIT kernel of a generic program.  Returns NT2G_ERR_UNSUPPORTED
// when no JIT kernel can be had; the caller then interprets.
nt2g_status launch_jit(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                       int64_t count, int precision, cudaStream_t st)
{
    static_assert(sizeof(DArgs) == 16 * sizeof(void *) + 3 * 16 * 4 + 8 && offsetof(DArgs, pos0) == 16 * 8 + 3 * 16 * 4,
                  "JitArgs layout");
    if (!jit_enabled()) return NT2G_ERR_UNSUPPORTED;
    JitEntry *e = jit_get(ops, logical, precision, nullptr);
    if (!e) return NT2G_ERR_UNSUPPORTED;
    if (count == 0) return NT2G_OK;
    // whole-vector accesses need every float table 16-byte and every uint8 table 4-byte aligned
    int vec = 1;
    for (int s = 0; s < kMaxSlots; ++s)
        if (args.ptr[s]) vec &= ((uintptr_t)args.ptr[s] & (args.dtype[s] == NT2G_F32 ? 15u : 3u)) == 0;
    int64_t full = (int64_t)device_sm_count() * (e->blocks_per_sm > 0 ? e->blocks_per_sm : 1);
    int64_t need = (count + 1023) / 1024;  // 256 threads x 4 elements
    int grid = (int)(need < full ? need : full);
    long long n = count;
    void *params[] = {(void *)&args, (void *)&n, (void *)&vec};
    cudaError_t ce = cudaLaunchKernel((const void *)e->kernel, dim3(grid), dim3(256), params, 0, st);
    if (ce != cudaSuccess) return cuda_status(ce, "JIT kernel launch");
    return NT2G_OK;
}

}  // namespace nt2g
