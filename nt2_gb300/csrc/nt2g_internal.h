// nt2g_internal.h -- declarations shared between the translation units of
// libnt2gpu (kernel launchers, the device program format, error helpers).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "nt2g.h"

namespace nt2g {

// ---------------------------------------------------------------- program --
// Device form of a compiled program: register-allocated three-address code,
// passed to the interpreter kernel by value (it lands in the constant bank,
// so every thread reads the same instruction word: no divergence).
constexpr int kMaxInstr = 160;
constexpr int kMaxRegs = 32;
constexpr int kMaxSlots = 16;

struct DInstr {
    uint8_t op;    // nt2g_opcode (fits in 8 bits)
    uint8_t dt;    // nt2g_dtype of the operands
    uint8_t dst;   // register
    uint8_t a, b, c;  // registers, or slot for LOAD/SCALAR/STORE (a)
    uint8_t logical;  // operand a of STORE holds a logical (0/1) value
    uint8_t pad;
    float imm;
};

struct DProgram {
    int32_t n;
    int32_t n_regs;
    DInstr ins[kMaxInstr];
};

struct DArgs {
    void *ptr[kMaxSlots];
    float scal[kMaxSlots];
    uint32_t scal_u8[kMaxSlots];
    int32_t dtype[kMaxSlots];
    int64_t pos0;  // linear position of element 0 of the evaluated range (INDEX leaves)
};

// Fused kernels a program can bind to.
enum FusedKernel {
    kGeneric = 0,
    kBlackScholes = 1,       // slots: S K T sigma(table|scalar) r | call put
    kBlackScholesDemo = 2,   // slots: S X T r v | R
    kSaxpy = 3,              // slots: alpha X Y | Y
    kExpr3 = 4,              // slots: x y z | out
    kRgb2Yuv = 5,            // slots: r g b | y u v
    kSigmaDelta = 6,         // slots: frame bkg var | bkg var label
};

// True when the current device can read and write the memory at p in place
// (device memory, pinned/registered host memory, or any host memory where the
// device has pageable memory access).  NULL counts as reachable.
bool reachable(const void *p);

// -------------------------------------------------------------- launchers --
nt2g_status launch_bs(const float *S, const float *K, const float *T, const float *sig, float sig_s, float r,
                      float *call, float *put, int64_t n, int precision, cudaStream_t st);
nt2g_status launch_bs_demo(const float *S, const float *X, const float *T, const float *rt, float r,
                           const float *vt, float v, float *R, int64_t n, int precision, cudaStream_t st);
nt2g_status launch_bs_vjp(const float *S, const float *K, const float *T, const float *sig, float r,
                          const float *gc, const float *gp, float *C, float *P, float *dS, float *dK,
                          float *dT, float *dsig, float *dr, int64_t n, cudaStream_t st);
nt2g_status launch_saxpy(float alpha, const float *X, const float *Y, float *O, int64_t n, cudaStream_t st);
nt2g_status reduce_workspace_bytes(size_t *bytes);
nt2g_status launch_reduce(const float *x, const float *y, int64_t n, void *ws, double *out64, float *out32,
                          cudaStream_t st);
nt2g_status launch_reduce_noalloc(const float *x, const float *y, int64_t n, double *out64, float *out32,
                                  cudaStream_t st);
nt2g_status launch_expr3(const float *x, const float *y, const float *z, float *out, int64_t n, int precision,
                         cudaStream_t st);
nt2g_status launch_rgb2yuv(const float *r, const float *g, const float *b, float *y, float *u, float *v,
                           int64_t n, int precision, cudaStream_t st);
nt2g_status launch_sigmadelta(const uint8_t *frame, uint8_t *bkg, uint8_t *var, uint8_t *label, int64_t n,
                              cudaStream_t st);
nt2g_status launch_sigmadelta_frames(const uint8_t *frames, uint8_t *bkg, uint8_t *var, uint8_t *labels,
                                     int64_t n, int frames_n, cudaStream_t st);
nt2g_status launch_map(int fn, const float *x, float *y, int64_t n, int precision, cudaStream_t st);
nt2g_status launch_interp(const DProgram &prog, const DArgs &args, int64_t count, int precision,
                          cudaStream_t st);
nt2g_status fold_partials_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status fold_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status scan_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status launch_scan(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws,
                        size_t ws_bytes, float *out, cudaStream_t st);
nt2g_status launch_fold(const float *x, int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws,
                        size_t ws_bytes, float *out, int64_t *index, cudaStream_t st);
// The same fold over the FOLD value of a program (its element function
// compiled at run time); out64 (optional, fast policy) receives the FP64
// results of sum-type and product folds.
nt2g_status launch_fold_expr(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                             int64_t lo, int64_t inner, int64_t hi, int op, int precision, void *ws, size_t ws_bytes,
                             float *out, int64_t *index, double *out64, cudaStream_t st);

// Run-time compiled kernels of generic programs (nt2g_jit.cu).  The program is
// the canonical SSA form; logical[k] marks comparison results.
//
// Fold kernels of a program with a FOLD instruction: the first-phase kernels
// of nt2g_fold_kernels.cuh (NT2-order, short-segment, contiguous inner[FINAL][IDX],
// strided outer[VEC == 4][FINAL]) instantiated over the program's element
// function, for one fold op; nullptr, with the reason in *why, when NVRTC is
// unavailable or rejects the source.
struct JitFoldKernels {
    cudaKernel_t nt2 = nullptr, shrt = nullptr;
    cudaKernel_t inner[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaKernel_t outer[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
};
const JitFoldKernels *jit_fold_kernels(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical,
                                       int precision, int op, std::string *why);
std::string jit_fold_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                            int op);
std::string jit_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision);
// A batch's programs linked into one persistent kernel per (dynamic | static
// tile schedule) x (1 | 2 float4 vectors per thread), compiled for one block
// size; per_sm holds each kernel's resident blocks per SM at that size.
struct ProgramCode {
    const std::vector<nt2g_op> *ops;
    const std::vector<uint8_t> *logical;
};
struct BatchJitKernels {
    cudaKernel_t k[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [dynamic][vectors - 1]
    int per_sm[2][2] = {{0, 0}, {0, 0}};
};
std::string jit_batch_source(const std::vector<ProgramCode> &progs, int precision, int block_threads);
const BatchJitKernels *jit_batch_kernels(const std::vector<ProgramCode> &progs, int precision, int block_threads,
                                         std::string *why);
// Reverse mode (nt2g_program_vjp): the run-time compiled kernel's source
// (empty, with the reason in *why, when an opcode has no adjoint rule), the
// float scalar slots whose gradients it sums, its workspace, its launch.
std::string jit_vjp_source(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision,
                           std::string *why);
std::vector<int> vjp_scalar_slots(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical);
size_t vjp_workspace_bytes(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int64_t count);
nt2g_status launch_vjp(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                       const float *const ct[kMaxSlots], float *const grad[kMaxSlots], double *scalar_grads,
                       const std::vector<int> &float_scalars, int64_t count, int precision, void *ws, size_t ws_bytes,
                       cudaStream_t st);
bool jit_enabled();
nt2g_status jit_prepare(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, int precision);
nt2g_status launch_jit(const std::vector<nt2g_op> &ops, const std::vector<uint8_t> &logical, const DArgs &args,
                       int64_t count, int precision, cudaStream_t st);

// Compiled programs as the batch sees them (nt2g_capi.cu owns their layout).
const std::vector<nt2g_op> &program_ops(const nt2g_program *p);
const std::vector<uint8_t> &program_logical(const nt2g_program *p);
bool program_folds(const nt2g_program *p);
// Bind n_args arguments over elements [0, count) (nt2g_eval's checks).
nt2g_status program_bind(const nt2g_program *p, const nt2g_arg *args, int32_t n_args, int64_t count, const char *who,
                         DArgs &da);
// Table bytes one element moves: each loaded slot read once, each stored slot written once.
int64_t program_bytes_per_element(const nt2g_program *p);
// The program's generic evaluation (run-time compiled kernel, else the
// interpreter): what nt2g_eval does with force_generic = 1.
nt2g_status program_eval(const nt2g_program *p, const DArgs &da, int64_t count, int precision, cudaStream_t st);

// trapz along a dimension (nt2g_fold.cu)
nt2g_status trapz_workspace_bytes(int64_t lo, int64_t inner, int64_t hi, size_t *bytes);
nt2g_status launch_trapz(const float *x, int64_t lo, int64_t inner, int64_t hi, int precision, void *ws,
                         size_t ws_bytes, float *out, cudaStream_t st);

// median / medianad along a dimension (nt2g_median.cu)
size_t median_workspace_bytes(int64_t lo, int64_t n, int64_t hi);
nt2g_status launch_median(const float *x, int64_t lo, int64_t n, int64_t hi, int32_t op, void *ws, float *out,
                          cudaStream_t st);

}  // namespace nt2g
