// nt2g_batched.cu -- thousands of independent tables of uneven sizes, each
// with its own expression, in one persistent launch.
//
// Every table is cut into tiles of tile_elems elements (a multiple of 4, so
// tiles start 16-byte aligned when the table does).  A prefix sum of tile
// counts maps a global tile id to (table, tile).  Blocks take tiles either in
// a fixed stride (static) or from an atomic counter (dynamic); a whole block
// works on one tile, so the expression switch is block-uniform.  A thread has
// one or two float4 vectors in flight per step (the second a block-width
// further, so warps stay contiguous).  Items of the three library expressions
// run in this file's kernel; items carrying a compiled program run in one
// run-time compiled kernel holding every distinct program of the batch
// (nt2g_jit.cu), launched after it on the same stream.  The run can be
// captured once into a CUDA graph and replayed.
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "nt2g_common.cuh"
#include "nt2g_exprs.cuh"
#include "nt2g_internal.h"
#include "nt2g_pair.cuh"

namespace nt2g {

struct DItem {
    int32_t expr;
    int32_t vec;
    int64_t n;
    const float *in[3];
    float *out[2];
    float s[2];
};

// A program item as the run-time compiled batch kernel reads it (BItem there).
struct PItem {
    DArgs a;
    int64_t n;
    int32_t prog;  // index of the item's program in the batch's program list
    int32_t vec;   // every table 16-byte (float) / 4-byte (uint8) aligned
};
static_assert(sizeof(PItem) == sizeof(DArgs) + 16 && offsetof(PItem, n) == sizeof(DArgs), "BItem layout");

// One tile [start, end) of a library-expression item; start is a multiple of
// 4.  Whole float4 vectors (aligned tables), VW per thread per step while a
// whole group lasts, then one at a time, then the scalar tail.
template <class P, int VW>
__device__ __forceinline__ void run_tile(const DItem &it, int64_t start, int64_t end)
{
    const int64_t v0 = start >> 2;
    const int64_t v1 = it.vec ? (end >> 2) : v0;
    const int64_t bd = blockDim.x;
    int64_t i = v0 + threadIdx.x;
    switch (it.expr) {
    case NT2G_BATCH_BLACKSCHOLES: {
        const float sig = it.s[0], r = it.s[1], inv_sig = P::exact ? 0.0f : inv_fast(sig);
        const float4 *S = (const float4 *)it.in[0], *K = (const float4 *)it.in[1], *T = (const float4 *)it.in[2];
        auto one = [&](const float4 s, const float4 k, const float4 t, int64_t at) {
            float4 c, p;
            if constexpr (!P::exact) {  // two options per packed instruction, as the plain kernel
                bs_vec4_fast(s, k, t, make_float4(sig, sig, sig, sig), make_float4(inv_sig, inv_sig, inv_sig, inv_sig),
                             r, c, p);
            } else {  // NT2's unfused arithmetic, two options per packed instruction
                bs_vec4_nt2(s, k, t, make_float4(sig, sig, sig, sig), r, c, p);
            }
            st_stream((float4 *)it.out[0] + at, c);
            st_stream((float4 *)it.out[1] + at, p);
        };
        if constexpr (VW == 2)
            for (; i + bd < v1; i += 2 * bd) {
                const float4 s0 = ld_stream(S + i), k0 = ld_stream(K + i), t0 = ld_stream(T + i);
                const float4 s1 = ld_stream(S + i + bd), k1 = ld_stream(K + i + bd), t1 = ld_stream(T + i + bd);
                one(s0, k0, t0, i);
                one(s1, k1, t1, i + bd);
            }
        for (; i < v1; i += bd) one(ld_stream(S + i), ld_stream(K + i), ld_stream(T + i), i);
        for (int64_t e = (v1 << 2) + threadIdx.x; e < end; e += bd)
            bs_option<P>(it.in[0][e], it.in[1][e], it.in[2][e], sig, inv_sig, r, it.out[0][e], it.out[1][e]);
        break;
    }
    case NT2G_BATCH_SAXPY: {
        const float a = it.s[0];
        const float4 *X = (const float4 *)it.in[0];
        float4 *Y = (float4 *)it.out[0];
        auto one = [&](const float4 x, const float4 y, int64_t at) {
            float4 o;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(o, j, saxpy_elem(a, get(x, j), get(y, j)));
            st_stream(Y + at, o);
        };
        if constexpr (VW == 2)
            for (; i + bd < v1; i += 2 * bd) {
                const float4 x0 = ld_stream(X + i), y0 = ld_stream(Y + i), x1 = ld_stream(X + i + bd),
                             y1 = ld_stream(Y + i + bd);
                one(x0, y0, i);
                one(x1, y1, i + bd);
            }
        for (; i < v1; i += bd) one(ld_stream(X + i), ld_stream(Y + i), i);
        for (int64_t e = (v1 << 2) + threadIdx.x; e < end; e += bd)
            it.out[0][e] = saxpy_elem(a, it.in[0][e], it.out[0][e]);
        break;
    }
    default: {
        const float4 *X = (const float4 *)it.in[0], *Y = (const float4 *)it.in[1], *Z = (const float4 *)it.in[2];
        auto one = [&](const float4 x, const float4 y, const float4 z, int64_t at) {
            float4 o;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(o, j, expr3_elem<P>(get(x, j), get(y, j), get(z, j)));
            st_stream((float4 *)it.out[0] + at, o);
        };
        if constexpr (VW == 2)
            for (; i + bd < v1; i += 2 * bd) {
                const float4 x0 = ld_stream(X + i), y0 = ld_stream(Y + i), z0 = ld_stream(Z + i);
                const float4 x1 = ld_stream(X + i + bd), y1 = ld_stream(Y + i + bd), z1 = ld_stream(Z + i + bd);
                one(x0, y0, z0, i);
                one(x1, y1, z1, i + bd);
            }
        for (; i < v1; i += bd) one(ld_stream(X + i), ld_stream(Y + i), ld_stream(Z + i), i);
        for (int64_t e = (v1 << 2) + threadIdx.x; e < end; e += bd)
            it.out[0][e] = expr3_elem<P>(it.in[0][e], it.in[1][e], it.in[2][e]);
        break;
    }
    }
}

__device__ __forceinline__ int find_item(const int64_t *prefix, int n_items, int64_t t)
{
    int lo = 0, hi = n_items;  // prefix[lo] <= t < prefix[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= t) lo = mid; else hi = mid;
    }
    return lo;
}

template <class P, bool DYNAMIC, int VW>
__global__ void k_batch(const DItem *__restrict__ items, const int64_t *__restrict__ prefix, int n_items,
                        int64_t total_tiles, int64_t tile_elems, unsigned long long *counter)
{
    __shared__ int64_t s_tile;
    int64_t t = DYNAMIC ? 0 : blockIdx.x;
    while (true) {
        if (DYNAMIC) {
            if (threadIdx.x == 0) s_tile = (int64_t)atomicAdd(counter, 1ull);
            __syncthreads();
            t = s_tile;
            __syncthreads();
        }
        if (t >= total_tiles) return;
        int k = find_item(prefix, n_items, t);
        const DItem it = items[k];
        int64_t start = (t - __ldg(prefix + k)) * tile_elems;
        int64_t end = start + tile_elems < it.n ? start + tile_elems : it.n;
        run_tile<P, VW>(it, start, end);
        if (!DYNAMIC) t += gridDim.x;
    }
}

}  // namespace nt2g

struct nt2g_batch {
    // items of the library expressions
    std::vector<nt2g::DItem> host_items;
    nt2g::DItem *d_items = nullptr;
    int64_t *d_prefix = nullptr;
    int n_items = 0;
    int64_t total_tiles = 0;
    // items carrying a program
    std::vector<nt2g::PItem> host_pitems;
    std::vector<const nt2g_program *> programs;  // distinct programs, in order of first use
    nt2g::PItem *d_pitems = nullptr;
    int64_t *d_pprefix = nullptr;
    int n_pitems = 0;
    int64_t total_ptiles = 0;
    const nt2g::BatchJitKernels *jit = nullptr;  // nullptr: each program item interpreted on its own
    // caller's item order: (0 library | 1 program, index within its kind)
    std::vector<std::pair<int, int>> order;
    unsigned long long *d_counter = nullptr;  // [0] library tiles, [1] program tiles
    int64_t tile_elems = 0;
    int64_t elements = 0, bytes = 0;
    nt2g_batch_tune tune{};
    int dynamic = 1;
    cudaGraphExec_t graph = nullptr;
};

using namespace nt2g;

static int64_t item_bytes(int expr, int64_t n)
{
    switch (expr) {
    case NT2G_BATCH_BLACKSCHOLES: return 20 * n;
    case NT2G_BATCH_SAXPY: return 12 * n;
    default: return 16 * n;
    }
}

static constexpr int kMaxBatchPrograms = 64;

extern "C" nt2g_status nt2g_batch_create(const nt2g_batch_item *items, int32_t n_items, const nt2g_batch_tune *tune,
                                         nt2g_batch **out)
{
    NT2G_CHECK_ARG(out != nullptr, "nt2g_batch_create: out is NULL");
    *out = nullptr;
    NT2G_CHECK_ARG(items != nullptr && n_items > 0, "nt2g_batch_create: no items");
    nt2g_batch_tune tn = tune ? *tune : nt2g_batch_tune{128, 0, 32, NT2G_PREC_FAST, 1, 0};
    if (tn.block_threads == 0) tn.block_threads = 128;
    if (tn.tile_vectors == 0) tn.tile_vectors = 32;
    if (tn.vector_width == 0) tn.vector_width = 1;
    NT2G_CHECK_ARG(tn.block_threads >= 64 && tn.block_threads <= 1024 && tn.block_threads % 32 == 0,
                   "nt2g_batch_create: block_threads %d not a multiple of 32 in [64,1024]", tn.block_threads);
    NT2G_CHECK_ARG(tn.tile_vectors >= 1 && tn.tile_vectors <= 64, "nt2g_batch_create: tile_vectors %d", tn.tile_vectors);
    NT2G_CHECK_ARG(tn.vector_width == 1 || tn.vector_width == 2, "nt2g_batch_create: vector_width %d (1 or 2)",
                   tn.vector_width);
    NT2G_CHECK_ARG(tn.precision == NT2G_PREC_FAST || tn.precision == NT2G_PREC_NT2, "nt2g_batch_create: precision %d",
                   tn.precision);
    nt2g_batch *b = new (std::nothrow) nt2g_batch();
    if (!b) { set_error("nt2g_batch_create: out of host memory"); return NT2G_ERR_NOMEM; }
    auto fail = [&](nt2g_status st) { nt2g_batch_destroy(b); return st; };
    b->tune = tn;
    b->dynamic = tn.blocks_per_sm >= 0 ? 1 : 0;  // negative blocks_per_sm selects static striding
    b->tile_elems = (int64_t)tn.block_threads * tn.tile_vectors * 4;
    std::vector<int64_t> prefix(1, 0), pprefix(1, 0);
    for (int i = 0; i < n_items; ++i) {
        const nt2g_batch_item &it = items[i];
        if (it.expr == NT2G_BATCH_PROGRAM) {
            if (!it.program || it.n < 0) {
                set_error("nt2g_batch_create: item %d is a program item without a program or with n < 0", i);
                return fail(NT2G_ERR_INVALID);
            }
            if (program_folds(it.program)) {
                set_error("nt2g_batch_create: item %d: the program folds its value (nt2g_eval_fold)", i);
                return fail(NT2G_ERR_INVALID);
            }
            PItem d{};
            char who[64];
            snprintf(who, sizeof who, "nt2g_batch_create: item %d", i);
            nt2g_status bs = program_bind(it.program, it.args, it.n_args, it.n, who, d.a);
            if (bs != NT2G_OK) return fail(bs);
            int k = 0;
            while (k < (int)b->programs.size() && b->programs[k] != it.program) ++k;
            if (k == (int)b->programs.size()) {
                if (k == kMaxBatchPrograms) {
                    set_error("nt2g_batch_create: more than %d distinct programs in one batch", kMaxBatchPrograms);
                    return fail(NT2G_ERR_UNSUPPORTED);
                }
                b->programs.push_back(it.program);
            }
            d.n = it.n;
            d.prog = k;
            int vec = 1;
            for (int s = 0; s < kMaxSlots; ++s)
                if (d.a.ptr[s]) vec &= ((uintptr_t)d.a.ptr[s] & (d.a.dtype[s] == NT2G_F32 ? 15u : 3u)) == 0;
            d.vec = vec;
            b->order.emplace_back(1, (int)b->host_pitems.size());
            b->host_pitems.push_back(d);
            pprefix.push_back(pprefix.back() + (it.n + b->tile_elems - 1) / b->tile_elems);
            b->elements += it.n;
            b->bytes += program_bytes_per_element(it.program) * it.n;
            continue;
        }
        bool ok = it.expr >= 0 && it.expr <= 2 && it.n >= 0 && it.in[0] && it.out[0] &&
                  (it.expr == NT2G_BATCH_SAXPY || (it.in[1] && it.in[2])) &&
                  (it.expr != NT2G_BATCH_BLACKSCHOLES || it.out[1]);
        if (!ok) {
            set_error("nt2g_batch_create: item %d is malformed (expr %d)", i, it.expr);
            return fail(NT2G_ERR_INVALID);
        }
        if (it.n > 0)
            for (int j = 0; j < 3; ++j)
                if (!reachable(it.in[j]) || (j < 2 && !reachable(it.out[j]))) {
                    set_error("nt2g_batch_create: item %d holds host memory the device cannot access", i);
                    return fail(NT2G_ERR_INVALID);
                }
        DItem d{};
        d.expr = it.expr;
        d.n = it.n;
        int vec = 1;
        for (int j = 0; j < 3; ++j) { d.in[j] = it.in[j]; if (it.in[j]) vec &= aligned16(it.in[j]); }
        for (int j = 0; j < 2; ++j) { d.out[j] = it.out[j]; if (it.out[j]) vec &= aligned16(it.out[j]); }
        d.vec = vec;
        d.s[0] = it.s[0];
        d.s[1] = it.s[1];
        b->order.emplace_back(0, (int)b->host_items.size());
        b->host_items.push_back(d);
        prefix.push_back(prefix.back() + (it.n + b->tile_elems - 1) / b->tile_elems);
        b->elements += it.n;
        b->bytes += item_bytes(it.expr, it.n);
    }
    b->n_items = (int)b->host_items.size();
    b->n_pitems = (int)b->host_pitems.size();
    b->total_tiles = prefix.back();
    b->total_ptiles = pprefix.back();
    if (b->n_pitems > 0) {
        // every program of the batch in one kernel, compiled here (not in a run
        // that may be under stream capture); without NVRTC the runs interpret
        // each program item on its own
        std::vector<ProgramCode> code;
        for (const nt2g_program *p : b->programs) code.push_back(ProgramCode{&program_ops(p), &program_logical(p)});
        std::string why;
        b->jit = jit_batch_kernels(code, tn.precision, tn.block_threads, &why);
    }
    cudaError_t e = cudaMalloc(&b->d_counter, 256);
    if (e == cudaSuccess && b->n_items > 0) {
        e = cudaMalloc(&b->d_items, sizeof(DItem) * b->n_items);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_prefix, sizeof(int64_t) * (b->n_items + 1));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_items, b->host_items.data(), sizeof(DItem) * b->n_items, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_prefix, prefix.data(), sizeof(int64_t) * (b->n_items + 1), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && b->n_pitems > 0) {
        e = cudaMalloc(&b->d_pitems, sizeof(PItem) * b->n_pitems);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_pprefix, sizeof(int64_t) * (b->n_pitems + 1));
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_pitems, b->host_pitems.data(), sizeof(PItem) * b->n_pitems, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_pprefix, pprefix.data(), sizeof(int64_t) * (b->n_pitems + 1), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return fail(cuda_status(e, "nt2g_batch_create: device upload"));
    *out = b;
    return NT2G_OK;
}

extern "C" void nt2g_batch_destroy(nt2g_batch *b)
{
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_items);
    cudaFree(b->d_prefix);
    cudaFree(b->d_pitems);
    cudaFree(b->d_pprefix);
    cudaFree(b->d_counter);
    delete b;
}

// Resident blocks per SM of a persistent grid: the tune's request (dynamic:
// > 0; static: -blocks_per_sm), capped by what the SM holds at this block size.
static int grid_blocks(const nt2g_batch *b, int limit)
{
    if (limit < 1) limit = 1;
    int per_sm = b->dynamic ? b->tune.blocks_per_sm : -b->tune.blocks_per_sm;
    if (per_sm < 1 || per_sm > limit) per_sm = limit;
    return device_sm_count() * per_sm;
}

template <class P, int VW>
static nt2g_status launch_library_items(nt2g_batch *b, cudaStream_t st)
{
    const int threads = b->tune.block_threads;
    int limit = 0;
    if (b->dynamic) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&limit, k_batch<P, true, VW>, threads, 0) != cudaSuccess)
            limit = 1;
        k_batch<P, true, VW><<<grid_blocks(b, limit), threads, 0, st>>>(b->d_items, b->d_prefix, b->n_items,
                                                                        b->total_tiles, b->tile_elems, b->d_counter);
    } else {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&limit, k_batch<P, false, VW>, threads, 0) != cudaSuccess)
            limit = 1;
        k_batch<P, false, VW><<<grid_blocks(b, limit), threads, 0, st>>>(b->d_items, b->d_prefix, b->n_items,
                                                                         b->total_tiles, b->tile_elems, b->d_counter);
    }
    NT2G_LAUNCH_CHECK("batch launch");
    return NT2G_OK;
}

static nt2g_status program_item_eval(nt2g_batch *b, int k, cudaStream_t st)
{
    const PItem &it = b->host_pitems[k];
    return program_eval(b->programs[it.prog], it.a, it.n, b->tune.precision, st);
}

static nt2g_status launch_program_items(nt2g_batch *b, cudaStream_t st)
{
    if (!b->jit) {  // no run-time compiler: each program item on its own
        for (int k = 0; k < b->n_pitems; ++k) {
            nt2g_status s = program_item_eval(b, k, st);
            if (s != NT2G_OK) return s;
        }
        return NT2G_OK;
    }
    const int d = b->dynamic, w = b->tune.vector_width - 1;
    int n = b->n_pitems;
    long long total = b->total_ptiles, tile = b->tile_elems;
    unsigned long long *counter = b->d_counter + 1;
    void *params[] = {(void *)&b->d_pitems, (void *)&b->d_pprefix, (void *)&n, (void *)&total, (void *)&tile,
                      (void *)&counter};
    cudaError_t ce = cudaLaunchKernel((const void *)b->jit->k[d][w], dim3(grid_blocks(b, b->jit->per_sm[d][w])),
                                      dim3(b->tune.block_threads), params, 0, st);
    if (ce != cudaSuccess) return cuda_status(ce, "batch program launch");
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_batch_run(nt2g_batch *b, void *stream)
{
    NT2G_CHECK_ARG(b != nullptr, "nt2g_batch_run: NULL batch");
    cudaStream_t st = (cudaStream_t)stream;
    if (b->dynamic) {
        cudaError_t e = cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(unsigned long long), st);
        if (e != cudaSuccess) return cuda_status(e, "batch counter reset");
    }
    if (b->n_items > 0) {
        const bool nt2 = b->tune.precision == NT2G_PREC_NT2, two = b->tune.vector_width == 2;
        nt2g_status s = nt2 ? (two ? launch_library_items<Nt2, 2>(b, st) : launch_library_items<Nt2, 1>(b, st))
                            : (two ? launch_library_items<Fast, 2>(b, st) : launch_library_items<Fast, 1>(b, st));
        if (s != NT2G_OK) return s;
    }
    if (b->n_pitems > 0) return launch_program_items(b, st);
    return NT2G_OK;
}

// The comparison path: each table through its expression's own plain kernel
// (nt2g_blackscholes_f32 / nt2g_saxpy_f32 / nt2g_expr3_f32 launchers, the
// program's generic kernel), one launch per table in the caller's order, as a
// caller without the batched path would issue them.
static nt2g_status per_table(nt2g_batch *b, cudaStream_t st)
{
    const int prec = b->tune.precision;
    for (const std::pair<int, int> &o : b->order) {
        nt2g_status s;
        if (o.first == 1) {
            s = program_item_eval(b, o.second, st);
        } else {
            const DItem &it = b->host_items[o.second];
            switch (it.expr) {
            case NT2G_BATCH_BLACKSCHOLES:
                s = launch_bs(it.in[0], it.in[1], it.in[2], nullptr, it.s[0], it.s[1], it.out[0], it.out[1], it.n, prec,
                              st);
                break;
            case NT2G_BATCH_SAXPY: s = launch_saxpy(it.s[0], it.in[0], it.out[0], it.out[0], it.n, st); break;
            default: s = launch_expr3(it.in[0], it.in[1], it.in[2], it.out[0], it.n, prec, st); break;
            }
        }
        if (s != NT2G_OK) return s;
    }
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_batch_run_per_table(nt2g_batch *b, void *stream)
{
    NT2G_CHECK_ARG(b != nullptr, "nt2g_batch_run_per_table: NULL batch");
    return per_table(b, (cudaStream_t)stream);
}

extern "C" nt2g_status nt2g_batch_run_graph(nt2g_batch *b, void *stream)
{
    NT2G_CHECK_ARG(b != nullptr, "nt2g_batch_run_graph: NULL batch");
    cudaStream_t st = (cudaStream_t)stream;
    NT2G_CHECK_ARG(st != nullptr, "nt2g_batch_run_graph: capture needs a non-default stream");
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_status(e, "batch graph: begin capture");
        nt2g_status s = nt2g_batch_run(b, stream);
        e = cudaStreamEndCapture(st, &g);
        if (s != NT2G_OK) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) return cuda_status(e, "batch graph: end capture");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { b->graph = nullptr; return cuda_status(e, "batch graph: instantiate"); }
    }
    cudaError_t e = cudaGraphLaunch(b->graph, st);
    if (e != cudaSuccess) return cuda_status(e, "batch graph: launch");
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_batch_stats(const nt2g_batch *b, int64_t *elements, int64_t *bytes)
{
    NT2G_CHECK_ARG(b != nullptr, "nt2g_batch_stats: NULL batch");
    if (elements) *elements = b->elements;
    if (bytes) *bytes = b->bytes;
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_batch_source(const nt2g_program *const *programs, int32_t n_programs, int32_t precision,
                                         int32_t block_threads, char *buf, size_t cap, size_t *len)
{
    NT2G_CHECK_ARG(programs != nullptr && n_programs >= 1 && n_programs <= kMaxBatchPrograms,
                   "nt2g_batch_source: %d programs (1..%d)", n_programs, kMaxBatchPrograms);
    NT2G_CHECK_ARG(precision == NT2G_PREC_FAST || precision == NT2G_PREC_NT2, "nt2g_batch_source: precision %d",
                   precision);
    NT2G_CHECK_ARG(block_threads >= 64 && block_threads <= 1024 && block_threads % 32 == 0,
                   "nt2g_batch_source: block_threads %d", block_threads);
    NT2G_CHECK_ARG(buf != nullptr || cap == 0, "nt2g_batch_source: NULL buffer");
    std::vector<ProgramCode> code;
    for (int k = 0; k < n_programs; ++k) {
        NT2G_CHECK_ARG(programs[k] != nullptr && !program_folds(programs[k]),
                       "nt2g_batch_source: program %d is NULL or folds its value", k);
        code.push_back(ProgramCode{&program_ops(programs[k]), &program_logical(programs[k])});
    }
    std::string src = jit_batch_source(code, precision, block_threads);
    if (len) *len = src.size() + 1;
    if (cap == 0) return NT2G_OK;
    NT2G_CHECK_ARG(cap > src.size(), "nt2g_batch_source: %zu-byte buffer, %zu needed", cap, src.size() + 1);
    memcpy(buf, src.c_str(), src.size() + 1);
    return NT2G_OK;
}

// ---------------------------------------------------------------- tuning --
// Times nt2g_batch_run for each candidate (block size, float4 vectors per
// thread per tile -- i.e. elements per thread --, resident blocks per SM,
// negative for the static tile stride, and float4 vectors in flight per
// thread) with CUDA events, reps runs after one warm-up each, and returns the
// fastest.  Each candidate builds its own plan, so device memory is allocated
// (and program kernels compiled, once per block size) here, at tuning time.
// Every run executes the whole batch: expressions that update a table in place
// (saxpy) are applied (1 + reps) times per candidate.
extern "C" nt2g_status nt2g_batch_autotune(const nt2g_batch_item *items, int32_t n_items,
                                           const nt2g_batch_tune *candidates, int32_t n_candidates, int32_t reps,
                                           int32_t precision, void *stream, nt2g_batch_tune *best, float *best_ms)
{
    NT2G_CHECK_ARG(best != nullptr, "nt2g_batch_autotune: best is NULL");
    NT2G_CHECK_ARG(reps >= 1 && reps <= 100, "nt2g_batch_autotune: reps %d outside [1,100]", reps);
    static const nt2g_batch_tune grid[] = {
        {128, 0, 8, 0, 1, 0},   {128, 0, 16, 0, 1, 0},  {128, 0, 32, 0, 1, 0},  {128, 0, 64, 0, 1, 0},
        {256, 0, 8, 0, 1, 0},   {256, 0, 16, 0, 1, 0},  {256, 0, 32, 0, 1, 0},  {256, 0, 64, 0, 1, 0},
        {512, 0, 16, 0, 1, 0},  {512, 0, 32, 0, 1, 0},  {128, -1, 32, 0, 1, 0}, {256, -1, 16, 0, 1, 0},
        {128, 0, 16, 0, 2, 0},  {128, 0, 32, 0, 2, 0},  {256, 0, 16, 0, 2, 0},  {256, 0, 32, 0, 2, 0},
        {512, 0, 16, 0, 2, 0},  {128, -1, 32, 0, 2, 0},
    };
    const nt2g_batch_tune *cand = candidates ? candidates : grid;
    const int nc = candidates ? n_candidates : (int)(sizeof grid / sizeof grid[0]);
    NT2G_CHECK_ARG(nc >= 1, "nt2g_batch_autotune: no candidates");
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return cuda_status(ce, "nt2g_batch_autotune: events");
    }
    float best_t = 0.f;
    int best_i = -1;
    nt2g_status status = NT2G_OK;
    for (int c = 0; c < nc && status == NT2G_OK; ++c) {
        nt2g_batch_tune t = cand[c];
        t.precision = precision;
        nt2g_batch *b = nullptr;
        status = nt2g_batch_create(items, n_items, &t, &b);
        if (status != NT2G_OK) break;
        status = nt2g_batch_run(b, stream);  // warm-up
        if (status == NT2G_OK) ce = cudaEventRecord(e0, st);
        for (int r = 0; r < reps && status == NT2G_OK && ce == cudaSuccess; ++r) status = nt2g_batch_run(b, stream);
        if (status == NT2G_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, st);
        if (status == NT2G_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (status == NT2G_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
        nt2g_batch_destroy(b);
        if (status == NT2G_OK && ce != cudaSuccess) status = cuda_status(ce, "nt2g_batch_autotune: timing");
        if (status == NT2G_OK && (best_i < 0 || ms < best_t)) { best_t = ms; best_i = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != NT2G_OK) return status;
    *best = cand[best_i];
    best->precision = precision;
    if (best->vector_width == 0) best->vector_width = 1;
    if (best_ms) *best_ms = best_t / reps;
    return NT2G_OK;
}
