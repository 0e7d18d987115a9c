// nt2g_batched.cu -- thousands of independent tables of uneven sizes, each
// with its own expression, in one persistent launch.
//
// Every table is cut into tiles of tile_elems elements (a multiple of 4, so
// tiles start 16-byte aligned when the table does).  A prefix sum of tile
// counts maps a global tile id to (table, tile).  Blocks take tiles either in
// a fixed stride (static) or from an atomic counter (dynamic); a whole block
// works on one tile, so the expression switch is block-uniform.  The run can
// be captured once into a CUDA graph and replayed.
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

template <class P>
__device__ __forceinline__ void run_tile(const DItem &it, int64_t start, int64_t end)
{
    // start is a multiple of 4; vector part then scalar tail
    const int64_t v0 = start >> 2;
    const int64_t v1 = it.vec ? (end >> 2) : v0;
    switch (it.expr) {
    case NT2G_BATCH_BLACKSCHOLES: {
        const float sig = it.s[0], r = it.s[1], inv_sig = P::exact ? 0.0f : inv_fast(sig);
        for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x) {
            float4 s = ld_stream((const float4 *)it.in[0] + i), k = ld_stream((const float4 *)it.in[1] + i),
                   t = ld_stream((const float4 *)it.in[2] + i), c, p;
            if constexpr (!P::exact) {  // two options per packed instruction, as the plain kernel
                bs_vec4_fast(s, k, t, make_float4(sig, sig, sig, sig), make_float4(inv_sig, inv_sig, inv_sig, inv_sig),
                             r, c, p);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float cj, pj;
                    bs_option<P>(get(s, j), get(k, j), get(t, j), sig, inv_sig, r, cj, pj);
                    set(c, j, cj); set(p, j, pj);
                }
            }
            st_stream((float4 *)it.out[0] + i, c);
            st_stream((float4 *)it.out[1] + i, p);
        }
        for (int64_t i = (v1 << 2) + threadIdx.x; i < end; i += blockDim.x)
            bs_option<P>(it.in[0][i], it.in[1][i], it.in[2][i], sig, inv_sig, r, it.out[0][i], it.out[1][i]);
        break;
    }
    case NT2G_BATCH_SAXPY: {
        const float a = it.s[0];
        for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x) {
            float4 x = ld_stream((const float4 *)it.in[0] + i), y = ld_stream((const float4 *)it.out[0] + i), o;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(o, j, saxpy_elem(a, get(x, j), get(y, j)));
            st_stream((float4 *)it.out[0] + i, o);
        }
        for (int64_t i = (v1 << 2) + threadIdx.x; i < end; i += blockDim.x)
            it.out[0][i] = saxpy_elem(a, it.in[0][i], it.out[0][i]);
        break;
    }
    default: {
        for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x) {
            float4 x = ld_stream((const float4 *)it.in[0] + i), y = ld_stream((const float4 *)it.in[1] + i),
                   z = ld_stream((const float4 *)it.in[2] + i), o;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(o, j, expr3_elem<P>(get(x, j), get(y, j), get(z, j)));
            st_stream((float4 *)it.out[0] + i, o);
        }
        for (int64_t i = (v1 << 2) + threadIdx.x; i < end; i += blockDim.x)
            it.out[0][i] = expr3_elem<P>(it.in[0][i], it.in[1][i], it.in[2][i]);
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

template <class P, bool DYNAMIC>
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
        run_tile<P>(it, start, end);
        if (!DYNAMIC) t += gridDim.x;
    }
}

}  // namespace nt2g

struct nt2g_batch {
    std::vector<nt2g::DItem> host_items;
    nt2g::DItem *d_items = nullptr;
    int64_t *d_prefix = nullptr;
    unsigned long long *d_counter = nullptr;
    int n_items = 0;
    int64_t total_tiles = 0;
    int64_t tile_elems = 0;
    int64_t elements = 0, bytes = 0;
    nt2g_batch_tune tune{};
    int dynamic = 1;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
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

extern "C" nt2g_status nt2g_batch_create(const nt2g_batch_item *items, int32_t n_items, const nt2g_batch_tune *tune,
                                         nt2g_batch **out)
{
    NT2G_CHECK_ARG(out != nullptr, "nt2g_batch_create: out is NULL");
    *out = nullptr;
    NT2G_CHECK_ARG(items != nullptr && n_items > 0, "nt2g_batch_create: no items");
    nt2g_batch_tune tn = tune ? *tune : nt2g_batch_tune{128, 0, 32, NT2G_PREC_FAST};
    if (tn.block_threads == 0) tn.block_threads = 128;
    if (tn.tile_vectors == 0) tn.tile_vectors = 32;
    NT2G_CHECK_ARG(tn.block_threads >= 64 && tn.block_threads <= 1024 && tn.block_threads % 32 == 0,
                   "nt2g_batch_create: block_threads %d not a multiple of 32 in [64,1024]", tn.block_threads);
    NT2G_CHECK_ARG(tn.tile_vectors >= 1 && tn.tile_vectors <= 64, "nt2g_batch_create: tile_vectors %d", tn.tile_vectors);
    nt2g_batch *b = new (std::nothrow) nt2g_batch();
    if (!b) { set_error("nt2g_batch_create: out of host memory"); return NT2G_ERR_NOMEM; }
    b->tune = tn;
    b->dynamic = tn.blocks_per_sm >= 0 ? 1 : 0;  // negative blocks_per_sm selects static striding
    b->tile_elems = (int64_t)tn.block_threads * tn.tile_vectors * 4;
    b->n_items = n_items;
    std::vector<int64_t> prefix(n_items + 1, 0);
    b->host_items.resize(n_items);
    for (int i = 0; i < n_items; ++i) {
        const nt2g_batch_item &it = items[i];
        bool ok = it.expr >= 0 && it.expr <= 2 && it.n >= 0 && it.in[0] && it.out[0] &&
                  (it.expr == NT2G_BATCH_SAXPY || (it.in[1] && it.in[2])) &&
                  (it.expr != NT2G_BATCH_BLACKSCHOLES || it.out[1]);
        if (ok && it.n > 0)
            for (int j = 0; j < 3; ++j)
                if (!reachable(it.in[j]) || (j < 2 && !reachable(it.out[j]))) {
                    delete b;
                    set_error("nt2g_batch_create: item %d holds host memory the device cannot access", i);
                    return NT2G_ERR_INVALID;
                }
        if (!ok) {
            delete b;
            set_error("nt2g_batch_create: item %d is malformed (expr %d)", i, it.expr);
            return NT2G_ERR_INVALID;
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
        b->host_items[i] = d;
        prefix[i + 1] = prefix[i] + (it.n + b->tile_elems - 1) / b->tile_elems;
        b->elements += it.n;
        b->bytes += item_bytes(it.expr, it.n);
    }
    b->total_tiles = prefix[n_items];
    cudaError_t e = cudaMalloc(&b->d_items, sizeof(DItem) * n_items);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_prefix, sizeof(int64_t) * (n_items + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, 256);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_items, b->host_items.data(), sizeof(DItem) * n_items, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_prefix, prefix.data(), sizeof(int64_t) * (n_items + 1), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        nt2g_batch_destroy(b);
        return cuda_status(e, "nt2g_batch_create: device upload");
    }
    *out = b;
    return NT2G_OK;
}

extern "C" void nt2g_batch_destroy(nt2g_batch *b)
{
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_items);
    cudaFree(b->d_prefix);
    cudaFree(b->d_counter);
    delete b;
}

template <class P>
static nt2g_status batch_launch(nt2g_batch *b, cudaStream_t st)
{
    const int threads = b->tune.block_threads;
    int grid;
    if (b->dynamic) {
        int per_sm = b->tune.blocks_per_sm;
        if (per_sm <= 0) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<P, true>, threads, 0) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
        }
        grid = device_sm_count() * per_sm;
        cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) return cuda_status(e, "batch counter reset");
        k_batch<P, true><<<grid, threads, 0, st>>>(b->d_items, b->d_prefix, b->n_items, b->total_tiles,
                                                   b->tile_elems, b->d_counter);
    } else {
        // -blocks_per_sm resident blocks per SM, capped by what the SM holds
        int per_sm = -b->tune.blocks_per_sm, limit = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&limit, k_batch<P, false>, threads, 0) != cudaSuccess ||
            limit < 1)
            limit = 1;
        if (per_sm < 1 || per_sm > limit) per_sm = limit;
        grid = device_sm_count() * per_sm;
        k_batch<P, false><<<grid, threads, 0, st>>>(b->d_items, b->d_prefix, b->n_items, b->total_tiles,
                                                    b->tile_elems, b->d_counter);
    }
    NT2G_LAUNCH_CHECK("batch launch");
    return NT2G_OK;
}

extern "C" nt2g_status nt2g_batch_run(nt2g_batch *b, void *stream)
{
    NT2G_CHECK_ARG(b != nullptr, "nt2g_batch_run: NULL batch");
    cudaStream_t st = (cudaStream_t)stream;
    return b->tune.precision == NT2G_PREC_NT2 ? batch_launch<Nt2>(b, st) : batch_launch<Fast>(b, st);
}

// The comparison path: each table through its expression's own plain kernel
// (nt2g_blackscholes_f32 / nt2g_saxpy_f32 / nt2g_expr3_f32 launchers), one
// launch per table, as a caller without the batched path would issue them.
static nt2g_status per_table(nt2g_batch *b, cudaStream_t st)
{
    const int prec = b->tune.precision;
    for (int k = 0; k < b->n_items; ++k) {
        const DItem &it = b->host_items[k];
        nt2g_status s;
        switch (it.expr) {
        case NT2G_BATCH_BLACKSCHOLES:
            s = launch_bs(it.in[0], it.in[1], it.in[2], nullptr, it.s[0], it.s[1], it.out[0], it.out[1], it.n, prec, st);
            break;
        case NT2G_BATCH_SAXPY: s = launch_saxpy(it.s[0], it.in[0], it.out[0], it.out[0], it.n, st); break;
        default: s = launch_expr3(it.in[0], it.in[1], it.in[2], it.out[0], it.n, prec, st); break;
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

// ---------------------------------------------------------------- tuning --
// Times nt2g_batch_run for each candidate (block size, float4 vectors per
// thread per tile -- i.e. elements per thread -- and resident blocks per SM,
// negative for the static tile stride) with CUDA events, reps runs after one
// warm-up each, and returns the fastest.  Each candidate builds its own plan,
// so device memory is allocated here, at tuning time.  Every run executes the
// whole batch: expressions that update a table in place (saxpy) are applied
// (1 + reps) times per candidate.
extern "C" nt2g_status nt2g_batch_autotune(const nt2g_batch_item *items, int32_t n_items,
                                           const nt2g_batch_tune *candidates, int32_t n_candidates, int32_t reps,
                                           int32_t precision, void *stream, nt2g_batch_tune *best, float *best_ms)
{
    NT2G_CHECK_ARG(best != nullptr, "nt2g_batch_autotune: best is NULL");
    NT2G_CHECK_ARG(reps >= 1 && reps <= 100, "nt2g_batch_autotune: reps %d outside [1,100]", reps);
    static const nt2g_batch_tune grid[] = {
        {128, 0, 8, 0},  {128, 0, 16, 0}, {128, 0, 32, 0}, {128, 0, 64, 0}, {256, 0, 8, 0},  {256, 0, 16, 0},
        {256, 0, 32, 0}, {256, 0, 64, 0}, {512, 0, 16, 0}, {512, 0, 32, 0}, {128, -1, 32, 0}, {256, -1, 16, 0},
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
    if (best_ms) *best_ms = best_t / reps;
    return NT2G_OK;
}
