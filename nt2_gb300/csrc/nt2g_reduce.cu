// nt2g_reduce.cu -- sum(x) and dot(x,y) over float tables.
//
// Replaces NT2's fold path (inner_fold_ on the shared_memory site,
// modules/arch/shared_memory/include/nt2/core/functions/shared_memory/
// inner_fold.hpp:25-64, OpenMP spawner modules/arch/openmp/include/nt2/sdk/
// openmp/spawner/fold.hpp:37-81), which folds 16-element blocks in naive
// FP32 and combines them under a critical section in thread-timing order.
//
// Here: each thread keeps four compensated FP32 accumulators (s, c) fed by
// TwoSum (Knuth) -- for dot the product error fma(x,y,-x*y) is folded in as
// well -- then (s, c) pairs are merged across the warp with shuffles and
// across the block through shared memory, still in FP32 TwoSum arithmetic.
// Each block writes s + c as one double; the last block to finish (atomic
// ticket after a release fence) adds the block partials in FP64 in a fixed
// order.  The result is deterministic for a given n and device.  No block
// ever waits on another.
#include <cuda.h>
#include <mutex>
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

static constexpr int kRThreads = 256;
static constexpr int kMaxPartials = 152 * 32;  // SMs x blocks per SM, upper bound

struct Acc {
    float s, c;
};

__device__ __forceinline__ void two_sum_add(Acc &a, float x)
{
    float s = __fadd_rn(a.s, x);
    float bb = __fsub_rn(s, a.s);
    float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    a.s = s;
    a.c = __fadd_rn(a.c, e);
}

__device__ __forceinline__ void two_prod_add(Acc &a, float x, float y)
{
    float p = __fmul_rn(x, y);
    float pe = __fmaf_rn(x, y, -p);
    float s = __fadd_rn(a.s, p);
    float bb = __fsub_rn(s, a.s);
    float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    a.s = s;
    a.c = __fadd_rn(a.c, __fadd_rn(e, pe));
}

__device__ __forceinline__ Acc merge(Acc a, Acc b)
{
    Acc r{a.s, __fadd_rn(a.c, b.c)};
    two_sum_add(r, b.s);
    return r;
}

__device__ __forceinline__ Acc warp_merge(Acc a)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Acc b{__shfl_xor_sync(0xffffffffu, a.s, o), __shfl_xor_sync(0xffffffffu, a.c, o)};
        // order the pair by lane so both lanes compute the same value
        a = (threadIdx.x & o) ? merge(b, a) : merge(a, b);
    }
    return a;
}

template <bool DOT>
__global__ void __launch_bounds__(kRThreads) k_reduce(const float *__restrict__ x, const float *__restrict__ y,
                                                      int64_t n, int vec, double *__restrict__ partials,
                                                      unsigned int *__restrict__ ticket, double *out64,
                                                      float *out32)
{
    Acc acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        int64_t i = tid;
        for (; i + stride < nv; i += 2 * stride) {
            float4 a0 = ld_stream((const float4 *)x + i), a1 = ld_stream((const float4 *)x + i + stride);
            if (DOT) {
                float4 b0 = ld_stream((const float4 *)y + i), b1 = ld_stream((const float4 *)y + i + stride);
#pragma unroll
                for (int j = 0; j < 4; ++j) two_prod_add(acc[j], get(a0, j), get(b0, j));
#pragma unroll
                for (int j = 0; j < 4; ++j) two_prod_add(acc[j], get(a1, j), get(b1, j));
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) two_sum_add(acc[j], get(a0, j));
#pragma unroll
                for (int j = 0; j < 4; ++j) two_sum_add(acc[j], get(a1, j));
            }
        }
        for (; i < nv; i += stride) {
            float4 a0 = ld_stream((const float4 *)x + i);
            if (DOT) {
                float4 b0 = ld_stream((const float4 *)y + i);
#pragma unroll
                for (int j = 0; j < 4; ++j) two_prod_add(acc[j], get(a0, j), get(b0, j));
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) two_sum_add(acc[j], get(a0, j));
            }
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) {
        if (DOT) two_prod_add(acc[0], x[i], y[i]);
        else two_sum_add(acc[0], x[i]);
    }
    Acc a = merge(merge(acc[0], acc[1]), merge(acc[2], acc[3]));
    a = warp_merge(a);

    __shared__ Acc wsum[kRThreads / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = a;
    __syncthreads();
    if (warp == 0) {
        Acc b = lane < (int)(blockDim.x >> 5) ? wsum[lane] : Acc{0.f, 0.f};
        b = warp_merge(b);
        if (lane == 0) {
            partials[blockIdx.x] = (double)b.s + (double)b.c;
            __threadfence();
            unsigned int t = atomicAdd(ticket, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return;
    // last block: FP64 combine of the block partials in a fixed order
    __threadfence();
    __shared__ double dsum[kRThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += ((volatile double *)partials)[i];
    dsum[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) dsum[threadIdx.x] += dsum[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *out64 = dsum[0];
        if (out32) *out32 = (float)dsum[0];
        *ticket = 0u;  // leave the workspace ready for the next call
    }
}

static int reduce_grid(bool dot, int64_t n)
{
    int g = dot ? persistent_blocks(k_reduce<true>, kRThreads, 0, kRThreads * 8, (n + 3) / 4)
                : persistent_blocks(k_reduce<false>, kRThreads, 0, kRThreads * 8, (n + 3) / 4);
    return g < kMaxPartials ? g : kMaxPartials;
}

// Workspace layout: [ticket (256 B)] [partials: kMaxPartials doubles]
static constexpr size_t kWsBytes = 256 + sizeof(double) * kMaxPartials;

nt2g_status reduce_workspace_bytes(size_t *bytes)
{
    *bytes = kWsBytes;
    return NT2G_OK;
}

nt2g_status launch_reduce(const float *x, const float *y, int64_t n, void *ws, double *out64, float *out32,
                          cudaStream_t st)
{
    unsigned int *ticket = (unsigned int *)ws;
    double *partials = (double *)((char *)ws + 256);
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return cuda_status(e, "reduce workspace reset");
    int vec = aligned16(x) && (!y || aligned16(y));
    int g = reduce_grid(y != nullptr, n);
    if (y) k_reduce<true><<<g, kRThreads, 0, st>>>(x, y, n, vec, partials, ticket, out64, out32);
    else k_reduce<false><<<g, kRThreads, 0, st>>>(x, y, n, vec, partials, ticket, out64, out32);
    NT2G_LAUNCH_CHECK("reduce launch");
    return NT2G_OK;
}

// ------------------------------------------------- no-allocation variant --
// Same kernel, but its scratch (the block ticket and one FP64 partial per
// block) lives in this file-scope device array instead of a caller workspace.
// It is for callers that cannot allocate device memory: hosts whose runtime
// owns every device allocation through its own pool and forbids others
// (language runtimes behind an FFI, engines with a fixed device-memory
// budget), code that must not risk cudaMalloc/cudaFree synchronizing the
// device, and thin wrappers with nowhere to keep a workspace between calls.
// Every GPU that loads the library holds these 39,168 bytes until exit.
static __device__ __align__(256) unsigned char g_reduce_scratch[kWsBytes];

// Identity of the calling thread's current context, through the driver entry
// points the runtime hands out (no link against the driver library).  Context
// IDs are unique for the life of the process, so a context created after
// cudaDeviceReset never matches the one an address was cached for.
static bool current_context_id(unsigned long long *id)
{
    typedef CUresult (*get_current_t)(CUcontext *);
    typedef CUresult (*get_id_t)(CUcontext, unsigned long long *);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (get_current_t)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (get_id_t)f;
        cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of g_reduce_scratch for the current device.  Host code only
// sees a host-side stand-in for the symbol, so the address is asked of the
// runtime with the device current and cached per device together with the
// identity of the context it belongs to; a new context on that device (after
// cudaDeviceReset) triggers a fresh lookup.  Without a context identity the
// lookup runs on every call.
static nt2g_status noalloc_scratch(void **out)
{
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static void *addr[kMaxDevices] = {};
    static unsigned long long ctx_of[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_reduce_f32_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("nt2g_reduce_f32_noalloc: device %d beyond the %d devices it tracks", dev, kMaxDevices);
        return NT2G_ERR_UNSUPPORTED;
    }
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(mu);
    if (!have_id || !addr[dev] || ctx_of[dev] != id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_reduce_scratch);
        if (e != cudaSuccess) return cuda_status(e, "nt2g_reduce_f32_noalloc: cudaGetSymbolAddress");
        if (!have_id) have_id = current_context_id(&id);  // the lookup made the device's context current
        addr[dev] = have_id ? p : nullptr;
        ctx_of[dev] = id;
        *out = p;
        return NT2G_OK;
    }
    *out = addr[dev];
    return NT2G_OK;
}

nt2g_status launch_reduce_noalloc(const float *x, const float *y, int64_t n, double *out64, float *out32,
                                  cudaStream_t st)
{
    void *ws = nullptr;
    nt2g_status s = noalloc_scratch(&ws);
    if (s != NT2G_OK) return s;
    const bool dot = y != nullptr;
    int g = dot ? persistent_blocks(k_reduce<true>, kRThreads, 0, kRThreads * 8, (n + 3) / 4)
                : persistent_blocks(k_reduce<false>, kRThreads, 0, kRThreads * 8, (n + 3) / 4);
    if (g > kMaxPartials) {
        set_error("nt2g_reduce_f32_noalloc: the launch needs %d block partials, the static scratch holds %d", g,
                  kMaxPartials);
        return NT2G_ERR_UNSUPPORTED;
    }
    unsigned int *ticket = (unsigned int *)ws;
    double *partials = (double *)((char *)ws + 256);
    // the array keeps the previous call's contents: the ticket must restart at 0
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return cuda_status(e, "nt2g_reduce_f32_noalloc: ticket reset");
    int vec = aligned16(x) && (!y || aligned16(y));
    if (dot) k_reduce<true><<<g, kRThreads, 0, st>>>(x, y, n, vec, partials, ticket, out64, out32);
    else k_reduce<false><<<g, kRThreads, 0, st>>>(x, y, n, vec, partials, ticket, out64, out32);
    NT2G_LAUNCH_CHECK("nt2g_reduce_f32_noalloc launch");
    return NT2G_OK;
}

}  // namespace nt2g
