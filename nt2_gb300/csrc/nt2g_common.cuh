// nt2g_common.cuh -- launch geometry, vector memory access and error plumbing
// shared by the kernels of libnt2gpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "nt2g.h"

namespace nt2g {

// Streaming accesses: inputs are read once (evict-first, no L1 allocation),
// outputs are written once.
__device__ __forceinline__ float4 ld_stream(const float4 *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }
__device__ __forceinline__ uint4 ld_stream(const uint4 *p) { return __ldcs(p); }
__device__ __forceinline__ void st_stream(float4 *p, float4 v) { __stcs(p, v); }
__device__ __forceinline__ void st_stream(float *p, float v) { __stcs(p, v); }
__device__ __forceinline__ void st_stream(uint4 *p, uint4 v) { __stcs(p, v); }

__device__ __forceinline__ float get(const float4 &v, int i)
{
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}
__device__ __forceinline__ void set(float4 &v, int i, float x)
{
    if (i == 0) v.x = x; else if (i == 1) v.y = x; else if (i == 2) v.z = x; else v.w = x;
}

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// Programmatic dependent launch (sm_90+): a kernel launched with
// launch_dependent() may start while the previous kernel in its stream is
// still running; pdl_wait() returns once that kernel has completed and its
// memory is visible (immediately when there is no such dependency).  A kernel
// reads only inputs no earlier kernel writes before pdl_wait(), and writes
// nothing before it.  pdl_trigger() lets the next dependent launch begin.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Persistent grid: resident blocks per SM (from the occupancy calculator)
// times the SM count, capped by the work available.
struct Geometry {
    int sms = 0;
};
int device_sm_count();
template <class K>
inline int persistent_blocks(K kernel, int threads, size_t smem, int64_t work_items_per_block_min,
                             int64_t work_items)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t full = (int64_t)device_sm_count() * per_sm;
    int64_t need = (work_items + work_items_per_block_min - 1) / work_items_per_block_min;
    if (need < 1) need = 1;
    return (int)(need < full ? need : full);
}

// Thread-local last-error text behind nt2g_last_error().
void set_error(const char *fmt, ...);
nt2g_status cuda_status(cudaError_t e, const char *what);

}  // namespace nt2g

#define NT2G_CHECK_ARG(cond, ...)                                                           \
    do {                                                                                    \
        if (!(cond)) { nt2g::set_error(__VA_ARGS__); return NT2G_ERR_INVALID; }             \
    } while (0)

#define NT2G_LAUNCH_CHECK(what)                                                             \
    do {                                                                                    \
        cudaError_t e_ = cudaGetLastError();                                                \
        if (e_ != cudaSuccess) return nt2g::cuda_status(e_, what);                          \
    } while (0)
