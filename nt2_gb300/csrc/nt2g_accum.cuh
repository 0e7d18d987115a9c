// nt2g_accum.cuh -- compensated FP32 accumulation shared by the fold and
// scan kernels: a running sum carried as s + c, c collecting the exact
// rounding error of every addition (TwoSum).
#pragma once
#if !defined(__CUDACC_RTC__)  // the run-time compiler (folds of expressions) embeds this header
#include <cuda_runtime.h>
#endif

namespace nt2g {

// Compensated sum: value = s + c, c collecting the exact rounding errors.
struct CSum {
    float s, c;
};
__device__ __forceinline__ void csum_add(CSum &a, float v)
{
    const float s = __fadd_rn(a.s, v);
    const float bb = __fsub_rn(s, a.s);
    const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    a.s = s;
    a.c = __fadd_rn(a.c, e);
}
__device__ __forceinline__ void csum_merge(CSum &a, const CSum &b)
{
    csum_add(a, b.s);
    a.c = __fadd_rn(a.c, b.c);
}

// Warp reduction of compensated sums (lane 0 receives the total).
__device__ __forceinline__ CSum warp_csum(CSum a)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        CSum b{__shfl_down_sync(0xffffffffu, a.s, off), __shfl_down_sync(0xffffffffu, a.c, off)};
        csum_merge(a, b);
    }
    return a;
}
}  // namespace nt2g
