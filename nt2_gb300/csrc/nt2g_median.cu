// nt2g_median.cu -- median(a, dim) and medianad(a, dim) along one dimension.
//
// NT2 (core/reduction/include/nt2/core/functions/expr/median.hpp:37-50) sorts
// each slice ascending along dim and takes the middle element for an odd
// length n, or meanof of the two middle ones for an even n; medianad
// (expr/medianad.hpp:38-54) is median(abs(a - expand_to(median(a, dim)))).
// Both results are order statistics, so here nothing is sorted: each slice's
// rank-(n-1)/2 element is found by radix selection on order-preserving
// 32-bit keys (four 8-bit digits, most significant first: a 256-bin
// histogram of the keys that share the digits found so far picks the next
// digit), and for an even n the next order statistic is either an equal key
// or the smallest key above it.
//
//  * slices of up to kSmemKeys elements: one block per slice, its keys held
//    in shared memory; the four histogram passes run over shared memory.
//  * longer slices: the same passes over global memory, many blocks per
//    slice, each adding its block histogram into the slice's histogram in
//    the workspace; a one-warp kernel per slice then picks the digit.
//
// A slice holding a NaN gives NaN (NT2 sorts with operator<, which orders no
// NaN, so its result there is unspecified).  -0 and +0 are distinct keys
// (-0 first); NT2's sort leaves their order unspecified, so where both sit
// at the middle the sign of a zero result may differ from NT2's.
#include "nt2g_common.cuh"
#include "nt2g_internal.h"

namespace nt2g {

constexpr int64_t kSmemKeys = 40960;  // 160 KB of keys per block
constexpr int64_t kChunk = 1 << 16;   // elements per block in the global passes
constexpr int kLoadBatch = 8;         // loads a thread issues before it uses them

// Order-preserving key: all bits of a negative float flipped, the sign bit
// of a positive one set; unsigned comparison of keys is the float order.
__device__ __forceinline__ uint32_t med_key(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float med_val(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// boost.simd's float meanof (arithmetic/functions/generic/meanof.hpp:21-33):
// m + (max - m) * 1/2 for finite arguments, else average = fma(a0, 1/2,
// a1 * 1/2), NT2's fma unfused.  a0 is the lower middle element.
__device__ __forceinline__ float nt2_meanof(float a0, float a1)
{
    const float m = a0 < a1 ? a0 : a1, M = a0 > a1 ? a0 : a1;
    const bool fin = __fsub_rn(a0, a0) == 0.0f && __fsub_rn(a1, a1) == 0.0f;
    return fin ? __fadd_rn(m, __fmul_rn(__fsub_rn(M, m), 0.5f))
               : __fadd_rn(__fmul_rn(a0, 0.5f), __fmul_rn(a1, 0.5f));
}

// Element k of slice s: x[l + lo*(k + n*h)], s = l + lo*h; medianad's
// elements are |x - centre(s)| (NT2: abs(a0 - expand_to(t0))).
template <bool AD>
__device__ __forceinline__ float med_elem(const float *__restrict__ base, int64_t lo, int64_t k, float c)
{
    const float v = base[lo * k];
    return AD ? fabsf(__fsub_rn(v, c)) : v;
}

// One warp: the bin of hist (256 counts) holding rank r, the rank left
// inside that bin and the bin's count.
template <class C>
__device__ __forceinline__ void med_find_bin(const C *hist, C r, int lane, uint32_t &bin, C &rest, C &cnt, bool &mine)
{
    C b[8], t = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        b[j] = hist[lane * 8 + j];
        t += b[j];
    }
    C inc = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const C v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    const C exc = inc - t;
    mine = r >= exc && r < inc;
    if (mine) {
        C acc = exc;
        int j = 0;
        while (j < 7 && acc + b[j] <= r) acc += b[j++];
        bin = (uint32_t)(lane * 8 + j);
        rest = r - acc;
        cnt = b[j];
    }
}

// ------------------------------------------------- slices in shared memory --
template <bool AD>
__global__ void k_median_smem(const float *__restrict__ x, int64_t lo, int64_t n, const float *centre,
                              float *out)
{
    extern __shared__ uint32_t keys[];  // [n] keys, then 256 bins
    uint32_t *hist = keys + n;
    __shared__ uint32_t sh_bin, sh_rest, sh_cnt, sh_min;
    const int64_t s = blockIdx.x, l = s % lo, h = s / lo;
    const float *base = x + l + lo * n * h;
    const float c = AD ? centre[s] : 0.0f;
    int nan = 0;
    // kLoadBatch loads in flight per thread before any is used: one at a time,
    // the loop would wait a memory latency per element
    for (int64_t k0 = threadIdx.x; k0 < n; k0 += kLoadBatch * (int64_t)blockDim.x) {
        float v[kLoadBatch];
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const int64_t k = k0 + j * (int64_t)blockDim.x;
            v[j] = k < n ? med_elem<AD>(base, lo, k, c) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const int64_t k = k0 + j * (int64_t)blockDim.x;
            if (k < n) {
                nan |= v[j] != v[j];
                keys[k] = med_key(v[j]);
            }
        }
    }
    if (__syncthreads_or(nan)) {
        if (threadIdx.x == 0) out[s] = __uint_as_float(0x7fc00000u);
        return;
    }
    const bool even = (n & 1) == 0;
    uint32_t r = (uint32_t)((n - (even ? 1 : 0)) >> 1), prefix = 0, mask = 0, cnt = 0;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
            const uint32_t key = keys[k];
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            uint32_t bin = 0, rest = 0, bc = 0;
            bool mine;
            med_find_bin<uint32_t>(hist, r, threadIdx.x, bin, rest, bc, mine);
            if (mine) {
                sh_bin = bin;
                sh_rest = rest;
                sh_cnt = bc;
            }
        }
        __syncthreads();
        prefix |= sh_bin << shift;
        mask |= 255u << shift;
        r = sh_rest;
        cnt = sh_cnt;
    }
    uint32_t key2 = prefix;
    if (even && r + 1 >= cnt) {  // no second copy of the lower middle key: the next key up
        if (threadIdx.x == 0) sh_min = 0xffffffffu;
        __syncthreads();
        uint32_t m = 0xffffffffu;
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
            const uint32_t key = keys[k];
            if (key > prefix && key < m) m = key;
        }
        m = __reduce_min_sync(0xffffffffu, m);
        if ((threadIdx.x & 31) == 0) atomicMin(&sh_min, m);
        __syncthreads();
        key2 = sh_min;
    }
    if (threadIdx.x == 0) out[s] = even ? nt2_meanof(med_val(prefix), med_val(key2)) : med_val(prefix);
}

// ------------------------------------------------ long slices, global passes --
struct MedState {
    unsigned long long r, cnt;  // rank left inside the keys matching prefix; their count
    uint32_t prefix, nan, key2, pad;
};

__global__ void k_median_init(MedState *st, int64_t S, int64_t n)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    const bool even = (n & 1) == 0;
    st[s].r = (unsigned long long)((n - (even ? 1 : 0)) >> 1);
    st[s].cnt = 0;
    st[s].prefix = 0;
    st[s].nan = 0;
    st[s].key2 = 0xffffffffu;
    st[s].pad = 0;
}

// Histogram of digit (key >> shift) & 255 of the keys matching the slice's
// prefix under mask, over chunk blockIdx.x of slice blockIdx.y; the first
// pass also flags NaNs.
template <bool AD>
__global__ void __launch_bounds__(256) k_median_hist(const float *__restrict__ x, int64_t lo, int64_t n,
                                                     const float *centre, MedState *st,
                                                     unsigned long long *ghist, int shift, uint32_t mask,
                                                     int64_t s0)
{
    __shared__ uint32_t hist[256];
    const int64_t s = s0 + blockIdx.y, l = s % lo, h = s / lo;
    const float *base = x + l + lo * n * h;
    const float c = AD ? centre[s] : 0.0f;
    const uint32_t prefix = st[s].prefix;
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t k0 = blockIdx.x * kChunk, k1 = k0 + kChunk < n ? k0 + kChunk : n;
    int nan = 0;
    for (int64_t kb = k0 + threadIdx.x; kb < k1; kb += kLoadBatch * (int64_t)blockDim.x) {
        float v[kLoadBatch];
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const int64_t k = kb + j * (int64_t)blockDim.x;
            v[j] = k < k1 ? med_elem<AD>(base, lo, k, c) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const int64_t k = kb + j * (int64_t)blockDim.x;
            if (k < k1) {
                nan |= v[j] != v[j];
                const uint32_t key = med_key(v[j]);
                if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
            }
        }
    }
    if (shift == 24 && __syncthreads_or(nan) && threadIdx.x == 0) atomicOr(&st[s].nan, 1u);
    __syncthreads();
    const uint32_t v = hist[threadIdx.x];
    if (v) atomicAdd(&ghist[s * 256 + threadIdx.x], (unsigned long long)v);
}

// One warp per slice: the digit holding the slice's rank, then the slice's
// histogram cleared for the next pass.
__global__ void k_median_pick(MedState *st, unsigned long long *ghist, int shift)
{
    const int64_t s = blockIdx.x;
    const int lane = threadIdx.x;
    uint32_t bin = 0;
    unsigned long long rest = 0, cnt = 0;
    bool mine;
    med_find_bin<unsigned long long>(ghist + s * 256, st[s].r, lane, bin, rest, cnt, mine);
    __syncwarp();
    if (mine) {
        st[s].prefix |= bin << shift;
        st[s].r = rest;
        st[s].cnt = cnt;
    }
    for (int j = 0; j < 8; ++j) ghist[s * 256 + lane * 8 + j] = 0;
}

// Even lengths whose lower middle key has no second copy: the smallest key
// above it.
template <bool AD>
__global__ void __launch_bounds__(256) k_median_next(const float *__restrict__ x, int64_t lo, int64_t n,
                                                     const float *centre, MedState *st, int64_t s0)
{
    const int64_t s = s0 + blockIdx.y, l = s % lo, h = s / lo;
    if ((n & 1) || st[s].r + 1 < st[s].cnt) return;
    const float *base = x + l + lo * n * h;
    const float c = AD ? centre[s] : 0.0f;
    const uint32_t prefix = st[s].prefix;
    const int64_t k0 = blockIdx.x * kChunk, k1 = k0 + kChunk < n ? k0 + kChunk : n;
    uint32_t m = 0xffffffffu;
    for (int64_t kb = k0 + threadIdx.x; kb < k1; kb += kLoadBatch * (int64_t)blockDim.x) {
        float v[kLoadBatch];
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const int64_t k = kb + j * (int64_t)blockDim.x;
            v[j] = k < k1 ? med_elem<AD>(base, lo, k, c) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kLoadBatch; ++j) {
            const uint32_t key = med_key(v[j]);
            if (kb + j * (int64_t)blockDim.x < k1 && key > prefix && key < m) m = key;
        }
    }
    m = __reduce_min_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m != 0xffffffffu) atomicMin(&st[s].key2, m);
}

__global__ void k_median_out(const MedState *st, int64_t S, int64_t n, float *out)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) return;
    const MedState m = st[s];
    float v;
    if (m.nan) v = __uint_as_float(0x7fc00000u);
    else if (n & 1) v = med_val(m.prefix);
    else v = nt2_meanof(med_val(m.prefix), med_val(m.r + 1 < m.cnt ? m.prefix : m.key2));
    out[s] = v;
}

__global__ void k_median_fill_nan(float *out, int64_t S)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s < S) out[s] = __uint_as_float(0x7fc00000u);
}

size_t median_workspace_bytes(int64_t lo, int64_t n, int64_t hi)
{
    if (n <= kSmemKeys) return 0;
    const int64_t S = lo * hi;
    return (size_t)S * (256 * sizeof(unsigned long long) + sizeof(MedState));
}

template <bool AD>
static nt2g_status median_pass(const float *x, int64_t lo, int64_t n, int64_t hi, const float *centre,
                               void *ws, float *out, cudaStream_t st)
{
    const int64_t S = lo * hi;
    if (n <= kSmemKeys) {
        const size_t smem = (size_t)n * 4 + 256 * 4;
        if (smem > 48 * 1024) {  // per device: set on every call that needs it
            cudaError_t e = cudaFuncSetAttribute(k_median_smem<AD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)(kSmemKeys * 4 + 256 * 4));
            if (e != cudaSuccess) return cuda_status(e, "median: shared memory attribute");
        }
        const int threads = n >= 256 ? 256 : (int)((n + 31) / 32 * 32);
        k_median_smem<AD><<<(unsigned)S, threads, smem, st>>>(x, lo, n, centre, out);
        NT2G_LAUNCH_CHECK("median (shared memory)");
        return NT2G_OK;
    }
    unsigned long long *ghist = (unsigned long long *)ws;
    MedState *state = (MedState *)(ghist + S * 256);
    cudaError_t e = cudaMemsetAsync(ghist, 0, (size_t)S * 256 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_status(e, "median: histogram clear");
    k_median_init<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(state, S, n);
    const unsigned chunks = (unsigned)((n + kChunk - 1) / kChunk);
    uint32_t mask = 0;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int64_t s0 = 0; s0 < S; s0 += 65535) {  // grid.y: at most 65535 slices per launch
            const dim3 grid(chunks, (unsigned)(S - s0 < 65535 ? S - s0 : 65535));
            k_median_hist<AD><<<grid, 256, 0, st>>>(x, lo, n, centre, state, ghist, shift, mask, s0);
        }
        k_median_pick<<<(unsigned)S, 32, 0, st>>>(state, ghist, shift);
        mask |= 255u << shift;
    }
    for (int64_t s0 = 0; s0 < S; s0 += 65535) {
        const dim3 grid(chunks, (unsigned)(S - s0 < 65535 ? S - s0 : 65535));
        k_median_next<AD><<<grid, 256, 0, st>>>(x, lo, n, centre, state, s0);
    }
    k_median_out<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(state, S, n, out);
    NT2G_LAUNCH_CHECK("median (global passes)");
    return NT2G_OK;
}

nt2g_status launch_median(const float *x, int64_t lo, int64_t n, int64_t hi, int32_t op, void *ws, float *out,
                          cudaStream_t st)
{
    const int64_t S = lo * hi;
    if (n == 0) {  // no middle element
        k_median_fill_nan<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(out, S);
        NT2G_LAUNCH_CHECK("median (empty slices)");
        return NT2G_OK;
    }
    nt2g_status r = median_pass<false>(x, lo, n, hi, nullptr, ws, out, st);
    if (r != NT2G_OK || op == NT2G_MEDIAN) return r;
    return median_pass<true>(x, lo, n, hi, out, ws, out, st);
}

}  // namespace nt2g
