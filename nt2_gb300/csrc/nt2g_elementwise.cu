// nt2g_elementwise.cu -- fused elementwise kernels other than Black-Scholes
// (saxpy, expr3, rgb2yuv, sigma-delta), element maps, and the generic
// program interpreter that evaluates any lowered nt2 expression in one pass.
#include <cuda_fp16.h>
#include <string.h>
#include "nt2g_common.cuh"
#include "nt2g_exprs.cuh"
#include "nt2g_internal.h"

namespace nt2g {

static constexpr int kThreads = 256;

template <class KERN>
static int grid_for(KERN k, int64_t units)
{
    return persistent_blocks(k, kThreads, 0, kThreads * 2, units);
}

// ------------------------------------------------------------------ saxpy --
// Y = alpha*X + Y with NT2's two roundings (demo/saxpy/nt2/saxpy_nt2.cpp:41).
__global__ void __launch_bounds__(kThreads) k_saxpy(float alpha, const float *__restrict__ X,
                                                    const float *Y, float *O, int64_t n, int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        int64_t i = tid;
        // two vectors in flight per thread
        for (; i + stride < nv; i += 2 * stride) {
            float4 x0 = ld_stream((const float4 *)X + i), y0 = ld_stream((const float4 *)Y + i);
            float4 x1 = ld_stream((const float4 *)X + i + stride), y1 = ld_stream((const float4 *)Y + i + stride);
            float4 o0, o1;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                set(o0, j, saxpy_elem(alpha, get(x0, j), get(y0, j)));
                set(o1, j, saxpy_elem(alpha, get(x1, j), get(y1, j)));
            }
            st_stream((float4 *)O + i, o0);
            st_stream((float4 *)O + i + stride, o1);
        }
        for (; i < nv; i += stride) {
            float4 x0 = ld_stream((const float4 *)X + i), y0 = ld_stream((const float4 *)Y + i), o0;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(o0, j, saxpy_elem(alpha, get(x0, j), get(y0, j)));
            st_stream((float4 *)O + i, o0);
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) O[i] = saxpy_elem(alpha, X[i], Y[i]);
}

// O may alias Y (the in-place form of the demo).
nt2g_status launch_saxpy(float alpha, const float *X, const float *Y, float *O, int64_t n, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(X) && aligned16(Y) && aligned16(O);
    k_saxpy<<<grid_for(k_saxpy, (n + 3) / 4), kThreads, 0, st>>>(alpha, X, Y, O, n, vec);
    NT2G_LAUNCH_CHECK("saxpy launch");
    return NT2G_OK;
}

// ------------------------------------------------------------------ expr3 --
template <class P>
__global__ void __launch_bounds__(kThreads) k_expr3(const float *__restrict__ x, const float *__restrict__ y,
                                                    const float *__restrict__ z, float *__restrict__ o,
                                                    int64_t n, int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        for (int64_t i = tid; i < nv; i += stride) {
            float4 a = ld_stream((const float4 *)x + i), b = ld_stream((const float4 *)y + i),
                   c = ld_stream((const float4 *)z + i), r;
#pragma unroll
            for (int j = 0; j < 4; ++j) set(r, j, expr3_elem<P>(get(a, j), get(b, j), get(c, j)));
            st_stream((float4 *)o + i, r);
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) o[i] = expr3_elem<P>(x[i], y[i], z[i]);
}

nt2g_status launch_expr3(const float *x, const float *y, const float *z, float *out, int64_t n, int precision,
                         cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(x) && aligned16(y) && aligned16(z) && aligned16(out);
    if (precision == NT2G_PREC_NT2)
        k_expr3<Nt2><<<grid_for(k_expr3<Nt2>, (n + 3) / 4), kThreads, 0, st>>>(x, y, z, out, n, vec);
    else
        k_expr3<Fast><<<grid_for(k_expr3<Fast>, (n + 3) / 4), kThreads, 0, st>>>(x, y, z, out, n, vec);
    NT2G_LAUNCH_CHECK("expr3 launch");
    return NT2G_OK;
}

// ---------------------------------------------------------------- rgb2yuv --
template <class P>
__global__ void __launch_bounds__(kThreads) k_rgb2yuv(const float *__restrict__ r, const float *__restrict__ g,
                                                      const float *__restrict__ b, float *__restrict__ y,
                                                      float *__restrict__ u, float *__restrict__ v, int64_t n,
                                                      int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 2;
        for (int64_t i = tid; i < nv; i += stride) {
            float4 R = ld_stream((const float4 *)r + i), G = ld_stream((const float4 *)g + i),
                   B = ld_stream((const float4 *)b + i), Y, U, V;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float yy, uu, vv;
                yuv_px<P>(get(R, j), get(G, j), get(B, j), yy, uu, vv);
                set(Y, j, yy); set(U, j, uu); set(V, j, vv);
            }
            st_stream((float4 *)y + i, Y);
            st_stream((float4 *)u + i, U);
            st_stream((float4 *)v + i, V);
        }
        done = nv << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) yuv_px<P>(r[i], g[i], b[i], y[i], u[i], v[i]);
}

nt2g_status launch_rgb2yuv(const float *r, const float *g, const float *b, float *y, float *u, float *v,
                           int64_t n, int precision, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(r) && aligned16(g) && aligned16(b) && aligned16(y) && aligned16(u) && aligned16(v);
    if (precision == NT2G_PREC_NT2)
        k_rgb2yuv<Nt2><<<grid_for(k_rgb2yuv<Nt2>, (n + 3) / 4), kThreads, 0, st>>>(r, g, b, y, u, v, n, vec);
    else
        k_rgb2yuv<Fast><<<grid_for(k_rgb2yuv<Fast>, (n + 3) / 4), kThreads, 0, st>>>(r, g, b, y, u, v, n, vec);
    NT2G_LAUNCH_CHECK("rgb2yuv launch");
    return NT2G_OK;
}

// ------------------------------------------------------------ sigma-delta --
// The vector paths evaluate the uint8 step in packed fp16 (half2): every value
// involved is an integer in [0, 1279], exact in fp16, and compare (1.0/0.0
// results), min, add and fma are single two-lane instructions where the byte
// SIMD intrinsics are multi-instruction sequences.  Pixels carry a +1024
// offset: the fp16 pattern 0x64pp is 1024 + pp, so a byte permute against
// 0x64 bytes unpacks four pixels into two half2 and another packs them back.
// Differences cancel the offset; m and the label compare add it back.
__device__ __forceinline__ __half2 h2_bits(uint32_t u)
{
    __half2 h;
    memcpy(&h, &u, 4);
    return h;
}
__device__ __forceinline__ uint32_t bits_h2(__half2 h)
{
    uint32_t u;
    memcpy(&u, &h, 4);
    return u;
}
// four pixels (bytes) -> (p0, p1) and (p2, p3), each as 1024 + p
__device__ __forceinline__ void sd_unpack(uint32_t w, __half2 &lo, __half2 &hi)
{
    lo = h2_bits(__byte_perm(w, 0x64646464u, 0x5140));
    hi = h2_bits(__byte_perm(w, 0x64646464u, 0x5342));
}
// inverse of sd_unpack (values 1024 + p, p in [0, 255])
__device__ __forceinline__ uint32_t sd_pack(__half2 lo, __half2 hi)
{
    return __byte_perm(bits_h2(lo), bits_h2(hi), 0x6420);
}

// One sigma-delta step on two pixels (demo/sigmadelta/nt2/sigmadelta_nt2.cpp:38-57),
// operands offset by 1024; lab receives 1024 + label.
__device__ __forceinline__ void sd_h2(__half2 f, __half2 &b, __half2 &v, __half2 &lab)
{
    const __half2 k1024 = __float2half2_rn(1024.0f), k1279 = __float2half2_rn(1279.0f);
    const __half2 k3 = __float2half2_rn(3.0f), k0 = __float2half2_rn(0.0f);
    b = __hadd2(b, __hsub2(__hlt2(b, f), __hgt2(b, f)));       // selinc/seldec toward the frame
    const __half2 d = __habs2(__hsub2(b, f));                  // max - min
    const __half2 m = __hmin2(__hfma2(d, k3, k1024), k1279);   // 1024 + adds(adds(d,d),d)
    const __half2 step = __hsub2(__hlt2(v, m), __hgt2(v, m));  // var toward m ...
    v = __hfma2(step, __hne2(d, k0), v);                       // ... where d != 0
    lab = __hadd2(__hle2(v, __hadd2(d, k1024)), k1024);        // if_zero_else_one(d < var)
}

// 16 pixels
__device__ __forceinline__ void sd_vec_h(const uint4 &f, uint4 &b, uint4 &v, uint4 &l)
{
    uint32_t *fb = (uint32_t *)&f, *bb = (uint32_t *)&b, *vb = (uint32_t *)&v, *lb = (uint32_t *)&l;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        __half2 f0, f1, b0, b1, v0, v1, l0, l1;
        sd_unpack(fb[w], f0, f1);
        sd_unpack(bb[w], b0, b1);
        sd_unpack(vb[w], v0, v1);
        sd_h2(f0, b0, v0, l0);
        sd_h2(f1, b1, v1, l1);
        bb[w] = sd_pack(b0, b1);
        vb[w] = sd_pack(v0, v1);
        lb[w] = sd_pack(l0, l1);
    }
}

__device__ __forceinline__ void sd_px(uint8_t f, uint8_t &b, uint8_t &v, uint8_t &lab)
{
    uint32_t bb = b, vv = v, l;
    sd_word(f, bb, vv, l);
    b = (uint8_t)bb; v = (uint8_t)vv; lab = (uint8_t)l;
}

__device__ __forceinline__ void sd_vec(const uint4 &f, uint4 &b, uint4 &v, uint4 &l)
{
    sd_word(f.x, b.x, v.x, l.x);
    sd_word(f.y, b.y, v.y, l.y);
    sd_word(f.z, b.z, v.z, l.z);
    sd_word(f.w, b.w, v.w, l.w);
}

// One frame step.  Consecutive steps are chained with programmatic dependent
// launch: a step's grid starts while the previous step runs, loads its frame
// (which no earlier step writes), and waits for the previous step only before
// it reads bkg/var.  One 16-pixel vector per thread, one wave.
__global__ void __launch_bounds__(kThreads, 4) k_sigmadelta(const uint8_t *__restrict__ fr, uint8_t *__restrict__ bkg,
                                                         uint8_t *__restrict__ var, uint8_t *__restrict__ lab,
                                                         int64_t n, int vec)
{
    pdl_trigger();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nv = n >> 4;  // 16 pixels per uint4
        uint4 f0 = make_uint4(0, 0, 0, 0);
        if (tid < nv) f0 = ld_stream((const uint4 *)fr + tid);
        pdl_wait();
        for (int64_t i = tid; i < nv; i += stride) {
            uint4 f = i == tid ? f0 : ld_stream((const uint4 *)fr + i), b = ld_stream((const uint4 *)bkg + i),
                  v = ld_stream((const uint4 *)var + i), l;
            sd_vec_h(f, b, v, l);
            st_stream((uint4 *)bkg + i, b);
            st_stream((uint4 *)var + i, v);
            st_stream((uint4 *)lab + i, l);
        }
        done = nv << 4;
    } else {
        pdl_wait();
    }
    for (int64_t i = done + tid; i < n; i += stride) sd_px(fr[i], bkg[i], var[i], lab[i]);
}

// Temporal fusion: a thread keeps 16 pixels' bkg/var (one uint4 each) in
// registers across all frames; eight frames' loads are issued before any is
// used.  Per pixel-frame HBM traffic drops from 6 B to 2 + 4/F B.  Planes
// that are not 16-byte aligned take a 4-pixel word path, then single pixels.
constexpr int kFramePrefetch = 8;

__global__ void __launch_bounds__(kThreads, 4) k_sigmadelta_frames(const uint8_t *__restrict__ frames,
                                                                uint8_t *__restrict__ bkg,
                                                                uint8_t *__restrict__ var,
                                                                uint8_t *__restrict__ labels, int64_t n,
                                                                int nf, int vec)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec == 2) {
        const int64_t nq = n >> 4;  // 16 pixels per uint4
        for (int64_t i = tid; i < nq; i += stride) {
            // bkg/var of 16 pixels as 8 + 8 offset half2, unpacked once
            uint4 bw = ld_stream((const uint4 *)bkg + i), vw = ld_stream((const uint4 *)var + i);
            __half2 b[8], v[8];
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                sd_unpack(((const uint32_t *)&bw)[w], b[2 * w], b[2 * w + 1]);
                sd_unpack(((const uint32_t *)&vw)[w], v[2 * w], v[2 * w + 1]);
            }
            auto frame_step = [&](const uint4 &f, int64_t k) {
                uint4 l;
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    __half2 f0, f1, l0, l1;
                    sd_unpack(((const uint32_t *)&f)[w], f0, f1);
                    sd_h2(f0, b[2 * w], v[2 * w], l0);
                    sd_h2(f1, b[2 * w + 1], v[2 * w + 1], l1);
                    ((uint32_t *)&l)[w] = sd_pack(l0, l1);
                }
                st_stream((uint4 *)(labels + k * n) + i, l);
            };
            int k = 0;
            for (; k + kFramePrefetch <= nf; k += kFramePrefetch) {
                uint4 f[kFramePrefetch];
#pragma unroll
                for (int j = 0; j < kFramePrefetch; ++j) f[j] = ld_stream((const uint4 *)(frames + (int64_t)(k + j) * n) + i);
#pragma unroll
                for (int j = 0; j < kFramePrefetch; ++j) frame_step(f[j], k + j);
            }
            for (; k < nf; ++k) frame_step(ld_stream((const uint4 *)(frames + (int64_t)k * n) + i), k);
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                ((uint32_t *)&bw)[w] = sd_pack(b[2 * w], b[2 * w + 1]);
                ((uint32_t *)&vw)[w] = sd_pack(v[2 * w], v[2 * w + 1]);
            }
            st_stream((uint4 *)bkg + i, bw);
            st_stream((uint4 *)var + i, vw);
        }
        done = nq << 4;
    } else if (vec == 1) {
        const int64_t nw = n >> 2;  // 4 pixels per word
        for (int64_t i = tid; i < nw; i += stride) {
            uint32_t b = __ldcs((const unsigned int *)bkg + i), v = __ldcs((const unsigned int *)var + i), l;
            int k = 0;
            for (; k + kFramePrefetch <= nf; k += kFramePrefetch) {
                uint32_t f[kFramePrefetch];
#pragma unroll
                for (int j = 0; j < kFramePrefetch; ++j)
                    f[j] = __ldcs((const unsigned int *)(frames + (int64_t)(k + j) * n) + i);
#pragma unroll
                for (int j = 0; j < kFramePrefetch; ++j) {
                    sd_word(f[j], b, v, l);
                    __stcs((unsigned int *)(labels + (int64_t)(k + j) * n) + i, l);
                }
            }
            for (; k < nf; ++k) {
                uint32_t f = __ldcs((const unsigned int *)(frames + (int64_t)k * n) + i);
                sd_word(f, b, v, l);
                __stcs((unsigned int *)(labels + (int64_t)k * n) + i, l);
            }
            __stcs((unsigned int *)bkg + i, b);
            __stcs((unsigned int *)var + i, v);
        }
        done = nw << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) {
        uint8_t b = bkg[i], v = var[i], l;
        for (int k = 0; k < nf; ++k) {
            sd_px(frames[(int64_t)k * n + i], b, v, l);
            labels[(int64_t)k * n + i] = l;
        }
        bkg[i] = b;
        var[i] = v;
    }
}

nt2g_status launch_sigmadelta(const uint8_t *frame, uint8_t *bkg, uint8_t *var, uint8_t *label, int64_t n,
                              cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    int vec = aligned16(frame) && aligned16(bkg) && aligned16(var) && aligned16(label);
    const int grid = persistent_blocks(k_sigmadelta, kThreads, 0, kThreads, (n + 15) / 16);
    cudaError_t e = launch_dependent(k_sigmadelta, grid, kThreads, st, frame, bkg, var, label, n, vec);
    if (e != cudaSuccess) return cuda_status(e, "sigmadelta launch");
    return NT2G_OK;
}

nt2g_status launch_sigmadelta_frames(const uint8_t *frames, uint8_t *bkg, uint8_t *var, uint8_t *labels,
                                     int64_t n, int nf, cudaStream_t st)
{
    if (n == 0 || nf == 0) return NT2G_OK;
    // every frame plane must start 16-byte (4-byte) aligned for the vector (word) path
    auto al = [](const void *p, unsigned m) { return ((uintptr_t)p & m) == 0; };
    int vec = 0;
    if (al(frames, 15) && al(bkg, 15) && al(var, 15) && al(labels, 15) && n % 16 == 0) vec = 2;
    else if (al(frames, 3) && al(bkg, 3) && al(var, 3) && al(labels, 3) && n % 4 == 0) vec = 1;
    const int64_t units = vec == 2 ? n / 16 : vec == 1 ? n / 4 : n;
    const int grid = persistent_blocks(k_sigmadelta_frames, kThreads, 0, kThreads, units);
    k_sigmadelta_frames<<<grid, kThreads, 0, st>>>(frames, bkg, var, labels, n, nf, vec);
    NT2G_LAUNCH_CHECK("sigmadelta frames launch");
    return NT2G_OK;
}

// ------------------------------------------------------------------- maps --
template <class P, int FN>
__device__ __forceinline__ float map_elem(float a)
{
    if (FN == 0) return exp<P>(a);
    if (FN == 1) return log<P>(a);
    if (FN == 2) return log1p<P>(a);
    if (FN == 3) return erfc<P>(a);
    if (FN == 4) return normcdf<P>(a);
    if (FN == 5) return fastnormcdf<P>(a);
    if (FN == 6) return P::sqrt(a);
    if (FN == 8) return exp2<P>(a);
    if (FN == 9) return exp10<P>(a);
    if (FN == 10) return expm1<P>(a);
    if (FN == 11) return log2<P>(a);
    if (FN == 12) return log10<P>(a);
    if (FN == 13) return sin<P>(a);
    if (FN == 14) return cos<P>(a);
    if (FN == 15) return tan<P>(a);
    if (FN == 16) return sinpi<P>(a);
    if (FN == 17) return cospi<P>(a);
    if (FN == 18) return sinh<P>(a);
    if (FN == 19) return cosh<P>(a);
    if (FN == 20) return tanh<P>(a);
    if (FN == 21) return asin<P>(a);
    if (FN == 22) return acos<P>(a);
    if (FN == 23) return atan<P>(a);
    if (FN == 24) return asinh<P>(a);
    if (FN == 25) return acosh<P>(a);
    if (FN == 26) return atanh<P>(a);
    if (FN == 27) return cbrt<P>(a);
    if (FN == 28) return cot<P>(a);
    if (FN == 29) return sec<P>(a);
    if (FN == 30) return csc<P>(a);
    if (FN == 31) return sind<P>(a);
    if (FN == 32) return cosd<P>(a);
    if (FN == 33) return tand<P>(a);
    if (FN == 34) return tanpi<P>(a);
    if (FN == 35) return cotpi<P>(a);
    if (FN == 36) return cotd<P>(a);
    if (FN == 37) return secpi<P>(a);
    if (FN == 38) return cscpi<P>(a);
    if (FN == 39) return secd<P>(a);
    if (FN == 40) return cscd<P>(a);
    if (FN == 41) return sinc<P>(a);
    if (FN == 42) return sincpi<P>(a);
    if (FN == 43) return acotd<P>(a);
    if (FN == 44) return asec<P>(a);
    if (FN == 45) return coth<P>(a);
    if (FN == 46) return sinhc<P>(a);
    if (FN == 47) return acsc<P>(a);
    if (FN == 48) return asech<P>(a);
    if (FN == 49) return acoth<P>(a);
    if (FN == 50) return acsch<P>(a);
    if (FN == 64) return erf<P>(a);
    if (FN == 65) return erfcx<P>(a);
    if (FN == 66) return expx2<P>(a);
    if (FN == 67) return gamma<P>(a);
    if (FN == 68) return gammaln<P>(a);
    if (FN == 69) return erfinv<P>(a);
    if (FN == 70) return erfcinv<P>(a);
    if (FN == 71) return digamma<P>(a);
    if (FN == 72) return signgam(a);
    if (FN == 73) return dawson<P>(a);
    if (FN == 74) return spence<P>(a);
    if (FN == 75) return stirling<P>(a);
    if (FN == 80) return exprecneg<P>(a);
    if (FN == 81) return exprecnegc<P>(a);
    if (FN == 82) return sqrt1pm1<P>(a);
    float p, q;
    normcdf_pair<P>(a, p, q);
    return q;
}

template <class P, int FN>
__global__ void __launch_bounds__(kThreads) k_map(const float *__restrict__ x, float *__restrict__ y, int64_t n)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = map_elem<P, FN>(x[i]);
}

template <class P>
static void map_dispatch(int fn, const float *x, float *y, int64_t n, cudaStream_t st)
{
#define NT2G_MAP(F) k_map<P, F><<<grid_for(k_map<P, F>, (n + 3) / 4), kThreads, 0, st>>>(x, y, n)
    switch (fn) {
    case 0: NT2G_MAP(0); break;
    case 1: NT2G_MAP(1); break;
    case 2: NT2G_MAP(2); break;
    case 3: NT2G_MAP(3); break;
    case 4: NT2G_MAP(4); break;
    case 5: NT2G_MAP(5); break;
    case 6: NT2G_MAP(6); break;
    case 8: NT2G_MAP(8); break;
    case 9: NT2G_MAP(9); break;
    case 10: NT2G_MAP(10); break;
    case 11: NT2G_MAP(11); break;
    case 12: NT2G_MAP(12); break;
    case 13: NT2G_MAP(13); break;
    case 14: NT2G_MAP(14); break;
    case 15: NT2G_MAP(15); break;
    case 16: NT2G_MAP(16); break;
    case 17: NT2G_MAP(17); break;
    case 18: NT2G_MAP(18); break;
    case 19: NT2G_MAP(19); break;
    case 20: NT2G_MAP(20); break;
    case 21: NT2G_MAP(21); break;
    case 22: NT2G_MAP(22); break;
    case 23: NT2G_MAP(23); break;
    case 24: NT2G_MAP(24); break;
    case 25: NT2G_MAP(25); break;
    case 26: NT2G_MAP(26); break;
    case 27: NT2G_MAP(27); break;
    case 28: NT2G_MAP(28); break;
    case 29: NT2G_MAP(29); break;
    case 30: NT2G_MAP(30); break;
    case 31: NT2G_MAP(31); break;
    case 32: NT2G_MAP(32); break;
    case 33: NT2G_MAP(33); break;
    case 34: NT2G_MAP(34); break;
    case 35: NT2G_MAP(35); break;
    case 36: NT2G_MAP(36); break;
    case 37: NT2G_MAP(37); break;
    case 38: NT2G_MAP(38); break;
    case 39: NT2G_MAP(39); break;
    case 40: NT2G_MAP(40); break;
    case 41: NT2G_MAP(41); break;
    case 42: NT2G_MAP(42); break;
    case 43: NT2G_MAP(43); break;
    case 44: NT2G_MAP(44); break;
    case 45: NT2G_MAP(45); break;
    case 46: NT2G_MAP(46); break;
    case 47: NT2G_MAP(47); break;
    case 48: NT2G_MAP(48); break;
    case 49: NT2G_MAP(49); break;
    case 50: NT2G_MAP(50); break;
    case 64: NT2G_MAP(64); break;
    case 65: NT2G_MAP(65); break;
    case 66: NT2G_MAP(66); break;
    case 67: NT2G_MAP(67); break;
    case 68: NT2G_MAP(68); break;
    case 69: NT2G_MAP(69); break;
    case 70: NT2G_MAP(70); break;
    case 71: NT2G_MAP(71); break;
    case 72: NT2G_MAP(72); break;
    case 73: NT2G_MAP(73); break;
    case 74: NT2G_MAP(74); break;
    case 75: NT2G_MAP(75); break;
    case 80: NT2G_MAP(80); break;
    case 81: NT2G_MAP(81); break;
    case 82: NT2G_MAP(82); break;
    default: NT2G_MAP(7); break;
    }
#undef NT2G_MAP
}

nt2g_status launch_map(int fn, const float *x, float *y, int64_t n, int precision, cudaStream_t st)
{
    if (n == 0) return NT2G_OK;
    if (precision == NT2G_PREC_NT2) map_dispatch<Nt2>(fn, x, y, n, st);
    else map_dispatch<Fast>(fn, x, y, n, st);
    NT2G_LAUNCH_CHECK("map launch");
    return NT2G_OK;
}

// ------------------------------------------------------------ interpreter --
// Each thread evaluates 4 consecutive elements per step; the register file
// R[reg][4] is per-thread local memory (L1-resident).  The program is a
// kernel parameter, so instruction fetch is a uniform constant-bank read and
// the opcode switch never diverges.
constexpr int kV = 4;

// The functors that work in double or loop (digamma, dawson, spence, stirling,
// nthroot, expni, gammainc, gammaincinv) are compiled only into the RARE instance of the interpreter, which
// runs the programs that use them: in the opcode switch of every program they
// would raise the kernel's register count from 42 to 62 and cut its
// occupancy.
NT2G_HD bool interp_rare_op(int op)
{
    return op == NT2G_OP_DIGAMMA || op == NT2G_OP_DAWSON || op == NT2G_OP_NTHROOT || op == NT2G_OP_EXPNI ||
           op == NT2G_OP_GAMMAINC || op == NT2G_OP_SPENCE || op == NT2G_OP_GAMMAINCINV || op == NT2G_OP_STIRLING;
}

template <class P, bool RARE>
__device__ __forceinline__ float f_unary(int op, float a)
{
    switch (op) {
    case NT2G_OP_NEG: return -a;
    case NT2G_OP_ABS: return fabsf(a);
    case NT2G_OP_SQR: return P::mul(a, a);
    case NT2G_OP_SQRT: return P::sqrt(a);
    case NT2G_OP_REC: return P::div(1.0f, a);
    case NT2G_OP_EXP: return exp<P>(a);
    case NT2G_OP_LOG: return log<P>(a);
    case NT2G_OP_LOG1P: return log1p<P>(a);
    case NT2G_OP_ERFC: return erfc<P>(a);
    case NT2G_OP_NORMCDF: return normcdf<P>(a);
    case NT2G_OP_EXP2: return exp2<P>(a);
    case NT2G_OP_EXP10: return exp10<P>(a);
    case NT2G_OP_EXPM1: return expm1<P>(a);
    case NT2G_OP_LOG2: return log2<P>(a);
    case NT2G_OP_LOG10: return log10<P>(a);
    case NT2G_OP_SIN: return sin<P>(a);
    case NT2G_OP_COS: return cos<P>(a);
    case NT2G_OP_TAN: return tan<P>(a);
    case NT2G_OP_SINPI: return sinpi<P>(a);
    case NT2G_OP_COSPI: return cospi<P>(a);
    case NT2G_OP_SINH: return sinh<P>(a);
    case NT2G_OP_COSH: return cosh<P>(a);
    case NT2G_OP_TANH: return tanh<P>(a);
    case NT2G_OP_ASIN: return asin<P>(a);
    case NT2G_OP_ACOS: return acos<P>(a);
    case NT2G_OP_ATAN: return atan<P>(a);
    case NT2G_OP_ASINH: return asinh<P>(a);
    case NT2G_OP_ACOSH: return acosh<P>(a);
    case NT2G_OP_ATANH: return atanh<P>(a);
    case NT2G_OP_CBRT: return cbrt<P>(a);
    case NT2G_OP_COT: return cot<P>(a);
    case NT2G_OP_SEC: return sec<P>(a);
    case NT2G_OP_CSC: return csc<P>(a);
    case NT2G_OP_SIND: return sind<P>(a);
    case NT2G_OP_COSD: return cosd<P>(a);
    case NT2G_OP_TAND: return tand<P>(a);
    case NT2G_OP_TANPI: return tanpi<P>(a);
    case NT2G_OP_PROPER_TANPI: return proper_tanpi<P>(a);
    case NT2G_OP_COTPI: return cotpi<P>(a);
    case NT2G_OP_COTD: return cotd<P>(a);
    case NT2G_OP_SECPI: return secpi<P>(a);
    case NT2G_OP_CSCPI: return cscpi<P>(a);
    case NT2G_OP_SECD: return secd<P>(a);
    case NT2G_OP_CSCD: return cscd<P>(a);
    case NT2G_OP_SINC: return sinc<P>(a);
    case NT2G_OP_SINCPI: return sincpi<P>(a);
    case NT2G_OP_ACOTD: return acotd<P>(a);
    case NT2G_OP_ASEC: return asec<P>(a);
    case NT2G_OP_COTH: return coth<P>(a);
    case NT2G_OP_SINHC: return sinhc<P>(a);
    case NT2G_OP_ACSC: return acsc<P>(a);
    case NT2G_OP_ASECH: return asech<P>(a);
    case NT2G_OP_ACOTH: return acoth<P>(a);
    case NT2G_OP_ACSCH: return acsch<P>(a);
    case NT2G_OP_ERF: return erf<P>(a);
    case NT2G_OP_ERFCX: return erfcx<P>(a);
    case NT2G_OP_EXPX2: return expx2<P>(a);
    case NT2G_OP_GAMMA: return gamma<P>(a);
    case NT2G_OP_GAMMALN: return gammaln<P>(a);
    case NT2G_OP_ERFINV: return erfinv<P>(a);
    case NT2G_OP_ERFCINV: return erfcinv<P>(a);
    case NT2G_OP_SIGNGAM: return signgam(a);
    case NT2G_OP_DIGAMMA: if constexpr (RARE) return digamma<P>(a); else return f_nan();
    case NT2G_OP_DAWSON: if constexpr (RARE) return dawson<P>(a); else return f_nan();
    case NT2G_OP_SPENCE: if constexpr (RARE) return spence<P>(a); else return f_nan();
    case NT2G_OP_STIRLING: if constexpr (RARE) return stirling<P>(a); else return f_nan();
    case NT2G_OP_FLOOR: return floorf(a);
    case NT2G_OP_CEIL: return ceilf(a);
    case NT2G_OP_TRUNC: return truncf(a);
    case NT2G_OP_ROUND: return roundf(a);
    case NT2G_OP_ROUND2EVEN: return nt2_round2even(a);
    case NT2G_OP_FRAC: return nt2_frac<P>(a);
    case NT2G_OP_SIGN: return nt2_sign(a);
    case NT2G_OP_SIGNNZ: return nt2_signnz(a);
    case NT2G_OP_EXPRECNEG: return exprecneg<P>(a);
    case NT2G_OP_EXPRECNEGC: return exprecnegc<P>(a);
    case NT2G_OP_SQRT1PM1: return sqrt1pm1<P>(a);
    default: return fastnormcdf<P>(a);
    }
}

template <class P, bool RARE>
__global__ void __launch_bounds__(128) k_interp(const DProgram prog, const DArgs args, int64_t n, int vec)
{
    uint32_t R[kMaxRegs][kV];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kV; base < n; base += stride * kV) {
        const int cnt = (int)((n - base) < kV ? (n - base) : kV);
        const bool full = vec && cnt == kV;
        for (int pc = 0; pc < prog.n; ++pc) {
            const DInstr in = prog.ins[pc];
            uint32_t *d = R[in.dst];
            const uint32_t *A = R[in.a], *B = R[in.b], *C = R[in.c];
            const bool f32 = in.dt == NT2G_F32;
            switch (in.op) {
            case NT2G_OP_LOAD:
                if (f32) {
                    const float *p = (const float *)args.ptr[in.a] + base;
                    if (full) {
                        float4 v = ld_stream((const float4 *)p);
                        d[0] = __float_as_uint(v.x); d[1] = __float_as_uint(v.y);
                        d[2] = __float_as_uint(v.z); d[3] = __float_as_uint(v.w);
                    } else {
#pragma unroll
                        for (int j = 0; j < kV; ++j) d[j] = j < cnt ? __float_as_uint(p[j]) : 0u;
                    }
                } else {
                    const uint8_t *p = (const uint8_t *)args.ptr[in.a] + base;
#pragma unroll
                    for (int j = 0; j < kV; ++j) d[j] = j < cnt ? p[j] : 0u;
                }
                break;
            case NT2G_OP_SCALAR:
#pragma unroll
                for (int j = 0; j < kV; ++j) d[j] = f32 ? __float_as_uint(args.scal[in.a]) : args.scal_u8[in.a];
                break;
            case NT2G_OP_CONST:
#pragma unroll
                for (int j = 0; j < kV; ++j) d[j] = f32 ? __float_as_uint(in.imm) : ((uint32_t)in.imm & 255u);
                break;
            case NT2G_OP_INDEX:  // enumerate<T>(p): float(p) rounds to nearest; uint8 wraps
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    const long long p = args.pos0 + base + j;
                    d[j] = f32 ? __float_as_uint(pos_to_float(p)) : (uint32_t)(p & 255);
                }
                break;
            case NT2G_OP_STORE:
                if (f32) {
                    float *p = (float *)args.ptr[in.b] + base;
                    float v[kV];
#pragma unroll
                    for (int j = 0; j < kV; ++j) v[j] = in.logical ? (float)A[j] : __uint_as_float(A[j]);
                    if (full) {
                        st_stream((float4 *)p, make_float4(v[0], v[1], v[2], v[3]));
                    } else {
#pragma unroll
                        for (int j = 0; j < kV; ++j)
                            if (j < cnt) p[j] = v[j];
                    }
                } else {
                    uint8_t *p = (uint8_t *)args.ptr[in.b] + base;
#pragma unroll
                    for (int j = 0; j < kV; ++j)
                        if (j < cnt) p[j] = (uint8_t)A[j];
                }
                break;
            case NT2G_OP_ADD: case NT2G_OP_SUB: case NT2G_OP_MUL: case NT2G_OP_DIV:
            case NT2G_OP_MIN: case NT2G_OP_MAX: case NT2G_OP_ADDS:
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    if (f32) {
                        float x = __uint_as_float(A[j]), y = __uint_as_float(B[j]), r;
                        switch (in.op) {
                        case NT2G_OP_ADD: r = P::add(x, y); break;
                        case NT2G_OP_SUB: r = P::sub(x, y); break;
                        case NT2G_OP_MUL: r = P::mul(x, y); break;
                        case NT2G_OP_DIV: r = P::div(x, y); break;
                        // boost/simd/arithmetic/functions/scalar/{min,max}.hpp
                        case NT2G_OP_MIN: r = (x < y) ? x : y; break;
                        default: r = (x > y) ? x : y; break;
                        }
                        d[j] = __float_as_uint(r);
                    } else {
                        uint32_t x = A[j], y = B[j], r;
                        switch (in.op) {
                        case NT2G_OP_ADD: r = (x + y) & 255u; break;
                        case NT2G_OP_SUB: r = (x - y) & 255u; break;
                        case NT2G_OP_MUL: r = (x * y) & 255u; break;
                        case NT2G_OP_MIN: r = x < y ? x : y; break;
                        case NT2G_OP_MAX: r = x > y ? x : y; break;
                        default: r = (x + y) > 255u ? 255u : (x + y); break;
                        }
                        d[j] = r;
                    }
                }
                break;
            case NT2G_OP_POW: case NT2G_OP_ATAN2: case NT2G_OP_HYPOT: case NT2G_OP_COPYSIGN: case NT2G_OP_MOD:
            case NT2G_OP_REM: case NT2G_OP_POW2:
                for (int j = 0; j < kV; ++j) {
                    const float x = __uint_as_float(A[j]), y = __uint_as_float(B[j]);
                    d[j] = __float_as_uint(in.op == NT2G_OP_POW     ? pow<P>(x, y)
                                           : in.op == NT2G_OP_ATAN2 ? atan2<P>(x, y)
                                           : in.op == NT2G_OP_HYPOT ? hypot<P>(x, y)
                                           : in.op == NT2G_OP_MOD   ? mod_<P>(x, y)
                                           : in.op == NT2G_OP_REM   ? rem_<P>(x, y)
                                           : in.op == NT2G_OP_POW2  ? pow2_<P>(x, y)
                                                                    : copysignf(x, y));
                }
                break;
            case NT2G_OP_NTHROOT: case NT2G_OP_EXPNI: case NT2G_OP_GAMMAINC: case NT2G_OP_GAMMAINCINV:
                for (int j = 0; j < kV; ++j) {
                    const float x = __uint_as_float(A[j]), y = __uint_as_float(B[j]);
                    float r = f_nan();
                    if constexpr (RARE)
                        r = in.op == NT2G_OP_NTHROOT ? nthroot<P>(x, int_operand(y))
                          : in.op == NT2G_OP_EXPNI   ? expni<P>(int_operand(x), y)
                          : in.op == NT2G_OP_GAMMAINC ? gammainc<P>(x, y)
                                                     : gammaincinv<P>(x, y);
                    d[j] = __float_as_uint(r);
                }
                break;
            case NT2G_OP_FMA: case NT2G_OP_FNMS:
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    float x = __uint_as_float(A[j]), y = __uint_as_float(B[j]), z = __uint_as_float(C[j]);
                    d[j] = __float_as_uint(in.op == NT2G_OP_FMA ? P::fma(x, y, z) : P::fma(-x, y, z));
                }
                break;
            case NT2G_OP_LT: case NT2G_OP_GT: case NT2G_OP_LE: case NT2G_OP_GE: case NT2G_OP_EQ:
            case NT2G_OP_NE:
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    bool r;
                    if (f32) {
                        float x = __uint_as_float(A[j]), y = __uint_as_float(B[j]);
                        r = in.op == NT2G_OP_LT ? x < y : in.op == NT2G_OP_GT ? x > y : in.op == NT2G_OP_LE ? x <= y
                          : in.op == NT2G_OP_GE ? x >= y : in.op == NT2G_OP_EQ ? x == y : x != y;
                    } else {
                        uint32_t x = A[j], y = B[j];
                        r = in.op == NT2G_OP_LT ? x < y : in.op == NT2G_OP_GT ? x > y : in.op == NT2G_OP_LE ? x <= y
                          : in.op == NT2G_OP_GE ? x >= y : in.op == NT2G_OP_EQ ? x == y : x != y;
                    }
                    d[j] = r ? 1u : 0u;
                }
                break;
            case NT2G_OP_IS_NAN: case NT2G_OP_IS_INF: case NT2G_OP_IS_FINITE: case NT2G_OP_IS_EQZ:
            case NT2G_OP_IS_NEZ: case NT2G_OP_IS_LTZ: case NT2G_OP_IS_GTZ:
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    const float x = __uint_as_float(A[j]);
                    const bool r = in.op == NT2G_OP_IS_NAN      ? x != x
                                 : in.op == NT2G_OP_IS_INF      ? fabsf(x) == f_inf()
                                 : in.op == NT2G_OP_IS_FINITE   ? (x - x) == 0.0f
                                 : in.op == NT2G_OP_IS_EQZ      ? x == 0.0f
                                 : in.op == NT2G_OP_IS_NEZ      ? x != 0.0f
                                 : in.op == NT2G_OP_IS_LTZ      ? x < 0.0f
                                                                : x > 0.0f;
                    d[j] = r ? 1u : 0u;
                }
                break;
            case NT2G_OP_IF_ELSE:
#pragma unroll
                for (int j = 0; j < kV; ++j) d[j] = A[j] ? B[j] : C[j];
                break;
            case NT2G_OP_SELINC: case NT2G_OP_SELDEC:
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    if (f32) {
                        float y = __uint_as_float(B[j]);
                        d[j] = __float_as_uint(A[j] ? P::add(y, in.op == NT2G_OP_SELINC ? 1.0f : -1.0f) : y);
                    } else {
                        d[j] = A[j] ? ((in.op == NT2G_OP_SELINC ? B[j] + 1u : B[j] - 1u) & 255u) : B[j];
                    }
                }
                break;
            case NT2G_OP_IF_ZERO_ELSE_ONE:
#pragma unroll
                for (int j = 0; j < kV; ++j) d[j] = f32 ? __float_as_uint(A[j] ? 0.0f : 1.0f) : (A[j] ? 0u : 1u);
                break;
            default:  // unary float functions
#pragma unroll
                for (int j = 0; j < kV; ++j) {
                    if (f32) d[j] = __float_as_uint(f_unary<P, RARE>(in.op, __uint_as_float(A[j])));
                    else d[j] = in.op == NT2G_OP_NEG ? ((0u - A[j]) & 255u)
                              : in.op == NT2G_OP_SQR ? ((A[j] * A[j]) & 255u) : A[j];  // ABS: identity
                }
                break;
            }
        }
    }
}

nt2g_status launch_interp(const DProgram &prog, const DArgs &args, int64_t count, int precision, cudaStream_t st)
{
    if (count == 0) return NT2G_OK;
    int vec = 1;
    for (int s = 0; s < kMaxSlots; ++s)
        if (args.ptr[s] && args.dtype[s] == NT2G_F32) vec &= aligned16(args.ptr[s]);
    int64_t units = (count + kV - 1) / kV;
    bool rare = false;
    for (int i = 0; i < prog.n; ++i) rare |= interp_rare_op(prog.ins[i].op);
#define NT2G_INTERP(PP, R)                                                                                      \
    k_interp<PP, R><<<persistent_blocks(k_interp<PP, R>, 128, 0, 128, units), 128, 0, st>>>(prog, args, count, vec)
    if (precision == NT2G_PREC_NT2) {
        if (rare) NT2G_INTERP(Nt2, true);
        else NT2G_INTERP(Nt2, false);
    } else {
        if (rare) NT2G_INTERP(Fast, true);
        else NT2G_INTERP(Fast, false);
    }
#undef NT2G_INTERP
    NT2G_LAUNCH_CHECK("interpreter launch");
    return NT2G_OK;
}

}  // namespace nt2g
