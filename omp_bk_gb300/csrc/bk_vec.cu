// bk_vec.cu -- vector kernels around the operator: STREAM-style bandwidth
// kernels (the roofline denominators, with the operator's own read:write
// mixes), and the FP64 dot product / axpy of the solvers.
//
// STREAM: the reference measures its roof with roofline/stream_omp.cpp
// (copy, scale, add, triad, "read9" = 9 reads per write for BK3's mix,
// :32-120).  Here: copy, triad and "mix" with R input arrays read per array
// written (R = 7 is BK5's u + 6 G against v; R = 9 BK3's), 16-byte accesses,
// a grid of whole waves.
//
// Dot products are deterministic: a fixed grid writes one partial sum per
// block into caller-provided workspace, a second one-block kernel adds the
// partials in a fixed order.  Sums are carried in FP64 (the solvers' residual
// arithmetic); FP32 vectors are widened as they are read.
#include <cstdint>

#include <cuda_runtime.h>

#include "bk_ff.cuh"
#include "bk_gpu.h"
#include "bk_vec.h"

namespace {

constexpr int kDotBlocks = 1216;   // 8 per SM of a GB300; partials in the workspace
constexpr int kDotThreads = 256;

int waves(long long n16)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n16 + 511) / 512;
    const long long cap = 8LL * sms;
    return int(want < cap ? (want > 0 ? want : 1) : cap);
}

__global__ void copy_kernel(const float4* __restrict__ a, float4* __restrict__ b, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i];
}

__global__ void triad_kernel(float4* __restrict__ a, const float4* __restrict__ b, const float4* __restrict__ c,
                             long long n, float q)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 x = b[i], y = c[i];
        a[i] = make_float4(x.x + q * y.x, x.y + q * y.y, x.z + q * y.z, x.w + q * y.w);
    }
}

// out[i] = sum_r in[r * n + i]: R reads per write
__global__ void mix_kernel(const float4* __restrict__ in, float4* __restrict__ out, long long n, int R)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 s = in[i];
        for (int r = 1; r < R; ++r) {
            const float4 x = in[r * n + i];
            s.x += x.x;
            s.y += x.y;
            s.z += x.z;
            s.w += x.w;
        }
        out[i] = s;
    }
}

template <class T>
__device__ __forceinline__ double widen(T x) { return double(x); }

// one partial sum per block (fixed order within the block)
template <class T>
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(const T* __restrict__ x, const T* __restrict__ y,
                                                                  long long n, double* __restrict__ part)
{
    __shared__ double red[kDotThreads];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)kDotThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kDotThreads)
        s = fma(widen(x[i]), widen(y[i]), s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kDotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out = (sum of the nb partials) (op: 0 the sum, 1 half of it)
__global__ void __launch_bounds__(kDotThreads) dot_final_kernel(const double* __restrict__ part, int nb,
                                                                double* __restrict__ out, int half)
{
    __shared__ double red[kDotThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kDotThreads) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kDotThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = half ? 0.5 * red[0] : red[0];
}

template <class T>
__global__ void axpby_kernel(long long n, double a, const T* __restrict__ x, double b, T* __restrict__ y)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = T(a * double(x[i]) + b * double(y[i]));
}

// G (binary64) -> float-float pairs, value by value (in place allowed): the
// float-float engine's own split, so that an apply on the pairs is bitwise
// the apply on the doubles.
__global__ void g_to_ff_kernel(const double* G, bkg::ff2* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const bkg::ff v = bkg::split(G[i]);
        out[i] = bkg::ff2{v.hi, v.lo};
    }
}

// transpose_jxw on the device: one block per element (grid-stride), the
// element's JxW(p, q, r) staged in shared memory with coalesced loads,
// JxW_t(r, q, p) written with coalesced stores.
template <class T>
__global__ void transpose_jxw_kernel(const T* __restrict__ jxw, T* __restrict__ jt, long long E, int q)
{
    extern __shared__ __align__(16) unsigned char sm[];
    T* s = reinterpret_cast<T*>(sm);
    const int q2 = q * q, q3 = q2 * q;
    for (long long e = blockIdx.x; e < E; e += gridDim.x) {
        const T* src = jxw + e * q3;
        for (int x = threadIdx.x; x < q3; x += blockDim.x) s[x] = src[x];
        __syncthreads();
        T* dst = jt + e * q3;
        for (int y = threadIdx.x; y < q3; y += blockDim.x) {
            const int r = y / q2, qq = (y / q) % q, pp = y % q;   // y = (r, q, p)
            dst[y] = s[(pp * q + qq) * q + r];
        }
        __syncthreads();
    }
}

// make_bk5_G on the device: one block per element (grid-stride), the
// element's six interleaved factors G6i(i, j, s, k) staged in shared memory
// with coalesced loads, the F factors of the target layout written with
// coalesced stores.  Full tensor (F = 9, row-major): factor f = (a, b) is the
// stored symmetric factor of (min(a, b), max(a, b)).
template <class T>
__global__ void make_g_kernel(const T* __restrict__ g6i, T* __restrict__ g, long long E, int q, int F, int layout)
{
    extern __shared__ __align__(16) unsigned char sm[];
    T* s = reinterpret_cast<T*>(sm);
    const int q2 = q * q, q3 = q2 * q, n6 = 6 * q3, nf = F * q3;
    for (long long e = blockIdx.x; e < E; e += gridDim.x) {
        const T* src = g6i + e * n6;
        for (int x = threadIdx.x; x < n6; x += blockDim.x) s[x] = src[x];
        __syncthreads();
        T* dst = g + e * nf;
        for (int y = threadIdx.x; y < nf; y += blockDim.x) {
            int f, i, j, k;
            if (layout == 0) {   // (f, i, j, k)
                f = y / q3;
                const int r = y - f * q3;
                i = r / q2;
                j = (r - i * q2) / q;
                k = r - i * q2 - j * q;
            } else if (layout == 1) {   // (i, j, f, k)
                k = y % q;
                const int r = y / q;
                f = r % F;
                j = (r / F) % q;
                i = r / (F * q);
            } else {   // (f, k, i, j)
                j = y % q;
                i = (y / q) % q;
                k = (y / q2) % q;
                f = y / q3;
            }
            int sf = f;
            if (F == 9) {
                const int a = f / 3, b = f - 3 * (f / 3);
                const int lo = a < b ? a : b, hi = a < b ? b : a;
                sf = (lo == 0) ? hi : (lo == 1 ? hi + 2 : 5);
            }
            dst[y] = s[((i * q + j) * 6 + sf) * q + k];
        }
        __syncthreads();
    }
}

int ok() { return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA; }

int dot_blocks(long long n)
{
    const long long want = (n + kDotThreads - 1) / kDotThreads;
    return int(want < kDotBlocks ? (want > 0 ? want : 1) : kDotBlocks);
}

}  // namespace

extern "C" {

int bk_stream_kernel(int kind, long long n_bytes, void* a, const void* b, const void* c, int reads,
                     bk_stream_t stream)
{
    if (n_bytes <= 0 || (n_bytes & 15)) return BK_ERR_SIZE;
    if (!a || !b) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c)) & 15)
        return BK_ERR_ALIGN;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = n_bytes / 16;
    const int g = waves(n);
    switch (kind) {
        case BK_STREAM_COPY:
            copy_kernel<<<g, 512, 0, s>>>(static_cast<const float4*>(b), static_cast<float4*>(a), n);
            return ok();
        case BK_STREAM_TRIAD:
            if (!c) return BK_ERR_NULL;
            triad_kernel<<<g, 512, 0, s>>>(static_cast<float4*>(a), static_cast<const float4*>(b),
                                           static_cast<const float4*>(c), n, 3.0f);
            return ok();
        case BK_STREAM_MIX:
            if (reads < 1 || reads > 64) return BK_ERR_ARG;
            mix_kernel<<<g, 512, 0, s>>>(static_cast<const float4*>(b), static_cast<float4*>(a), n, reads);
            return ok();
        default:
            return BK_ERR_ARG;
    }
}

long long bk_dot_workspace_bytes(long long n) { return (long long)dot_blocks(n) * (long long)sizeof(double); }

int bk_dot(long long n, const void* x, const void* y, int f64, double* result, void* workspace,
           long long workspace_bytes, int half, bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (!result || !workspace) return BK_ERR_NULL;
    if (n > 0 && (!x || !y)) return BK_ERR_NULL;
    const int nb = dot_blocks(n);
    if (workspace_bytes < (long long)nb * (long long)sizeof(double)) return BK_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double* part = static_cast<double*>(workspace);
    if (f64)
        dot_partial_kernel<double><<<nb, kDotThreads, 0, s>>>(static_cast<const double*>(x),
                                                              static_cast<const double*>(y), n, part);
    else
        dot_partial_kernel<float><<<nb, kDotThreads, 0, s>>>(static_cast<const float*>(x),
                                                             static_cast<const float*>(y), n, part);
    dot_final_kernel<<<1, kDotThreads, 0, s>>>(part, nb, result, half);
    return ok();
}

int bk_axpby(long long n, double a, const void* x, double b, void* y, int f64, bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (n == 0) return BK_OK;
    if (!x || !y) return BK_ERR_NULL;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int g = waves(n / 2 + 1);
    if (f64)
        axpby_kernel<double><<<g, 256, 0, s>>>(n, a, static_cast<const double*>(x), b, static_cast<double*>(y));
    else
        axpby_kernel<float><<<g, 256, 0, s>>>(n, a, static_cast<const float*>(x), b, static_cast<float*>(y));
    return ok();
}

int bk5_make_g(int p, int64_t E, const void* G6i, void* G, int nfactors, int layout, int prec, bk_stream_t stream)
{
    if (p < 1 || p > 8) return BK_ERR_ORDER;
    if (E < 0) return BK_ERR_SIZE;
    if ((nfactors != 6 && nfactors != 9) || layout < 0 || layout > 2) return BK_ERR_PREC;
    if (prec != BK_PREC_FP64 && prec != BK_PREC_FP32 && prec != BK_PREC_MIXED) return BK_ERR_PREC;
    if (E == 0) return BK_OK;
    if (!G6i || !G) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(G6i) | reinterpret_cast<uintptr_t>(G)) & 15) return BK_ERR_ALIGN;
    const int q = p + 1;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cap = 8LL * sms;
    const int grid = int(E < cap ? E : cap);
    if (prec == BK_PREC_FP64)
        make_g_kernel<double><<<grid, 256, 6 * q * q * q * sizeof(double), s>>>(
            static_cast<const double*>(G6i), static_cast<double*>(G), E, q, nfactors, layout);
    else
        make_g_kernel<float><<<grid, 256, 6 * q * q * q * sizeof(float), s>>>(
            static_cast<const float*>(G6i), static_cast<float*>(G), E, q, nfactors, layout);
    return ok();
}

int bk1_transpose_jxw(int p, int64_t E, const void* jxw, void* jxw_t, int prec, bk_stream_t stream)
{
    if (p < 1 || p > 8) return BK_ERR_ORDER;
    if (E < 0) return BK_ERR_SIZE;
    if (prec != BK_PREC_FP64 && prec != BK_PREC_FP32 && prec != BK_PREC_MIXED) return BK_ERR_PREC;
    if (E == 0) return BK_OK;
    if (!jxw || !jxw_t) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(jxw) | reinterpret_cast<uintptr_t>(jxw_t)) & 15) return BK_ERR_ALIGN;
    if (jxw == jxw_t) return BK_ERR_ARG;
    const int q = p + 2;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cap = 8LL * sms;
    const int grid = int(E < cap ? E : cap);
    if (prec == BK_PREC_FP64)
        transpose_jxw_kernel<double><<<grid, 256, q * q * q * sizeof(double), s>>>(
            static_cast<const double*>(jxw), static_cast<double*>(jxw_t), E, q);
    else
        transpose_jxw_kernel<float><<<grid, 256, q * q * q * sizeof(float), s>>>(
            static_cast<const float*>(jxw), static_cast<float*>(jxw_t), E, q);
    return ok();
}

int bk_g_to_ff(const void* G, void* Gff, int64_t n, bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (n == 0) return BK_OK;
    if (!G || !Gff) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(Gff)) & 15) return BK_ERR_ALIGN;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    g_to_ff_kernel<<<waves(n / 2 + 1), 256, 0, s>>>(static_cast<const double*>(G), static_cast<bkg::ff2*>(Gff), n);
    return ok();
}

}  // extern "C"
