// bk_probe.cu -- one 1-D contraction y = D x of Q = 8 values per line (the BK5
// p = 7 derivative) in FP64 accuracy, by two arithmetic routes, so that the
// routes can be timed and counted against each other on the same data:
//
//   BK_PROBE_COPY  load, split into float-float, join, store (the part both
//                  routes share);
//   BK_PROBE_FF    the float-float route of the BK5 kernels: each double split
//                  into two floats, the even-odd contraction with Dot2-style
//                  accumulators on the FP32 pipes (eo_line, EngFF);
//   BK_PROBE_MMA   the tensor cores, by exact slices (the scheme of Ozaki,
//                  Ogita, Oishi, Rump, "Error-free transformations of matrix
//                  multiplication", Numer. Algorithms 2012, with the slices of
//                  Mukunoki et al.'s FP16 DGEMM emulation):
//                    - per line, the 53-bit mantissas of its 8 doubles are
//                      aligned to the line's largest exponent E (56 bits,
//                      V = |x| 2^(55-E) truncated), and V is cut into 7 bytes;
//                      the bytes, signed, are exact bf16 values (|b| <= 255);
//                    - D is cut the same way per row (exponent F_i) on the host;
//                    - the products of a byte of x and a byte of D are exact
//                      (16 bits), and all products of one level L = a + k
//                      (L = 0..6, 28 pairs) are summed by mma.sync
//                      m16n8k16.bf16 into FP32 accumulators: at most 7 pairs x 8
//                      terms x 255^2 < 2^22, so every level sum is an exact
//                      integer (16 MMAs per 16 lines x 8 outputs);
//                    - y = 2^(E + F_i - 14) sum_L 2^(-8 L) T_L, formed as a
//                      float-float pair (levels 0..2 by two TwoSums, which are
//                      exact; levels 3..6 by FMA into the low part, rounding at
//                      about 2^-46 of the leading level) and joined to a
//                      double.
//                  Levels L >= 7 and the mantissa bits below 2^(E-55) are
//                  dropped: relative to max|D||x| of the line, 2^-53 or less.
//
// The probe is a measurement entry point, not part of the operator path.
#include <cmath>
#include <cstdint>
#include <cstring>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "bk_gpu.h"
#include "bk_kernels.cuh"
#include "bk_probe.h"

namespace {

using namespace bkg;

constexpr int kQ = 8;
constexpr int kLevels = 7;   // bytes per aligned mantissa, and slice levels kept
constexpr int kThreads = 256;

struct ProbeFF {
    EOMat<ff, kQ> eo;
};

// Per thread of a warp (g = lane / 4, t = lane % 4): the B fragments of the
// 7 byte slices of D, b(a) = (d_a(g, 2t), d_a(g, 2t + 1)) as bf16 pairs, and
// the row exponents F_i.
struct ProbeMMA {
    uint32_t bfrag[kLevels][8][4];
    int F[kQ];
};

__global__ void __launch_bounds__(kThreads) probe_copy(long long nlines, const double* __restrict__ x,
                                                       double* __restrict__ y)
{
    for (long long l = blockIdx.x * (long long)kThreads + threadIdx.x; l < nlines; l += (long long)gridDim.x * kThreads) {
        const double2* xl = reinterpret_cast<const double2*>(x + l * kQ);
        double2* yl = reinterpret_cast<double2*>(y + l * kQ);
#pragma unroll
        for (int h = 0; h < kQ / 2; ++h) {
            const double2 v = xl[h];
            yl[h] = make_double2(join(split(v.x)), join(split(v.y)));
        }
    }
}

__global__ void __launch_bounds__(kThreads) probe_ff(const __grid_constant__ ProbeFF prm, long long nlines,
                                                     const double* __restrict__ x, double* __restrict__ y)
{
    for (long long l = blockIdx.x * (long long)kThreads + threadIdx.x; l < nlines; l += (long long)gridDim.x * kThreads) {
        const double2* xl = reinterpret_cast<const double2*>(x + l * kQ);
        double2* yl = reinterpret_cast<double2*>(y + l * kQ);
        ff a[kQ], b[kQ];
#pragma unroll
        for (int h = 0; h < kQ / 2; ++h) {
            const double2 v = xl[h];
            a[2 * h] = EngFF::load(v.x);
            a[2 * h + 1] = EngFF::load(v.y);
        }
        eo_line<EngFF, kQ>(a, b, prm.eo);
#pragma unroll
        for (int h = 0; h < kQ / 2; ++h) yl[h] = make_double2(EngFF::store(b[2 * h]), EngFF::store(b[2 * h + 1]));
    }
}

__device__ __forceinline__ int biased_exp(double v) { return (__double2hiint(v) >> 20) & 0x7FF; }

// The aligned mantissa of v for a line whose largest biased exponent is eb:
// V = |v| 2^(55 - E) truncated (56 bits at most), zero for zeros and
// subnormals.
__device__ __forceinline__ unsigned long long aligned_mantissa(double v, int eb)
{
    const int e = biased_exp(v);
    if (e == 0) return 0ull;
    const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(v));
    const unsigned long long m = (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const int sh = eb - e;
    return sh >= 64 ? 0ull : ((m << 3) >> sh);
}

// Byte k (0: the top) of a 56-bit aligned mantissa, signed, as an exact float.
__device__ __forceinline__ float mant_byte(unsigned long long V, int k, float sgn)
{
    const uint32_t b = static_cast<uint32_t>(V >> (48 - 8 * k)) & 0xFFu;
    return sgn * (__uint_as_float(0x4B000000u | b) - 8388608.0f);
}

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi)
{
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);   // lo -> low 16 bits
    return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// 2^k as a float (normal range only; outside it the probe's inputs do not go).
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

__device__ __forceinline__ float two_sum(float a, float b, float& err)
{
    const float s = a + b;
    const float bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}

// sum_L 2^(-8L) T_L scaled by 2^k, as a double: levels 0..2 by TwoSum
// (exact), levels 3..6 by FMA into the low part, then FastTwoSum and join.
__device__ __forceinline__ double recombine(const float (&T)[kLevels], int k)
{
    float e1, e2;
    const float s1 = two_sum(T[0], T[1] * 0.00390625f, e1);         // 2^-8
    const float s = two_sum(s1, T[2] * 1.52587890625e-05f, e2);     // 2^-16
    float e = e1 + e2;
    e = fmaf(T[3], 5.9604644775390625e-08f, e);                // 2^-24
    e = fmaf(T[4], 2.3283064365386963e-10f, e);                // 2^-32
    e = fmaf(T[5], 9.094947017729282e-13f, e);                 // 2^-40
    e = fmaf(T[6], 3.552713678800501e-15f, e);                 // 2^-48
    const float h = s + e;
    const float l = e - (h - s);
    const float sc = pow2f(k);
    return join(ff{h * sc, l * sc});
}

// One warp per 16 lines (grid-stride over groups): thread (g, t) holds the
// values n = 2t, 2t+1 of lines g and g + 8 -- exactly its A fragment -- and
// gets outputs i = 2t, 2t+1 of the same lines in its accumulators.
__global__ void __launch_bounds__(kThreads) probe_mma(const __grid_constant__ ProbeMMA prm, long long nlines,
                                                      const double* __restrict__ x, double* __restrict__ y)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    uint32_t B[kLevels];
#pragma unroll
    for (int a = 0; a < kLevels; ++a) B[a] = prm.bfrag[a][g][t];
    const int F0 = prm.F[2 * t], F1 = prm.F[2 * t + 1];
    const long long ngroups = nlines / 16;   // whole groups of 16 lines (the entry point checks)
    const long long warp = (blockIdx.x * (long long)kThreads + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * kThreads) >> 5;
    for (long long grp = warp; grp < ngroups; grp += nwarps) {
        const long long l0 = grp * 16 + g, l1 = l0 + 8;
        const double2 v0 = reinterpret_cast<const double2*>(x + l0 * kQ)[t];
        const double2 v1 = reinterpret_cast<const double2*>(x + l1 * kQ)[t];
        // largest biased exponent of each line (its 8 values over 4 threads)
        int e0 = max(biased_exp(v0.x), biased_exp(v0.y));
        int e1 = max(biased_exp(v1.x), biased_exp(v1.y));
        e0 = max(e0, __shfl_xor_sync(0xffffffffu, e0, 1));
        e0 = max(e0, __shfl_xor_sync(0xffffffffu, e0, 2));
        e1 = max(e1, __shfl_xor_sync(0xffffffffu, e1, 1));
        e1 = max(e1, __shfl_xor_sync(0xffffffffu, e1, 2));
        const unsigned long long m00 = aligned_mantissa(v0.x, e0), m01 = aligned_mantissa(v0.y, e0);
        const unsigned long long m10 = aligned_mantissa(v1.x, e1), m11 = aligned_mantissa(v1.y, e1);
        const float s00 = v0.x < 0 ? -1.f : 1.f, s01 = v0.y < 0 ? -1.f : 1.f;
        const float s10 = v1.x < 0 ? -1.f : 1.f, s11 = v1.y < 0 ? -1.f : 1.f;
        // A fragments per slice k: row g (a_lo) and row g + 8 (a_hi), columns 2t, 2t+1
        uint32_t Alo[kLevels], Ahi[kLevels];
#pragma unroll
        for (int k = 0; k < kLevels; ++k) {
            Alo[k] = bf16x2(mant_byte(m00, k, s00), mant_byte(m01, k, s01));
            Ahi[k] = bf16x2(mant_byte(m10, k, s10), mant_byte(m11, k, s11));
        }
        // level L = a + k: pairs (a, k), two per MMA (K = 16 = 2 x 8)
        float T[kLevels][4];
#pragma unroll
        for (int L = 0; L < kLevels; ++L) {
#pragma unroll
            for (int r = 0; r < 4; ++r) T[L][r] = 0.f;
#pragma unroll
            for (int a = 0; a <= L; a += 2) {
                const int k1 = L - a;
                if (a + 1 <= L) {
                    const int k2 = L - a - 1;
                    mma_bf16(T[L], Alo[k1], Ahi[k1], Alo[k2], Ahi[k2], B[a], B[a + 1]);
                } else {
                    mma_bf16(T[L], Alo[k1], Ahi[k1], 0u, 0u, B[a], 0u);
                }
            }
        }
        // outputs (line, i): c0 = (g, 2t), c1 = (g, 2t+1), c2 = (g+8, 2t), c3 = (g+8, 2t+1)
        double out[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float Tr[kLevels];
#pragma unroll
            for (int L = 0; L < kLevels; ++L) Tr[L] = T[L][r];
            const int eb = (r < 2) ? e0 : e1;
            const int F = (r & 1) ? F1 : F0;
            out[r] = recombine(Tr, (eb - 1023) + F - 14);
        }
        reinterpret_cast<double2*>(y + l0 * kQ)[t] = make_double2(out[0], out[1]);
        reinterpret_cast<double2*>(y + l1 * kQ)[t] = make_double2(out[2], out[3]);
    }
}

uint16_t bf16_bits_of_int(int v)
{
    // integers |v| <= 256 are exact in bf16: the top half of the float's bits
    const float f = static_cast<float>(v);
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return static_cast<uint16_t>(b >> 16);
}

// D(i, n) = D[i*8 + n]: its byte slices per row in the B fragment order.
bool make_mma_params(const double* D, ProbeMMA& P)
{
    int8_t sgn[kQ][kQ];
    int w[kLevels][kQ][kQ];
    for (int i = 0; i < kQ; ++i) {
        double big = 0;
        for (int n = 0; n < kQ; ++n) big = big > std::abs(D[i * kQ + n]) ? big : std::abs(D[i * kQ + n]);
        if (!(big > 0) || big > 1e30) return false;
        int ex = 0;
        std::frexp(big, &ex);      // big = f 2^ex, f in [0.5, 1): unbiased exponent ex - 1
        const int F = ex - 1;
        P.F[i] = F;
        for (int n = 0; n < kQ; ++n) {
            const double a = std::abs(D[i * kQ + n]);
            const unsigned long long W = static_cast<unsigned long long>(std::ldexp(a, 55 - F));   // truncates
            sgn[i][n] = D[i * kQ + n] < 0 ? -1 : 1;
            for (int k = 0; k < kLevels; ++k) w[k][i][n] = static_cast<int>((W >> (48 - 8 * k)) & 0xFFu);
        }
    }
    for (int a = 0; a < kLevels; ++a)
        for (int g = 0; g < 8; ++g)
            for (int t = 0; t < 4; ++t) {
                const uint32_t lo = bf16_bits_of_int(sgn[g][2 * t] * w[a][g][2 * t]);
                const uint32_t hi = bf16_bits_of_int(sgn[g][2 * t + 1] * w[a][g][2 * t + 1]);
                P.bfrag[a][g][t] = lo | (hi << 16);
            }
    return true;
}

int probe_grid(long long work, int sms)
{
    const long long g = (work + kThreads - 1) / kThreads;
    const long long cap = 8LL * sms;
    return int(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

extern "C" {

// method: BK_PROBE_COPY, BK_PROBE_FF or BK_PROBE_MMA; nlines lines of 8
// doubles (x, y device, 16-byte aligned; MMA: nlines a multiple of 16); D
// host, 8 x 8, D(i, n) = D[i*8 + n], centro-antisymmetric for BK_PROBE_FF.
int bk_probe_contract(int method, long long nlines, const double* D, const void* x, void* y, bk_stream_t stream)
{
    if (nlines < 0) return BK_ERR_SIZE;
    if (method < BK_PROBE_COPY || method > BK_PROBE_MMA) return BK_ERR_ARG;
    if (method == BK_PROBE_MMA && (nlines % 16) != 0) return BK_ERR_SIZE;
    if (nlines == 0) return BK_OK;
    if (!D || !x || !y) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) return BK_ERR_ALIGN;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const double* xd = static_cast<const double*>(x);
    double* yd = static_cast<double*>(y);
    if (method == BK_PROBE_COPY) {
        probe_copy<<<probe_grid(nlines, sms), kThreads, 0, s>>>(nlines, xd, yd);
    } else if (method == BK_PROBE_FF) {
        ProbeFF P;
        if (!make_eo<ff, kQ>(D, false, P.eo, &EngFF::coef)) return BK_ERR_ARG;
        probe_ff<<<probe_grid(nlines, sms), kThreads, 0, s>>>(P, nlines, xd, yd);
    } else {
        ProbeMMA P;
        if (!make_mma_params(D, P)) return BK_ERR_ARG;
        probe_mma<<<probe_grid(nlines * 2, sms), kThreads, 0, s>>>(P, nlines, xd, yd);
    }
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

}  // extern "C"
