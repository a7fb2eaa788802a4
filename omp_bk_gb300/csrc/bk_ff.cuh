// bk_ff.cuh -- float-float ("double-float") arithmetic on the FP32 pipes.
//
// The GB300's FP64 pipe runs at 1/64 of the FP32 rate (measured: 0.5 T DFMA/s
// against 34 T FFMA/s), so an FP64-accurate operator apply that must keep up
// with HBM cannot use native DFMA.  A value is carried as the unevaluated sum
// hi + lo of two floats (about 48 significant bits, float's exponent range).
// This is the technique of the reference's openmp/float_float.h (used by
// openmp/BK1_ff.cpp); the code below is written from the published
// error-free transformations:
//   TwoSum      Knuth, TAOCP vol. 2 (6 flops, no ordering condition);
//   FastTwoSum  Dekker 1971 (3 flops, |a| >= |b|);
//   TwoProd     via FMA: p = fl(a*b), e = fma(a, b, -p) exact.
// Dot products use the compensated scheme of Ogita, Rump and Oishi
// ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005: Dot2),
// extended with the cross terms of the lo parts: the hi sum is carried with
// TwoSum, all error terms in one FP32 accumulator, and the pair is
// renormalised once at the end (12 flops per term instead of 15 for a
// renormalising multiply-add).
//
// Conversions never touch the FP64 pipe on the fast path: split() cuts the
// binary64 bit pattern into a truncated 24-bit hi and the remaining 29
// mantissa bits (rounded to a float) with integer operations and one I2F;
// join() adds the lo part to the bit pattern of hi as a count of double ulps.
// Values outside [2^-74, 2^128) (split) or [2^-74, 2^127) (join) take a slow
// path through the FP64 pipe.
//
// Every operation uses the __f*_rn intrinsics, which the compiler never
// contracts into FMAs: the transformations need IEEE round-to-nearest.
#pragma once

#include <cstdint>

namespace bkg {

struct ff {
    float hi;
    float lo;
};

__device__ __forceinline__ ff ff_make(float hi, float lo) { return ff{hi, lo}; }

// A float-float value stored in memory (8 bytes, 8-byte aligned so that it
// moves as one 64-bit access): the form of a geometric-factor array that has
// been split once ahead of the applies (bk_g_to_ff), in place of the split of
// every binary64 value as it is loaded.
struct alignas(8) ff2 {
    float hi;
    float lo;
};

// s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e == a + b exactly when |a| >= |b| (Dekker's FastTwoSum).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// Compensated accumulator of a dot product: the value is s + c.
struct ffacc {
    float s;
    float c;
};

__device__ __forceinline__ ffacc acc_zero() { return ffacc{0.0f, 0.0f}; }

// acc += a * x, a and x float-float.
__device__ __forceinline__ void acc_madd(ffacc& acc, const ff a, const ff x)
{
    const float p = __fmul_rn(a.hi, x.hi);
    float pe = __fmaf_rn(a.hi, x.hi, -p);          // exact error of the hi product
    pe = __fmaf_rn(a.hi, x.lo, pe);                // cross terms (lo*lo dropped)
    pe = __fmaf_rn(a.lo, x.hi, pe);
    float s, e;
    two_sum(acc.s, p, s, e);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, pe));
}

// The accumulator holding a * x alone: the product as p + pe (no TwoSum
// into zero).
__device__ __forceinline__ ffacc acc_first(const ff a, const ff x)
{
    const float p = __fmul_rn(a.hi, x.hi);
    float pe = __fmaf_rn(a.hi, x.hi, -p);
    pe = __fmaf_rn(a.hi, x.lo, pe);
    pe = __fmaf_rn(a.lo, x.hi, pe);
    return ffacc{p, pe};
}

// acc += x (float-float).
__device__ __forceinline__ void acc_add(ffacc& acc, const ff x)
{
    float s, e;
    two_sum(acc.s, x.hi, s, e);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, x.lo));
}

// acc += a * x, a and x plain floats (the product is exact as p + pe).
__device__ __forceinline__ void acc_madd_f(ffacc& acc, const float a, const float x)
{
    const float p = __fmul_rn(a, x);
    const float pe = __fmaf_rn(a, x, -p);
    float s, e;
    two_sum(acc.s, p, s, e);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, pe));
}

// The accumulated value as a normalised pair (|lo| <= ulp(hi)/2); TwoSum
// because after cancellation |c| may exceed |s|.
__device__ __forceinline__ ff acc_result(const ffacc& acc)
{
    ff r;
    two_sum(acc.s, acc.c, r.hi, r.lo);
    return r;
}

// a * b, both float-float (the lo*lo term dropped), as the unevaluated pair
// p + pe (p the rounded hi product, pe its exact error plus the cross
// terms), not renormalised: every consumer (multiply-adds, accumulators,
// join) takes hi and lo separately.
__device__ __forceinline__ ff ff_mul(const ff a, const ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float pe = __fmaf_rn(a.hi, b.hi, -p);
    pe = __fmaf_rn(a.hi, b.lo, pe);
    pe = __fmaf_rn(a.lo, b.hi, pe);
    return ff{p, pe};
}

// The accumulated value as the unevaluated pair s + c, not renormalised
// (after cancellation |c| may exceed |s|).  Only for values that are summed
// or stored next, never multiplied: the FP32 rounding of a product with a
// loose pair's lo part is an error relative to the magnitudes summed before
// the cancellation (measured: 5e-12 relative on a strongly cancelling BK1
// result), where a renormalised pair keeps 2^-48 of the value itself.
// join() renormalises with TwoSum.
__device__ __forceinline__ ff acc_loose(const ffacc& acc) { return ff{acc.s, acc.c}; }

// a + b without the final renormalisation: hi = fl(a.hi + b.hi) and lo the
// exact error of that sum plus the lo parts, so |lo| may reach a few ulp(hi).
// For operands of multiply-adds, which use hi and lo separately (the sweeps'
// even and odd combinations): 8 flops instead of 11.
__device__ __forceinline__ ff ff_add_loose(const ff a, const ff b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return ff{s, __fadd_rn(e, __fadd_rn(a.lo, b.lo))};
}

// a + b and b - a from two compensated accumulators, each renormalised once
// with TwoSum (safe after cancellation, where the compensation may exceed
// the sum) instead of normalising a and b first and then adding them: 28
// flops for the pair instead of 34.  The results feed further products, so
// they are renormalised (see acc_loose).
__device__ __forceinline__ void acc_sum_diff(const ffacc& a, const ffacc& b, ff& sum, ff& diff)
{
    float s, e, t, f;
    two_sum(a.s, b.s, s, e);
    two_sum(b.s, -a.s, t, f);
    const float cs = __fadd_rn(e, __fadd_rn(a.c, b.c));
    const float cd = __fadd_rn(f, __fsub_rn(b.c, a.c));
    two_sum(s, cs, sum.hi, sum.lo);
    two_sum(t, cd, diff.hi, diff.lo);
}

// a + b and b - a from two compensated accumulators as unevaluated pairs,
// not renormalised (16 flops for the pair instead of 28): for values that
// are only summed or stored next, never multiplied (see acc_loose).
__device__ __forceinline__ void acc_sum_diff_loose(const ffacc& a, const ffacc& b, ff& sum, ff& diff)
{
    float e, f;
    two_sum(a.s, b.s, sum.hi, e);
    two_sum(b.s, -a.s, diff.hi, f);
    sum.lo = __fadd_rn(e, __fadd_rn(a.c, b.c));
    diff.lo = __fadd_rn(f, __fsub_rn(b.c, a.c));
}

// a + b, both float-float, normalised (TwoSum of the hi parts, lo parts added).
__device__ __forceinline__ ff ff_add(const ff a, const ff b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    ff r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}

// ---- binary64 <-> float-float ------------------------------------------------

// The rare out-of-range cases, out of line: kept off the fast path so that
// the compiler cannot predicate their FP64-pipe instructions into it.
static __device__ __noinline__ ff split_slow(const double x)
{
    ff r;
    r.hi = __double2float_rz(x);
    r.lo = __double2float_rn(x - static_cast<double>(r.hi));
    return r;
}

static __device__ __noinline__ double join_slow(const float s, const float t)
{
    return static_cast<double>(s) + static_cast<double>(t);
}

// Split x into hi (x truncated to 24 significant bits) and lo (the remaining
// 29 mantissa bits rounded to a float).  Fast path for biased exponents
// 949..1150 (2^-74 <= |x| < 2^128): pure integer work plus one I2F and one
// FMUL.
__device__ __forceinline__ ff split(const double x)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t whi = static_cast<uint32_t>(b >> 32);
    const uint32_t wlo = static_cast<uint32_t>(b);
    const uint32_t e = (whi >> 20) & 0x7ffu;
    const uint32_t sign = whi & 0x80000000u;
    ff r;
    if (e - 949u <= 1150u - 949u) {
        // bits 60..29 of x: the low 9 exponent bits and the top 23 mantissa
        // bits; rebias the exponent by 896 (mod 2^9 it is exact here).
        const uint32_t w = __funnelshift_r(wlo, whi, 29);
        r.hi = __uint_as_float(((w - 0xC0000000u) & 0x7fffffffu) | sign);
        // x - hi = +-(low 29 mantissa bits) * 2^(e - 1075)
        const float scale = __uint_as_float(((e - 948u) << 23) | sign);
        r.lo = __fmul_rn(__uint2float_rn(wlo & 0x1fffffffu), scale);
    } else {
        r = split_slow(x);
    }
    return r;
}

// hi + lo rounded to the nearest double.  The pair is first renormalised
// with TwoSum (it may be loose: |lo| > |hi| after cancellation).  Fast path:
// the normalised hi has a biased float exponent 53..254; lo becomes an
// integer count k of double ulps of hi (|k| <= 2^28) added to hi's binary64
// pattern.  When hi is a power of two and lo points below it, the sum lies in
// the binade below, whose ulp is half as large.
__device__ __forceinline__ double join(const ff v)
{
    float s, t;
    two_sum(v.hi, v.lo, s, t);
    const uint32_t sb = __float_as_uint(s);
    const uint32_t e8 = (sb >> 23) & 0xffu;
    if (e8 - 53u <= 254u - 53u) {
        const uint32_t tb = __float_as_uint(t);
        const uint32_t down = ((sb & 0x7fffffu) == 0u && ((tb ^ sb) & 0x80000000u) != 0u && (tb & 0x7fffffffu) != 0u)
                                  ? 1u
                                  : 0u;
        // 2^(52 - E + down), E = e8 - 127
        const float scale = __uint_as_float((306u - e8 + down) << 23);
        int k = __float2int_rn(__fmul_rn(t, scale));
        if (sb & 0x80000000u) {
            k = -k;
        }
        const uint32_t dhi = (sb & 0x80000000u) | ((e8 + 896u) << 20) | ((sb >> 3) & 0xfffffu);
        const uint32_t dlo = sb << 29;
        const unsigned long long bits = ((static_cast<unsigned long long>(dhi) << 32) | dlo) +
                                        static_cast<unsigned long long>(static_cast<long long>(k));
        return __longlong_as_double(static_cast<long long>(bits));
    }
    return join_slow(s, t);
}

}  // namespace bkg
