// bk_engine.cuh -- the arithmetic "engines" of the operator kernels.
//
// Every kernel is written once over an engine that fixes
//   S  the storage type in HBM (double or float),
//   V  the working type in shared memory and registers,
//   C  the type of the 1-D matrix coefficients (kernel parameters),
//   A  the accumulator of a contraction,
// and the operations on them.  Engines:
//   EngDfma   FP64 storage, native FP64 FMA (1/64 of the FP32 rate on GB300);
//   EngFF     FP64 storage, float-float arithmetic on the FP32 pipes;
//   EngF32    FP32 storage and FMA: the reference drivers' T = float;
//   EngMixed  FP32 storage and FMA, with the final sum of the three
//             directional terms of BK3/BK5 compensated (TwoSum).
#pragma once

#include "bk_ff.cuh"

namespace bkg {

struct EngDfma {
    using S = double;
    using V = double;
    using C = double;
    using A = double;
    static constexpr int kId = BK_ENGINE_DFMA;
    __device__ static __forceinline__ V load(S x) { return x; }
    __device__ static __forceinline__ S store(V x) { return x; }
    __device__ static __forceinline__ A zero() { return 0.0; }
    // an accumulator started with a first product / value (no add to zero)
    __device__ static __forceinline__ A first(C c, V x) { return c * x; }
    __device__ static __forceinline__ A vfirst(V a, V x) { return a * x; }
    __device__ static __forceinline__ A from(V x) { return x; }
    __device__ static __forceinline__ void madd(A& acc, C c, V x) { acc = fma(c, x, acc); }
    __device__ static __forceinline__ void vmadd(A& acc, V a, V x) { acc = fma(a, x, acc); }
    __device__ static __forceinline__ void add(A& acc, V x) { acc += x; }
    __device__ static __forceinline__ V result(A acc) { return acc; }
    __device__ static __forceinline__ V loose(A acc) { return acc; }
    __device__ static __forceinline__ V mul(V a, V b) { return a * b; }
    __device__ static __forceinline__ V vadd(V a, V b) { return a + b; }
    __device__ static __forceinline__ V vsub(V a, V b) { return a - b; }
    __device__ static __forceinline__ V vadd_in(V a, V b) { return a + b; }
    __device__ static __forceinline__ V vsub_in(V a, V b) { return a - b; }
    __device__ static __forceinline__ void sum_diff(const A& a, const A& b, V& s, V& d)
    {
        s = a + b;
        d = b - a;
    }
    __device__ static __forceinline__ void sum_diff_loose(const A& a, const A& b, V& s, V& d) { sum_diff(a, b, s, d); }
    static C coef(double d) { return d; }
};

struct EngFF {
    using S = double;
    using V = ff;
    using C = ff;
    using A = ffacc;
    static constexpr int kId = BK_ENGINE_FF;
    __device__ static __forceinline__ V load(S x) { return split(x); }
    // a value split ahead of time (bk_g_to_ff): no work
    __device__ static __forceinline__ V load(ff2 x) { return ff{x.hi, x.lo}; }
    __device__ static __forceinline__ S store(V x) { return join(x); }
    __device__ static __forceinline__ A zero() { return acc_zero(); }
    // the first product needs no TwoSum into an empty accumulator
    __device__ static __forceinline__ A first(C c, V x) { return acc_first(c, x); }
    __device__ static __forceinline__ A vfirst(V a, V x) { return acc_first(a, x); }
    __device__ static __forceinline__ A from(V x) { return ffacc{x.hi, x.lo}; }
    __device__ static __forceinline__ void madd(A& acc, C c, V x) { acc_madd(acc, c, x); }
    __device__ static __forceinline__ void vmadd(A& acc, V a, V x) { acc_madd(acc, a, x); }
    __device__ static __forceinline__ void add(A& acc, V x) { acc_add(acc, x); }
    __device__ static __forceinline__ V result(A acc) { return acc_result(acc); }
    // for values that are only summed or stored next: not renormalised
    __device__ static __forceinline__ V loose(A acc) { return acc_loose(acc); }
    __device__ static __forceinline__ V mul(V a, V b) { return ff_mul(a, b); }
    __device__ static __forceinline__ V vadd(V a, V b) { return ff_add(a, b); }
    __device__ static __forceinline__ V vsub(V a, V b) { return ff_add(a, ff{-b.hi, -b.lo}); }
    // operands of multiply-adds only: not renormalised
    __device__ static __forceinline__ V vadd_in(V a, V b) { return ff_add_loose(a, b); }
    __device__ static __forceinline__ V vsub_in(V a, V b) { return ff_add_loose(a, ff{-b.hi, -b.lo}); }
    // a + b and b - a of two accumulators
    __device__ static __forceinline__ void sum_diff(const A& a, const A& b, V& s, V& d) { acc_sum_diff(a, b, s, d); }
    // the same as unevaluated pairs, for outputs that are only summed next
    __device__ static __forceinline__ void sum_diff_loose(const A& a, const A& b, V& s, V& d)
    {
        acc_sum_diff_loose(a, b, s, d);
    }
    static C coef(double d)
    {
        C c;
        c.hi = static_cast<float>(d);
        c.lo = static_cast<float>(d - static_cast<double>(c.hi));
        return c;
    }
};

struct EngF32 {
    using S = float;
    using V = float;
    using C = float;
    using A = float;
    static constexpr int kId = 100;
    __device__ static __forceinline__ V load(S x) { return x; }
    __device__ static __forceinline__ S store(V x) { return x; }
    __device__ static __forceinline__ A zero() { return 0.0f; }
    __device__ static __forceinline__ A first(C c, V x) { return c * x; }
    __device__ static __forceinline__ A vfirst(V a, V x) { return a * x; }
    __device__ static __forceinline__ A from(V x) { return x; }
    __device__ static __forceinline__ void madd(A& acc, C c, V x) { acc = fmaf(c, x, acc); }
    __device__ static __forceinline__ void vmadd(A& acc, V a, V x) { acc = fmaf(a, x, acc); }
    __device__ static __forceinline__ void add(A& acc, V x) { acc += x; }
    __device__ static __forceinline__ V result(A acc) { return acc; }
    __device__ static __forceinline__ V loose(A acc) { return acc; }
    __device__ static __forceinline__ V mul(V a, V b) { return a * b; }
    __device__ static __forceinline__ V vadd(V a, V b) { return a + b; }
    __device__ static __forceinline__ V vsub(V a, V b) { return a - b; }
    __device__ static __forceinline__ V vadd_in(V a, V b) { return a + b; }
    __device__ static __forceinline__ V vsub_in(V a, V b) { return a - b; }
    __device__ static __forceinline__ void sum_diff(const A& a, const A& b, V& s, V& d)
    {
        s = a + b;
        d = b - a;
    }
    __device__ static __forceinline__ void sum_diff_loose(const A& a, const A& b, V& s, V& d) { sum_diff(a, b, s, d); }
    static C coef(double d) { return static_cast<float>(d); }
};

// Plain FP32 everywhere except the final combination of the three directional
// terms, which is summed with TwoSum and rounded once.
struct EngMixed : EngF32 {
    static constexpr int kId = 101;
    __device__ static __forceinline__ float sum3(float a, float b, float c)
    {
        float s, e, s2, e2;
        two_sum(a, b, s, e);
        two_sum(s, c, s2, e2);
        return __fadd_rn(s2, __fadd_rn(e, e2));
    }
};

template <class Eng>
struct HasSum3 {
    static constexpr bool value = false;
};
template <>
struct HasSum3<EngMixed> {
    static constexpr bool value = true;
};

}  // namespace bkg
