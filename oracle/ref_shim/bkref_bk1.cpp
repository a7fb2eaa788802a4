// bkref_bk1.cpp -- C entry points over the reference's own BK1 kernel,
// bk::SumFactorization<T, nq> of openmp/bk1_sumfact.h:17-159, compiled from
// the reference's sources by include path (oracle/Makefile, target ref).
// Test infrastructure: generates the golden vectors the oracle is pinned to.
#include <cstddef>
#include "bk_common.h"
#include "bk1_sumfact.h"

template <typename T>
static int run(int p, std::size_t E, const T* basis, const T* jxw, const T* in, T* out)
{
    const bool ok = bk::with_order<1, 8>("polynomial order p", p, [&](auto P) {
        bk::SumFactorization<T, decltype(P)::value + 2>(E, basis, jxw, in, out);
    });
    return ok ? 0 : 1;
}

extern "C" int bkref_bk1_f64(int p, std::size_t E, const double* basis, const double* jxw,
                             const double* in, double* out)
{
    return run<double>(p, E, basis, jxw, in, out);
}

extern "C" int bkref_bk1_f32(int p, std::size_t E, const float* basis, const float* jxw,
                             const float* in, float* out)
{
    return run<float>(p, E, basis, jxw, in, out);
}
