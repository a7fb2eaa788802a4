// bkref_bk3.cpp -- C entry points over the reference's own BK3 kernel,
// bk::SumFactorization<T, nq> of openmp/bk3_sumfact.h:18-187, compiled from
// the reference's sources by include path (oracle/Makefile, target ref).
// Test infrastructure: generates the golden vectors the oracle is pinned to.
#include <cstddef>
#include "bk_common.h"
#include "bk3_sumfact.h"

template <typename T>
static int run(int p, std::size_t E, const T* basis, const T* dbasis, const T* G, const T* in, T* out)
{
    const bool ok = bk::with_order<1, 8>("polynomial order p", p, [&](auto P) {
        bk::SumFactorization<T, decltype(P)::value + 2>(E, basis, dbasis, G, in, out);
    });
    return ok ? 0 : 1;
}

extern "C" int bkref_bk3_f64(int p, std::size_t E, const double* basis, const double* dbasis,
                             const double* G, const double* in, double* out)
{
    return run<double>(p, E, basis, dbasis, G, in, out);
}

extern "C" int bkref_bk3_f32(int p, std::size_t E, const float* basis, const float* dbasis,
                             const float* G, const float* in, float* out)
{
    return run<float>(p, E, basis, dbasis, G, in, out);
}
