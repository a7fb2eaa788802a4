// bkref_bk5.cpp -- C entry points over the reference's own BK5 kernel,
// bk::SumFactorization<T, nq> of openmp/BK5.cpp:19-103.  The kernel lives in
// the driver's .cpp, so that file is compiled here with its main renamed
// (oracle/Makefile, target ref).  The reference driver stops at p = 7; the
// template itself is instantiated here for p = 1..8 (nq = p + 1).
// Test infrastructure: generates the golden vectors the oracle is pinned to.
#define main bk5_reference_driver_main
#include "BK5.cpp"
#undef main

template <typename T>
static int run5(int p, std::size_t E, const T* dbasis, const T* G, const T* in, T* out)
{
    const bool ok = bk::with_order<1, 8>("polynomial order p", p, [&](auto P) {
        bk::SumFactorization<T, decltype(P)::value + 1>(E, dbasis, G, in, out);
    });
    return ok ? 0 : 1;
}

extern "C" int bkref_bk5_f64(int p, std::size_t E, const double* dbasis, const double* G,
                             const double* in, double* out)
{
    return run5<double>(p, E, dbasis, G, in, out);
}

extern "C" int bkref_bk5_f32(int p, std::size_t E, const float* dbasis, const float* G,
                             const float* in, float* out)
{
    return run5<float>(p, E, dbasis, G, in, out);
}
