// bkref_harness.cpp -- C entry points over the reference's host harness,
// include/bk_harness.h (FP64 references, layouts) and include/bk_common.h
// (test data, norm), compiled from the reference's sources by include path
// (oracle/Makefile, target ref).  Test infrastructure only.
#include <cstddef>
#include <cstdint>
#include <vector>
#include "bk_common.h"
#include "bk_harness.h"

namespace {
std::vector<float> vf(const float* p, std::size_t n) { return std::vector<float>(p, p + n); }
}

extern "C" void bkref_reference_bk1(int nq, std::size_t E, const float* basis, const float* jxw,
                                    const float* in, double* out)
{
    const int nm = nq - 1;
    std::vector<double> o(E * nm * nm * nm);
    bk::reference_bk1(nq, E, vf(basis, nm * nq), vf(jxw, E * nq * nq * nq), vf(in, E * nm * nm * nm), o);
    for (std::size_t i = 0; i < o.size(); ++i) out[i] = o[i];
}

extern "C" void bkref_reference_bk3(int nq, std::size_t E, const float* basis, const float* D,
                                    const float* G, const float* in, double* out)
{
    const int nm = nq - 1;
    std::vector<double> o(E * nm * nm * nm);
    bk::reference_bk3(nq, E, vf(basis, nm * nq), vf(D, nq * nq), vf(G, E * 6 * nq * nq * nq),
                      vf(in, E * nm * nm * nm), o);
    for (std::size_t i = 0; i < o.size(); ++i) out[i] = o[i];
}

extern "C" void bkref_reference_bk5(int nq, std::size_t E, const float* D, const float* G6i,
                                    const float* in, double* out)
{
    const std::size_t nq3 = std::size_t(nq) * nq * nq;
    std::vector<double> o(E * nq3);
    bk::reference_bk5(nq, E, vf(D, nq * nq), vf(G6i, E * 6 * nq3), vf(in, E * nq3), o);
    for (std::size_t i = 0; i < o.size(); ++i) out[i] = o[i];
}

extern "C" void bkref_make_bk5_G(const float* G6i, std::size_t E, int nq, int F, int layout, float* G)
{
    const std::size_t nq3 = std::size_t(nq) * nq * nq;
    const std::vector<float> g = bk::make_bk5_G(vf(G6i, E * 6 * nq3), E, nq, F, layout);
    for (std::size_t i = 0; i < g.size(); ++i) G[i] = g[i];
}

extern "C" void bkref_transpose_jxw(const float* jxw, std::size_t E, int nq, float* out)
{
    const std::size_t nq3 = std::size_t(nq) * nq * nq;
    const std::vector<float> t = bk::transpose_jxw(vf(jxw, E * nq3), E, nq);
    for (std::size_t i = 0; i < t.size(); ++i) out[i] = t[i];
}

extern "C" void bkref_fill_random_f64(double* in, std::size_t nin, double* jxw, std::size_t njxw,
                                      uint32_t seed)
{
    std::vector<double> a(nin), b(njxw);
    bk::fill_random_test_data(a, b, seed);
    for (std::size_t i = 0; i < nin; ++i) in[i] = a[i];
    for (std::size_t i = 0; i < njxw; ++i) jxw[i] = b[i];
}

extern "C" void bkref_make_test_basis_f64(int rows, int cols, double* m)
{
    const std::vector<double> b = bk::make_test_basis<double>(rows, cols);
    for (std::size_t i = 0; i < b.size(); ++i) m[i] = b[i];
}

extern "C" void bkref_make_test_basis_f32(int rows, int cols, float* m)
{
    const std::vector<float> b = bk::make_test_basis<float>(rows, cols);
    for (std::size_t i = 0; i < b.size(); ++i) m[i] = b[i];
}

extern "C" double bkref_norm2_f64(const double* v, std::size_t n) { return bk::norm2(v, n); }
extern "C" double bkref_norm2_f32(const float* v, std::size_t n) { return bk::norm2(v, n); }
