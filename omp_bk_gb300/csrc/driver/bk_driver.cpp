// bk_driver.cpp -- the reference drivers' command line on the GB300 kernels.
//
//   bk_cuda BK1|BK3|BK5 <p> [nelmt] [ntests]
//   bk_cuda BK1_ff <p> [nelmt] [ntests]      (openmp/BK1_ff.cpp: run_bk1_ff)
//
// Keeps the surface of openmp/BK1.cpp, BK3.cpp and BK5.cpp and of the variant
// harnesses: the positional arguments and defaults of bk::parse_args
// (include/bk_common.h:127-141: nelmt 524288, ntests 5), the order dispatch
// with its "unsupported polynomial order p" message (bk::with_order,
// :162-178), the constant test data (in = 3, JxW = 1, G = 2 and the basis
// cos(a*cols + b), openmp/BK1.cpp:40-44, BK3.cpp:56-60, BK5.cpp:118-120), the
// result line "SumFactorization -> nelmt = .. GDoF/s = .. GB/s = .." and
// "norm = .." (bk::print_rates :196-202, bk::norm2 :44-52), the minimum time
// over ntests (bk::time_min :182-192, here CUDA-event device time), and the
// variant selection BK_KERNEL="a b -c" (bk::selected, include/bk_harness.h:
// 20-40).  Environment:
//   BK_KERNEL  variants to run among fp32 mixed dfma ff (default: the
//              precision of BK_PREC)
//   BK_PREC    fp32 (default, the drivers' T = float) or fp64
//   BK_RANDOM  set: pseudo-random in and JxW/G (the LCG of
//              fill_random_test_data, include/bk_common.h:92-107)
//   BK_CHECK   set: compare every variant with a double-precision host
//              reference, one element per OpenMP iteration (the harness check
//              of include/bk_harness.h:74-85); prints relerr and FAIL at 1e-5
//              (FP32) or 1e-12 (FP64) and exits 1 on a failure
// The host reference here is the driver's own check (as the reference's
// harnesses carry theirs); it is not a compute path of the library.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "bk_gpu.h"

namespace {

bool env_set(const char* n) { return std::getenv(n) != nullptr; }

std::string env_str(const char* n, const char* d)
{
    const char* v = std::getenv(n);
    return v ? std::string(v) : std::string(d);
}

// BK_KERNEL="a b -c" (include/bk_harness.h:20-40)
bool selected(const std::string& list, const char* name)
{
    bool any = false, named = false;
    std::istringstream ss(list);
    std::string w;
    while (ss >> w) {
        if (w[0] == '-') {
            if (w.compare(1, std::string::npos, name) == 0) return false;
        } else {
            any = true;
            named = named || (w == name);
        }
    }
    return !any || named;
}

std::vector<double> test_basis(int rows, int cols, bool as_float)
{
    std::vector<double> m(size_t(rows) * cols);
    for (int a = 0; a < rows; ++a)
        for (int b = 0; b < cols; ++b)
            m[a * cols + b] = as_float ? double(std::cos(float(a * cols + b))) : std::cos(double(a * cols + b));
    return m;
}

void fill_random(std::vector<double>& in, std::vector<double>& geo, uint32_t seed = 12345u)
{
    uint32_t s = seed;
    auto next = [&] {
        s = 1664525u * s + 1013904223u;
        return double(s >> 8) / double(1 << 23) - 1.0;
    };
    for (auto& v : in) v = next();
    for (auto& v : geo) v = 1.5 + next();
}

// ---- host reference (double), one element per OpenMP iteration ------------------

void interp(int nm, int nq, const double* B, const double* in, double* w0, double* w1, double* out)
{
    // out(p,q,r) = sum_ijk in(i,j,k) B(i,p) B(j,q) B(k,r)
    for (int p = 0; p < nq; ++p)
        for (int j = 0; j < nm; ++j)
            for (int k = 0; k < nm; ++k) {
                double s = 0;
                for (int i = 0; i < nm; ++i) s += in[(i * nm + j) * nm + k] * B[i * nq + p];
                w0[(p * nm + j) * nm + k] = s;
            }
    for (int p = 0; p < nq; ++p)
        for (int q = 0; q < nq; ++q)
            for (int k = 0; k < nm; ++k) {
                double s = 0;
                for (int j = 0; j < nm; ++j) s += w0[(p * nm + j) * nm + k] * B[j * nq + q];
                w1[(p * nq + q) * nm + k] = s;
            }
    for (int p = 0; p < nq; ++p)
        for (int q = 0; q < nq; ++q)
            for (int r = 0; r < nq; ++r) {
                double s = 0;
                for (int k = 0; k < nm; ++k) s += w1[(p * nq + q) * nm + k] * B[k * nq + r];
                out[(p * nq + q) * nq + r] = s;
            }
}

void interp_back(int nm, int nq, const double* B, const double* u, double* w0, double* w1, double* out)
{
    for (int p = 0; p < nq; ++p)
        for (int q = 0; q < nq; ++q)
            for (int k = 0; k < nm; ++k) {
                double s = 0;
                for (int r = 0; r < nq; ++r) s += u[(p * nq + q) * nq + r] * B[k * nq + r];
                w1[(p * nq + q) * nm + k] = s;
            }
    for (int p = 0; p < nq; ++p)
        for (int j = 0; j < nm; ++j)
            for (int k = 0; k < nm; ++k) {
                double s = 0;
                for (int q = 0; q < nq; ++q) s += w1[(p * nq + q) * nm + k] * B[j * nq + q];
                w0[(p * nm + j) * nm + k] = s;
            }
    for (int i = 0; i < nm; ++i)
        for (int j = 0; j < nm; ++j)
            for (int k = 0; k < nm; ++k) {
                double s = 0;
                for (int p = 0; p < nq; ++p) s += w0[(p * nm + j) * nm + k] * B[i * nq + p];
                out[(i * nm + j) * nm + k] = s;
            }
}

// grad with D(n,p) (BK3: Dconv = 0) or D(i,n) (BK5: Dconv = 1) at nq^3 points,
// fluxes with G (factor-major stride gs, factor stride gf), transposed grad
void laplace(int nq, int Dconv, const double* D, const double* u, const double* G, long gstride_f,
             bool interleaved, double* out)
{
    const int n3 = nq * nq * nq;
    std::vector<double> fr(n3), fs(n3), ft(n3);
    auto d = [&](int a, int b) { return Dconv ? D[a * nq + b] : D[b * nq + a]; };   // d(point, node)
    for (int i = 0; i < nq; ++i)
        for (int j = 0; j < nq; ++j)
            for (int k = 0; k < nq; ++k) {
                double qr = 0, qs = 0, qt = 0;
                for (int n = 0; n < nq; ++n) {
                    qr += u[(n * nq + j) * nq + k] * d(i, n);
                    qs += u[(i * nq + n) * nq + k] * d(j, n);
                    qt += u[(i * nq + j) * nq + n] * d(k, n);
                }
                const int x = (i * nq + j) * nq + k;
                auto g = [&](int f) {
                    return interleaved ? G[((i * nq + j) * 6 + f) * nq + k] : G[f * gstride_f + x];
                };
                fr[x] = g(0) * qr + g(1) * qs + g(2) * qt;
                fs[x] = g(1) * qr + g(3) * qs + g(4) * qt;
                ft[x] = g(2) * qr + g(4) * qs + g(5) * qt;
            }
    for (int i = 0; i < nq; ++i)
        for (int j = 0; j < nq; ++j)
            for (int k = 0; k < nq; ++k) {
                double s = 0;
                for (int n = 0; n < nq; ++n) {
                    s += fr[(n * nq + j) * nq + k] * d(n, i);
                    s += fs[(i * nq + n) * nq + k] * d(n, j);
                    s += ft[(i * nq + j) * nq + n] * d(n, k);
                }
                out[(i * nq + j) * nq + k] = s;
            }
}

void host_reference(int bk, int nq, size_t E, const std::vector<double>& B, const std::vector<double>& D,
                    const std::vector<double>& geo, const std::vector<double>& in, std::vector<double>& out)
{
    const int nm = (bk == 5) ? nq : nq - 1;
    const size_t n3 = size_t(nq) * nq * nq, m3 = size_t(nm) * nm * nm;
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < (long long)E; ++e) {
        std::vector<double> w0(n3), w1(n3), uq(n3), vq(n3);
        if (bk == 5) {
            laplace(nq, 1, D.data(), &in[e * n3], &geo[e * 6 * n3], 0, true, &out[e * n3]);
            continue;
        }
        interp(nm, nq, B.data(), &in[e * m3], w0.data(), w1.data(), uq.data());
        if (bk == 1) {
            for (size_t x = 0; x < n3; ++x) uq[x] *= geo[e * n3 + x];
            interp_back(nm, nq, B.data(), uq.data(), w0.data(), w1.data(), &out[e * m3]);
        } else {
            laplace(nq, 0, D.data(), uq.data(), &geo[e * 6 * n3], long(n3), false, vq.data());
            interp_back(nm, nq, B.data(), vq.data(), w0.data(), w1.data(), &out[e * m3]);
        }
    }
}

struct Variant {
    const char* name;
    int prec;
    int engine;
};

const Variant kVariants[] = {
    {"fp32", BK_PREC_FP32, BK_ENGINE_AUTO},
    {"mixed", BK_PREC_MIXED, BK_ENGINE_AUTO},
    {"ff", BK_PREC_FP64, BK_ENGINE_FF},
    {"dfma", BK_PREC_FP64, BK_ENGINE_DFMA},
};

#define CK(x)                                                                                  \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) {                                                               \
            std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, \
                         __LINE__);                                                            \
            std::exit(2);                                                                      \
        }                                                                                      \
    } while (0)

// ||x - ref|| / ||ref|| in double (the reference's relative_error,
// openmp/BK1_ff.cpp:751-764)
double rel_l2(const std::vector<double>& x, const std::vector<double>& ref)
{
    double num = 0, den = 0;
    for (size_t i = 0; i < ref.size(); ++i) {
        const double d = x[i] - ref[i];
        num += d * d;
        den += ref[i] * ref[i];
    }
    return std::sqrt(num) / std::sqrt(den);
}

// BK1_ff <p> [nelmt] [ntests]: the precision harness of openmp/BK1_ff.cpp
// (run_test :799-845, main :847-862) on the GPU kernels.  The same data (the
// double test basis, in = 3, JxW = 1, or BK_RANDOM's LCG) through BK1 in
// double (the DFMA engine), float (FP32 storage, the double data rounded)
// and float-float (the FF engine); one row per precision with GDoF/s, GB/s
// and the norm; the float and float-float relative L2 errors against the
// double result; ok or FAIL at BK_TOL (default 1e-10) for the float-float
// result, and the exit code 0 or 1.  The reference's ff-teams and ff-plane
// rows are loop organisations of the same float-float arithmetic on the
// host; the GPU has one float-float kernel, reported once.
int run_bk1_ff(int argc, char** argv)
{
    const int p = (argc > 2) ? std::atoi(argv[2]) : 2;
    const size_t nelmt = (argc > 3) ? size_t(std::atoll(argv[3])) : (size_t(1) << 19);
    const int ntests = (argc > 4) ? std::atoi(argv[4]) : 5;
    if (p < 1 || p > 8) {
        std::fprintf(stderr, "unsupported polynomial order p = %d (supported: 1..8)\n", p);
        return 1;
    }
    const bool random_data = env_set("BK_RANDOM");
    const double tol = std::atof(env_str("BK_TOL", "1e-10").c_str());
    const int nq = p + 2, nm = nq - 1;
    const size_t n_in = nelmt * size_t(nm) * nm * nm, n_geo = nelmt * size_t(nq) * nq * nq;
    const std::vector<double> B = test_basis(nm, nq, false);
    std::vector<double> in(n_in, 3.0), jxw(n_geo, 1.0);
    if (random_data) fill_random(in, jxw);
    std::printf("SumFactorization -> nelmt = %zu nq = %d data = %s fma = hardware\n", nelmt, nq,
                random_data ? "random" : "constant");
    void *d_in = nullptr, *d_geo = nullptr, *d_out = nullptr;
    CK(cudaMalloc(&d_in, n_in * 8));
    CK(cudaMalloc(&d_geo, n_geo * 8));
    CK(cudaMalloc(&d_out, n_in * 8));
    cudaStream_t s;
    CK(cudaStreamCreate(&s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const Variant rows[] = {{"double", BK_PREC_FP64, BK_ENGINE_DFMA},
                            {"float", BK_PREC_FP32, BK_ENGINE_AUTO},
                            {"float-float", BK_PREC_FP64, BK_ENGINE_FF}};
    std::vector<double> out[3];
    int status = BK_OK;
    for (int r = 0; r < 3; ++r) {
        const Variant& v = rows[r];
        const bool f32 = v.prec == BK_PREC_FP32;
        const size_t vb = f32 ? 4 : 8;
        auto upload = [&](void* dst, const std::vector<double>& h) {
            if (f32) {
                std::vector<float> t(h.begin(), h.end());
                CK(cudaMemcpy(dst, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
            } else {
                CK(cudaMemcpy(dst, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
            }
        };
        upload(d_in, in);
        upload(d_geo, jxw);
        bk_options o = bk_default_options();
        o.prec = v.prec;
        o.engine = v.engine;
        // float: the double basis rounded, as the reference's float row sees it
        std::vector<double> Bv = B;
        if (f32)
            for (double& b : Bv) b = double(float(b));
        auto run = [&]() { return bk1_apply_opt(p, int64_t(nelmt), Bv.data(), d_geo, d_in, d_out, &o, s); };
        int rc = run();
        if (rc != BK_OK) {
            std::fprintf(stderr, "%s: status %d\n", v.name, rc);
            status = rc;
            break;
        }
        float best = 1e30f;
        for (int t = 0; t < ntests; ++t) {
            CK(cudaEventRecord(e0, s));
            run();
            CK(cudaEventRecord(e1, s));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        int st = 0;
        bk_device_status(&st, 1, s);
        if (st != BK_OK) status = st;
        out[r].resize(n_in);
        if (f32) {
            std::vector<float> t(n_in);
            CK(cudaMemcpy(t.data(), d_out, n_in * 4, cudaMemcpyDeviceToHost));
            std::copy(t.begin(), t.end(), out[r].begin());
        } else {
            CK(cudaMemcpy(out[r].data(), d_out, n_in * 8, cudaMemcpyDeviceToHost));
        }
        const double sec = best * 1e-3;
        double nrm = 0;
        for (double x : out[r]) nrm += x * x;
        std::printf("%-12s GDoF/s = %9.4g GB/s = %9.4g norm = %.10g\n", v.name, 1e-9 * n_in / sec,
                    1e-9 * double(vb) * (2.0 * n_in + n_geo) / sec, std::sqrt(nrm));
    }
    cudaFree(d_in);
    cudaFree(d_geo);
    cudaFree(d_out);
    if (status != BK_OK) return 1;
    const double err_float = rel_l2(out[1], out[0]);
    const double err_ff = rel_l2(out[2], out[0]);
    const bool ok = err_ff <= tol;
    std::printf("float        rel. error vs double = %g\n", err_float);
    std::printf("%s: float-float rel. error vs double = %g (tol = %g)\n", ok ? "ok" : "FAIL", err_ff, tol);
    return ok ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s BK1|BK3|BK5|BK1_ff <p> [nelmt] [ntests]\n", argv[0]);
        return 1;
    }
    const std::string op = argv[1];
    if (op == "BK1_ff") return run_bk1_ff(argc, argv);
    const int bk = (op == "BK1") ? 1 : (op == "BK3") ? 3 : (op == "BK5") ? 5 : 0;
    if (bk == 0) {
        std::fprintf(stderr, "unknown operator %s (BK1, BK3, BK5 or BK1_ff)\n", op.c_str());
        return 1;
    }
    // bk::parse_args: <order> [nelmt] [ntests], defaults 2 (3 for BK5), 2^19, 5
    const int p = (argc > 2) ? std::atoi(argv[2]) : (bk == 5 ? 3 : 2);
    const size_t nelmt = (argc > 3) ? size_t(std::atoll(argv[3])) : (size_t(1) << 19);
    const int ntests = (argc > 4) ? std::atoi(argv[4]) : 5;
    if (p < 1 || p > 8) {
        std::fprintf(stderr, "unsupported polynomial order p = %d (supported: 1..8)\n", p);
        return 1;
    }
    const bool fp64 = env_str("BK_PREC", "fp32") == "fp64";
    const std::string kernels = env_str("BK_KERNEL", fp64 ? "ff" : "fp32");
    const bool random_data = env_set("BK_RANDOM");
    const bool check = env_set("BK_CHECK");

    const int nq = (bk == 5) ? p + 1 : p + 2;
    const int nm = (bk == 5) ? nq : nq - 1;
    const size_t n_in = nelmt * size_t(nm) * nm * nm;
    const size_t n_geo = nelmt * size_t(nq) * nq * nq * (bk == 1 ? 1 : 6);
    // the float drivers build their basis in float (make_test_basis<float>)
    std::vector<double> B = (bk != 5) ? test_basis(nm, nq, !fp64) : std::vector<double>();
    std::vector<double> D = (bk != 1) ? test_basis(nq, nq, !fp64) : std::vector<double>();
    std::vector<double> in(n_in, 3.0), geo(n_geo, bk == 1 ? 1.0 : 2.0);
    if (random_data) fill_random(in, geo);
    std::vector<double> ref;
    double big = 0;
    if (check) {
        ref.resize(n_in);
        host_reference(bk, nq, nelmt, B, D, geo, in, ref);
        for (double r : ref) big = std::max(big, std::fabs(r));
    }

    void *d_in = nullptr, *d_geo = nullptr, *d_out = nullptr;
    CK(cudaMalloc(&d_in, n_in * 8));
    CK(cudaMalloc(&d_geo, n_geo * 8));
    CK(cudaMalloc(&d_out, n_in * 8));
    cudaStream_t s;
    CK(cudaStreamCreate(&s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    bool failed = false;
    std::printf("%s CUDA: p = %d, nq = %d, nelmt = %zu, ntests = %d, data = %s\n", op.c_str(), p, nq, nelmt, ntests,
                random_data ? "random" : "constant");
    for (const Variant& v : kVariants) {
        if (!selected(kernels, v.name)) continue;
        const bool f32 = (v.prec != BK_PREC_FP64);
        const size_t vb = f32 ? 4 : 8;
        // upload in the variant's storage type
        auto upload = [&](void* dst, const std::vector<double>& h) {
            if (f32) {
                std::vector<float> t(h.begin(), h.end());
                CK(cudaMemcpy(dst, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
            } else {
                CK(cudaMemcpy(dst, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
            }
        };
        upload(d_in, in);
        upload(d_geo, geo);
        CK(cudaMemset(d_out, 0, n_in * vb));
        bk_options o = bk_default_options();
        o.prec = v.prec;
        o.engine = v.engine;
        o.layout = BK_LAYOUT_INTERLEAVED;
        auto run = [&]() {
            if (bk == 1) return bk1_apply_opt(p, int64_t(nelmt), B.data(), d_geo, d_in, d_out, &o, s);
            if (bk == 3) return bk3_apply_opt(p, int64_t(nelmt), B.data(), D.data(), d_geo, d_in, d_out, &o, s);
            return bk5_apply_opt(p, int64_t(nelmt), D.data(), d_geo, d_in, d_out, &o, s);
        };
        int rc = run();   // warm-up
        if (rc != BK_OK) {
            std::printf("%-6s skipped (status %d)\n", v.name, rc);
            continue;
        }
        float best = 1e30f;
        for (int t = 0; t < ntests; ++t) {
            CK(cudaEventRecord(e0, s));
            run();
            CK(cudaEventRecord(e1, s));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        int st = 0;
        bk_device_status(&st, 1, s);
        std::vector<double> out(n_in);
        if (f32) {
            std::vector<float> t(n_in);
            CK(cudaMemcpy(t.data(), d_out, n_in * 4, cudaMemcpyDeviceToHost));
            std::copy(t.begin(), t.end(), out.begin());
        } else {
            CK(cudaMemcpy(out.data(), d_out, n_in * 8, cudaMemcpyDeviceToHost));
        }
        const double sec = best * 1e-3;
        const double bytes = double(vb) * (2.0 * n_in + n_geo);
        std::printf("%-6s SumFactorization -> nelmt = %zu GDoF/s = %g GB/s = %g\n", v.name, nelmt,
                    1e-9 * n_in / sec, 1e-9 * bytes / sec);
        double nrm = 0;
        for (double x : out) nrm += x * x;
        std::printf("%-6s norm = %.10g", v.name, std::sqrt(nrm));
        if (check) {
            double diff = 0;
            for (size_t i = 0; i < n_in; ++i) diff = std::max(diff, std::fabs(out[i] - ref[i]));
            const double rel = big > 0 ? diff / big : diff;
            const double tol = f32 ? 1e-5 : 1e-12;
            const bool bad = !(rel < tol) || st != BK_OK;
            failed = failed || bad;
            std::printf("  relerr = %.1e%s", rel, bad ? "  FAIL" : "");
        }
        std::printf("\n");
    }
    cudaFree(d_in);
    cudaFree(d_geo);
    cudaFree(d_out);
    return failed ? 1 : 0;
}
