// bk_basis.cpp -- 1-D quadrature rules and Lagrange matrices for the benchmark
// configurations.  The reference has none of these (its drivers use the test
// basis cos(a*cols + b), include/bk_common.h:60-86); the standard
// constructions are written here from the mathematics:
//   Gauss-Legendre points: roots of P_n by Newton's method, weights
//     2 / ((1 - x^2) P_n'(x)^2);
//   Gauss-Lobatto-Legendre points: +-1 and the roots of P_{n-1}', weights
//     2 / (n (n - 1) P_{n-1}(x)^2);
//   Lagrange interpolation l_i(x) as a product, derivatives by the
//   barycentric formula D_in = (lambda_n / lambda_i) / (x_i - x_n), with the
//   diagonal as minus the row sum (so that D 1 = 0 to rounding).
#include <cmath>
#include <vector>

#include "bk_data.h"

namespace {

// P_n(x) and P_n'(x) by the three-term recurrence.
void legendre(int n, double x, double& p, double& dp)
{
    double p0 = 1.0, p1 = x;
    if (n == 0) {
        p = 1.0;
        dp = 0.0;
        return;
    }
    for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
    }
    p = p1;
    // (1 - x^2) P_n' = n (P_{n-1} - x P_n); valid away from +-1
    dp = n * (p0 - x * p1) / (1.0 - x * x);
}

}  // namespace

extern "C" {

int bk_gauss_points(int n, double* x, double* w)
{
    if (n < 1 || n > 64 || x == nullptr || w == nullptr) return BK_ERR_ARG;
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i) {
        double z = std::cos(pi * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p, dp;
            legendre(n, z, p, dp);
            const double dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        double p, dp;
        legendre(n, z, p, dp);
        // ascending order
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    return BK_OK;
}

int bk_gll_points(int n, double* x, double* w)
{
    if (n < 2 || n > 64 || x == nullptr || w == nullptr) return BK_ERR_ARG;
    const int N = n - 1;   // polynomial degree
    const double pi = 3.14159265358979323846;
    x[0] = -1.0;
    x[N] = 1.0;
    for (int i = 1; i < N; ++i) {
        // Chebyshev-Gauss-Lobatto guess, Newton on q(z) = P_N'(z) with
        // q'(z) = (2 z P_N' - N (N + 1) P_N) / (1 - z^2)
        double z = -std::cos(pi * i / N);
        for (int it = 0; it < 100; ++it) {
            double p, dp;
            legendre(N, z, p, dp);
            const double d2p = (2.0 * z * dp - N * (N + 1.0) * p) / (1.0 - z * z);
            const double dz = dp / d2p;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = z;
    }
    for (int i = 0; i <= N; ++i) {
        double p, dp;
        legendre(N, x[i], p, dp);
        w[i] = 2.0 / (N * (N + 1.0) * p * p);
    }
    return BK_OK;
}

// B[i*npts + p] = l_i(pts[p]), l_i the Lagrange polynomial of nodes[i]:
// the reference's basis(i, p) convention (openmp/bk1_sumfact.h:39).
int bk_lagrange_interp(int nnodes, const double* nodes, int npts, const double* pts, double* B)
{
    if (nnodes < 1 || npts < 1 || !nodes || !pts || !B) return BK_ERR_ARG;
    for (int i = 0; i < nnodes; ++i) {
        for (int p = 0; p < npts; ++p) {
            double v = 1.0;
            for (int m = 0; m < nnodes; ++m) {
                if (m != i) v *= (pts[p] - nodes[m]) / (nodes[i] - nodes[m]);
            }
            B[i * npts + p] = v;
        }
    }
    return BK_OK;
}

// D[i*n + j] = l_j'(x_i): the collocation derivative on the points x
// (BK5's D(i, n), openmp/BK5.cpp:290; BK3 uses the transpose, D(n, p) =
// l_n'(x_p), openmp/bk3_sumfact.h:41).
int bk_lagrange_deriv(int n, const double* x, double* D)
{
    if (n < 1 || !x || !D) return BK_ERR_ARG;
    std::vector<double> lam(n);
    for (int i = 0; i < n; ++i) {
        double prod = 1.0;
        for (int m = 0; m < n; ++m) {
            if (m != i) prod *= (x[i] - x[m]);
        }
        lam[i] = 1.0 / prod;
    }
    for (int i = 0; i < n; ++i) {
        double diag = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            const double d = (lam[j] / lam[i]) / (x[i] - x[j]);
            D[i * n + j] = d;
            diag -= d;
        }
        D[i * n + i] = diag;
    }
    return BK_OK;
}

}  // extern "C"
