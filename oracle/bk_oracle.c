/* bk_oracle.c -- CPU oracle of the bake-off operator apply (BK1, BK3, BK5).
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  This library is the checker of the
 * CUDA kernels: only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark load it.  Nothing in the omp_bk_gb300 package links or calls
 * it, and the GPU path has no CPU fallback to it.
 *
 * What it restates (plain C, one element per OpenMP iteration, the
 * reference's loop order and order of summation in every sum):
 *   - bk::SumFactorization for BK1 (openmp/bk1_sumfact.h:17-159), BK3
 *     (openmp/bk3_sumfact.h:18-187) and BK5 (openmp/BK5.cpp:19-103), in double
 *     and in float (bk_oracle_body.inc);
 *   - the harness references bk::reference_bk1/bk3/bk5
 *     (include/bk_harness.h:186-205, 299-355, 247-293): float inputs, double
 *     arithmetic -- same sums in the same order as SumFactorization<double>;
 *   - the data layouts: make_bk5_G (include/bk_harness.h:220-244, g6i_index
 *     :210, bk5_sym :215) and transpose_jxw (:89-102);
 *   - the test data: make_test_basis (include/bk_common.h:63-86), the LCG of
 *     fill_random_test_data (:92-107) and norm2 (:44-52);
 *   - the accuracy check rel_maxdiff / max_abs (include/bk_harness.h:65-83).
 * And, with no reference counterpart (the reference has no variable
 * coefficient, no gradient and no Helmholtz term), the FP64 host forms of the
 * variable-coefficient BK3 operator, its adjoint gradient with respect to the
 * coefficient and the geometric factors, and BK5 plus a diagonal mass term.
 *
 * Pinned against the reference itself: tests/golden holds outputs of the
 * reference's own kernels compiled from its sources (oracle/Makefile, target
 * ref), and tests/test_oracle.py checks this file against them. */

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define BKO_MAX_NQ 10
#define BKO_BOX (BKO_MAX_NQ * BKO_MAX_NQ * BKO_MAX_NQ)
#define X3(a, b, c) (((a) * nq + (b)) * nq + (c))

/* double: a run-time-nq instance and one instance per fixed nq, then the
 * entry points that dispatch to them */
#define NQ_OF(x) (x)
#define REAL double
#define SFX(name) name##_generic
#define NQ_FIXED
#include "bk_oracle_body.inc"
#undef NQ_FIXED
#undef SFX
#undef NQ_OF

#define NQ_FIXED
#define NQ_OF(x) 2
#define SFX(name) name##_nq2
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 3
#define SFX(name) name##_nq3
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 4
#define SFX(name) name##_nq4
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 5
#define SFX(name) name##_nq5
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 6
#define SFX(name) name##_nq6
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 7
#define SFX(name) name##_nq7
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 8
#define SFX(name) name##_nq8
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 9
#define SFX(name) name##_nq9
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#define NQ_OF(x) 10
#define SFX(name) name##_nq10
#include "bk_oracle_body.inc"
#undef SFX
#undef NQ_OF
#undef NQ_FIXED
#undef REAL

#define DISPATCH(fn, nq, args)                 \
    switch (nq) {                              \
        case 2: fn##_nq2 args; return;         \
        case 3: fn##_nq3 args; return;         \
        case 4: fn##_nq4 args; return;         \
        case 5: fn##_nq5 args; return;         \
        case 6: fn##_nq6 args; return;         \
        case 7: fn##_nq7 args; return;         \
        case 8: fn##_nq8 args; return;         \
        case 9: fn##_nq9 args; return;         \
        case 10: fn##_nq10 args; return;       \
        default: fn##_generic args; return;    \
    }

void bko_bk1_sumfact(int nq, size_t nelmt, const double* basis, const double* JxW, const double* in, double* out)
{
    DISPATCH(bko_bk1_sumfact, nq, (nq, nelmt, basis, JxW, in, out))
}

void bko_bk3_sumfact_k(int nq, size_t nelmt, const double* basis, const double* dbasis, const double* G,
                       const double* kq, const double* in, double* out)
{
    DISPATCH(bko_bk3_sumfact_k, nq, (nq, nelmt, basis, dbasis, G, kq, in, out))
}

void bko_bk3_sumfact(int nq, size_t nelmt, const double* basis, const double* dbasis, const double* G,
                     const double* in, double* out)
{
    bko_bk3_sumfact_k(nq, nelmt, basis, dbasis, G, NULL, in, out);
}

void bko_bk5_sumfact_h(int nq, size_t nelmt, const double* dbasis, const double* G, const double* mass,
                       double lambda, const double* in, double* out)
{
    DISPATCH(bko_bk5_sumfact_h, nq, (nq, nelmt, dbasis, G, mass, lambda, in, out))
}

void bko_bk5_sumfact(int nq, size_t nelmt, const double* dbasis, const double* G, const double* in, double* out)
{
    bko_bk5_sumfact_h(nq, nelmt, dbasis, G, NULL, 0.0, in, out);
}

#define NQ_OF(x) (x)
#define REAL float
#define SFX(name) name##_f32
#include "bk_oracle_body.inc"
#undef REAL
#undef SFX
#undef NQ_OF

int bko_max_nq(void) { return BKO_MAX_NQ; }

/* ---- harness references: float inputs, double arithmetic ---------------- */

static double* widen(const float* x, size_t n)
{
    double* y = (double*)malloc(n * sizeof(double));
    size_t i;
    for (i = 0; i < n; ++i) y[i] = (double)x[i];
    return y;
}

/* bk::reference_bk1 (include/bk_harness.h:186-205 with ref_interp :106-143
 * and ref_interp_back :146-183): the same sums, index by index and in the same
 * summation order, as bk1_sumfact.h's nine steps in double. */
void bko_reference_bk1(int nq, size_t nelmt, const float* basis, const float* JxW,
                       const float* in, double* out)
{
    const int nm = nq - 1;
    const size_t nq3 = (size_t)nq * nq * nq, nm3 = (size_t)nm * nm * nm;
    double *b = widen(basis, (size_t)nm * nq), *j = widen(JxW, nelmt * nq3), *u = widen(in, nelmt * nm3);
    bko_bk1_sumfact(nq, nelmt, b, j, u, out);
    free(b); free(j); free(u);
}

/* bk::reference_bk3 (include/bk_harness.h:299-355). */
void bko_reference_bk3(int nq, size_t nelmt, const float* basis, const float* D, const float* G,
                       const float* in, double* out)
{
    const int nm = nq - 1;
    const size_t nq3 = (size_t)nq * nq * nq, nm3 = (size_t)nm * nm * nm;
    double *b = widen(basis, (size_t)nm * nq), *d = widen(D, (size_t)nq * nq);
    double *g = widen(G, nelmt * 6 * nq3), *u = widen(in, nelmt * nm3);
    bko_bk3_sumfact(nq, nelmt, b, d, g, u, out);
    free(b); free(d); free(g); free(u);
}

/* bk::reference_bk5 (include/bk_harness.h:247-293), G6i interleaved. */
void bko_reference_bk5(int nq, size_t nelmt, const float* D, const float* G6i, const float* in,
                       double* out)
{
    const size_t nq3 = (size_t)nq * nq * nq;
    double *d = widen(D, (size_t)nq * nq), *g = widen(G6i, nelmt * 6 * nq3), *u = widen(in, nelmt * nq3);
    bko_bk5_sumfact(nq, nelmt, d, g, u, out);
    free(d); free(g); free(u);
}

/* ---- layouts -------------------------------------------------------------- */

/* include/bk_harness.h:215 */
static const int bk5_sym[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};

/* make_bk5_G (include/bk_harness.h:220-244): G with F = 6 or 9 factors per
 * point, layout 0 factor-major G(f,i,j,k), 1 interleaved G(i,j,f,k), 2 column
 * G(f,k,i,j), from G6i(e,i,j,s,k) (g6i_index :210). */
void bko_make_bk5_G(const double* G6i, size_t nelmt, int nq, int F, int layout, double* G)
{
    const size_t nq3 = (size_t)nq * nq * nq;
    long long e;
#pragma omp parallel for schedule(static)
    for (e = 0; e < (long long)nelmt; ++e) {
        int i, j, k, f;
        for (i = 0; i < nq; ++i) for (j = 0; j < nq; ++j) for (k = 0; k < nq; ++k)
            for (f = 0; f < F; ++f) {
                const int s = (F == 6) ? f : bk5_sym[f];
                int dst = ((f * nq + i) * nq + j) * nq + k;
                if (layout == 1) dst = ((i * nq + j) * F + f) * nq + k;
                else if (layout == 2) dst = ((f * nq + k) * nq + i) * nq + j;
                G[(size_t)e * F * nq3 + dst] = G6i[(size_t)e * 6 * nq3 + ((i * nq + j) * 6 + s) * nq + k];
            }
    }
}

/* transpose_jxw (include/bk_harness.h:89-102): JxW(e,p,q,r) -> JxW_t(e,r,q,p). */
void bko_transpose_jxw(const double* JxW, size_t nelmt, int nq, double* JxW_t)
{
    size_t e;
    int p, q, r;
    for (e = 0; e < nelmt; ++e)
        for (p = 0; p < nq; ++p) for (q = 0; q < nq; ++q) for (r = 0; r < nq; ++r)
            JxW_t[((e * nq + r) * nq + q) * nq + p] = JxW[((e * nq + p) * nq + q) * nq + r];
}

/* ---- test data ------------------------------------------------------------ */

/* make_test_basis (include/bk_common.h:63-86): M(a,b) = cos(a*cols + b). */
void bko_make_test_basis(int rows, int cols, double* m)
{
    int a, b;
    for (a = 0; a < rows; ++a) for (b = 0; b < cols; ++b) m[a * cols + b] = cos((double)(a * cols + b));
}

void bko_make_test_basis_f32(int rows, int cols, float* m)
{
    int a, b;
    for (a = 0; a < rows; ++a) for (b = 0; b < cols; ++b) m[a * cols + b] = cosf((float)(a * cols + b));
}

/* fill_random_test_data (include/bk_common.h:92-107): one LCG stream fills
 * in with [-1,1] and then JxW (or G) with 1.5 + [-1,1]; every draw is a 24-bit
 * integer over 2^23, so the float and double values are identical. */
void bko_fill_random_test_data(double* in, size_t nin, double* jxw, size_t njxw, uint32_t seed)
{
    uint32_t s = seed;
    size_t i;
    for (i = 0; i < nin; ++i) {
        s = 1664525u * s + 1013904223u;
        in[i] = (double)(s >> 8) / (double)(1 << 23) - 1.0;
    }
    for (i = 0; i < njxw; ++i) {
        s = 1664525u * s + 1013904223u;
        jxw[i] = 1.5 + ((double)(s >> 8) / (double)(1 << 23) - 1.0);
    }
}

/* norm2 (include/bk_common.h:44-52): sequential double sum of squares. */
double bko_norm2(const double* v, size_t n)
{
    double s = 0;
    size_t i;
    for (i = 0; i < n; ++i) s += v[i] * v[i];
    return sqrt(s);
}

double bko_norm2_f32(const float* v, size_t n)
{
    double s = 0;
    size_t i;
    for (i = 0; i < n; ++i) s += (double)v[i] * (double)v[i];
    return sqrt(s);
}

/* max_abs and rel_maxdiff (include/bk_harness.h:65-83): largest |out - ref|
 * over the largest |ref|. */
double bko_rel_maxdiff(const double* out, const double* ref, size_t n)
{
    double big = 0, diff = 0;
    size_t i;
    for (i = 0; i < n; ++i) {
        const double a = fabs(ref[i]), d = fabs(out[i] - ref[i]);
        if (a > big) big = a;
        if (d > diff) diff = d;
    }
    return big > 0 ? diff / big : diff;
}

/* ---- adjoint of the variable-coefficient BK3 operator (no reference
 * counterpart) ------------------------------------------------------------- */

/* Per element: g(x) = D B w at every quadrature point x, the three reference
 * derivatives of the interpolant of w (the first two stages of bk3_sumfact.h,
 * :63-125, before the fluxes). */
static void bko_grad_q(int nq, const double* basis, const double* dbasis, const double* ein,
                       double* gr, double* gs, double* gt)
{
    const int nm = nq - 1;
    double w0[BKO_BOX], w1[BKO_BOX];
    int i, j, k, p, q, r, n;
    for (i = 0; i < nm; ++i) for (j = 0; j < nm; ++j) for (k = 0; k < nm; ++k)
        w0[X3(i, j, k)] = ein[(i * nm + j) * nm + k];
    for (p = 0; p < nq; ++p) for (k = 0; k < nm; ++k) for (j = 0; j < nm; ++j) {
        double t = 0;
        for (i = 0; i < nm; ++i) t += w0[X3(i, j, k)] * basis[i * nq + p];
        w1[X3(p, j, k)] = t;
    }
    for (q = 0; q < nq; ++q) for (p = 0; p < nq; ++p) for (k = 0; k < nm; ++k) {
        double t = 0;
        for (j = 0; j < nm; ++j) t += w1[X3(p, j, k)] * basis[j * nq + q];
        w0[X3(q, p, k)] = t;
    }
    for (r = 0; r < nq; ++r) for (q = 0; q < nq; ++q) for (p = 0; p < nq; ++p) {
        double t = 0;
        for (k = 0; k < nm; ++k) t += w0[X3(q, p, k)] * basis[k * nq + r];
        w1[X3(p, q, r)] = t;
    }
    for (p = 0; p < nq; ++p) for (q = 0; q < nq; ++q) for (r = 0; r < nq; ++r) {
        double a = 0, b = 0, c = 0;
        for (n = 0; n < nq; ++n) a += w1[X3(n, q, r)] * dbasis[n * nq + p];
        for (n = 0; n < nq; ++n) b += w1[X3(p, n, r)] * dbasis[n * nq + q];
        for (n = 0; n < nq; ++n) c += w1[X3(p, q, n)] * dbasis[n * nq + r];
        gr[X3(p, q, r)] = a; gs[X3(p, q, r)] = b; gt[X3(p, q, r)] = c;
    }
}

/* Loss L = 1/2 |A(k) u - f|^2 with the residual res = A(k) u - f given:
 * dL/dk(x) = g_res(x)^T G(x) g_u(x) and, for the six stored symmetric factors
 * (rr rs rt ss st tt, each off-diagonal factor standing for both of its
 * entries), dL/dG_ab(x) = k(x) (g_res,a g_u,b + g_res,b g_u,a) for a != b and
 * k(x) g_res,a g_u,a on the diagonal.  G factor-major (e,f,p,q,r). */
void bko_bk3_adjoint(int nq, size_t nelmt, const double* basis, const double* dbasis,
                     const double* G, const double* kq, const double* u, const double* res,
                     double* dk, double* dG)
{
    const int nm = nq - 1;
    const size_t nq3 = (size_t)nq * nq * nq, nm3 = (size_t)nm * nm * nm;
    long long e;
#pragma omp parallel for schedule(static)
    for (e = 0; e < (long long)nelmt; ++e) {
        double ur[BKO_BOX], us[BKO_BOX], ut[BKO_BOX], rr[BKO_BOX], rs[BKO_BOX], rt[BKO_BOX];
        size_t x;
        bko_grad_q(nq, basis, dbasis, u + (size_t)e * nm3, ur, us, ut);
        bko_grad_q(nq, basis, dbasis, res + (size_t)e * nm3, rr, rs, rt);
        for (x = 0; x < nq3; ++x) {
            const double* g = G + (size_t)e * 6 * nq3 + x;
            const double kk = kq[(size_t)e * nq3 + x];
            const double fr = g[0] * ur[x] + g[nq3] * us[x] + g[2 * nq3] * ut[x];
            const double fs = g[nq3] * ur[x] + g[3 * nq3] * us[x] + g[4 * nq3] * ut[x];
            const double ft = g[2 * nq3] * ur[x] + g[4 * nq3] * us[x] + g[5 * nq3] * ut[x];
            double* o = dG + (size_t)e * 6 * nq3 + x;
            dk[(size_t)e * nq3 + x] = rr[x] * fr + rs[x] * fs + rt[x] * ft;
            o[0] = kk * rr[x] * ur[x];
            o[nq3] = kk * (rr[x] * us[x] + rs[x] * ur[x]);
            o[2 * nq3] = kk * (rr[x] * ut[x] + rt[x] * ur[x]);
            o[3 * nq3] = kk * rs[x] * us[x];
            o[4 * nq3] = kk * (rs[x] * ut[x] + rt[x] * us[x]);
            o[5 * nq3] = kk * rt[x] * ut[x];
        }
    }
}
