/* bk_geom_oracle.c -- CPU oracle of the synthetic inputs of the benchmark
 * configurations: seeded fields, 1-D rules and matrices, and the geometric
 * data of the affine and jittered-trilinear meshes, in FP64.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  The tests hold the GPU generators
 * of the library to these functions, and the CPU legs of the benchmark build
 * their host inputs with them (so that the reference arm runs on the same
 * seeded data as the GPU without loading the GPU library).  Nothing in the
 * omp_bk_gb300 package links or calls this file.
 *
 * The reference has no geometry (its drivers use constant G = 2, JxW = 1 or
 * an LCG, include/bk_common.h:60-107), so everything here is written from the
 * definitions alone:
 *
 *   stream s, value i:  U(s, i) = top 53 bits of splitmix64(splitmix64(s) + i)
 *                       over 2^53 (splitmix64: Steele, Lea, Flood, "Fast
 *                       splittable pseudorandom number generators", 2014)
 *   uniform field:      lo + (hi - lo) U(s, i)
 *   log-normal field:   exp(sigma z_i), z_i = sqrt(-2 ln(1 - U(s, 2i)))
 *                       cos(2 pi U(s, 2i + 1))  (Box-Muller)
 *   affine element e:   x(xi) = c_e + (h/2)(I + P_e) xi, P_e[a][b] =
 *                       pert (2 U(s, 9e + 3a + b) - 1), c_e the centre of cell
 *                       (e mod nx, e/nx mod ny, e/(nx ny)) of spacing h
 *   trilinear element:  x(xi) = sum over the 8 corners of the cell of
 *                       N(xi) X_corner, N the product of (1 -+ xi_d)/2;
 *                       corner (vx, vy, vz) of the (nx+1) x (ny+1) x .. vertex
 *                       grid sits at h (v_c + jit (2 U(s, 3 id + c) - 1)),
 *                       id = vx + (nx+1)(vy + (ny+1) vz)
 *   point (i, j, k):    xi = (x_i, x_j, x_k), w = w_i w_j w_k
 *   geometric factors:  qdata = mass = w det J,
 *                       G = w det J J^-1 J^-T, stored as rr rs rt ss st tt
 *                       in layout 0 (f,i,j,k), 1 (i,j,f,k) or 2 (f,k,i,j)
 *
 * J^-1 is formed from the cross products of J's columns t_b = dx/dxi_b: row b
 * of J^-1 is (t_{b+1} x t_{b+2}) / det J, so G_bc = w (n_b . n_c) / det J
 * with n_b those cross products.  (The GPU generator inverts J by cofactors
 * per point and recomputes the corners at every point; the two agree to
 * rounding, not bit for bit.)
 *
 * Rules: Gauss-Legendre points are the roots of P_n, Gauss-Lobatto-Legendre
 * points +-1 and the roots of P'_{n-1}, both by Newton's method on the
 * three-term recurrence; Lagrange matrices by the barycentric formulas
 * (Berrut, Trefethen, "Barycentric Lagrange interpolation", SIAM Review
 * 2004). */

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#define PI_D 3.14159265358979323846

uint64_t bko_splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* U(s, i) with the stream's key k = splitmix64(s) already formed. */
static double u01(uint64_t key, uint64_t i)
{
    const uint64_t bits = bko_splitmix64(key + i) >> 11;
    return (double)bits / 9007199254740992.0;
}

double bko_uniform01(uint64_t seed, uint64_t i) { return u01(bko_splitmix64(seed), i); }

void bko_fill_uniform(double* out, size_t n, uint64_t seed, double lo, double hi)
{
    const uint64_t key = bko_splitmix64(seed);
    long long i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (long long)n; ++i) out[i] = lo + (hi - lo) * u01(key, (uint64_t)i);
}

void bko_fill_lognormal(double* out, size_t n, uint64_t seed, double sigma)
{
    const uint64_t key = bko_splitmix64(seed);
    long long i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (long long)n; ++i) {
        const double a = 1.0 - u01(key, 2 * (uint64_t)i);
        const double b = u01(key, 2 * (uint64_t)i + 1);
        out[i] = exp(sigma * (sqrt(-2.0 * log(a)) * cos(2.0 * PI_D * b)));
    }
}

/* ---- 1-D rules -------------------------------------------------------------- */

/* P_n(x) and P_n'(x) by the recurrence (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}. */
static void legendre(int n, double x, double* p, double* dp)
{
    double p0 = 1.0, p1 = x;
    int k;
    if (n == 0) {
        *p = 1.0;
        *dp = 0.0;
        return;
    }
    for (k = 1; k < n; ++k) {
        const double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
        p0 = p1;
        p1 = p2;
    }
    *p = p1;
    /* (1 - x^2) P_n' = n (P_{n-1} - x P_n) */
    *dp = n * (p0 - x * p1) / (1.0 - x * x);
}

/* Gauss-Legendre: n points, ascending. */
int bko_gauss(int n, double* x, double* w)
{
    int i, it;
    if (n < 1 || n > 64) return -1;
    for (i = 0; i < n; ++i) {
        /* Chebyshev-like first guess of the (n - i)-th root, descending */
        double r = cos(PI_D * (i + 0.75) / (n + 0.5)), p, dp;
        for (it = 0; it < 100; ++it) {
            double d;
            legendre(n, r, &p, &dp);
            d = p / dp;
            r -= d;
            if (fabs(d) < 1e-17) break;
        }
        legendre(n, r, &p, &dp);
        x[n - 1 - i] = r;
        w[n - 1 - i] = 2.0 / ((1.0 - r * r) * dp * dp);
    }
    return 0;
}

/* Gauss-Lobatto-Legendre: n >= 2 points, ascending; interior points are the
 * roots of P'_{n-1}, weights 2 / (n (n-1) P_{n-1}(x)^2). */
int bko_gll(int n, double* x, double* w)
{
    const int m = n - 1;
    int i, it;
    if (n < 2 || n > 64) return -1;
    x[0] = -1.0;
    x[m] = 1.0;
    for (i = 1; i < m; ++i) {
        /* roots of P'_m interleave those of P_m: start from the Chebyshev-
         * Gauss-Lobatto point, Newton on q(x) = (1 - x^2) P'_m(x), whose
         * derivative is -m (m + 1) P_m(x) */
        double r = -cos(PI_D * i / m), p, dp;
        for (it = 0; it < 100; ++it) {
            double q, d;
            legendre(m, r, &p, &dp);
            q = (1.0 - r * r) * dp;
            d = q / (-(double)m * (m + 1) * p);
            r -= d;
            if (fabs(d) < 1e-17) break;
        }
        x[i] = r;
    }
    for (i = 0; i < n; ++i) {
        double p, dp;
        if (i == 0 || i == m) {
            p = (i == 0 && (m & 1)) ? -1.0 : 1.0;
        } else {
            legendre(m, x[i], &p, &dp);
        }
        w[i] = 2.0 / ((double)m * n * p * p);
    }
    return 0;
}

static void bary_weights(int n, const double* x, double* lam)
{
    int i, j;
    for (i = 0; i < n; ++i) {
        double prod = 1.0;
        for (j = 0; j < n; ++j)
            if (j != i) prod *= (x[i] - x[j]);
        lam[i] = 1.0 / prod;
    }
}

/* B[i*np + p] = l_i(pts[p]), l_i the Lagrange polynomials of `nodes`. */
int bko_lagrange_interp(int nn, const double* nodes, int np, const double* pts, double* B)
{
    double lam[64];
    int i, p;
    if (nn < 1 || nn > 64 || np < 1) return -1;
    bary_weights(nn, nodes, lam);
    for (p = 0; p < np; ++p) {
        int hit = -1;
        double den = 0.0;
        for (i = 0; i < nn; ++i)
            if (pts[p] == nodes[i]) hit = i;
        if (hit >= 0) {
            for (i = 0; i < nn; ++i) B[i * np + p] = (i == hit) ? 1.0 : 0.0;
            continue;
        }
        for (i = 0; i < nn; ++i) den += lam[i] / (pts[p] - nodes[i]);
        for (i = 0; i < nn; ++i) B[i * np + p] = lam[i] / (pts[p] - nodes[i]) / den;
    }
    return 0;
}

/* D[i*n + j] = l_j'(x_i): off the diagonal (lam_j / lam_i) / (x_i - x_j), on it
 * minus the sum of the row's other entries (the derivative of a constant). */
int bko_lagrange_deriv(int n, const double* x, double* D)
{
    double lam[64];
    int i, j;
    if (n < 1 || n > 64) return -1;
    bary_weights(n, x, lam);
    for (i = 0; i < n; ++i) {
        double s = 0.0;
        for (j = 0; j < n; ++j) {
            if (j == i) continue;
            D[i * n + j] = (lam[j] / lam[i]) / (x[i] - x[j]);
            s += D[i * n + j];
        }
        D[i * n + i] = -s;
    }
    return 0;
}

/* ---- geometry --------------------------------------------------------------- */

static void cross3(const double* a, const double* b, double* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Columns t[b] = dx/dxi_b of J, weight w -> det J and the six factors of
 * G = w det J J^-1 J^-T (rr rs rt ss st tt). */
static double factors(const double t[3][3], double w, double g[6])
{
    double n[3][3];
    double det;
    cross3(t[1], t[2], n[0]);
    cross3(t[2], t[0], n[1]);
    cross3(t[0], t[1], n[2]);
    det = dot3(t[0], n[0]);
    g[0] = w * dot3(n[0], n[0]) / det;
    g[1] = w * dot3(n[0], n[1]) / det;
    g[2] = w * dot3(n[0], n[2]) / det;
    g[3] = w * dot3(n[1], n[1]) / det;
    g[4] = w * dot3(n[1], n[2]) / det;
    g[5] = w * dot3(n[2], n[2]) / det;
    return det;
}

static size_t g_index(int Q, int layout, int i, int j, int f, int k)
{
    if (layout == 0) return (((size_t)f * Q + i) * Q + j) * Q + k;
    if (layout == 1) return (((size_t)i * Q + j) * 6 + f) * Q + k;
    return (((size_t)f * Q + k) * Q + i) * Q + j;
}

static void store_point(int Q, int layout, double* Ge, int i, int j, int k, const double g[6])
{
    int f;
    for (f = 0; f < 6; ++f) Ge[g_index(Q, layout, i, j, f, k)] = g[f];
}

/* Affine mesh, elements e0 .. e0 + ne - 1 of the configuration (the outputs
 * hold those elements only): qdata (ne x Q^3) and G (ne x 6 Q^3 in `layout`),
 * each may be NULL. */
void bko_geom_affine(int Q, size_t e0, size_t ne, const double* x, const double* w, uint64_t seed, double h,
                     double pert, double* qdata, double* G, int layout)
{
    const uint64_t key = bko_splitmix64(seed);
    const size_t Q3 = (size_t)Q * Q * Q;
    long long le;
    (void)x; /* J is constant over an affine element */
#pragma omp parallel for schedule(static)
    for (le = 0; le < (long long)ne; ++le) {
        const uint64_t e = e0 + (uint64_t)le;
        double t[3][3];
        int a, b, i, j, k;
        /* column b of J: (h/2)(e_b + P_e[:, b]) */
        for (b = 0; b < 3; ++b)
            for (a = 0; a < 3; ++a)
                t[b][a] = 0.5 * h * ((a == b ? 1.0 : 0.0) + pert * (2.0 * u01(key, e * 9 + 3 * a + b) - 1.0));
        for (i = 0; i < Q; ++i) for (j = 0; j < Q; ++j) for (k = 0; k < Q; ++k) {
            double g[6];
            const double wp = w[i] * w[j] * w[k];
            const double det = factors(t, wp, g);
            const size_t pt = ((size_t)i * Q + j) * Q + k;
            if (qdata) qdata[(size_t)le * Q3 + pt] = wp * det;
            if (G) store_point(Q, layout, G + (size_t)le * 6 * Q3, i, j, k, g);
        }
    }
}

/* Physical coordinates (ne x Q^3 x 3) of the affine mesh's points. */
void bko_coords_affine(int Q, size_t e0, size_t ne, int nx, int ny, const double* x, uint64_t seed, double h,
                       double pert, double* coords)
{
    const uint64_t key = bko_splitmix64(seed);
    const size_t Q3 = (size_t)Q * Q * Q;
    long long le;
#pragma omp parallel for schedule(static)
    for (le = 0; le < (long long)ne; ++le) {
        const uint64_t e = e0 + (uint64_t)le;
        const double cell[3] = {(double)(e % (uint64_t)nx), (double)((e / (uint64_t)nx) % (uint64_t)ny),
                                (double)(e / ((uint64_t)nx * (uint64_t)ny))};
        double J[3][3];
        int a, b, i, j, k;
        for (a = 0; a < 3; ++a)
            for (b = 0; b < 3; ++b)
                J[a][b] = 0.5 * h * ((a == b ? 1.0 : 0.0) + pert * (2.0 * u01(key, e * 9 + 3 * a + b) - 1.0));
        for (i = 0; i < Q; ++i) for (j = 0; j < Q; ++j) for (k = 0; k < Q; ++k) {
            const double xi[3] = {x[i], x[j], x[k]};
            double* o = coords + 3 * ((size_t)le * Q3 + ((size_t)i * Q + j) * Q + k);
            for (a = 0; a < 3; ++a) o[a] = (cell[a] + 0.5) * h + dot3(J[a], xi);
        }
    }
}

/* Jittered trilinear mesh on an nx x ny x .. grid, elements e0 .. e0+ne-1:
 * G (layout), mass = w det J and coordinates, each may be NULL. */
void bko_geom_trilinear(int Q, size_t e0, size_t ne, int nx, int ny, const double* x, const double* w,
                        uint64_t seed, double h, double jit, double* G, int layout, double* mass, double* coords)
{
    const uint64_t key = bko_splitmix64(seed);
    const size_t Q3 = (size_t)Q * Q * Q;
    long long le;
#pragma omp parallel for schedule(static)
    for (le = 0; le < (long long)ne; ++le) {
        const uint64_t e = e0 + (uint64_t)le;
        const uint64_t cx = e % (uint64_t)nx, cy = (e / (uint64_t)nx) % (uint64_t)ny,
                       cz = e / ((uint64_t)nx * (uint64_t)ny);
        double V[2][2][2][3]; /* V[c][b][a] = corner (cx + a, cy + b, cz + c) */
        int a, b, c, d, i, j, k;
        for (c = 0; c < 2; ++c) for (b = 0; b < 2; ++b) for (a = 0; a < 2; ++a) {
            const uint64_t v[3] = {cx + a, cy + b, cz + c};
            const uint64_t id = v[0] + ((uint64_t)nx + 1) * (v[1] + ((uint64_t)ny + 1) * v[2]);
            for (d = 0; d < 3; ++d)
                V[c][b][a][d] = h * ((double)v[d] + jit * (2.0 * u01(key, 3 * id + d) - 1.0));
        }
        for (i = 0; i < Q; ++i) for (j = 0; j < Q; ++j) for (k = 0; k < Q; ++k) {
            /* linear shape functions per direction and their derivatives */
            const double s0[2] = {0.5 * (1.0 - x[i]), 0.5 * (1.0 + x[i])};
            const double s1[2] = {0.5 * (1.0 - x[j]), 0.5 * (1.0 + x[j])};
            const double s2[2] = {0.5 * (1.0 - x[k]), 0.5 * (1.0 + x[k])};
            double t[3][3], X[3] = {0.0, 0.0, 0.0};
            const size_t pt = ((size_t)i * Q + j) * Q + k;
            for (d = 0; d < 3; ++d) {
                /* dx/dxi_0: half the differences along a, weighted in b, c */
                t[0][d] = 0.0;
                t[1][d] = 0.0;
                t[2][d] = 0.0;
                for (c = 0; c < 2; ++c) for (b = 0; b < 2; ++b)
                    t[0][d] += s1[b] * s2[c] * 0.5 * (V[c][b][1][d] - V[c][b][0][d]);
                for (c = 0; c < 2; ++c) for (a = 0; a < 2; ++a)
                    t[1][d] += s0[a] * s2[c] * 0.5 * (V[c][1][a][d] - V[c][0][a][d]);
                for (b = 0; b < 2; ++b) for (a = 0; a < 2; ++a)
                    t[2][d] += s0[a] * s1[b] * 0.5 * (V[1][b][a][d] - V[0][b][a][d]);
                for (c = 0; c < 2; ++c) for (b = 0; b < 2; ++b) for (a = 0; a < 2; ++a)
                    X[d] += s0[a] * s1[b] * s2[c] * V[c][b][a][d];
            }
            {
                double g[6];
                const double wp = w[i] * w[j] * w[k];
                const double det = factors(t, wp, g);
                if (G) store_point(Q, layout, G + (size_t)le * 6 * Q3, i, j, k, g);
                if (mass) mass[(size_t)le * Q3 + pt] = wp * det;
                if (coords) memcpy(coords + 3 * ((size_t)le * Q3 + pt), X, sizeof X);
            }
        }
    }
}
