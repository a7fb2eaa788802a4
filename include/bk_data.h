/* bk_data.h -- C ABI of the input generators of the benchmark configurations
 * (1-D rules and Lagrange matrices on the host; seeded fields and mesh
 * geometry on the GPU, in FP64).  The reference has no counterpart: its
 * drivers use a cosine test basis and constant or LCG data
 * (include/bk_common.h:60-107), which the oracle restates.  Return values are
 * bk_status codes (bk_gpu.h). */
#ifndef BK_DATA_H
#define BK_DATA_H

#include "bk_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Gauss-Legendre points/weights on [-1,1], ascending (n = 1..64). */
int bk_gauss_points(int n, double* x, double* w);
/* Gauss-Lobatto-Legendre points/weights on [-1,1], ascending (n = 2..64). */
int bk_gll_points(int n, double* x, double* w);
/* B[i*npts + p] = l_i(pts[p]) for the Lagrange polynomials of `nodes`. */
int bk_lagrange_interp(int nnodes, const double* nodes, int npts, const double* pts, double* B);
/* D[i*n + j] = l_j'(x_i), the collocation derivative on the points x. */
int bk_lagrange_deriv(int n, const double* x, double* D);

/* Device fields (f64 != 0: double, else float), seeded by index. */
int bk_fill_uniform(void* out, long long n, unsigned long long seed, double lo, double hi, int f64,
                    bk_stream_t stream);
int bk_fill_lognormal(void* out, long long n, unsigned long long seed, double sigma, int f64,
                      bk_stream_t stream);

/* Affine mesh (x = c_e + (h/2)(I + delta_e) xi, delta ~ U[-pert, pert]):
 * qdata = w detJ (E x Q^3) and/or G = w detJ J^-1 J^-T (E x 6 x Q^3, layout
 * 0/1/2 as bk_layout); x, w: host, Q points and weights. */
int bk_geom_affine(int Q, long long E, const double* x, const double* w, unsigned long long seed,
                   double h, double pert, double* qdata, double* G, int layout, bk_stream_t stream);
int bk_coords_affine(int Q, long long E, int nx, int ny, const double* x, unsigned long long seed,
                     double h, double pert, double* coords, bk_stream_t stream);
/* Trilinear mesh of a jittered nx x ny x .. grid (vertex jitter U[-jit h, jit h]):
 * G (layout), mass = w detJ, coordinates (E x Q^3 x 3); each may be NULL. */
int bk_geom_trilinear(int Q, long long E, int nx, int ny, const double* x, const double* w,
                      unsigned long long seed, double h, double jit, double* G, int layout,
                      double* mass, double* coords, bk_stream_t stream);
/* double -> float (to_f32 != 0) or float -> double on the device. */
int bk_convert(const void* in, void* out, long long n, int to_f32, bk_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BK_DATA_H */
