/* bk_solver.h -- C ABI of the batched mixed-order Helmholtz operator and its
 * CG solver (no reference counterpart: the reference has neither mixed orders
 * nor a solver).  Return values are bk_status codes (bk_gpu.h).
 *
 * Data: the elements of each order are stored one order after another, in
 * the order of the plan's ranges: u, v, mass (the collocated GLL mass w detJ)
 * with E_p (p+1)^3 values per order, G with E_p 6 (p+1)^3 values per order in
 * the column layout G(e, f, k, i, j) (BK_LAYOUT_COLUMN).  The operator is
 *     v = D^T G D u + lambda mass .* u
 * (BK5, openmp/BK5.cpp:19-103, plus the diagonal term), orders p = 2..8. */
#ifndef BK_SOLVER_H
#define BK_SOLVER_H

#include "bk_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { BK_ERR_NOCONV = 9 };   /* the solver stopped above its tolerance */

typedef struct bk_order_range {
    int p;               /* polynomial order, 2..8 (q = p + 1 points) */
    int64_t E;           /* elements of this order */
    int elems_per_tile;  /* elements per tile of the persistent launch, with
                            elems_per_tile * q^2 <= 1024 (the column body:
                            <= 256, one thread per column); 0: about 128 / q^2 */
} bk_order_range;

typedef struct bk_hplan* bk_hplan_t;

/* A plan over norders (1..7) ranges; D[r] is the host (p+1) x (p+1) GLL
 * derivative of range r, D(i,n) = D[r][i*q + n].  Allocates the tile list
 * and the solver's work vectors on the current device (once, here: the
 * applies and solves allocate nothing).  Synchronizes `stream`. */
int bk_hplan_create(bk_hplan_t* plan, int norders, const bk_order_range* orders, const double* const* D,
                    bk_stream_t stream);
int bk_hplan_destroy(bk_hplan_t plan);
/* what = 0: values of a vector (sum E_p q^3); 1: values of G; 2: tiles;
 * 3: the kernel shape of the applies (BK_KERNEL_SWEEP or BK_KERNEL_COLUMN);
 * 4, 5: shared memory per block of the sweep body's launch for FP64 / FP32
 * storage (a launch needs at most 232448 bytes); 6, 7: the threads and G
 * staging set by bk_hplan_set_shape; 8, 9: the tiles and threads of the
 * FP64-storage launches (bk_hplan_set_fp64_shape). */
long long bk_hplan_size(bk_hplan_t plan, int what);

/* The body of the persistent launch: BK_KERNEL_SWEEP (line sweeps in the
 * even-odd form, half the multiply-adds; needs every D centro-antisymmetric,
 * which GLL derivatives are, BK_ERR_ARG otherwise), BK_KERNEL_COLUMN (one
 * thread per k-column, any D) or BK_KERNEL_AUTO (SWEEP when possible: the
 * default of a new plan). */
int bk_hplan_set_kernel(bk_hplan_t plan, int kernel);

/* The shape of the even-odd sweep body's persistent launch.  threads: per
 * block, a multiple of 32 in 64..256, or 0 (the default) for the largest
 * tile's lines (elements x q^2, at most 256); tiles with more lines than
 * threads loop over their lines, so tile sizes per order and the block are
 * chosen apart.  The FP64 launch runs three thread groups of that size (one
 * per direction).  gstage (FP32 storage): 1 stages each tile's G into shared
 * memory by TMA, 0 (the default) reads it in the pointwise stage straight
 * from global memory, prefetched into L2 one tile ahead.  omp_bk_gb300.tune
 * chooses both by measurement.  BK_ERR_ARG for other values. */
int bk_hplan_set_shape(bk_hplan_t plan, int threads, int gstage);

/* The shape of the sweep body's FP64-storage launches (the float-float and
 * DFMA applies, among them the solver's FP64 residual) apart from the FP32
 * storage launches, whose arithmetic costs differ: elems_per_tile[r] for
 * range r (elems_per_tile * q^2 <= 1024; 0 keeps the range's own) and
 * threads as in bk_hplan_set_shape.  elems_per_tile NULL returns the FP64
 * launches to the plan's tiles and threads.  Builds the FP64 tile list on
 * the device (allocates; synchronizes `stream`, and the device when a list
 * is replaced).  bk_hplan_set_shape sets the threads of both launches: call
 * this after it.  BK_ERR_ARG for sizes out of range. */
int bk_hplan_set_fp64_shape(bk_hplan_t plan, const int* elems_per_tile, int threads, bk_stream_t stream);

/* v = A u for all orders in ONE persistent launch.  prec BK_PREC_FP64 (engine
 * AUTO/FF: float-float, DFMA: native), BK_PREC_MIXED or BK_PREC_FP32 (float
 * storage).  mass may be NULL (plain BK5). */
int bk_hplan_apply(bk_hplan_t plan, const void* G, const void* mass, double lambda, const void* u, void* v,
                   int prec, int engine, bk_stream_t stream);

enum { BK_PRECOND_NONE = 0, BK_PRECOND_JACOBI = 1 };

typedef struct bk_cg_options {
    double rtol;        /* stop at |f - A x| <= rtol |f| (FP64 residual); default 1e-10 */
    int max_outer;      /* refinement steps; default 8 */
    double inner_rtol;  /* inner FP32 CG tolerance, relative, on r.z (the
                           residual in the preconditioner's norm); default 1e-5 */
    int max_inner;      /* inner iterations per refinement step; default 10000 */
    int precond;        /* inner CG preconditioner: BK_PRECOND_JACOBI (the
                           default with opt NULL: z = r / diag(A)) or
                           BK_PRECOND_NONE */
} bk_cg_options;

typedef struct bk_cg_stats {
    int outer;          /* refinement steps taken */
    int inner;          /* inner CG iterations, all steps */
    double relres;      /* final |f - A x| / |f| in FP64 */
} bk_cg_stats;

/* The diagonal of A = K + lambda M at every point (FP64; G, mass as for
 * bk_hplan_apply in double, mass may be NULL): the sums of D(n,i)^2 times the
 * diagonal factors along the three lines through the point and the mixed
 * factors at the point (the element operators are independent, so this is
 * the assembled diagonal too).  The inner CG's Jacobi preconditioner. */
int bk_hplan_diagonal(bk_hplan_t plan, const void* G, const void* mass, double lambda, double* diag,
                      bk_stream_t stream);

/* Solves A x = f (x holds the initial guess; f, x FP64 device vectors).
 * The residual is formed in FP64 with G64/mass64 (double); the inner CG
 * applies the FP32-storage operator G32/mass32 (float) with FP64 dot
 * products, its iterations captured once per operator in a CUDA graph with a
 * conditional WHILE node (no host round trip inside a solve).  Returns BK_OK,
 * BK_ERR_NOCONV if rtol was not reached, or an error.  opt, stats may be NULL. */
int bk_hplan_cg(bk_hplan_t plan, const void* G64, const void* mass64, const void* G32, const void* mass32,
                double lambda, const double* f, double* x, const bk_cg_options* opt, bk_cg_stats* stats,
                bk_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BK_SOLVER_H */
