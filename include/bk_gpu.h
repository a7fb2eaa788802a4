/* bk_gpu.h -- C ABI of the GB300 bake-off operator apply (BK1 mass, BK3
 * Poisson, BK5 collocated Laplacian) on element-major hexahedral E-vectors.
 *
 * The reference (ivan-pi/omp_bk) has no library and no FFI: its "interface"
 * is the kernel template
 *     template <typename T, int nq> void bk::SumFactorization(
 *         std::size_t nelmt, const T* basis, const T* JxW|G, const T* in, T* out)
 * (openmp/bk1_sumfact.h:16-22, openmp/bk3_sumfact.h:17-24 with basis and
 * dbasis, openmp/BK5.cpp:18-24 with dbasis), called by the drivers through the
 * function-pointer type sumfact_kernel<T> (openmp/bk1_sumfact.h:161-163) and
 * the variant tables of the GPU harnesses.  Each entry point below replaces one
 * of those templates for every order p = 1..8 at once (run-time p dispatched to
 * a compile-time nq, as bk::with_order does, include/bk_common.h:148-178).
 *
 * Conventions (all entry points):
 *   - p is the polynomial order; BK1/BK3 use P = p + 1 nodes and Q = p + 2
 *     points per direction (openmp/BK1.cpp:41), BK5 uses Q = p + 1
 *     (openmp/BK5.cpp:153).  E is the number of elements (0 is a no-op).
 *   - The 1-D matrices (B, D) are HOST pointers to row-major doubles in the
 *     reference's convention: B(i,p) = B[i*Q + p] (P x Q, node-major,
 *     bk1_sumfact.h:39); BK3's D(n,p) = D[n*Q + p] (bk3_sumfact.h:41); BK5's
 *     D(i,n) = D[i*Q + n] (BK5.cpp:290).  They are at most 10 x 10 and are
 *     passed by value into the launch (constant bank): no device copy, no
 *     allocation, safe to capture in a CUDA graph.
 *   - All other arrays are DEVICE pointers, 16-byte aligned, element-major with
 *     the last index fastest, in the storage type of `prec`: double for
 *     BK_PREC_FP64, float for BK_PREC_FP32 and BK_PREC_MIXED.
 *   - The call is asynchronous on `stream` (0: the legacy default stream),
 *     allocates nothing and synchronizes nothing.  Calls on distinct streams
 *     may run concurrently.
 *   - Return value: BK_OK or one of the BK_ERR_* codes below.  Argument errors
 *     are detected on the host before any launch.  Errors that only the GPU
 *     can see (a bounded wait that gave up) are recorded in a device status
 *     word read by bk_device_status().
 */
#ifndef BK_GPU_H
#define BK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A CUDA stream (cudaStream_t); declared here so that callers need no CUDA
 * header. */
typedef struct CUstream_st* bk_stream_t;

/* ---- status codes --------------------------------------------------------- */
enum bk_status {
    BK_OK = 0,
    BK_ERR_ORDER = 1,    /* p outside 1..8: the reference's with_order prints
                            "unsupported polynomial order p" (bk_common.h:170-177) */
    BK_ERR_SIZE = 2,     /* E < 0, or an index would overflow 64 bits */
    BK_ERR_ALIGN = 3,    /* a device pointer is not 16-byte aligned */
    BK_ERR_NULL = 4,     /* a required pointer is NULL (E > 0) */
    BK_ERR_PREC = 5,     /* unknown precision, engine, layout or factor count */
    BK_ERR_CUDA = 6,     /* a CUDA launch or copy failed */
    BK_ERR_TIMEOUT = 7,  /* a device-side wait gave up (device status only) */
    BK_ERR_ARG = 8       /* another invalid argument */
};

/* ---- precision forms ------------------------------------------------------ */
enum bk_prec {
    BK_PREC_FP64 = 0,   /* FP64 storage, FP64-accurate arithmetic (engine below) */
    BK_PREC_FP32 = 1,   /* FP32 storage and arithmetic: the reference drivers'
                           T = float (openmp/BK1.cpp:41, BK3.cpp:60, BK5.cpp:153) */
    BK_PREC_MIXED = 2   /* FP32 storage and FP32 FMA contractions, the final
                           sum of the three directional terms compensated
                           (float-float); used inside FP64-refined solvers */
};

/* ---- FP64 arithmetic engines (BK_PREC_FP64 only) -------------------------- */
enum bk_engine {
    BK_ENGINE_AUTO = 0, /* the fastest engine that meets 1e-12 (float-float) */
    BK_ENGINE_DFMA = 1, /* native FP64 FMA */
    BK_ENGINE_FF = 2    /* float-float on the FP32 pipes: values split into
                           two floats (~48 significant bits) as they are
                           loaded, joined back to double as they are stored
                           (the technique of openmp/float_float.h) */
};

/* BK5 geometric-factor layouts (make_bk5_G, include/bk_harness.h:217-219). */
enum bk_layout {
    BK_LAYOUT_FACTOR = 0,      /* G(e, f, i, j, k) */
    BK_LAYOUT_INTERLEAVED = 1, /* G(e, i, j, f, k): BK5.cpp's layout (:42, :296) */
    BK_LAYOUT_COLUMN = 2       /* G(e, f, k, i, j) */
};

/* Options of the extended entry points; a NULL bk_options* means defaults. */
typedef struct bk_options {
    int prec;      /* bk_prec */
    int engine;    /* bk_engine (FP64 only) */
    int layout;    /* BK5: bk_layout; BK3 reads G factor-major (bk3_sumfact.h:53) */
    int nfactors;  /* BK5: 6 (symmetric rr rs rt ss st tt) or 9 (full 3x3,
                      row-major; bk5_offload.cpp "F") */
    int elems_per_block; /* BK5 column kernel: elements per thread block, 0
                            or its default (other values BK_ERR_ARG); the
                            sweep kernels use per-order tables measured on
                            GB300 and ignore it */
    int kernel;    /* bk_kernel_shape (BK5); BK1/BK3 have the sweep kernel only */
    int gform;     /* bk_gform (BK5, BK3, the adjoint): how G is stored */
    int jxw_layout; /* bk_jxw_layout (BK1): the order of qdata's points */
} bk_options;

/* BK1 qdata ("JxW") layouts. */
enum bk_jxw_layout {
    BK_JXW_PQR = 0,  /* JxW(e, p, q, r), r fastest: bk1_sumfact.h's layout (:53) */
    BK_JXW_RQP = 1   /* JxW_t(e, r, q, p), p fastest: the layout transpose_jxw
                        makes (include/bk_harness.h:89-102) and the SYCL BK1
                        variants read (sycl/bk1_sycl.cpp:74-98) */
};

/* Geometric-factor storage forms (BK5, BK3). */
enum bk_gform {
    BK_G_STORAGE = 0, /* the storage type of prec (double for FP64) */
    BK_G_FF = 1       /* float-float pairs (float hi, float lo; 8 bytes per
                         value, the same footprint as double) made once by
                         bk_g_to_ff: the float-float engine then skips the
                         split of every G value it loads.  The pair is the
                         split the engine applies to a double, so the apply's
                         result is bitwise that of the double G.  FP64 with
                         engine AUTO or FF and the even-odd path: BK5 with 6
                         factors, D on points symmetric about 0 (GLL), sweep
                         kernel; BK3 and its adjoint with B and D of GLL
                         nodes and Gauss points.  Otherwise (and for BK1,
                         which takes no G) BK_ERR_PREC */
};

/* BK5 kernel shapes. */
enum bk_kernel_shape {
    BK_KERNEL_AUTO = 0,   /* the faster of the two as measured on GB300: the
                             column kernel for the FP32-storage forms with G
                             in the column layout at p <= 3 and at p = 5
                             with a mass term, the sweep kernel otherwise */
    BK_KERNEL_SWEEP = 1,  /* one thread per line of the box per 1-D contraction,
                             all intermediates in shared memory */
    BK_KERNEL_COLUMN = 2  /* one thread per k-column of an element, the
                             k-direction and the pointwise products in
                             registers, TMA double buffering */
};

/* bk_options with the defaults: prec FP64, engine AUTO, BK5 layout
 * INTERLEAVED with 6 factors, elems_per_block 0, kernel AUTO, gform
 * STORAGE, jxw_layout PQR. */
bk_options bk_default_options(void);

/* ---- operator apply ------------------------------------------------------- */

/* BK1 mass operator v = B^T diag(qdata) B u per element
 * (replaces bk::SumFactorization<T, nq>, openmp/bk1_sumfact.h:16-159).
 *   B      host, P x Q doubles, B(i,p) = B[i*Q+p]
 *   qdata  device, E x Q^3 (quadrature weight x detJ, "JxW" in the reference),
 *          JxW(e,p,q,r); bk1_apply_opt with jxw_layout BK_JXW_RQP reads
 *          JxW_t(e,r,q,p) instead
 *   u, v   device, E x P^3 */
int bk1_apply(int p, int64_t E, const double* B, const void* qdata, const void* u, void* v,
              int prec, bk_stream_t stream);

/* BK3 Poisson operator v = B^T D^T G D B u per element
 * (replaces bk::SumFactorization<T, nq>, openmp/bk3_sumfact.h:17-187).
 *   B      host, P x Q doubles; D host, Q x Q doubles, D(n,p) = D[n*Q+p]
 *   G      device, E x 6 x Q^3, factor-major (rr rs rt ss st tt)
 *   u, v   device, E x P^3 */
int bk3_apply(int p, int64_t E, const double* B, const double* D, const void* G, const void* u,
              void* v, int prec, bk_stream_t stream);

/* BK5 collocated Laplacian v = D^T G D u per element
 * (replaces bk::SumFactorization<T, nq>, openmp/BK5.cpp:18-103).
 *   D      host, Q x Q doubles, D(i,n) = D[i*Q+n]
 *   G      device, E x 6 x Q^3 interleaved G(e,i,j,f,k) (BK5.cpp:296)
 *   u, v   device, E x Q^3 */
int bk5_apply(int p, int64_t E, const double* D, const void* G, const void* u, void* v, int prec,
              bk_stream_t stream);

/* The same with options (engine, BK5 layout and factor count, block shape):
 * the variants of the reference's kernel harnesses (bk5_offload.cpp:7-28,
 * variant table :716-772) behind one entry point.  opt may be NULL. */
int bk1_apply_opt(int p, int64_t E, const double* B, const void* qdata, const void* u, void* v,
                  const bk_options* opt, bk_stream_t stream);
int bk3_apply_opt(int p, int64_t E, const double* B, const double* D, const void* G,
                  const void* u, void* v, const bk_options* opt, bk_stream_t stream);
int bk5_apply_opt(int p, int64_t E, const double* D, const void* G, const void* u, void* v,
                  const bk_options* opt, bk_stream_t stream);

/* BK5 plus a diagonal term: v = D^T G D u + lambda * mass .* u (the
 * Helmholtz operator with the collocated GLL mass, no reference counterpart).
 * mass: device, E x Q^3 in the storage type, or NULL for plain BK5. */
int bk5_apply_ex(int p, int64_t E, const double* D, const void* G, const void* u, const void* mass,
                 double lambda, void* v, const bk_options* opt, bk_stream_t stream);

/* BK3 with a coefficient at the quadrature points: the fluxes are
 * k(x) G(x) grad u(x) (no reference counterpart; the forward operator of the
 * adjoint below).  k: device, E x Q^3, or NULL for plain BK3. */
int bk3_apply_k(int p, int64_t E, const double* B, const double* D, const void* G, const void* k,
                const void* u, void* v, const bk_options* opt, bk_stream_t stream);

/* Backward of the variable-coefficient BK3 operator (no reference
 * counterpart).  For L = 1/2 |A(k) u - f|^2 and res = A(k) u - f (computed
 * by the caller with bk3_apply_k and an axpby):
 *   dk(e, x)    = dL/dk at every quadrature point           (E x Q^3)
 *   dG(e, f, x) = dL/dG for the six stored symmetric factors  (E x 6 x Q^3,
 *                 factor-major; an off-diagonal factor stands for both of
 *                 its entries)
 * The gradients of u and res at the points are recomputed, not stored.  The
 * operator is symmetric, so dL/du = A(k) res is bk3_apply_k itself. */
int bk3_adjoint(int p, int64_t E, const double* B, const double* D, const void* G, const void* k,
                const void* u, const void* res, void* dk, void* dG, const bk_options* opt,
                bk_stream_t stream);

/* BK5's BK_KERNEL_AUTO per order p, precision, engine, layout and mass term
 * (with_mass 0/1: bk5_apply_ex with or without a mass array): kernel
 * BK_KERNEL_SWEEP or BK_KERNEL_COLUMN fixes the shape AUTO uses there,
 * BK_KERNEL_AUTO restores the built-in choice (the column kernel for FP32
 * storage with G in the column layout at p <= 3 and at p = 5 with a mass
 * term, the sweep kernel otherwise).  A tuner sets these from measurements (omp_bk_gb300.tune:
 * tune_apply); the table is process-wide, so a process should set it before
 * its applies run concurrently with the change.  G split ahead of time
 * (BK_G_FF) always takes the sweep kernel.  No reference counterpart: it
 * plays the part of the harnesses' per-order variant pick
 * (openmp/offload/bk5_offload.cpp:750-772). */
int bk5_set_auto_kernel(int p, int prec, int engine, int layout, int with_mass, int kernel);
/* The kernel shape BK_KERNEL_AUTO takes for these arguments, or minus a
 * bk_status code for invalid ones. */
int bk5_auto_kernel(int p, int prec, int engine, int layout, int with_mass);

/* make_bk5_G on the device (replaces include/bk_harness.h:220-244): G6i,
 * the six symmetric factors interleaved as BK5.cpp stores them,
 * G6i(e, i, j, s, k) (g6i_index, bk_harness.h:210), into G with nfactors = 6
 * (rr rs rt ss st tt) or 9 (the full 3 x 3 tensor, row-major, bk5_sym :215)
 * in layout 0, 1 or 2 (bk_layout), for BK5 with Q = p + 1 points per
 * direction.  Both in the storage type of prec (double for FP64, float
 * otherwise), device, 16-byte aligned, distinct.  Asynchronous on stream. */
int bk5_make_g(int p, int64_t E, const void* G6i, void* G, int nfactors, int layout, int prec,
               bk_stream_t stream);

/* transpose_jxw on the device (replaces include/bk_harness.h:89-102):
 * JxW(e, p, q, r) -> JxW_t(e, r, q, p) for BK1 with Q = p + 2 points per
 * direction, in the storage type of prec; device, 16-byte aligned, distinct.
 * BK1 reads the result with jxw_layout = BK_JXW_RQP.  Asynchronous on
 * stream. */
int bk1_transpose_jxw(int p, int64_t E, const void* jxw, void* jxw_t, int prec, bk_stream_t stream);

/* Splits n doubles G (device) into float-float pairs Gff (device, n x 8
 * bytes; may be G itself: the conversion is in place value by value): hi =
 * the value truncated to 24 significant bits, lo = the rest rounded to a
 * float, exactly as the float-float engine splits a double it loads.  For
 * BK5 applies with gform = BK_G_FF; a one-time preparation of the operator,
 * like the reference's relayout of G (make_bk5_G, include/bk_harness.h:220).
 * Asynchronous on stream. */
int bk_g_to_ff(const void* G, void* Gff, int64_t n, bk_stream_t stream);

/* ---- device status -------------------------------------------------------- */

/* Reads (and, if reset != 0, clears) the status word of the current device:
 * BK_OK or the first device-side error (BK_ERR_TIMEOUT) recorded since the
 * last reset.  Synchronizes `stream`. */
int bk_device_status(int* status, int reset, bk_stream_t stream);

/* Test hook: the cycle limit of every bounded device-side wait on the current
 * device (default 4e9, about two seconds).  0 restores the default. */
int bk_set_wait_limit(long long cycles);

/* Test hook: launches one block that waits on a barrier nothing arrives on,
 * with the current wait limit; the wait gives up, records BK_ERR_TIMEOUT in
 * the status word and the kernel returns normally. */
int bk_test_wait_timeout(bk_stream_t stream);

/* Library version string. */
const char* bk_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BK_GPU_H */
