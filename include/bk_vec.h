/* bk_vec.h -- C ABI of the vector kernels around the operator apply: STREAM
 * bandwidth kernels (the in-run roofline denominators; the reference's
 * roofline/stream_omp.cpp:32-120 is the counterpart) and the FP64 dot product
 * and axpby of the solvers (no reference counterpart: the reference has no
 * solver).  Return values are bk_status codes (bk_gpu.h). */
#ifndef BK_VEC_H
#define BK_VEC_H

#include "bk_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum bk_stream_kind {
    BK_STREAM_COPY = 0,   /* a = b */
    BK_STREAM_TRIAD = 1,  /* a = b + 3 c */
    BK_STREAM_MIX = 2     /* a[i] = sum_r b[r*n + i], r < reads: `reads` arrays read per array written */
};

/* One STREAM kernel over n_bytes per array (a multiple of 16); device
 * pointers 16-byte aligned; for MIX, b holds `reads` arrays of n_bytes. */
int bk_stream_kernel(int kind, long long n_bytes, void* a, const void* b, const void* c, int reads,
                     bk_stream_t stream);

/* Bytes of device workspace bk_dot needs for n values (one double per block
 * of the first pass; at most 1216 doubles). */
long long bk_dot_workspace_bytes(long long n);

/* *result (device) = sum_i x[i] y[i] (half != 0: half of it), accumulated in
 * FP64 in a fixed order (deterministic).  x, y: double (f64 != 0) or float.
 * workspace: device, at least bk_dot_workspace_bytes(n) bytes, owned by the
 * caller; its contents are overwritten. */
int bk_dot(long long n, const void* x, const void* y, int f64, double* result, void* workspace,
           long long workspace_bytes, int half, bk_stream_t stream);

/* The same dot product with no workspace argument and no allocation, for
 * callers that cannot allocate device memory (no counterpart in the
 * reference, whose host loops need no scratch).  Its partial sums live in a
 * fixed 32 KiB array of this library on each device (4096 doubles, one per
 * chunk of 65536 values): n <= BK_DOT_NOALLOC_MAX_N = 268,435,456, larger n
 * returns BK_ERR_SIZE.  The first call on a device looks the array's device
 * address up (cudaGetSymbolAddress): make it before capturing a stream.
 * Calls share the array: calls that overlap on the GPU race on it. */
#define BK_DOT_NOALLOC_MAX_N 268435456LL
int bk_dot_noalloc(long long n, const void* x, const void* y, int f64, double* result, int half,
                   bk_stream_t stream);

/* y = a x + b y (double or float vectors, FP64 scalars). */
int bk_axpby(long long n, double a, const void* x, double b, void* y, int f64, bk_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BK_VEC_H */
