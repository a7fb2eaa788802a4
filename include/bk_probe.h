/* bk_probe.h -- a measurement entry point (no reference counterpart): one
 * 1-D contraction y = D x over lines of 8 doubles (the BK5 p = 7 derivative
 * direction) in FP64 accuracy by the float-float route of the operator
 * kernels or by exact byte slices on the tensor cores (mma.sync, bf16
 * products summed exactly in FP32), so that the two routes can be timed and
 * counted on the same data.  Not part of the operator path.  Return values
 * are bk_status codes (bk_gpu.h). */
#ifndef BK_PROBE_H
#define BK_PROBE_H

#include "bk_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum bk_probe_method {
    BK_PROBE_COPY = 0, /* load, split into float-float, join, store */
    BK_PROBE_FF = 1,   /* float-float even-odd contraction (FP32 pipes) */
    BK_PROBE_MMA = 2   /* exact byte slices on the tensor cores */
};

/* nlines lines of 8 doubles, x and y device arrays (16-byte aligned; for
 * BK_PROBE_MMA nlines a multiple of 16); D host, 8 x 8, D(i, n) = D[i*8 + n]
 * (centro-antisymmetric for BK_PROBE_FF).  y(l, i) = sum_n D(i, n) x(l, n).
 * Asynchronous on stream. */
int bk_probe_contract(int method, long long nlines, const double* D, const void* x, void* y, bk_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BK_PROBE_H */
