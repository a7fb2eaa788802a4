/* bk_host.h -- C ABI of the operator applies on HOST arrays: the drop-in for
 * the reference's host-pointer kernel signature, whose OpenMP offload maps
 * `in` to the device and `out` back on every call
 * (SumFactorization(nelmt, basis, JxW|G, in, out): openmp/bk1_sumfact.h:16-22,
 * openmp/bk3_sumfact.h:17-24, openmp/BK5.cpp:18-24 with the `map` clauses of
 * openmp/offload/bk5_offload.cpp).  The operator data (qdata or G, and k)
 * stay resident on the device; u comes from host memory and v goes back to
 * host memory in element chunks: chunk c+1's copy in, chunk c's apply and
 * chunk c-1's copy out run at the same time on two copy streams and the
 * caller's stream.  Host arrays should be pinned (cudaHostAlloc or
 * cudaHostRegister) for the copies to overlap; pageable memory works but
 * copies synchronously.  Return values are bk_status codes (bk_gpu.h). */
#ifndef BK_HOST_H
#define BK_HOST_H

#include "bk_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bk_host_plan* bk_host_plan_t;

/* A plan for operator `op` (1, 3 or 5) at order p over E elements with
 * storage precision prec: device buffers for u and v (E elements each), two
 * copy streams and one event per chunk, on the current device; chunks of
 * chunk_elems elements (0: E / 16 rounded up; at most 64 chunks; rounded up
 * to keep chunk offsets 16-byte aligned).  The applies allocate nothing. */
int bk_host_plan_create(bk_host_plan_t* plan, int op, int p, int64_t E, int prec, int64_t chunk_elems);
int bk_host_plan_destroy(bk_host_plan_t plan);

/* v_host = A u_host over the plan's E elements; B, D host as in bk_gpu.h;
 * qdata, G, k device (resident).  Asynchronous: enqueued on `stream` (which
 * completes after the last copy into v_host), u_host and v_host must stay
 * valid until then; synchronize the stream to read v_host.  opt as in
 * bk*_apply_opt (prec must be the plan's); opt->nfactors 9 for BK5's full
 * tensor.  Consecutive calls on one plan are ordered. */
int bk1_apply_host(bk_host_plan_t plan, const double* B, const void* qdata, const void* u_host, void* v_host,
                   const bk_options* opt, bk_stream_t stream);
int bk3_apply_host(bk_host_plan_t plan, const double* B, const double* D, const void* G, const void* k,
                   const void* u_host, void* v_host, const bk_options* opt, bk_stream_t stream);
int bk5_apply_host(bk_host_plan_t plan, const double* D, const void* G, const void* u_host, void* v_host,
                   const bk_options* opt, bk_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BK_HOST_H */
