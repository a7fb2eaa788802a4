// bk_host.cu -- the operator applies on host arrays (include/bk_host.h).
//
// The reference's kernels take host pointers and map `in` to the device and
// `out` back on every call (openmp/offload/bk5_offload.cpp's `map` clauses).
// Here the element range is cut into chunks, and a call is three passes over
// them on three streams: every chunk's copy in (stream s_in), every chunk's
// apply (the caller's stream, each after its own copy in), every chunk's
// copy out (stream s_out, each after its own apply); the caller's stream
// then waits for the last copy out, and the next call's copies wait for the
// caller's stream (stream order).  Chunk c+1's copy in, chunk c's apply and
// chunk c-1's copy out run at the same time.  u and v have device buffers of the full size:
// with a ring of chunk slots the copies in had to wait for applies and, on
// this part, the copy engines' queues then held the copies out behind them
// (measured: the copies serialised, 15 ms per BK5 p=7 apply instead of 7.9).
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "bk_host.h"
#include "bk_internal.h"

namespace {

constexpr int kMaxChunks = 64;

long long gcd_ll(long long a, long long b)
{
    while (b) {
        const long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// the smallest element count whose byte size in every array (values per
// element given) is a multiple of 16: chunk offsets keep the 16-byte
// alignment the applies require
long long align_elems(int vbytes, const long long* per_elem, int n)
{
    long long m = 1;
    for (int i = 0; i < n; ++i) {
        const long long b = per_elem[i] * vbytes;
        const long long need = 16 / gcd_ll(16, b);
        m = m / gcd_ll(m, need) * need;
    }
    return m;
}

}  // namespace

struct bk_host_plan {
    int op, p, prec, vbytes;
    long long E, chunk;
    int nchunk;
    long long nin, nq;   // values per element of u/v and of one quadrature field
    void* du;
    void* dv;
    cudaStream_t s_in, s_out;
    cudaEvent_t ev_start;
    cudaEvent_t ev_in[kMaxChunks], ev_done[kMaxChunks], ev_out[kMaxChunks];
};

namespace {

int ck(cudaError_t e)
{
    if (e == cudaSuccess) return BK_OK;
    cudaGetLastError();
    return BK_ERR_CUDA;
}

// the chunk pipeline; apply(e0, ne, u_dev, v_dev, stream) runs one chunk
template <class F>
int run_chunks(bk_host_plan* h, const void* u_host, void* v_host, cudaStream_t s, F apply)
{
    if (h->E == 0) return BK_OK;
    const size_t eb = size_t(h->nin) * h->vbytes;   // bytes of u (and v) per element
    const char* uh = static_cast<const char*>(u_host);
    char* vh = static_cast<char*>(v_host);
    char* du = static_cast<char*>(h->du);
    char* dv = static_cast<char*>(h->dv);
    int rc;
    // stream order: the copies in start after the caller's earlier work on
    // `s` (an earlier call included: its copies out may write the host
    // array this call reads, and it still uses du and dv)
    if ((rc = ck(cudaEventRecord(h->ev_start, s)))) return rc;
    if ((rc = ck(cudaStreamWaitEvent(h->s_in, h->ev_start, 0)))) return rc;
    for (int c = 0; c < h->nchunk; ++c) {
        const long long e0 = c * h->chunk;
        const long long ne = (h->E - e0) < h->chunk ? (h->E - e0) : h->chunk;
        const size_t off = size_t(e0) * eb, bytes = size_t(ne) * eb;
        if ((rc = ck(cudaMemcpyAsync(du + off, uh + off, bytes, cudaMemcpyHostToDevice, h->s_in)))) return rc;
        if ((rc = ck(cudaEventRecord(h->ev_in[c], h->s_in)))) return rc;
    }
    for (int c = 0; c < h->nchunk; ++c) {
        const long long e0 = c * h->chunk;
        const long long ne = (h->E - e0) < h->chunk ? (h->E - e0) : h->chunk;
        const size_t off = size_t(e0) * eb;
        if ((rc = ck(cudaStreamWaitEvent(s, h->ev_in[c], 0)))) return rc;
        if ((rc = apply(e0, ne, du + off, dv + off, s))) return rc;
        if ((rc = ck(cudaEventRecord(h->ev_done[c], s)))) return rc;
    }
    for (int c = 0; c < h->nchunk; ++c) {
        const long long e0 = c * h->chunk;
        const long long ne = (h->E - e0) < h->chunk ? (h->E - e0) : h->chunk;
        const size_t off = size_t(e0) * eb, bytes = size_t(ne) * eb;
        if ((rc = ck(cudaStreamWaitEvent(h->s_out, h->ev_done[c], 0)))) return rc;
        if ((rc = ck(cudaMemcpyAsync(vh + off, dv + off, bytes, cudaMemcpyDeviceToHost, h->s_out)))) return rc;
        if ((rc = ck(cudaEventRecord(h->ev_out[c], h->s_out)))) return rc;
    }
    // the caller's stream completes after the last copy out
    return ck(cudaStreamWaitEvent(s, h->ev_out[h->nchunk - 1], 0));
}

int check_plan(const bk_host_plan* h, int op, const void* u_host, void* v_host, const bk_options* opt)
{
    if (!h) return BK_ERR_NULL;
    if (h->op != op) return BK_ERR_ARG;
    if (h->E > 0 && (!u_host || !v_host)) return BK_ERR_NULL;
    const int prec = opt ? opt->prec : BK_PREC_FP64;
    if (prec != h->prec) return BK_ERR_PREC;
    return BK_OK;
}

}  // namespace

extern "C" {

int bk_host_plan_create(bk_host_plan_t* out, int op, int p, int64_t E, int prec, int64_t chunk_elems)
{
    if (!out) return BK_ERR_NULL;
    *out = nullptr;
    if (op != 1 && op != 3 && op != 5) return BK_ERR_ARG;
    if (p < 1 || p > 8) return BK_ERR_ORDER;
    if (E < 0 || chunk_elems < 0) return BK_ERR_SIZE;
    if (prec != BK_PREC_FP64 && prec != BK_PREC_FP32 && prec != BK_PREC_MIXED) return BK_ERR_PREC;
    bk_host_plan* h = new bk_host_plan();
    std::memset(h, 0, sizeof(*h));
    h->op = op;
    h->p = p;
    h->prec = prec;
    h->vbytes = prec == BK_PREC_FP64 ? 8 : 4;
    h->E = E;
    const long long P = p + 1, Q = (op == 5) ? p + 1 : p + 2;
    h->nin = P * P * P;
    h->nq = Q * Q * Q;
    // u/v, qdata or G (up to 9 factors for BK5), k
    const long long per[4] = {h->nin, h->nq, 6 * h->nq, 9 * h->nq};
    const long long m = align_elems(h->vbytes, per, 4);
    long long c = chunk_elems > 0 ? chunk_elems : (E + 15) / 16;
    if (c < 1) c = 1;
    if ((E + c - 1) / c > kMaxChunks) c = (E + kMaxChunks - 1) / kMaxChunks;
    c = (c + m - 1) / m * m;
    h->chunk = c;
    h->nchunk = int((E + c - 1) / c);
    const size_t bytes = size_t(E > 0 ? E : 1) * size_t(h->nin) * h->vbytes;
    int rc = ck(cudaMalloc(&h->du, bytes));
    if (rc == BK_OK) rc = ck(cudaMalloc(&h->dv, bytes));
    if (rc == BK_OK) rc = ck(cudaEventCreateWithFlags(&h->ev_start, cudaEventDisableTiming));
    for (int k = 0; k < h->nchunk && rc == BK_OK; ++k) {
        rc = ck(cudaEventCreateWithFlags(&h->ev_in[k], cudaEventDisableTiming));
        if (rc == BK_OK) rc = ck(cudaEventCreateWithFlags(&h->ev_done[k], cudaEventDisableTiming));
        if (rc == BK_OK) rc = ck(cudaEventCreateWithFlags(&h->ev_out[k], cudaEventDisableTiming));
    }
    if (rc == BK_OK) rc = ck(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));
    if (rc == BK_OK) rc = ck(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    if (rc != BK_OK) {
        bk_host_plan_destroy(h);
        return rc;
    }
    *out = h;
    return BK_OK;
}

int bk_host_plan_destroy(bk_host_plan_t h)
{
    if (!h) return BK_OK;
    if (h->s_in) cudaStreamSynchronize(h->s_in);
    if (h->s_out) cudaStreamSynchronize(h->s_out);
    for (int k = 0; k < kMaxChunks; ++k) {
        if (h->ev_done[k]) cudaEventSynchronize(h->ev_done[k]);
        if (h->ev_in[k]) cudaEventDestroy(h->ev_in[k]);
        if (h->ev_done[k]) cudaEventDestroy(h->ev_done[k]);
        if (h->ev_out[k]) cudaEventDestroy(h->ev_out[k]);
    }
    if (h->ev_start) cudaEventDestroy(h->ev_start);
    cudaFree(h->du);
    cudaFree(h->dv);
    if (h->s_in) cudaStreamDestroy(h->s_in);
    if (h->s_out) cudaStreamDestroy(h->s_out);
    delete h;
    return BK_OK;
}

int bk1_apply_host(bk_host_plan_t h, const double* B, const void* qdata, const void* u_host, void* v_host,
                   const bk_options* opt, bk_stream_t stream)
{
    int rc = check_plan(h, 1, u_host, v_host, opt);
    if (rc) return rc;
    if (!B || (h->E > 0 && !qdata)) return BK_ERR_NULL;
    const char* q = static_cast<const char*>(qdata);
    const size_t qb = size_t(h->nq) * h->vbytes;
    return run_chunks(h, u_host, v_host, reinterpret_cast<cudaStream_t>(stream),
                      [&](long long e0, long long ne, void* du, void* dv, cudaStream_t s) {
                          return bk1_apply_opt(h->p, ne, B, q + size_t(e0) * qb, du, dv, opt,
                                               reinterpret_cast<bk_stream_t>(s));
                      });
}

int bk3_apply_host(bk_host_plan_t h, const double* B, const double* D, const void* G, const void* k,
                   const void* u_host, void* v_host, const bk_options* opt, bk_stream_t stream)
{
    int rc = check_plan(h, 3, u_host, v_host, opt);
    if (rc) return rc;
    if (!B || !D || (h->E > 0 && !G)) return BK_ERR_NULL;
    const char* g = static_cast<const char*>(G);
    const char* kk = static_cast<const char*>(k);
    const size_t qb = size_t(h->nq) * h->vbytes;
    return run_chunks(h, u_host, v_host, reinterpret_cast<cudaStream_t>(stream),
                      [&](long long e0, long long ne, void* du, void* dv, cudaStream_t s) {
                          return bk3_apply_k(h->p, ne, B, D, g + size_t(e0) * 6 * qb,
                                             kk ? kk + size_t(e0) * qb : nullptr, du, dv, opt,
                                             reinterpret_cast<bk_stream_t>(s));
                      });
}

int bk5_apply_host(bk_host_plan_t h, const double* D, const void* G, const void* u_host, void* v_host,
                   const bk_options* opt, bk_stream_t stream)
{
    int rc = check_plan(h, 5, u_host, v_host, opt);
    if (rc) return rc;
    if (!D || (h->E > 0 && !G)) return BK_ERR_NULL;
    const int F = (opt && opt->nfactors == 9) ? 9 : 6;
    const char* g = static_cast<const char*>(G);
    const size_t qb = size_t(h->nq) * h->vbytes;
    return run_chunks(h, u_host, v_host, reinterpret_cast<cudaStream_t>(stream),
                      [&](long long e0, long long ne, void* du, void* dv, cudaStream_t s) {
                          return bk5_apply_opt(h->p, ne, D, g + size_t(e0) * F * qb, du, dv, opt,
                                               reinterpret_cast<bk_stream_t>(s));
                      });
}

}  // extern "C"
