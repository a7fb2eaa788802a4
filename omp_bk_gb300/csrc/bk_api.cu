// bk_api.cu -- the C ABI of include/bk_gpu.h: argument checks on the host,
// order/precision/engine dispatch, the device status word.
#include <atomic>
#include <cstdint>
#include <cstring>

#include <cuda_runtime.h>

#include "bk_device.cuh"
#include "bk_gpu.h"
#include "bk_internal.h"

#define BK_VERSION "omp_bk_gb300 0.1 (sm_103a)"

namespace bkg {

// First device-side error since the last reset, one word per device (the
// copy of this module on each device holds its own).
__device__ int g_status_word;

namespace {
constexpr long long kDefaultWaitLimit = 4000000000LL;   // SM cycles, ~2 s
// Per-device values filled in on first use.  Host threads may make their
// first calls on a device at the same time: each slot is an atomic, and two
// threads that both look a value up store the same value.  The status word's
// address is that of this module's copy in the device's primary context; the
// library is not meant to outlive a reset of that context (cudaDeviceReset).
std::atomic<long long> g_wait_limit[kMaxDevices];
// BK5's BK_KERNEL_AUTO as measured by a tuner, per order, engine, layout and
// mass term (0: the built-in rule, bk5_builtin_auto); process-wide.
std::atomic<int> g_auto_kernel[9][4][3][2];
std::atomic<int*> g_status_ptr[kMaxDevices];
std::atomic<int> g_sm_count[kMaxDevices];
}  // namespace

int current_device()
{
    int d = -1;
    if (cudaGetDevice(&d) != cudaSuccess) return -1;
    return d;
}

int sm_count()
{
    const int d = current_device();
    if (d < 0 || d >= kMaxDevices) return 1;
    int n = g_sm_count[d].load(std::memory_order_acquire);
    if (n == 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
        n = n > 0 ? n : 1;
        g_sm_count[d].store(n, std::memory_order_release);
    }
    return n;
}

static int* status_ptr()
{
    const int d = current_device();
    if (d < 0 || d >= kMaxDevices) return nullptr;
    int* ptr = g_status_ptr[d].load(std::memory_order_acquire);
    if (ptr == nullptr) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_status_word) != cudaSuccess) return nullptr;
        ptr = static_cast<int*>(p);
        g_status_ptr[d].store(ptr, std::memory_order_release);
    }
    return ptr;
}

DevCtx dev_ctx()
{
    const int d = current_device();
    DevCtx c;
    c.status = status_ptr();
    const long long lim = (d >= 0 && d < kMaxDevices) ? g_wait_limit[d].load(std::memory_order_relaxed) : 0;
    c.wait_limit = lim > 0 ? lim : kDefaultWaitLimit;
    return c;
}

__global__ void wait_timeout_kernel(const DevCtx ctx)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // nothing arrives on the barrier: the bounded wait must give up
    if (!mbar_wait_bounded(&bar, 0, ctx.wait_limit)) {
        if (threadIdx.x == 0) set_status(ctx, BK_ERR_TIMEOUT);
    }
}

}  // namespace bkg

using namespace bkg;

namespace {

bool misaligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; }

// Common checks; returns BK_OK or an error code.
int check_common(int p, int pmax, int64_t E)
{
    if (p < 1 || p > pmax) return BK_ERR_ORDER;
    if (E < 0 || E > (int64_t(1) << 40)) return BK_ERR_SIZE;
    return BK_OK;
}

int check_ptrs(int64_t E, std::initializer_list<const void*> ptrs)
{
    if (E == 0) return BK_OK;
    for (const void* q : ptrs) {
        if (q == nullptr) return BK_ERR_NULL;
        if (misaligned(q)) return BK_ERR_ALIGN;
    }
    return BK_OK;
}

int engine_of(const bk_options& o)
{
    if (o.prec == BK_PREC_FP32) return 2;
    if (o.prec == BK_PREC_MIXED) return 3;
    if (o.prec != BK_PREC_FP64) return -1;
    if (o.engine == BK_ENGINE_DFMA) return 0;
    if (o.engine == BK_ENGINE_FF || o.engine == BK_ENGINE_AUTO) return 1;
    return -1;
}

int status_or_null()
{
    return dev_ctx().status == nullptr ? BK_ERR_CUDA : BK_OK;
}

}  // namespace

extern "C" {

bk_options bk_default_options(void)
{
    bk_options o;
    o.prec = BK_PREC_FP64;
    o.engine = BK_ENGINE_AUTO;
    o.layout = BK_LAYOUT_INTERLEAVED;
    o.nfactors = 6;
    o.elems_per_block = 0;
    o.kernel = BK_KERNEL_AUTO;
    o.gform = BK_G_STORAGE;
    o.jxw_layout = BK_JXW_PQR;
    return o;
}

const char* bk_version(void) { return BK_VERSION; }

int bk5_apply_ex(int p, int64_t E, const double* D, const void* G, const void* u, const void* mass, double lambda,
                 void* v, const bk_options* opt, bk_stream_t stream)
{
    const bk_options o = opt ? *opt : bk_default_options();
    int rc = check_common(p, 8, E);
    if (rc) return rc;
    if (D == nullptr) return BK_ERR_NULL;
    if ((rc = check_ptrs(E, {G, u, v}))) return rc;
    if (mass != nullptr && misaligned(mass)) return BK_ERR_ALIGN;
    if (o.nfactors != 6 && o.nfactors != 9) return BK_ERR_PREC;
    if (o.layout < 0 || o.layout > 2) return BK_ERR_PREC;
    if (o.kernel < 0 || o.kernel > 2) return BK_ERR_PREC;
    if (o.elems_per_block < 0 || o.elems_per_block > 64) return BK_ERR_ARG;
    const int eng = engine_of(o);
    if (eng < 0) return BK_ERR_PREC;
    // G split ahead of time: the float-float engine (FP64, engine AUTO or FF),
    // 6 factors, sweep kernel
    if (o.gform != BK_G_STORAGE &&
        (o.gform != BK_G_FF || eng != 1 || o.nfactors != 6 || o.kernel == BK_KERNEL_COLUMN))
        return BK_ERR_PREC;
    if (E == 0) return BK_OK;
    if ((rc = status_or_null())) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // AUTO: the tuned shape where a tuner set one, else the built-in rule
    int kernel = o.kernel;
    if (kernel == BK_KERNEL_AUTO) {
        const int t = g_auto_kernel[p][eng][o.layout][mass != nullptr ? 1 : 0].load(std::memory_order_relaxed);
        kernel = (o.gform == BK_G_STORAGE && t != 0) ? t : bk5_builtin_auto(p, eng, o.layout, mass != nullptr);
        if (o.gform != BK_G_STORAGE) kernel = BK_KERNEL_SWEEP;
    }
    switch (eng) {
        case 0: return launch_bk5_dfma(p, E, D, G, u, mass, lambda, v, o.nfactors, o.layout, o.elems_per_block, kernel,
                                      o.gform, s);
        case 1: return launch_bk5_ff(p, E, D, G, u, mass, lambda, v, o.nfactors, o.layout, o.elems_per_block, kernel,
                                      o.gform, s);
        case 2: return launch_bk5_f32(p, E, D, G, u, mass, lambda, v, o.nfactors, o.layout, o.elems_per_block, kernel,
                                      o.gform, s);
        default: return launch_bk5_mixed(p, E, D, G, u, mass, lambda, v, o.nfactors, o.layout, o.elems_per_block, kernel,
                                      o.gform, s);
    }
}

int bk5_set_auto_kernel(int p, int prec, int engine, int layout, int with_mass, int kernel)
{
    if (p < 1 || p > 8) return BK_ERR_ORDER;
    bk_options o = bk_default_options();
    o.prec = prec;
    o.engine = engine;
    const int eng = engine_of(o);
    if (eng < 0 || layout < 0 || layout > 2 || (with_mass != 0 && with_mass != 1)) return BK_ERR_PREC;
    if (kernel != BK_KERNEL_AUTO && kernel != BK_KERNEL_SWEEP && kernel != BK_KERNEL_COLUMN) return BK_ERR_ARG;
    g_auto_kernel[p][eng][layout][with_mass].store(kernel, std::memory_order_relaxed);
    return BK_OK;
}

int bk5_auto_kernel(int p, int prec, int engine, int layout, int with_mass)
{
    if (p < 1 || p > 8) return -BK_ERR_ORDER;
    bk_options o = bk_default_options();
    o.prec = prec;
    o.engine = engine;
    const int eng = engine_of(o);
    if (eng < 0 || layout < 0 || layout > 2 || (with_mass != 0 && with_mass != 1)) return -BK_ERR_PREC;
    const int t = g_auto_kernel[p][eng][layout][with_mass].load(std::memory_order_relaxed);
    return t != 0 ? t : bk5_builtin_auto(p, eng, layout, with_mass != 0);
}

int bk5_apply_opt(int p, int64_t E, const double* D, const void* G, const void* u, void* v, const bk_options* opt,
                  bk_stream_t stream)
{
    return bk5_apply_ex(p, E, D, G, u, nullptr, 0.0, v, opt, stream);
}

int bk5_apply(int p, int64_t E, const double* D, const void* G, const void* u, void* v, int prec,
              bk_stream_t stream)
{
    bk_options o = bk_default_options();
    o.prec = prec;
    return bk5_apply_opt(p, E, D, G, u, v, &o, stream);
}

int bk1_apply_opt(int p, int64_t E, const double* B, const void* qdata, const void* u, void* v,
                  const bk_options* opt, bk_stream_t stream)
{
    const bk_options o = opt ? *opt : bk_default_options();
    int rc = check_common(p, 8, E);
    if (rc) return rc;
    if (B == nullptr) return BK_ERR_NULL;
    if ((rc = check_ptrs(E, {qdata, u, v}))) return rc;
    const int eng = engine_of(o);
    if (eng < 0 || o.gform != BK_G_STORAGE) return BK_ERR_PREC;
    if (o.jxw_layout != BK_JXW_PQR && o.jxw_layout != BK_JXW_RQP) return BK_ERR_ARG;
    if (E == 0) return BK_OK;
    if ((rc = status_or_null())) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int jt = o.jxw_layout == BK_JXW_RQP;
    switch (eng) {
        case 0: return launch_bk1_dfma(p, E, B, qdata, u, v, o.elems_per_block, jt, s);
        case 1: return launch_bk1_ff(p, E, B, qdata, u, v, o.elems_per_block, jt, s);
        case 2: return launch_bk1_f32(p, E, B, qdata, u, v, o.elems_per_block, jt, s);
        default: return launch_bk1_mixed(p, E, B, qdata, u, v, o.elems_per_block, jt, s);
    }
}

int bk1_apply(int p, int64_t E, const double* B, const void* qdata, const void* u, void* v, int prec,
              bk_stream_t stream)
{
    bk_options o = bk_default_options();
    o.prec = prec;
    return bk1_apply_opt(p, E, B, qdata, u, v, &o, stream);
}

int bk3_apply_k(int p, int64_t E, const double* B, const double* D, const void* G, const void* k, const void* u,
                void* v, const bk_options* opt, bk_stream_t stream)
{
    const bk_options o = opt ? *opt : bk_default_options();
    int rc = check_common(p, 8, E);
    if (rc) return rc;
    if (B == nullptr || D == nullptr) return BK_ERR_NULL;
    if ((rc = check_ptrs(E, {G, u, v}))) return rc;
    if (k != nullptr && misaligned(k)) return BK_ERR_ALIGN;
    const int eng = engine_of(o);
    if (eng < 0) return BK_ERR_PREC;
    // G split ahead of time: the float-float engine (FP64, engine AUTO or FF)
    if (o.gform != BK_G_STORAGE && (o.gform != BK_G_FF || eng != 1)) return BK_ERR_PREC;
    if (E == 0) return BK_OK;
    if ((rc = status_or_null())) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    switch (eng) {
        case 0: return launch_bk3_dfma(p, E, B, D, G, k, u, v, o.elems_per_block, o.gform, s);
        case 1: return launch_bk3_ff(p, E, B, D, G, k, u, v, o.elems_per_block, o.gform, s);
        case 2: return launch_bk3_f32(p, E, B, D, G, k, u, v, o.elems_per_block, o.gform, s);
        default: return launch_bk3_mixed(p, E, B, D, G, k, u, v, o.elems_per_block, o.gform, s);
    }
}

int bk3_apply_opt(int p, int64_t E, const double* B, const double* D, const void* G, const void* u, void* v,
                  const bk_options* opt, bk_stream_t stream)
{
    return bk3_apply_k(p, E, B, D, G, nullptr, u, v, opt, stream);
}

int bk3_apply(int p, int64_t E, const double* B, const double* D, const void* G, const void* u, void* v, int prec,
              bk_stream_t stream)
{
    bk_options o = bk_default_options();
    o.prec = prec;
    return bk3_apply_opt(p, E, B, D, G, u, v, &o, stream);
}

int bk3_adjoint(int p, int64_t E, const double* B, const double* D, const void* G, const void* k, const void* u,
                const void* res, void* dk, void* dG, const bk_options* opt, bk_stream_t stream)
{
    const bk_options o = opt ? *opt : bk_default_options();
    int rc = check_common(p, 8, E);
    if (rc) return rc;
    if (B == nullptr || D == nullptr) return BK_ERR_NULL;
    if ((rc = check_ptrs(E, {G, k, u, res, dk, dG}))) return rc;
    const int eng = engine_of(o);
    if (eng < 0) return BK_ERR_PREC;
    // G split ahead of time: the float-float engine (FP64, engine AUTO or FF)
    if (o.gform != BK_G_STORAGE && (o.gform != BK_G_FF || eng != 1)) return BK_ERR_PREC;
    if (E == 0) return BK_OK;
    if ((rc = status_or_null())) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    switch (eng) {
        case 0: return launch_bk3_adjoint_dfma(p, E, B, D, G, k, u, res, dk, dG, o.gform, s);
        case 1: return launch_bk3_adjoint_ff(p, E, B, D, G, k, u, res, dk, dG, o.gform, s);
        case 2: return launch_bk3_adjoint_f32(p, E, B, D, G, k, u, res, dk, dG, o.gform, s);
        default: return launch_bk3_adjoint_mixed(p, E, B, D, G, k, u, res, dk, dG, o.gform, s);
    }
}

int bk_device_status(int* status, int reset, bk_stream_t stream)
{
    if (status == nullptr) return BK_ERR_NULL;
    int* dp = status_ptr();
    if (dp == nullptr) return BK_ERR_CUDA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(status, dp, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return BK_ERR_CUDA;
    if (reset && cudaMemsetAsync(dp, 0, sizeof(int), s) != cudaSuccess) return BK_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return BK_ERR_CUDA;
    return BK_OK;
}

int bk_set_wait_limit(long long cycles)
{
    const int d = current_device();
    if (d < 0 || d >= kMaxDevices) return BK_ERR_CUDA;
    if (cycles < 0) return BK_ERR_ARG;
    g_wait_limit[d].store(cycles, std::memory_order_relaxed);
    return BK_OK;
}

int bk_test_wait_timeout(bk_stream_t stream)
{
    const DevCtx c = dev_ctx();
    if (c.status == nullptr) return BK_ERR_CUDA;
    wait_timeout_kernel<<<1, 32, 0, reinterpret_cast<cudaStream_t>(stream)>>>(c);
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

}  // extern "C"
