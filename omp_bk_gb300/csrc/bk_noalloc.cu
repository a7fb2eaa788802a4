// bk_noalloc.cu -- the FP64 dot product for callers that cannot allocate
// device memory.
//
// bk_dot (bk_vec.cu) needs a workspace for its per-block partial sums, which
// the caller allocates.  Some callers cannot: code that runs while a stream
// is being captured into a CUDA graph (cudaMalloc is not allowed there), host
// programs whose device memory is owned by another runtime's pool and that
// may not call cudaMalloc/cudaFree themselves, and callers that reach this
// library only through its C ABI without any CUDA memory management of their
// own.  bk_dot_noalloc gives them the same reduction with its scratch in a
// fixed array of this library's module on the device: 4096 doubles (32 KiB,
// held by every GPU that loads the library until the process exits), one
// partial sum per chunk of 65536 values, so at most 4096 x 65536 =
// 268,435,456 values per call; longer vectors are rejected with BK_ERR_SIZE.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in): the device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, on the first
// call made on it -- so make a first call before capturing a stream.  The
// address cached per device is an atomic, so host threads that make their
// first calls at the same time are safe; it belongs to the device's primary
// context, so the library must not be used across a cudaDeviceReset.  Every
// call shares the array and leaves its last partial sums in it; a call reads
// back only the partials it has just written, so nothing has to start at
// zero.  Calls whose kernels overlap on the GPU (different streams, no
// ordering between them) race on the array.
#include <atomic>
#include <cstdint>

#include <cuda_runtime.h>

#include "bk_internal.h"
#include "bk_vec.h"

namespace {

constexpr int kNoAllocPartials = 4096;
constexpr long long kNoAllocChunk = 65536;
constexpr long long kNoAllocMaxN = kNoAllocPartials * kNoAllocChunk;
static_assert(kNoAllocMaxN == BK_DOT_NOALLOC_MAX_N, "the limit stated in bk_vec.h");
constexpr int kThreads = 256;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocPartials];

std::atomic<double*> g_scratch_ptr[bkg::kMaxDevices];

template <class T>
__global__ void __launch_bounds__(kThreads) chunk_dot_kernel(const T* __restrict__ x, const T* __restrict__ y,
                                                             long long n, double* __restrict__ part)
{
    __shared__ double sh[kThreads];
    const long long lo = blockIdx.x * kNoAllocChunk;
    const long long hi = (lo + kNoAllocChunk < n) ? lo + kNoAllocChunk : n;
    double s = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) s = fma(double(x[i]), double(y[i]), s);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kThreads) chunk_final_kernel(const double* __restrict__ part, int nb,
                                                               double* __restrict__ out, int half)
{
    __shared__ double sh[kThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = half ? 0.5 * sh[0] : sh[0];
}

// The device address of the scratch array on the current device, looked up
// on the first call made on that device (nullptr if the lookup failed).
double* scratch_on_current_device()
{
    const int dev = bkg::current_device();
    if (dev < 0 || dev >= bkg::kMaxDevices) return nullptr;
    double* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (p == nullptr) {
        if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        // two threads that race here store the same address
        g_scratch_ptr[dev].store(p, std::memory_order_release);
    }
    return p;
}

}  // namespace

extern "C" {

int bk_dot_noalloc(long long n, const void* x, const void* y, int f64, double* result, int half,
                   bk_stream_t stream)
{
    if (n < 0 || n > kNoAllocMaxN) return BK_ERR_SIZE;
    if (!result) return BK_ERR_NULL;
    if (n > 0 && (!x || !y)) return BK_ERR_NULL;
    double* part = scratch_on_current_device();
    if (part == nullptr) return BK_ERR_CUDA;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int nb = (n > 0) ? int((n + kNoAllocChunk - 1) / kNoAllocChunk) : 1;
    if (f64)
        chunk_dot_kernel<double><<<nb, kThreads, 0, s>>>(static_cast<const double*>(x), static_cast<const double*>(y),
                                                         n, part);
    else
        chunk_dot_kernel<float><<<nb, kThreads, 0, s>>>(static_cast<const float*>(x), static_cast<const float*>(y), n,
                                                        part);
    chunk_final_kernel<<<1, kThreads, 0, s>>>(part, nb, result, half);
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

}  // extern "C"
