// bk_device.cuh -- device-side plumbing shared by every kernel: the device
// status word, bounded waits, mbarriers and 1-D TMA bulk copies (sm_90+ PTX,
// compiled for sm_103a only).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "bk_gpu.h"

namespace bkg {

// Per-launch context of the device-side error handling: the status word of
// the device (first error wins) and the cycle limit of every bounded wait.
struct DevCtx {
    int* status;
    long long wait_limit;
};

__device__ __forceinline__ void set_status(const DevCtx& ctx, int code)
{
    atomicCAS(ctx.status, 0, code);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier ---------------------------------------------------------------

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the async proxy (TMA).
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses to the same memory.
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Adds `bytes` to the transaction count of the current phase without an
// arrival (copies issued before the phase's arrive.expect_tx).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of the barrier for at most `limit` SM cycles.
// Returns false when it gave up.  Never spins without bound.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit)
{
    if (mbar_try_wait(bar, parity)) {
        return true;
    }
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) {
            return false;
        }
    }
    return true;
}

// ---- 1-D TMA bulk copies -----------------------------------------------------

// Global -> shared, completion counted in bytes on `bar`.  dst, src and bytes
// must be multiples of 16.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Shared -> global through a bulk async-group.  dst, src and bytes multiples of 16.
__device__ __forceinline__ void tma_store_1d(void* dst, const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_store_commit()
{
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Waits until the committed bulk stores have finished READING shared memory.
__device__ __forceinline__ void tma_store_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Waits until the committed bulk stores are complete.
__device__ __forceinline__ void tma_store_wait_all()
{
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// One arrival on the barrier (no transaction bytes).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// A hint: brings [p, p + bytes) into L2 by one bulk prefetch (no shared
// memory, no completion to wait for).  The range is widened to 16-byte
// boundaries but never past `end` rounded down, so it stays inside the array
// p points into (whose start is 16-byte aligned).
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes, const void* end)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15);
    uintptr_t b = (reinterpret_cast<uintptr_t>(p) + bytes + 15) & ~uintptr_t(15);
    const uintptr_t cap = reinterpret_cast<uintptr_t>(end) & ~uintptr_t(15);
    if (b > cap) b = cap;
    if (b > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(uint32_t(b - a)) : "memory");
}

}  // namespace bkg
