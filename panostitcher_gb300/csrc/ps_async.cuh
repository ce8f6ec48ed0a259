// ps_async.cuh -- bulk asynchronous copies (the TMA engine's non-tensor mode)
// and mbarrier completion tracking, as inline PTX for sm_90+ / sm_103a.
//
// Every wait is bounded: after kMaxPolls unsuccessful polls the caller gets
// false, records an error in the frame's status word and carries on with
// whatever is in shared memory, so a CTA never hangs and every thread still
// reaches each __syncthreads.
#pragma once

#include <cstdint>

namespace ps {

constexpr long long kMaxPolls = 1LL << 24;

__device__ __forceinline__ uint32_t smemAddr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarArriveExpectTx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbarArrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar)) : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity, long long maxPolls = kMaxPolls)
{
    for (long long i = 0; i < maxPolls; i++)
        if (mbarTryWait(bar, parity)) return true;
    return false;
}

// Global -> shared bulk copy completing on an mbarrier.  dst, src and bytes
// must be multiples of 16.
__device__ __forceinline__ void bulkCopy(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
        : "memory");
}

// Bulk tensor copies (TMA, tile mode, no swizzle) of one box of a 3-D or
// 2-D tensor map into shared memory, completing on an mbarrier.  The map
// (a CUtensorMap) lives in global memory; dst must be 128-byte aligned and
// the box's first coordinate times the element size a multiple of 16 bytes.
__device__ __forceinline__ void tmaLoad3d(void* dst, const void* tmap, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smemAddr(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smemAddr(bar))
        : "memory");
}

__device__ __forceinline__ void tmaLoad2d(void* dst, const void* tmap, int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smemAddr(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smemAddr(bar))
        : "memory");
}

// Named barrier over the first `count` threads of the CTA (id 1..15).
__device__ __forceinline__ void namedBarrier(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same buffers.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace ps
