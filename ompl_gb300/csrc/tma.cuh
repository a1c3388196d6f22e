// Shared-memory staging of world data with the bulk-copy engine (cp.async.bulk, completion on an
// mbarrier). Every wait is bounded: on expiry the kernel raises the timeout flag and returns.
#pragma once
#include <cstdint>

namespace gbo
{

constexpr unsigned long long kWaitNs = 1000000000ull;  // a bounded wait gives up after one second

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    uint64_t st;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(st)
                 : "r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    (void)st;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for phase `parity` of the barrier for at most limit_ns nanoseconds (global timer): false when
// the time ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, unsigned long long limit_ns = kWaitNs)
{
    const unsigned long long t0 = global_ns();
    while (true)
    {
        if (mbar_try_wait(bar, parity))
            return true;
        if (global_ns() - t0 > limit_ns)
            return false;
    }
}

__device__ __forceinline__ unsigned dynamic_smem_bytes()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
    return r;
}

// Copy `bytes` (multiple of 16, 16-byte aligned on both sides) from global to shared memory with the
// bulk-copy engine. All threads of the block must call it. A copy larger than the launch's dynamic
// shared memory, or an unaligned one, is refused: *error is raised and false returned. Returns false
// after raising *timeout if the copy did not complete within the wait limit (after a second bounded
// wait for the copy in flight).
__device__ __forceinline__ bool stage_bulk(void *dst, const void *src, unsigned bytes, uint64_t *bar,
                                           unsigned *timeout, unsigned *error)
{
    if (bytes == 0)
        return true;
    if (bytes > dynamic_smem_bytes() || (bytes & 15u) || (((uintptr_t)src) & 15u) || (smem_addr(dst) & 15u))
    {
        if (threadIdx.x == 0)
            atomicExch(error, 1u);
        return false;
    }
    if (threadIdx.x == 0)
        mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0)
    {
        mbar_expect_tx(bar, bytes);
        constexpr unsigned kChunk = 16384;
        for (unsigned off = 0; off < bytes; off += kChunk)
            bulk_g2s((char *)dst + off, (const char *)src + off, bytes - off < kChunk ? bytes - off : kChunk, bar);
    }
    bool ok = mbar_wait_bounded(bar, 0);
    if (!ok)
    {
        atomicExch(timeout, 1u);
        mbar_wait_bounded(bar, 0);
    }
    return __syncthreads_and(ok);
}

}  // namespace gbo
