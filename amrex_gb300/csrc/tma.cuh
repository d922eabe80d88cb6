// Tensor Memory Accelerator and mbarrier primitives (inline PTX, sm_90+),
// with bounded waits.
#pragma once

#include <cuda.h>

namespace mlmg {

namespace tma {

__device__ __forceinline__ unsigned smem_addr (const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init (unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx (unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" :: "r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void load_3d (void* dst, const void* map, unsigned long long* bar, int c0, int c1, int c2)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];\n"
                 :: "r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar)) : "memory");
}

// prefetch a tensor-map box into L2 (no shared memory, no barrier); parts of
// the box outside the tensor are not fetched
__device__ __forceinline__ void prefetch_3d (const void* map, int c0, int c1, int c2)
{
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];\n"
                 :: "l"(map), "r"(c0), "r"(c1), "r"(c2) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait (unsigned long long* bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// bounded wait for phase `parity` of the barrier: false after `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded (unsigned long long* bar, unsigned parity, long long limit)
{
    for (long long it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) { return true; }
    }
    return false;
}

constexpr long long WAIT_LIMIT = 1LL << 24;   // polls (each try_wait blocks for a short while)
constexpr int ERR_TMA_TIMEOUT = 1;            // the tile's copy did not complete
constexpr int ERR_TMA_ALIGN = 2;              // a box would start off a 16-byte boundary (never issued)

} // namespace tma

} // namespace mlmg
