// Asynchronous copies for sm_100 and later, as inline PTX: mbarrier phases, and tensor-memory-
// accelerator (TMA) tile loads from a tensor map into shared memory.
//
// A TMA load is issued by one thread; it arrives on an mbarrier with the number of bytes it wrote
// (the thread first arms the barrier with that count through arrive.expect_tx), and the consumers
// wait on the barrier's phase parity. Waits are bounded: mbar_wait gives up after `limit` polls and
// returns false, so that a kernel can record the failure and return instead of spinning forever.
#pragma once

#include <cstdint>

namespace ntg {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// After initialising barriers, before any thread or the async proxy uses them.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the completion of the phase with the given parity (`limit` polls; 0 gives up at once).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Arms the barrier's current phase with the bytes the coming TMA loads will deliver (one arrival).
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// A tensor map in global memory written by a host copy: make its current contents visible to the
// TMA unit before the first load through it.
__device__ __forceinline__ void tensormap_acquire(const void *map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// Box of a 3-D tensor map at element coordinates (x innermost) into shared memory, completing on
// `bar`. The shared-memory destination must be 128-byte aligned and x times the element size a
// multiple of 16 bytes (x may be negative); elements outside the tensor read 0.
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace ntg
