// zs_ptx.cuh -- inline-PTX helpers shared by the pipelined kernels: mbarriers with
// bounded waits, bulk and tensor (TMA) copies into shared memory, the global timer.
#pragma once
#include <stdint.h>

#define ZS_WAIT_NS 1000000000ull   // limit of every bounded wait: one second of global time

__device__ __forceinline__ uint32_t zs_smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void zs_mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void zs_mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool zs_mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t zs_globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase of `bar` with the given parity to complete; false when
// `limit_ns` of global time passed first.
__device__ __forceinline__ bool zs_mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns = ZS_WAIT_NS) {
    if (zs_mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = zs_globaltimer();
    for (;;) {
        if (zs_mbar_try_wait(bar, parity)) return true;
        if (zs_globaltimer() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void zs_bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void zs_mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 2-D tiled tensor copy (box of the tensor map at element coordinates x, y) into shared memory.
__device__ __forceinline__ void zs_tma_2d(uint32_t dst, const void *tmap, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(tmap), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
