// tma.cuh -- bulk-copy (TMA) and mbarrier helpers in inline PTX (sm_90 and later).
//
// Every wait is bounded: a wait that runs out of iterations reports false, and the
// caller records an error in the solver's health word and leaves the work undone,
// so a copy that never lands cannot hang the GPU.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hgpu {

__device__ __forceinline__ unsigned smemAddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbarInit(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

// the barrier's current phase completes when `bytes` have landed (one arrival)
__device__ __forceinline__ void mbarExpectTx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbarTryWait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// wait for the phase of parity `parity` to complete; false after `limit` polls
__device__ __forceinline__ bool mbarWait(unsigned long long* bar, unsigned parity, int limit = 1 << 24) {
    for (int i = 0; i < limit; ++i)
        if (mbarTryWait(bar, parity)) return true;
    return false;
}

// order this thread's earlier generic-proxy accesses of shared memory before later
// async-proxy (bulk copy) accesses of it
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// make mbarrier initialisation visible to the async proxy
__device__ __forceinline__ void fenceBarrierInit() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// contiguous global -> shared copy of `bytes` (multiple of 16; both addresses 16-byte aligned)
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
        : "memory");
}

// 2D tiled tensor load of the box at element coordinates (x, y) of `map` (a
// __grid_constant__ CUtensorMap) into shared memory (128-byte aligned)
__device__ __forceinline__ void tensorLoad2D(void* dst, const void* map, int x, int y, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smemAddr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smemAddr(bar))
        : "memory");
}

}  // namespace hgpu
