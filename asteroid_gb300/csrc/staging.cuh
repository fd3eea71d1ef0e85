// staging.cuh -- bulk-copy staging of an object's observations into shared memory.
//
// One elected thread arms an mbarrier with the byte count and issues a single
// cp.async.bulk global -> shared copy of the whole SoA block (every array 16-byte aligned,
// total a multiple of 16); every thread then waits on the barrier's phase.  The wait is
// bounded: after kWaitLimit polls the CTA records kErrStageTimeout, keeps reading the global
// copy instead, and before exiting waits (bounded again) for the copy it issued.
#pragma once
#include <stdint.h>
#include "model.cuh"

namespace ast {

constexpr int kWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
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

// Stage [g_obs, g_obs + L.bytes) into smem.  Must be called by every thread of the CTA.
// `bar` is an 8-byte shared word; each thread polls the barrier at most `wait_limit` times.
// Returns true when the shared copy is complete.
__device__ __forceinline__ bool bulk_stage(void* smem, const void* g_src, uint32_t bytes, uint64_t* bar,
                                           unsigned long long* err, int wait_limit = kWaitLimit)
{
    const uint32_t b = smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(smem)),
            "l"(g_src), "r"(bytes), "r"(b)
            : "memory");
    }
    bool ok = false;
    for (int it = 0; it < wait_limit; ++it)
        if (mbar_try_wait(b, 0)) { ok = true; break; }
    // Every thread must agree; one that gave up makes the whole CTA use global memory.
    ok = __syncthreads_and(ok);
    if (!ok && threadIdx.x == 0 && err) atomicCAS(err, 0ull, (unsigned long long)kErrStageTimeout);
    return ok;
}

// Before a CTA whose staging wait ran out exits, give the copy it issued a bounded wait.
__device__ __forceinline__ void bulk_drain(uint64_t* bar, bool staged)
{
    if (staged || threadIdx.x != 0) return;
    const uint32_t b = smem_u32(bar);
    for (int it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(b, 0)) break;
}

}  // namespace ast
