// tma.cuh -- mbarrier / bulk-copy (TMA) helpers for sm_103a, inline PTX.
//
// Every wait is bounded in wall-clock time: a wait that gives up returns
// false, the kernel records an error code in a device word the host reads
// (gfft_device_error), waits (again bounded) for its own copies in flight
// and returns.  No wait can hang the GPU.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace gfft {

// ~1 s: far above any legitimate copy latency, short enough to keep the
// context usable if a copy never lands
constexpr unsigned long long TMA_WAIT_NS = 1000000000ull;

enum DeviceError : unsigned { DEV_ERR_TMA_TIMEOUT = 1u, DEV_ERR_TC_TIMEOUT = 2u };

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this CTA's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) accesses
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
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

// wait for phase `parity` of the barrier; false after TMA_WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > TMA_WAIT_NS) return false;
    return true;
}

// contiguous global -> shared copy of `bytes` (multiple of 16, both
// addresses 16-byte aligned), completing on `bar`
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// 3D tiled tensor load of one box at coordinates (c0, c1, c2); c0 * element
// size must be a multiple of 16 bytes (checked on the host)
__device__ __forceinline__ void tensor_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                               uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// L2 eviction-priority policies (createpolicy) for the hinted accesses
// below: evict_first for data read or written once, evict_last for data
// that must stay in L2 until it is read back
__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// tensor_load_3d with an L2 cache policy
__device__ __forceinline__ void tensor_load_3d_hint(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                                    uint64_t *bar, uint64_t policy)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
        "%3, %4}], [%5], %6;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// 16-byte global store with an L2 cache policy
__device__ __forceinline__ void st_global_v4_hint(void *p, float4 v, uint64_t policy)
{
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w), "l"(policy)
                 : "memory");
}

}  // namespace gfft
