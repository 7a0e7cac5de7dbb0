// tc.cuh -- tcgen05 (5th-generation tensor core) helpers for sm_103a, inline
// PTX: tensor-memory allocation, shared-memory matrix descriptors, the
// kind::f16 MMA (FP16 or BF16 operands, FP32 accumulate), commit to an
// mbarrier and the tensor-memory load of the accumulator.
#pragma once

#include <stdint.h>

#include "tma.cuh"

namespace gfft {
namespace tc {

// ---- tensor memory -------------------------------------------------------
// allocate `ncols` columns (power of two >= 32); one whole warp executes it;
// the TMEM address is written to the shared word `dst`
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors ---------------------------------------------------------
// Shared-memory matrix descriptor, K-major, no swizzle: the operand is an
// array of 8-row x 16-byte core matrices; `lbo` is the byte distance between
// core matrices adjacent along K, `sbo` between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // bits 0-13: start address >> 4
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;      // bits 16-29: leading byte offset >> 4
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;      // bits 32-45: stride byte offset >> 4
    d |= (uint64_t)1 << 46;                            // bits 46-48: descriptor version 0b001
    // bits 49-51 base offset 0, bit 52 relative LBO, bits 61-63 layout 0 (no swizzle)
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, A and B of the same
// 16-bit type (bf16 = false: FP16; true: BF16), both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_f16(bool bf16, int M, int N)
{
    return (1u << 4)                                   // D format: F32
           | ((bf16 ? 1u : 0u) << 7)                   // A format
           | ((bf16 ? 1u : 0u) << 10)                  // B format
           | ((uint32_t)(N >> 3) << 17)                // N >> 3
           | ((uint32_t)(M >> 4) << 24);               // M >> 4
}

// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        bool accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// arrive once on `bar` when every MMA this thread issued so far is complete
__device__ __forceinline__ void commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive 32-bit columns of this thread's TMEM lane (warp w reads
// lanes 32 (w % 4) .. + 31; `taddr` carries the warp's lane base)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&r)[32])
{
    uint32_t u[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
          "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
          "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) r[i] = __uint_as_float(u[i]);
}

}  // namespace tc
}  // namespace gfft
