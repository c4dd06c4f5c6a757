// 5th-generation tensor core (tcgen05) building blocks for sm_103a: TMEM
// allocation, shared-memory matrix descriptors, the instruction descriptor of a
// BF16 x BF16 -> FP32 MMA, the MMA itself, its commit to an mbarrier, and
// TMEM -> register loads. Inline PTX only (no CUTLASS/CuTe).
//
// Operand layout used throughout: K-major, no swizzle. A tile of R rows x K
// columns of 16-bit elements is stored as "core matrices" of 8 rows x 16 bytes
// (8 elements), each core matrix 128 contiguous bytes (row r of it at r*16):
//     byte offset of (row, k) = (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2
// with LBO = 128 (next core matrix along K) and SBO = K * 16 (next group of 8
// rows). One MMA consumes K = 16, i.e. two core matrices along K; MMA s of a
// tile starts at byte 256 * s.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace senkgpu {
namespace tc {

constexpr uint32_t kLbo = 128;

// Shared-memory matrix descriptor (tcgen05 format):
//   [0,14)  start address >> 4      [16,30) leading byte offset >> 4
//   [32,46) stride byte offset >> 4 [46,48) version (1 for tcgen05)
//   [49,52) base offset (0)         [52]    LBO mode (0)
//   [61,64) layout: 0 = no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator,
// both operands K-major, dense:
//   [4,6) D format (1 = F32)   [7,10) A format (1 = BF16)   [10,13) B format (1 = BF16)
//   [15] A major (0 = K)       [16] B major (0 = K)
//   [17,23) N >> 3             [24,29) M >> 4
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM allocation of `ncols` columns (power of two, >= 32) by one whole warp;
// the TMEM address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Makes this thread's generic-proxy shared-memory writes visible to the tensor
// core (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued before
// has completed.
__device__ __forceinline__ void mma_commit(unsigned long long *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 32 lanes x 16 columns of 32-bit values: lane t of the warp gets the 16
// columns of TMEM lane (taddr.lane + t), starting at column taddr.col.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) in a K-major no-swizzle tile with K columns.
__host__ __device__ constexpr uint32_t kmajor_offset(int row, int k, int K)
{
    return (uint32_t)((row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

}  // namespace tc
}  // namespace senkgpu
