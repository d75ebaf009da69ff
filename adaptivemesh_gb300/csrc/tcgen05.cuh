// tcgen05.cuh -- the fifth-generation tensor-core instructions of the sm_100 family (tcgen05) that
// this library's BF16 GEMM uses: Tensor Memory (TMEM) allocation, the MMA whose A and B operands
// sit in shared memory (described by 64-bit matrix descriptors) and whose accumulator lives in
// TMEM, its completion signalled on an mbarrier, and loads of the accumulator back to registers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tma.cuh"

namespace amr {

// Shared-memory matrix descriptor of a K-major operand without swizzling.  The operand is stored
// as core matrices of 8 rows x 16 bytes (8 BF16 of K per row, rows 16 bytes apart, 128 bytes per
// core matrix); lbo = bytes between core matrices adjacent along K, sbo = bytes between core
// matrices adjacent along M (or N).  Bits: start address >> 4 [0, 14), lbo >> 4 [16, 30), sbo >> 4
// [32, 46), descriptor version 1 [46, 48), base offset 0, layout 0 (no swizzle) [61, 64).
__device__ __forceinline__ uint64_t umma_desc_kmajor(uint32_t smem_byte_addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((smem_byte_addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits [4, 6) = 1), BF16 A and
// B (bits [7, 10) = 1, [10, 13) = 1), both K-major (bits 15, 16 = 0), N >> 3 at [17, 23), M >> 4 at
// [24, 29).
__host__ __device__ constexpr uint32_t umma_idesc_bf16_f32(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp; the TMEM address is
// written to *smem_dst.  The warp then gives up its allocation permit so that other CTAs on the SM
// can allocate; the same warp frees the columns before the CTA exits.
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(smem_dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A x B (+ D when accumulate), issued by one thread; asynchronous.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate) : "memory");
}
// The mbarrier's current phase completes (one arrival) once every MMA this thread issued before is
// done: their shared-memory operands have been read and their results are in TMEM.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_addr(bar)) : "memory");
}
// Ordering of tcgen05 operations across a thread barrier.
__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Shared-memory writes of this thread (generic proxy) made visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive 32-bit TMEM columns of one lane per thread: warp w of a 4-warp group reads lanes
// 32 (w % 4) .. 32 (w % 4) + 31 (taddr carries the lane in bits 16+, the column below).  The wait
// is in the same statement, so that no use of the registers can move before it.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace amr
