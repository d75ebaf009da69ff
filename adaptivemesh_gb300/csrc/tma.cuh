// tma.cuh -- bulk asynchronous copies (cp.async.bulk, the 1-D form of the Tensor Memory
// Accelerator) into shared memory, tracked by transaction-count mbarriers.
//
// Every wait is bounded: after kMaxSpins polls the waiter reports failure so the kernel can
// raise its error flag and leave instead of hanging the GPU.  A poll suspends the thread until the
// phase completes or kSuspendHintNs pass, so waiting warps leave the issue slots to working ones
// and a wait gives up after about kMaxSpins * kSuspendHintNs (~1 s).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace amr {

constexpr uint32_t kMaxSpins = 1u << 22;
constexpr uint32_t kSuspendHintNs = 256;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Make initialised barriers visible to the asynchronous proxy before the first copy.
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Wait for phase `parity` of the barrier; true once it completed, false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kMaxSpins) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(a), "r"(parity), "n"(kSuspendHintNs) : "memory");
        if (done) return true;
    }
    return false;
}
// Copy `bytes` (multiple of 16, both addresses 16-byte aligned) from global to shared memory;
// completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Copy `bytes` (multiple of 16, both addresses 16-byte aligned) from shared to global memory as
// part of the issuing thread's current bulk group; bulk_commit closes the group.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                 ::"l"(dst), "r"(smem_addr(src)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until every committed group of this thread has read its shared-memory source ...
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... or has completed its writes.
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace amr
