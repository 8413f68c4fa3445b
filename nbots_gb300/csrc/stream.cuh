// Per-warp bulk-copy streaming of the 2x2-block SELL matrix into shared
// memory (cp.async.bulk + mbarrier, inline PTX for sm_103a).
//
// Every slice of the layout is contiguous in each array (its entries run
// from 32 * slice_off[s] to 32 * slice_off[s+1]), 16-byte aligned and a
// multiple of 16 bytes long, so one bulk copy per array moves a whole slice.
// A warp owns a contiguous run of slices and a ring of kStages stage buffers;
// lane 0 keeps the next slices' copies in flight while the warp computes on
// the current one, so the matrix stream needs no registers and little
// occupancy.  Each stage has its own mbarrier (one arrival plus the byte
// count); its phase parity flips on every reuse.  Waits are bounded by
// %globaltimer and record NBG_ERR_TIMEOUT instead of spinning forever.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace nbg {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for a stage; returns false (and records a timeout) on expiry.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    while (!mbar_try_wait(bar, parity)) {
        if (globaltimer() - t0 > kSpinLimitNs) {
            atomicCAS(status, 0, NBG_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// Stage geometry of one warp: kStages buffers of up to kMaxW block entries
// per lane (wider slices fall back to direct loads).
template <int kStages, int kMaxW, int kBytesPerEntry>
struct WarpStream {
    static constexpr uint32_t kStageBytes = (uint32_t)kMaxW * 32u * kBytesPerEntry;
    static constexpr uint32_t kBytes = kStages * kStageBytes;
};

}  // namespace nbg
