// tc_tma.cuh -- Tensor Memory Accelerator (TMA) tile loads into shared
// memory, completed on mbarriers, in hand-written inline PTX for sm_100-class
// GPUs.  Every wait is bounded by the device's global timer: a wait that runs
// out returns false instead of spinning forever.
#pragma once

#include <cuda.h>   // CUtensorMap (the descriptor type; no driver call is made here)

namespace tcgb {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long tma_now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One arrival expected per phase (the thread that posts the byte count).
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the TMA unit (async proxy).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrive once and add `bytes` to the transaction count of the current phase:
// the phase completes when the TMA loads posted against it have written that
// many bytes.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity to complete; false if it has not
// after limit_ns nanoseconds.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = tma_now_ns();
    while (!mbar_try_wait(bar, parity))
        if (tma_now_ns() - t0 > limit_ns) return false;
    return true;
}

// Arrive once on the barrier (release: the thread's earlier reads of the
// buffer the barrier guards are done).
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// mbar_wait that also gives up as soon as *abort is set (by a thread of
// the block whose own wait ran out); sets *abort when it runs out itself.
__device__ __forceinline__ bool mbar_wait_or_abort(unsigned bar, unsigned parity, unsigned long long limit_ns,
                                                   volatile int* abort) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = tma_now_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort) return false;
        if (tma_now_ns() - t0 > limit_ns) {
            *abort = 1;
            return false;
        }
    }
    return true;
}

// Tiled 3-D load of the tensor map's box at element coordinates (x, y, z)
// into shared memory at dst (128-byte aligned), completing on bar.
// Coordinates outside the tensor read as zero; x must be a multiple of
// 16 bytes / element size (the box start is then 16-byte aligned).
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

}  // namespace tcgb
