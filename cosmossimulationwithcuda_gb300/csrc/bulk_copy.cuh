// Bulk asynchronous copies (the Blackwell/Hopper copy engine inside each SM,
// "TMA") from global into shared memory, completed through mbarriers, and
// bounded waits on those barriers.  Inline PTX only.
//
// A stage of shared memory is filled by one thread: it announces the bytes
// the stage will receive (arrive.expect_tx on the stage's "full" barrier) and
// issues cp.async.bulk copies that count those bytes down as they land; the
// barrier's phase completes when every byte has arrived.  Consumers wait on
// the phase's parity.  When they are done reading a stage they arrive on its
// "empty" barrier, which the filling thread waits on before it reuses the
// stage.  Every wait is bounded in wall time (globaltimer) and in iterations,
// and reports a timeout instead of spinning forever.
#pragma once

#include <stdint.h>

namespace cpm {
namespace bulk {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the asynchronous (copy) proxy.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces `bytes` more bytes for the current phase.
__device__ __forceinline__ void arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Global -> shared copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) whose completion counts down the transaction bytes of `bar`.
__device__ __forceinline__ void copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// L2 policy for data read once per step (the particle state): evicted first,
// so that it does not push the step's lattices out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// copy_g2s with an L2 cache-eviction policy for the source lines.
__device__ __forceinline__ void copy_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

__device__ __forceinline__ bool try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase of parity `parity` of `bar` to complete: at most
// `limit_ns` of wall time and kWaitMaxIters polls; false on timeout.
constexpr uint64_t kWaitLimitNs = 500000000ull;  // 0.5 s: far beyond any copy of this library
constexpr int kWaitMaxIters = 1 << 26;
__device__ __forceinline__ bool wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
    if (try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (int it = 0; it < kWaitMaxIters; ++it) {
        if (try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Named barrier over the first `threads` threads of the CTA (id 1; id 0 is
// __syncthreads), so that a subset of warps can synchronise without the rest.
__device__ __forceinline__ void named_sync(int threads) {
    asm volatile("bar.sync 1, %0;" ::"r"(threads) : "memory");
}

}  // namespace bulk
}  // namespace cpm
