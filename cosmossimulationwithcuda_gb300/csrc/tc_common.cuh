// tcgen05 helpers (5th-generation tensor cores, sm_100a family): tensor
// memory allocation, MMA issue with shared-memory operand descriptors,
// completion through an mbarrier, and tensor-memory loads.  Inline PTX only.
//
// Operand layout used throughout: "K-major, no swizzle" core matrices.  A
// core matrix is 8 rows x 16 bytes (8 x 8 16-bit elements) stored as 128
// contiguous bytes; element (row r, k) of an R x K operand sits at
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 bytes (core matrices adjacent along K are contiguous) and
// SBO = K * 16 bytes (then the next group of 8 rows).  One MMA consumes a
// K = 16 slice, i.e. the start address advances by 2 * LBO per slice.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace cpm {
namespace tc {

constexpr int kLBO = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__host__ __device__ constexpr int kmajor_offset(int r, int k, int K) {
    return (r >> 3) * (K * 16) + (k >> 3) * kLBO + (r & 7) * 16 + (k & 7) * 2;
}
// The same layout with any LBO / SBO (multiples of 16 bytes): spacing the
// core matrices adjacent along K by 144 bytes instead of 128 spreads a warp's
// writes of one row's K elements over distinct shared-memory banks.
__host__ __device__ constexpr int kmajor_offset(int r, int k, int lbo, int sbo) {
    return (r >> 3) * sbo + (k >> 3) * lbo + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), the
// descriptor version (1) at bits 46-47, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int lbo, int sbo) {
    return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((uint32_t(lbo) >> 4) & 0x3FFFu) << 16) |
           (uint64_t((uint32_t(sbo) >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int K) { return smem_desc(saddr, kLBO, K * 16); }

// Instruction descriptor, kind::f16: FP32 accumulator, A and B both FP16 or
// both BF16, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int bf16, int M, int N) {
    return (1u << 4) | (uint32_t(bf16) << 7) | (uint32_t(bf16) << 10) | (uint32_t(N >> 3) << 17) |
           (uint32_t(M >> 4) << 24);
}

// D(tmem) (+)= A(smem) * B(smem)^T, one K = 16 slice.  Issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

// Arrive on `mbar` when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for phase `parity` of `mbar`: non-blocking tests with a short
// sleep between them, for at most `limit_ns` of wall time (and max_iters
// tests); false if the phase did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, int max_iters,
                                          uint64_t limit_ns = 200000000ull) {
    const uint64_t t0 = globaltimer_ns();
    for (int it = 0; it < max_iters; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
        __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes made visible to the tensor cores.
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole warp: allocate `ncols` tensor-memory columns, base address to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t base, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols));
}

// Whole warp: 16 consecutive 32-bit columns of the warp's 32 lanes (lane =
// thread), starting at `taddr` (lane << 16 | column).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Split v into a 16-bit high part and the 16-bit rounding of the remainder.
template <int BF16>
__device__ __forceinline__ void split16(float v, uint16_t& hi, uint16_t& lo);

// Eight values split and packed as two 16-byte rows of a core matrix.
template <int BF16>
__device__ __forceinline__ void split16x8(const float (&v)[8], uint4& hi, uint4& lo) {
    uint16_t h[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) split16<BF16>(v[j], h[j], l[j]);
    hi = make_uint4(h[0] | (uint32_t(h[1]) << 16), h[2] | (uint32_t(h[3]) << 16), h[4] | (uint32_t(h[5]) << 16),
                    h[6] | (uint32_t(h[7]) << 16));
    lo = make_uint4(l[0] | (uint32_t(l[1]) << 16), l[2] | (uint32_t(l[3]) << 16), l[4] | (uint32_t(l[5]) << 16),
                    l[6] | (uint32_t(l[7]) << 16));
}

template <int BF16>
__device__ __forceinline__ void split16(float v, uint16_t& hi, uint16_t& lo) {
    if (BF16) {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        hi = __bfloat16_as_ushort(h);
        lo = __bfloat16_as_ushort(l);
    } else {
        const __half h = __float2half_rn(v);
        const __half l = __float2half_rn(v - __half2float(h));
        hi = __half_as_ushort(h);
        lo = __half_as_ushort(l);
    }
}

}  // namespace tc
}  // namespace cpm
