// Spectral-force column pass on the tensor cores, split precision.
//
// Same job as k_cols_spectral (pm_fft.cu): per half-spectrum line kx, the
// forward FFT over y (length L = N), the filter K, the three y-edge sums, and
// the two inverse FFTs Phi = IFFT(phi_hat) and Psi = IFFT(phi_hat * i S g).
// Here every length-L transform is a four-step FFT, L = L1 * L2, whose two
// DFT stages are tcgen05 GEMMs:
//   stage A  rows (line b, n2), 128 per MMA: Y[k1] = sum_n1 x[n1*L2 + n2] W_L1^(n1 k1)
//   twiddle  Y'[k1][n2] = Y * W_L^(n2 k1)   (FP32, while draining tensor memory)
//   stage C  rows (line b, k1):              X[k1 + L1 k2] = sum_n2 Y'[k1][n2] W_L2^(n2 k2)
// A complex DFT of size R is the real 2R x 2R matrix [[C, S], [-S, C]]
// (C = cos 2 pi k n / R, S = sin 2 pi k n / R) applied to (Re, Im): the data
// is the MMA's A operand (rows x 2R, K-major), the DFT matrix the B operand.
// Split precision: data and DFT matrix are each a 16-bit high part plus the
// 16-bit rounding of the remainder (FP16 or BF16); three MMA chains
// hi*hi + lo*hi + hi*lo accumulate in FP32 in tensor memory.  FP16 needs a
// range scale: the input is scaled by a power of two to |v| < 2^14 and stage
// C's input by a further 1/L1 (stage A grows values by at most L1).
// Inverse transforms use IFFT(x) = conj(FFT(conj x)), so only forward DFT
// matrices are kept in shared memory.
//
// Shapes: L = 1024 (32 x 32, 4 lines per CTA), 2048 (64 x 32, 4 lines),
// 4096 (64 x 64, 2 lines).  One CTA holds the DFT matrices, its lines (FP32)
// and one operand buffer: 89 / 217 / 201 KB of shared memory, 128 tensor-memory
// columns.  Waits on the MMA completion barrier are bounded (200 ms of wall
// time); a timeout sets *status and the CTA skips its remaining MMAs, and the
// batch it had committed gets one more bounded wait before tensor memory is
// freed (a second timeout leaves the columns allocated, *status = 2).
#include <cmath>
#include <cstring>
#include <vector>

#include "fft_engine.cuh"
#include "pm_internal.h"
#include "tc_common.cuh"

namespace cpm {

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcWaitIters = 1 << 20;

template <int L>
struct TcShape {
    static constexpr int L1 = L == 1024 ? 32 : 64;
    static constexpr int L2 = L / L1;
    static constexpr int B = 128 / L2;            // lines per CTA
    static constexpr int KA = 2 * L1;             // stage A: K and N of the MMA
    static constexpr int RC = B * L1;             // stage C rows
    static constexpr int GC = RC / 128;           // stage C MMA groups of 128 rows
    static constexpr int KC = 2 * L2;             // stage C: K and N
    static constexpr bool SHARED_F = L1 == L2;
    static constexpr int F1_BYTES = 2 * KA * KA * 2;                  // hi + lo
    static constexpr int F2_BYTES = SHARED_F ? 0 : 2 * KC * KC * 2;
    static constexpr int D0_BYTES = B * L * 8;
    // data operands: core matrices adjacent along K 144 bytes apart (bank spread)
    static constexpr int LBO_OP = 144;
    static constexpr int SBO_A = (KA / 8) * LBO_OP, SBO_C = (KC / 8) * LBO_OP;
    static constexpr int OPA_BYTES = (128 / 8) * SBO_A, OPC_BYTES = (RC / 8) * SBO_C;
    static constexpr int OP_BYTES = OPA_BYTES > OPC_BYTES ? OPA_BYTES : OPC_BYTES;  // per hi / lo
    static constexpr int OFF_F2 = F1_BYTES;
    static constexpr int OFF_D0 = F1_BYTES + F2_BYTES;
    static constexpr int OFF_OPHI = OFF_D0 + D0_BYTES;
    static constexpr int OFF_OPLO = OFF_OPHI + OP_BYTES;
    static constexpr int SMEM = OFF_OPLO + OP_BYTES;
    static constexpr int TCOLS = 128;
    static_assert(L1 * L2 == L && KA <= 128 && KC <= 128 && GC * KC <= TCOLS && KA <= TCOLS, "tc shape");
};

__device__ __forceinline__ float warp_max(float v) {
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

// One complex length-L transform of the CTA's B lines through both MMA stages.
// in(b, i) gives element i of line b (already conjugated for an inverse),
// out(b, k, v) receives output k (to be conjugated by the caller for an inverse).
// A completion wait that runs out sets *fail (the CTA issues no further MMAs)
// and, when an MMA batch was committed, records its parity in *pending so that
// the CTA waits for that batch once more before it frees tensor memory.
template <int L, int BF16, class In, class Out>
__device__ void tc_fft(unsigned char* smem, uint32_t tmem, uint64_t* mbar, uint32_t& phase, int* fail,
                       int* pending, float* red, const float2* __restrict__ tw, In in, Out out, int* status,
                       int skip_mma) {
    using S = TcShape<L>;
    constexpr int L1 = S::L1, L2 = S::L2, B = S::B;
    uint16_t* ophi = reinterpret_cast<uint16_t*>(smem + S::OFF_OPHI);
    uint16_t* oplo = reinterpret_cast<uint16_t*>(smem + S::OFF_OPLO);
    const unsigned char* f1 = smem;
    const unsigned char* f2 = smem + (S::SHARED_F ? 0 : S::OFF_F2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // ---- range scale (FP16): max |component| over the CTA's lines ----
    float scale_a = 1.0f, scale_c = 1.0f;
    if (!BF16) {
        float m = 0.0f;
        for (int i = tid; i < B * L; i += kTcThreads) {
            const float2 v = in(i / L, i % L);
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        m = warp_max(m);
        if (lane == 0) red[warp] = m;
        __syncthreads();
        float mm = 0.0f;
#pragma unroll
        for (int w = 0; w < kTcThreads / 32; ++w) mm = fmaxf(mm, red[w]);
        __syncthreads();
        if (mm > 0.0f) {
            int e;
            frexpf(mm, &e);  // mm < 2^e
            scale_a = ldexpf(1.0f, 14 - e);
        }
        scale_c = scale_a / float(L1);
    }

    // ---- stage A operand: row r = b*L2 + n2, K = (Re n1 | Im n1); a thread
    // packs 8 consecutive n1 of one row into 16-byte core-matrix rows ----
    {
        unsigned char* hib = reinterpret_cast<unsigned char*>(ophi);
        unsigned char* lob = reinterpret_cast<unsigned char*>(oplo);
        for (int idx = tid; idx < 128 * (L1 / 8); idx += kTcThreads) {
            const int r = idx & 127, kb = idx >> 7;
            const int b = r / L2, n2 = r - b * L2;
            float re[8], im[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float2 v = in(b, (kb * 8 + j) * L2 + n2);
                re[j] = v.x * scale_a;
                im[j] = v.y * scale_a;
            }
            uint4 h, l;
            tc::split16x8<BF16>(re, h, l);
            const int o_re = tc::kmajor_offset(r, kb * 8, S::LBO_OP, S::SBO_A);
            *reinterpret_cast<uint4*>(hib + o_re) = h;
            *reinterpret_cast<uint4*>(lob + o_re) = l;
            tc::split16x8<BF16>(im, h, l);
            const int o_im = tc::kmajor_offset(r, L1 + kb * 8, S::LBO_OP, S::SBO_A);
            *reinterpret_cast<uint4*>(hib + o_im) = h;
            *reinterpret_cast<uint4*>(lob + o_im) = l;
        }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !*fail && !skip_mma) {
        const uint32_t idesc = tc::idesc_f16(BF16, 128, S::KA);
        const uint32_t a_hi = tc::smem_u32(ophi), a_lo = tc::smem_u32(oplo);
        const uint32_t b_hi = tc::smem_u32(f1), b_lo = tc::smem_u32(f1 + S::KA * S::KA * 2);
        uint32_t acc = 0;
        constexpr int AS = 2 * S::LBO_OP;  // bytes per K = 16 slice of a data operand
        for (int kk = 0; kk < S::KA / 16; ++kk, acc = 1)
            tc::mma_f16(tmem, tc::smem_desc(a_hi + kk * AS, S::LBO_OP, S::SBO_A), tc::smem_desc(b_hi + kk * 256, S::KA),
                        idesc, acc);
        for (int kk = 0; kk < S::KA / 16; ++kk)
            tc::mma_f16(tmem, tc::smem_desc(a_lo + kk * AS, S::LBO_OP, S::SBO_A), tc::smem_desc(b_hi + kk * 256, S::KA),
                        idesc, 1);
        for (int kk = 0; kk < S::KA / 16; ++kk)
            tc::mma_f16(tmem, tc::smem_desc(a_hi + kk * AS, S::LBO_OP, S::SBO_A), tc::smem_desc(b_lo + kk * 256, S::KA),
                        idesc, 1);
        tc::commit(mbar);
    }
    if (!*fail && !tc::mbar_wait(mbar, phase, kTcWaitIters)) {
        *fail = 1;
        if (!skip_mma) *pending = int(phase);
        atomicMax(status, 1);
    }
    phase ^= 1u;
    tc::fence_after_sync();

    // ---- drain stage A, twiddle, stage C operand: row (b, k1), K = (Re n2 | Im n2) ----
    {
        const int r = 32 * (warp & 3) + lane;  // tensor-memory lane = stage A row
        const int b = r / L2, n2 = r - b * L2;
        const uint32_t lane_addr = tmem + (uint32_t(32 * (warp & 3)) << 16);
        constexpr int HALF = L1 / 2;
        const float rescale = scale_c / scale_a;
        for (int c0 = (warp >> 2) * HALF; c0 < (warp >> 2) * HALF + HALF; c0 += 16) {
            float re[16], im[16];
            tc::tmem_ld16(lane_addr + uint32_t(c0), re);
            tc::tmem_ld16(lane_addr + uint32_t(L1 + c0), im);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int k1 = c0 + j;
                const float2 w = __ldg(tw + ((n2 * k1) & (L - 1)));
                const float yr = (re[j] * w.x - im[j] * w.y) * rescale;
                const float yi = (re[j] * w.y + im[j] * w.x) * rescale;
                const int rc = b * L1 + k1;  // stage C row (groups of 128 follow each other)
                uint16_t h, l;
                tc::split16<BF16>(yr, h, l);
                const int o_re = tc::kmajor_offset(rc, n2, S::LBO_OP, S::SBO_C) >> 1;
                ophi[o_re] = h;
                oplo[o_re] = l;
                tc::split16<BF16>(yi, h, l);
                const int o_im = tc::kmajor_offset(rc, L2 + n2, S::LBO_OP, S::SBO_C) >> 1;
                ophi[o_im] = h;
                oplo[o_im] = l;
            }
        }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && !*fail && !skip_mma) {
        const uint32_t idesc = tc::idesc_f16(BF16, 128, S::KC);
        const uint32_t b_hi = tc::smem_u32(f2), b_lo = tc::smem_u32(f2 + S::KC * S::KC * 2);
        constexpr int AS = 2 * S::LBO_OP;
        for (int g = 0; g < S::GC; ++g) {
            const uint32_t d = tmem + uint32_t(g * S::KC);
            const uint32_t gofs = uint32_t(g * 16 * S::SBO_C);  // 128 rows = 16 groups of 8
            const uint32_t a_hi = tc::smem_u32(ophi) + gofs, a_lo = tc::smem_u32(oplo) + gofs;
            uint32_t acc = 0;
            for (int kk = 0; kk < S::KC / 16; ++kk, acc = 1)
                tc::mma_f16(d, tc::smem_desc(a_hi + kk * AS, S::LBO_OP, S::SBO_C), tc::smem_desc(b_hi + kk * 256, S::KC),
                            idesc, acc);
            for (int kk = 0; kk < S::KC / 16; ++kk)
                tc::mma_f16(d, tc::smem_desc(a_lo + kk * AS, S::LBO_OP, S::SBO_C), tc::smem_desc(b_hi + kk * 256, S::KC),
                            idesc, 1);
            for (int kk = 0; kk < S::KC / 16; ++kk)
                tc::mma_f16(d, tc::smem_desc(a_hi + kk * AS, S::LBO_OP, S::SBO_C), tc::smem_desc(b_lo + kk * 256, S::KC),
                            idesc, 1);
        }
        tc::commit(mbar);
    }
    if (!*fail && !tc::mbar_wait(mbar, phase, kTcWaitIters)) {
        *fail = 1;
        if (!skip_mma) *pending = int(phase);
        atomicMax(status, 1);
    }
    phase ^= 1u;
    tc::fence_after_sync();

    // ---- drain stage C: row (b, k1) of group g, columns (Re k2 | Im k2) -> X[k1 + L1 k2] ----
    {
        const uint32_t lane_addr = tmem + (uint32_t(32 * (warp & 3)) << 16);
        const float inv = 1.0f / scale_c;
        constexpr int HALF = L2 / 2;
        for (int g = 0; g < S::GC; ++g) {
            const int rc = g * 128 + 32 * (warp & 3) + lane;
            const int b = rc / L1, k1 = rc - b * L1;
            for (int c0 = (warp >> 2) * HALF; c0 < (warp >> 2) * HALF + HALF; c0 += 16) {
                float re[16], im[16];
                tc::tmem_ld16(lane_addr + uint32_t(g * S::KC + c0), re);
                tc::tmem_ld16(lane_addr + uint32_t(g * S::KC + L2 + c0), im);
#pragma unroll
                for (int j = 0; j < 16; ++j) out(b, k1 + L1 * (c0 + j), make_float2(re[j] * inv, im[j] * inv));
            }
        }
    }
    // tensor memory and the operand buffer are reused by the next transform
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

}  // namespace

// Host image of the forward DFT matrices (real embedding, K-major core-matrix
// layout, 16-bit hi then lo), in the order the kernel's shared memory holds them.
template <int L, int BF16>
static std::vector<uint16_t> tc_dft_image() {
    using S = TcShape<L>;
    std::vector<uint16_t> img((S::F1_BYTES + S::F2_BYTES) / 2, 0);
    auto put = [&](int base_elems, int R) {
        const int K = 2 * R;
        for (int c = 0; c < K; ++c)
            for (int j = 0; j < K; ++j) {
                const int k = c % R, n = j % R;
                const double a = 2.0 * M_PI * double((int64_t(k) * n) % R) / double(R);
                const double cs = std::cos(a), sn = std::sin(a);
                double v;
                if (c < R) v = j < R ? cs : sn;
                else v = j < R ? -sn : cs;
                uint16_t h, l;
                if (BF16) {
                    const __nv_bfloat16 bh = __double2bfloat16(v);
                    const __nv_bfloat16 bl = __double2bfloat16(v - double(__bfloat162float(bh)));
                    std::memcpy(&h, &bh, 2);
                    std::memcpy(&l, &bl, 2);
                } else {
                    const __half fh = __double2half(v);
                    const __half fl = __double2half(v - double(__half2float(fh)));
                    std::memcpy(&h, &fh, 2);
                    std::memcpy(&l, &fl, 2);
                }
                const int o = tc::kmajor_offset(c, j, K) / 2;
                img[base_elems + o] = h;
                img[base_elems + K * K + o] = l;
            }
    };
    put(0, S::L1);
    if (!S::SHARED_F) put(S::F1_BYTES / 2, S::L2);
    return img;
}

template <int L, int BF16>
__global__ void __launch_bounds__(kTcThreads, 1) k_cols_spectral_tc(float2* __restrict__ spec,
                                                                     float2* __restrict__ spec2,
                                                                     float2* __restrict__ edge,
                                                                     const float* __restrict__ kq,
                                                                     const float2* __restrict__ tw,
                                                                     const uint4* __restrict__ fimg, float g,
                                                                     int* __restrict__ status, int skip_mma) {
    using S = TcShape<L>;
    constexpr int B = S::B, M = L / 2;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int fail;
    __shared__ int pending;  // parity of a committed MMA batch whose wait ran out (-1: none)
    __shared__ float red[6 * (kTcThreads / 32)];
    const int tid = threadIdx.x, warp = tid >> 5;
    spec += size_t(blockIdx.y) * M * L;
    spec2 += size_t(blockIdx.y) * M * L;
    edge += size_t(blockIdx.y) * M * 4;
    const int kx0 = int(blockIdx.x) * B;
    float2* d0 = reinterpret_cast<float2*>(smem + S::OFF_D0);

    {  // DFT matrices and the CTA's lines into shared memory
        uint4* fs = reinterpret_cast<uint4*>(smem);
        for (int i = tid; i < (S::F1_BYTES + S::F2_BYTES) / 16; i += kTcThreads) fs[i] = __ldg(fimg + i);
        const float4* src = reinterpret_cast<const float4*>(spec + size_t(kx0) * L);
        float4* dst = reinterpret_cast<float4*>(d0);
        for (int i = tid; i < B * L / 2; i += kTcThreads) dst[i] = src[i];
    }
    if (tid == 0) {
        fail = 0;
        pending = -1;
        tc::mbar_init(&mbar, 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, S::TCOLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;

    // forward FFT over y, in place
    tc_fft<L, BF16>(
        smem, tmem, &mbar, phase, &fail, &pending, red, tw, [d0](int b, int i) { return d0[b * L + i]; },
        [d0](int b, int k, float2 v) { d0[b * L + k] = v; }, status, skip_mma);

    // x K (line kx = 0 packs the real spectra of kx = 0 and kx = N/2)
    for (int idx = tid; idx < B * (M + 1); idx += kTcThreads) {
        const int b = idx / (M + 1);
        const int ky = idx - b * (M + 1);
        const int kx = kx0 + b;
        const int i1 = b * L + ky;
        const int i2 = b * L + ((L - ky) & (L - 1));
        if (kx != 0) {
            const float kv = __ldg(kq + size_t(kx) * (M + 1) + ky);
            d0[i1] = cscale(d0[i1], kv);
            if (ky != 0 && ky != M) d0[i2] = cscale(d0[i2], kv);
        } else {
            const float k0 = __ldg(kq + ky);
            const float km = __ldg(kq + size_t(M) * (M + 1) + ky);
            const float p = 0.5f * (k0 + km), q = 0.5f * (k0 - km);
            const float2 z1 = d0[i1], z2 = d0[i2];
            d0[i1] = cadd(cscale(z1, p), cscale(cconj(z2), q));
            if (ky != 0 && ky != M) d0[i2] = cadd(cscale(z2, p), cscale(cconj(z1), q));
        }
    }
    __syncthreads();
    // the three y-edge sums of every line
    for (int b = 0; b < B; ++b) {
        float acc[6] = {0, 0, 0, 0, 0, 0};
        for (int ky = tid; ky < L; ky += kTcThreads) {
            const float2 v = d0[b * L + ky];
            const float2 t1 = tw[ky & (L - 1)], t2 = tw[(2 * ky) & (L - 1)];
            const float2 w01 = make_float2(1.0f - t1.x, -t1.y);
            const float2 w02 = make_float2(1.0f - t2.x, -t2.y);
            const float2 w13 = make_float2(0.0f, -2.0f * t1.y);
            const float2 a = cmul(v, w01), c = cmul(v, w02), d = cmul(v, w13);
            acc[0] += a.x; acc[1] += a.y; acc[2] += c.x; acc[3] += c.y; acc[4] += d.x; acc[5] += d.y;
        }
#pragma unroll
        for (int j = 0; j < 6; ++j)
            for (int off = 16; off > 0; off >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], off);
        if ((tid & 31) == 0)
#pragma unroll
            for (int j = 0; j < 6; ++j) red[warp * 6 + j] = acc[j];
        __syncthreads();
        if (tid == 0) {
            float s[6] = {0, 0, 0, 0, 0, 0};
            for (int w = 0; w < kTcThreads / 32; ++w)
#pragma unroll
                for (int j = 0; j < 6; ++j) s[j] += red[w * 6 + j];
            float2* e = edge + size_t(kx0 + b) * 4;
            e[0] = make_float2(s[0], s[1]);
            e[1] = make_float2(s[2], s[3]);
            e[2] = make_float2(s[4], s[5]);
        }
        __syncthreads();
    }

    // Psi = IFFT(phi_hat * i S g) -> spec2, then Phi = IFFT(phi_hat) -> spec
    float2* out2 = spec2 + size_t(kx0) * L;
    tc_fft<L, BF16>(
        smem, tmem, &mbar, phase, &fail, &pending, red, tw,
        [d0, tw, g](int b, int i) {
            const float2 v = d0[b * L + i];
            const float S = g * (tw[(2 * i) & (L - 1)].y - 8.0f * tw[i].y) * (1.0f / 6.0f);
            return make_float2(-S * v.y, -S * v.x);  // conj(i S v)
        },
        [out2](int b, int k, float2 v) { out2[size_t(b) * L + k] = make_float2(v.x, -v.y); }, status, skip_mma);
    float2* out1 = spec + size_t(kx0) * L;
    tc_fft<L, BF16>(
        smem, tmem, &mbar, phase, &fail, &pending, red, tw, [d0](int b, int i) { return cconj(d0[b * L + i]); },
        [out1](int b, int k, float2 v) { out1[size_t(b) * L + k] = make_float2(v.x, -v.y); }, status, skip_mma);

    // Tensor memory is freed only once no MMA can still write it: after a wait
    // that ran out, the committed batch gets one more bounded wait; if that
    // runs out too, the columns stay allocated and *status = 2 reports it.
    if (warp == 0) {
        bool idle = true;
        if (pending >= 0) idle = tc::mbar_wait(&mbar, uint32_t(pending), kTcWaitIters);
        idle = __all_sync(0xffffffffu, idle);
        if (idle)
            tc::tmem_dealloc(tmem, S::TCOLS);
        else if ((tid & 31) == 0)
            atomicMax(status, 2);
    }
}

// ---- host side ---------------------------------------------------------------------------
bool tc_fft_supported(int N) { return N == 1024 || N == 2048 || N == 4096; }

size_t tc_dft_bytes(int N) {
    switch (N) {
        case 1024: return TcShape<1024>::F1_BYTES + TcShape<1024>::F2_BYTES;
        case 2048: return TcShape<2048>::F1_BYTES + TcShape<2048>::F2_BYTES;
        case 4096: return TcShape<4096>::F1_BYTES + TcShape<4096>::F2_BYTES;
        default: return 0;
    }
}

template <int L, int BF16>
static cudaError_t upload_image(void* dev, cudaStream_t st) {
    const std::vector<uint16_t> img = tc_dft_image<L, BF16>();
    cudaError_t e = cudaMemcpyAsync(dev, img.data(), img.size() * 2, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // img is a local
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_cols_spectral_tc<L, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<L>::SMEM);
    return e;
}

cudaError_t prepare_tc_columns(int N, int bf16, void* dft_dev, cudaStream_t st) {
#define CPM_TC(n)                                                                              \
    if (N == n) return bf16 ? upload_image<n, 1>(dft_dev, st) : upload_image<n, 0>(dft_dev, st);
    CPM_TC(1024) CPM_TC(2048) CPM_TC(4096)
#undef CPM_TC
    return cudaErrorInvalidValue;
}

cudaError_t launch_cols_spectral_tc(int N, int bf16, float2* spec, float2* spec2, float2* edge, const float* kq,
                                    const float2* tw, const void* dft_dev, float g, int* status, int skip_mma,
                                    int batch, cudaStream_t st) {
#define CPM_TC(n)                                                                                                 \
    if (N == n) {                                                                                                 \
        using S = TcShape<n>;                                                                                     \
        const dim3 grid((n / 2) / S::B, batch);                                                                   \
        if (bf16)                                                                                                 \
            k_cols_spectral_tc<n, 1><<<grid, kTcThreads, S::SMEM, st>>>(spec, spec2, edge, kq, tw,                \
                                                                        static_cast<const uint4*>(dft_dev), g, status, skip_mma); \
        else                                                                                                      \
            k_cols_spectral_tc<n, 0><<<grid, kTcThreads, S::SMEM, st>>>(spec, spec2, edge, kq, tw,                \
                                                                        static_cast<const uint4*>(dft_dev), g, status, skip_mma); \
        return cudaGetLastError();                                                                                \
    }
    CPM_TC(1024) CPM_TC(2048) CPM_TC(4096)
#undef CPM_TC
    return cudaErrorInvalidValue;
}

}  // namespace cpm
