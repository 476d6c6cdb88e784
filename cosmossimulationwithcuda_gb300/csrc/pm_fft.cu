// FFT convolution passes of the particle-mesh step and the FP64 filter build.
//
// The reference convolves the density with the Green's lattice through
// cuFFT: copy to complex (CosmosCuda.cuh:596-612), forward C2C FFT (:1266),
// multiply by FFT(G) (:149-173), divide by the FFT of the mass-assignment
// kernel with 0.001 regularisation (:120-148), inverse C2C FFT (:1291), shift
// by N/2 and divide by N^2 (:333-355).  With G real and even and the
// assignment kernel a (shifted) delta or 2x2 box, all of that collapses to
//     phi = IFFT2( FFT2(rho) * K ),   K = Ghat * W / (W^2 + 0.001) / N^2,
// W = 1 (NGP) or cos(pi kx/N) cos(pi ky/N) (CIC), K real and even in both
// axes.  The N/2 shifts of the reference cancel (the (-1)^(kx+ky) factor of
// the assignment kernel's spectrum undoes k_shiftLattice).
//
// Passes (all hand-written, no cuFFT):
//  1. k_rows_r2c   : B density rows per CTA -> real FFT of each row (one
//                    N/2-point complex FFT + split), stored TRANSPOSED as
//                    spec[kx][y] so that the column pass reads contiguous
//                    lines.  kx = 0 and kx = N/2 (both real along x) share
//                    line 0 as X0 + i*XN/2.
//  2. k_cols_conv  : per line kx: forward FFT over y, multiply by K (line 0
//                    unpacks / repacks its two real spectra), inverse FFT over
//                    y, written back in place.
//  3. k_rows_c2r   : B rows per CTA, Hermitian pre-split + N/2-point inverse
//                    FFT, the potential row written as float2 pairs.
// The filter build runs passes 1-2 in FP64 on the Green's lattice.
//
// Batches: every pass takes gridDim.y independent lattices of the same N
// stored back to back (an ensemble of simulations); blockIdx.y selects the
// lattice, and the filter K and the twiddles are shared.
#include <cmath>
#include <vector>

#include "fft_engine.cuh"
#include "pm_internal.h"
#include "tma.cuh"

namespace cpm {

// ---- launch shapes ------------------------------------------------------------------
// Launch shapes (chosen by timing variants at 2048^2): radix-16 Stockham
// stages with one radix-16 butterfly per thread per stage of the forward
// transforms, about 4096 points per row CTA (at least 4 rows, so that the
// transposed spectrum moves in 32-byte sectors) and one 2048-point line per
// column CTA, so that 2-4 CTAs are resident per SM and their load /
// transform / store phases overlap; the spectral passes' two inverse
// transforms per CTA run two butterflies per thread (128 registers), except
// up to 512^2 (SpecShape).  Below 2048^2 the rows and lines per CTA shrink
// so that one lattice still spreads over at least 128 CTAs (N/128 rows,
// N/256 lines).  FP64 (filter build) halves the rows to keep shared memory
// in range.
constexpr int kMaxRadix = 16;
constexpr int ceil_pow2_min(int v, int lo) { return v < lo ? lo : v; }
constexpr int clamp_threads(int v) { return v < 64 ? 64 : (v > 1024 ? 1024 : v); }

template <class T, int N>
struct RowShape {
    static constexpr int M = N / 2;
    static constexpr int Bw = 4096 / M < N / 128 ? 4096 / M : N / 128;  // work per CTA vs CTA count
    static constexpr int Bf0 = ceil_pow2_min(Bw, 4);
    static constexpr int Bf = Bf0 > N ? N : Bf0;
    static constexpr int B = (sizeof(T) == 8 && Bf > 1) ? (Bf / 2) : Bf;  // rows per CTA
    static constexpr int NT = clamp_threads(B * M / kMaxRadix);
    static constexpr size_t smem = size_t(B) * LinePad<M>::value * sizeof(cplx_t<T>);
};

template <class T, int N>
struct ColShape {
    static constexpr int M = N / 2;
    static constexpr int Bw = 2048 / N < M / 128 ? 2048 / N : M / 128;
    static constexpr int B0 = ceil_pow2_min(Bw, 1);
    static constexpr int B = B0 > M ? M : B0;  // lines per CTA
    static constexpr int NT = clamp_threads(B * N / kMaxRadix);
    static constexpr size_t smem = size_t(B) * LinePad<N>::value * sizeof(cplx_t<T>);
};

// Register limits (resident CTAs per SM) of the spectral passes.
#ifndef CPM_COLS_SPECTRAL_MINB
#define CPM_COLS_SPECTRAL_MINB 3
#endif
#ifndef CPM_C2R_SPECTRAL_MINB
#define CPM_C2R_SPECTRAL_MINB 2
#endif
// Up to this lattice size the column pass also runs one butterfly per thread
// (twice the threads, ~90 registers instead of ~155): measured 38.3 -> 36.2 us
// for the 512^2 force passes, +2% at 1024^2 and +4% at 2048^2.
#ifndef CPM_COLS_FULL_MAX_N
#define CPM_COLS_FULL_MAX_N 512
#endif


// Minimum resident CTAs per SM for a block size (register limit of launch bounds).
template <int NT>
struct MinBlocks {
    static constexpr int value = NT <= 128 ? 6 : (NT <= 256 ? 4 : (NT <= 512 ? 2 : 1));
};

// Resident CTAs per SM asked of the register allocator: WANT, but no more
// than SMEM bytes of shared memory per CTA let reside, and never so many that
// a thread is left fewer than FLOOR registers (a tighter limit only spills:
// at 4096^2 and 8192^2 the long lines need 512-thread CTAs, which shared
// memory already holds to one or two per SM).
template <int NT, size_t SMEM, int WANT, int FLOOR>
struct FitBlocks {
    static constexpr int by_regs = 65536 / (NT * FLOOR);
    static constexpr int by_smem = int((228u * 1024u) / (SMEM + 1024u));
    static constexpr int v0 = WANT < by_regs ? WANT : by_regs;
    static constexpr int v1 = v0 < by_smem ? v0 : by_smem;
    static constexpr int value = v1 < 1 ? 1 : v1;
};

// ---- pass 1: rows, real -> half spectrum, transposed store --------------------------------
// Body of the row pass: B rows from `src(line, i)` (row `line` as M complex
// values z[n] = (x[2n], x[2n+1])), transformed in shared memory `s`.
template <class T, int N, int B, int NT, class Src>
__device__ __forceinline__ void r2c_rows(const Src& src, cplx_t<T>* s, cplx_t<T>* __restrict__ spec,
                                         const cplx_t<T>* __restrict__ tw, T* clear, int y0) {
    using C = cplx_t<T>;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<M>::value;
    auto dst = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<M, B, NT, -1, C, kMaxRadix>(s, src, dst, tw, 2);
    if (clear) {  // the rows were read (fft_lines ends with a barrier): zero them for the next deposit
        C* z = reinterpret_cast<C*>(clear + size_t(blockIdx.y) * N * N + size_t(y0) * N);
        for (int i = threadIdx.x; i < B * M; i += NT) z[i] = cmake<C>(T(0), T(0));
    }
    // X[k] = (Z[k] + conj Z[M-k])/2 - i/2 W^k (Z[k] - conj Z[M-k]),  W = exp(-2 pi i/N)
    for (int idx = threadIdx.x; idx < M * B; idx += NT) {
        const int k = idx / B;
        const int b = idx - k * B;
        const C zk = s[b * LP + pad16(k)];
        C out;
        if (k == 0) {
            out = cmake<C>(zk.x + zk.y, zk.x - zk.y);  // (X[0], X[N/2]) packed
        } else {
            const C zm = cconj(s[b * LP + pad16(M - k)]);
            const C a = cadd(zk, zm);
            const C wd = cmul(tw[k], csub(zk, zm));
            out = cmake<C>(T(0.5) * (a.x + wd.y), T(0.5) * (a.y - wd.x));
        }
        spec[size_t(k) * N + y0 + b] = out;
    }
}

template <class T, int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N / 2>::value * sizeof(cplx_t<T>),
                                                 MinBlocks<NT>::value, sizeof(T) == 8 ? 128 : 64>::value))
    k_rows_r2c(const T* __restrict__ in, cplx_t<T>* __restrict__ spec,
                                                 const cplx_t<T>* __restrict__ tw, T* clear) {
    using C = cplx_t<T>;
    constexpr int M = N / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    dependency_wait();
    allow_dependents();
    const int y0 = int(blockIdx.x) * B;
    in += size_t(blockIdx.y) * N * N;
    spec += size_t(blockIdx.y) * M * N;
    const C* rows = reinterpret_cast<const C*>(in + size_t(y0) * N);
    auto src = [rows](int line, int i) { return rows[line * M + i]; };
    r2c_rows<T, N, B, NT>(src, s, spec, tw, clear, y0);
}

// The dynamic shared memory of a kernel is only guaranteed 16-byte alignment;
// a tensor-map load needs a 128-byte aligned destination.  TMA kernels ask for
// kTmaAlignPad extra bytes and start their tiles at the next 128-byte boundary.
constexpr size_t kTmaAlignPad = 128;
__device__ __forceinline__ unsigned char* align128(unsigned char* p) {
    const uint32_t a = bulk::smem_u32(p);
    return p + ((128u - (a & 127u)) & 127u);
}

// Self-check before a tensor-map load: a destination off the 128-byte grid is
// recorded (*status = 3) and the tile skipped, never handed to the copy engine
// (the same answer in every thread of the CTA).
__device__ __forceinline__ bool tma_dst_ok(const void* dst, int* status) {
    if ((bulk::smem_u32(dst) & 127u) == 0u) return true;
    if (threadIdx.x == 0) atomicMax(status, 3);
    return false;
}

// A bounded TMA wait, decided for the whole CTA: false (every thread) when any
// thread's wait ran out; thread 0 then records it and waits once more for the
// copy in flight, so that it has landed before the CTA releases its shared memory.
__device__ __forceinline__ bool tile_landed(bool ok, uint64_t* bar, int* status) {
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) atomicMax(status, bulk::wait(bar, 0) ? 1 : 2);
    return ok;
}

// The row pass with its B rows staged by one tensor-map load (TMA) into the
// same shared memory the transform then works in: the first radix stage reads
// every input value into registers before it stores (fft_stage), so the dense
// tile and the padded lines can share the space.
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N / 2>::value * sizeof(float2),
                                                 MinBlocks<NT>::value, 64>::value))
    k_rows_r2c_tma(const __grid_constant__ CUtensorMap rho_map, float2* __restrict__ spec,
                   const float2* __restrict__ tw, float* clear, int* status) {
    using C = float2;
    constexpr int M = N / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    C* s = reinterpret_cast<C*>(align128(smem_raw));
    if (threadIdx.x == 0) {
        bulk::mbar_init(&bar, 1);
        bulk::fence_barrier_init();
        tma::prefetch_map(&rho_map);
    }
    __syncthreads();
    dependency_wait();
    allow_dependents();
    const int y0 = int(blockIdx.x) * B;
    if (!tma_dst_ok(s, status)) return;
    if (!tile_landed(tma::load_rows_sync(s, &rho_map, y0, int(blockIdx.y), uint32_t(B) * N * 4u, &bar, 0), &bar,
                     status))
        return;
    spec += size_t(blockIdx.y) * M * N;
    const C* land = s;
    auto src = [land](int line, int i) { return land[line * M + i]; };
    r2c_rows<float, N, B, NT>(src, s, spec, tw, clear, y0);
}

// ---- pass 2: columns, forward FFT x K x inverse FFT ----------------------------------------
// kq: (N/2+1) x (N/2+1) floats, kq[kx*(M+1) + min(ky, N-ky)].
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N>::value * sizeof(float2),
                                                 MinBlocks<NT>::value, 80>::value))
    k_cols_conv(float2* __restrict__ spec, const float* __restrict__ kq,
                                                  const float2* __restrict__ tw) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<N>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx0 = int(blockIdx.x) * B;
    C* lines = spec + size_t(blockIdx.y) * M * N + size_t(kx0) * N;
    auto gload = [lines](int line, int i) { return lines[size_t(line) * N + i]; };
    auto gstore = [lines](int line, int i, C v) { lines[size_t(line) * N + i] = v; };
    auto sload = [s](int line, int i) { return s[line * LP + pad16(i)]; };
    auto sstore = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<N, B, NT, -1, C, kMaxRadix>(s, gload, sstore, tw, 1);
    for (int idx = threadIdx.x; idx < B * (M + 1); idx += NT) {
        const int b = idx / (M + 1);
        const int ky = idx - b * (M + 1);
        const int kx = kx0 + b;
        const int i1 = b * LP + pad16(ky);
        const int i2 = b * LP + pad16((N - ky) & (N - 1));
        if (kx != 0) {
            const float kv = __ldg(kq + size_t(kx) * (M + 1) + ky);
            s[i1] = cscale(s[i1], kv);
            if (ky != 0 && ky != M) s[i2] = cscale(s[i2], kv);
        } else {
            // line 0 holds P = X0 + i XM with X0, XM Hermitian in ky:
            // P' = (K0+KM)/2 * P[ky] + (K0-KM)/2 * conj(P[N-ky])
            const float k0 = __ldg(kq + ky);
            const float km = __ldg(kq + size_t(M) * (M + 1) + ky);
            const float p = 0.5f * (k0 + km), q = 0.5f * (k0 - km);
            const C z1 = s[i1], z2 = s[i2];
            s[i1] = cadd(cscale(z1, p), cscale(cconj(z2), q));
            if (ky != 0 && ky != M) s[i2] = cadd(cscale(z2, p), cscale(cconj(z1), q));
        }
    }
    __syncthreads();
    fft_lines<N, B, NT, +1, C, kMaxRadix>(s, sload, gstore, tw, 1);
}

// FP64 forward column FFT for the filter build: writes the real part of the
// 2-D spectrum of a real, even input as ghat[kx][ky], kx in [0, N/2], ky in [0, N).
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, 1) k_cols_fwd_real64(const double2* __restrict__ spec, double* __restrict__ ghat,
                                                        const double2* __restrict__ tw) {
    using C = double2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<N>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx0 = int(blockIdx.x) * B;
    const C* lines = spec + size_t(kx0) * N;
    auto gload = [lines](int line, int i) { return lines[size_t(line) * N + i]; };
    auto sstore = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<N, B, NT, -1, C, kMaxRadix>(s, gload, sstore, tw, 1);
    for (int idx = threadIdx.x; idx < B * N; idx += NT) {
        const int b = idx / N;
        const int ky = idx - b * N;
        const int kx = kx0 + b;
        const C z1 = s[b * LP + pad16(ky)];
        if (kx != 0) {
            ghat[size_t(kx) * N + ky] = z1.x;
        } else {
            const C z2 = s[b * LP + pad16((N - ky) & (N - 1))];
            ghat[ky] = 0.5 * (z1.x + z2.x);                     // spectrum of line kx = 0
            ghat[size_t(M) * N + ky] = 0.5 * (z1.y + z2.y);     // spectrum of line kx = N/2
        }
    }
}

// ---- pass 3: rows, half spectrum (transposed) -> real potential rows -----------------------
// Hermitian pre-split of `lines` half spectra in shared memory (line stride
// LinePad<M>): Z[k] = (X[k] + conj X[M-k]) + i W^-k (X[k] - conj X[M-k]) is
// twice the spectrum of z[n] = x[2n] + i x[2n+1]; pairs (k, M-k) in one thread.
// Line element 0 holds the packed (X[0], X[N/2]).
template <int M, int NT>
__device__ __forceinline__ void c2r_presplit(float2* s, int lines, const float2* __restrict__ tw) {
    using C = float2;
    constexpr int LP = LinePad<M>::value;
    constexpr int H = M / 2 + 1;
    for (int idx = threadIdx.x; idx < H * lines; idx += NT) {
        const int b = idx / H;
        const int k = idx - b * H;
        C* row = s + b * LP;
        if (k == 0) {
            const C x = row[0];
            row[0] = cmake<C>(x.x + x.y, x.x - x.y);
        } else {
            const C xk = row[pad16(k)];
            const C xm = row[pad16(M - k)];
            {
                const C a = cadd(xk, cconj(xm));
                const C d = cmul(cconj(tw[k]), csub(xk, cconj(xm)));
                row[pad16(k)] = cmake<C>(a.x - d.y, a.y + d.x);
            }
            if (k != M - k) {
                const C a = cadd(xm, cconj(xk));
                const C d = cmul(cconj(tw[M - k]), csub(xm, cconj(xk)));
                row[pad16(M - k)] = cmake<C>(a.x - d.y, a.y + d.x);
            }
        }
    }
}

// B rows per CTA; the half spectrum is transposed: element (k, row) at
// spec[k * STRIDE + row].
template <int N, int B, int NT, int STRIDE = N>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N / 2>::value * sizeof(float2),
                                                 MinBlocks<NT>::value, 64>::value))
    k_rows_c2r(const float2* __restrict__ spec, float* __restrict__ out,
                                                 const float2* __restrict__ tw) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<M>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int y0 = int(blockIdx.x) * B;
    spec += size_t(blockIdx.y) * M * STRIDE;              // M lines of STRIDE per lattice
    out += size_t(blockIdx.y) * gridDim.x * B * N;        // gridDim.x * B rows per lattice
    for (int idx = threadIdx.x; idx < M * B; idx += NT) {
        const int k = idx / B;
        const int b = idx - k * B;
        s[b * LP + pad16(k)] = spec[size_t(k) * STRIDE + y0 + b];
    }
    __syncthreads();
    c2r_presplit<M, NT>(s, B, tw);
    __syncthreads();
    float2* orow = reinterpret_cast<float2*>(out + size_t(y0) * N);
    auto sload = [s](int line, int i) { return s[line * LP + pad16(i)]; };
    auto gstore = [orow](int line, int i, C v) { orow[size_t(line) * M + i] = v; };
    fft_lines<M, B, NT, +1, C, kMaxRadix>(s, sload, gstore, tw, 2);
}

// ---- spectral force ---------------------------------------------------------------------------
// The reference's 4th-order difference (CosmosCuda.cuh:174-229) is the
// convolution with a stencil whose symbol is i*S(k), S = (8 sin t - sin 2t)/6,
// t = 2 pi k / N.  Applying it in Fourier space gives the periodic force
// straight out of the inverse FFT.  The reference clamps out-of-range
// neighbours to the centre value instead of wrapping, which differs from the
// periodic stencil only at x (or y) in {0, 1, N-2, N-1}; there the difference
// is a combination of three potential differences along the line,
//   D01 = phi(0) - phi(N-1),  D02 = phi(0) - phi(N-2),  D13 = phi(1) - phi(N-1),
//   dF(0) = (-8 D01 + D02)/12,  dF(1) = D13/12,  dF(N-2) = D02/12,
//   dF(N-1) = (D13 - 8 D01)/12   (times the gravity multiplier),
// evaluated here as spectral sums so that no FP32 potential is differenced.
//
// Edge-difference weights at frequency k (table tw[k] = exp(-2 pi i k/N)):
//   w01 = 1 - tw[k],  w02 = 1 - tw[2k],  w13 = conj(tw[k]) - tw[k].
__device__ __forceinline__ void edge_weights(const float2* __restrict__ tw, int k, int N, float2& w01, float2& w02,
                                             float2& w13) {
    const float2 t1 = tw[k & (N - 1)];
    const float2 t2 = tw[(2 * k) & (N - 1)];
    w01 = make_float2(1.0f - t1.x, -t1.y);
    w02 = make_float2(1.0f - t2.x, -t2.y);
    w13 = make_float2(0.0f, -2.0f * t1.y);
}

// Sum of `v` over the CTA (NT threads); result valid in every thread.
template <int NT, int K>
__device__ __forceinline__ void block_sum(float (&v)[K], float* red) {
    constexpr int NW = NT / 32;
#pragma unroll
    for (int j = 0; j < K; ++j)
        for (int off = 16; off > 0; off >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int j = 0; j < K; ++j) red[(threadIdx.x >> 5) * K + j] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < K; ++j) {
        float s = 0.0f;
        for (int w = 0; w < NW; ++w) s += red[w * K + j];
        v[j] = s;
    }
    __syncthreads();
}

// Columns, spectral force: forward FFT over y, x K, then two inverse FFTs over
// y: Phi = IFFT_y(phi_hat) (back into spec) and Psi = IFFT_y(phi_hat * i S(ky) * g)
// (into spec2); and the three y-edge differences of every line,
// edge[kx * 4 + j] = sum_ky phi_hat(kx, ky) w_j(ky).
// Body for B lines from `src(line, i)`; `lines` / `lines2` receive Phi / Psi.
template <int N, int B, int NT, class Src>
__device__ __forceinline__ void cols_spectral_lines(const Src& src, float2* s, float2* __restrict__ lines,
                                                    float2* __restrict__ lines2, float2* __restrict__ edge,
                                                    const float* __restrict__ kq, const float2* __restrict__ tw,
                                                    float g, int kx0) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<N>::value;
    float* red = reinterpret_cast<float*>(s + 2 * B * LP);
    auto sstore = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<N, B, NT, -1, C, kMaxRadix>(s, src, sstore, tw, 1);
    for (int idx = threadIdx.x; idx < B * (M + 1); idx += NT) {
        const int b = idx / (M + 1);
        const int ky = idx - b * (M + 1);
        const int kx = kx0 + b;
        const int i1 = b * LP + pad16(ky);
        const int i2 = b * LP + pad16((N - ky) & (N - 1));
        if (kx != 0) {
            const float kv = __ldg(kq + size_t(kx) * (M + 1) + ky);
            s[i1] = cscale(s[i1], kv);
            if (ky != 0 && ky != M) s[i2] = cscale(s[i2], kv);
        } else {
            const float k0 = __ldg(kq + ky);
            const float km = __ldg(kq + size_t(M) * (M + 1) + ky);
            const float p = 0.5f * (k0 + km), q = 0.5f * (k0 - km);
            const C z1 = s[i1], z2 = s[i2];
            s[i1] = cadd(cscale(z1, p), cscale(cconj(z2), q));
            if (ky != 0 && ky != M) s[i2] = cadd(cscale(z2, p), cscale(cconj(z1), q));
        }
    }
    __syncthreads();
    for (int b = 0; b < B; ++b) {
        float acc[6] = {0, 0, 0, 0, 0, 0};
        for (int ky = threadIdx.x; ky < N; ky += NT) {
            const C v = s[b * LP + pad16(ky)];
            C w01, w02, w13;
            edge_weights(tw, ky, N, w01, w02, w13);
            const C a = cmul(v, w01), c = cmul(v, w02), d = cmul(v, w13);
            acc[0] += a.x; acc[1] += a.y; acc[2] += c.x; acc[3] += c.y; acc[4] += d.x; acc[5] += d.y;
            // i * S(ky) * g, S = (8 sin t - sin 2t) / 6 with sin t = -tw[ky].y
            const float S = g * (tw[(2 * ky) & (N - 1)].y - 8.0f * tw[ky].y) * (1.0f / 6.0f);
            s[(B + b) * LP + pad16(ky)] = cmake<C>(-S * v.y, S * v.x);
        }
        block_sum<NT, 6>(acc, red);
        if (threadIdx.x == 0) {
            float2* e = edge + size_t(kx0 + b) * 4;
            e[0] = make_float2(acc[0], acc[1]);
            e[1] = make_float2(acc[2], acc[3]);
            e[2] = make_float2(acc[4], acc[5]);
        }
    }
    __syncthreads();
    auto sload = [s](int line, int i) { return s[line * LP + pad16(i)]; };
    auto gstore2 = [lines, lines2](int line, int i, C v) {
        if (line < B)
            lines[size_t(line) * N + i] = v;
        else
            lines2[size_t(line - B) * N + i] = v;
    };
    fft_lines<N, 2 * B, NT, +1, C, kMaxRadix>(s, sload, gstore2, tw, 1);
}

template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, 2 * size_t(B) * LinePad<N>::value * sizeof(float2),
                                                 CPM_COLS_SPECTRAL_MINB, (N <= CPM_COLS_FULL_MAX_N ? 64 : 128)>::value))
    k_cols_spectral(float2* __restrict__ spec, float2* __restrict__ spec2,
                                                         float2* __restrict__ edge, const float* __restrict__ kq,
                                                         const float2* __restrict__ tw, float g) {
    using C = float2;
    constexpr int M = N / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);  // lines [0, B): phi_hat; [B, 2B): phi_hat * iS
    dependency_wait();
    allow_dependents();
    const int kx0 = int(blockIdx.x) * B;
    spec += size_t(blockIdx.y) * M * N;
    spec2 += size_t(blockIdx.y) * M * N;
    edge += size_t(blockIdx.y) * M * 4;
    C* lines = spec + size_t(kx0) * N;
    auto gload = [lines](int line, int i) { return lines[size_t(line) * N + i]; };
    cols_spectral_lines<N, B, NT>(gload, s, lines, spec2 + size_t(kx0) * N, edge, kq, tw, g, kx0);
}

// Byte offset (from the 128-byte aligned base) of the TMA landing tile of the
// spectral column pass: the B dense lines land in the upper half of the shared
// lines (phi_hat * iS, unused until after the forward transform), on a
// 128-byte boundary.
template <int N, int B>
constexpr size_t cols_land_offset() {
    return ((2 * size_t(B) * LinePad<N>::value - size_t(B) * N) * sizeof(float2)) & ~size_t(127);
}

// The spectral column pass with its B lines staged by one tensor-map load.
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, 2 * size_t(B) * LinePad<N>::value * sizeof(float2),
                                                 CPM_COLS_SPECTRAL_MINB, (N <= CPM_COLS_FULL_MAX_N ? 64 : 128)>::value))
    k_cols_spectral_tma(const __grid_constant__ CUtensorMap spec_map, float2* __restrict__ spec,
                        float2* __restrict__ spec2, float2* __restrict__ edge, const float* __restrict__ kq,
                        const float2* __restrict__ tw, float g, int* status) {
    using C = float2;
    constexpr int M = N / 2;
    static_assert(cols_land_offset<N, B>() >= size_t(B) * LinePad<N>::value * sizeof(float2), "landing tile");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    unsigned char* base = align128(smem_raw);
    C* s = reinterpret_cast<C*>(base);
    C* land = reinterpret_cast<C*>(base + cols_land_offset<N, B>());
    if (threadIdx.x == 0) {
        bulk::mbar_init(&bar, 1);
        bulk::fence_barrier_init();
        tma::prefetch_map(&spec_map);
    }
    __syncthreads();
    dependency_wait();
    allow_dependents();
    const int kx0 = int(blockIdx.x) * B;
    if (!tma_dst_ok(land, status)) return;
    if (!tile_landed(tma::load_rows_sync(land, &spec_map, kx0, int(blockIdx.y), uint32_t(B) * N * 8u, &bar, 0),
                     &bar, status))
        return;
    spec += size_t(blockIdx.y) * M * N;
    spec2 += size_t(blockIdx.y) * M * N;
    edge += size_t(blockIdx.y) * M * 4;
    auto lload = [land](int line, int i) { return land[line * N + i]; };
    cols_spectral_lines<N, B, NT>(lload, s, spec + size_t(kx0) * N, spec2 + size_t(kx0) * N, edge, kq, tw, g, kx0);
}

// Rows, spectral force: C2R of Fx = IFFT_x(i S(kx) g Phi) and Fy = IFFT_x(Psi)
// with the x-edge corrections from Phi, written as interleaved (fx, fy).  The
// y-edge corrections of rows 0, 1, N-2, N-1 follow in k_apply_edge_rows.
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, 2 * size_t(B) * LinePad<N / 2>::value * sizeof(float2),
                                                 CPM_C2R_SPECTRAL_MINB, (N <= 512 ? 64 : 128)>::value))
    k_rows_c2r_spectral(const float2* __restrict__ spec,
                                                             const float2* __restrict__ spec2,
                                                             float4* __restrict__ force,
                                                             const float2* __restrict__ tw, float g) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<M>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);  // lines [0, B): Fx spectra, [B, 2B): Fy spectra
    float* red = reinterpret_cast<float*>(s + 2 * B * LP);
    __shared__ float dx[B][3];
    dependency_wait();
    allow_dependents();
    const int y0 = int(blockIdx.x) * B;
    spec += size_t(blockIdx.y) * M * N;
    spec2 += size_t(blockIdx.y) * M * N;
    force += size_t(blockIdx.y) * M * N;  // float4 = two cells
#pragma unroll 4  // several transposed loads in flight per thread (measured: -2 us per step at 2048^2)
    for (int idx = threadIdx.x; idx < M * B; idx += NT) {
        const int k = idx / B;
        const int b = idx - k * B;
        s[b * LP + pad16(k)] = spec[size_t(k) * N + y0 + b];
        s[(B + b) * LP + pad16(k)] = spec2[size_t(k) * N + y0 + b];
    }
    __syncthreads();
    // One pass over the potential half spectra Phi: the x-edge differences
    //   D = Phi(M) ((-1)^a - (-1)^b) + 2 sum_{k=1}^{M-1} Re(Phi(k) w(k))
    // of every row, and the Fx spectrum i S(kx) g Phi in place (S(0) = S(N/2) = 0
    // empties the packed element 0).
    float acc[3 * B];
#pragma unroll
    for (int j = 0; j < 3 * B; ++j) acc[j] = 0.0f;
    for (int k = threadIdx.x; k < M; k += NT) {
        C w01, w02, w13;
        edge_weights(tw, k, N, w01, w02, w13);
        const float S = g * (tw[(2 * k) & (N - 1)].y - 8.0f * tw[k].y) * (1.0f / 6.0f);
#pragma unroll
        for (int b = 0; b < B; ++b) {
            C* p = s + b * LP + pad16(k);
            const C v = *p;
            if (k != 0) {
                acc[3 * b + 0] += v.x * w01.x - v.y * w01.y;
                acc[3 * b + 1] += v.x * w02.x - v.y * w02.y;
                acc[3 * b + 2] += v.x * w13.x - v.y * w13.y;
                *p = cmake<C>(-S * v.y, S * v.x);
            } else {
                acc[3 * b + 0] += v.y;  // Phi(N/2): (-1)^0 - (-1)^(N-1) = 2 with the factor 2 below
                *p = cmake<C>(0.0f, 0.0f);
            }
        }
    }
    block_sum<NT, 3 * B>(acc, red);
    if (threadIdx.x < B) {
        dx[threadIdx.x][0] = 2.0f * acc[3 * threadIdx.x + 0];
        dx[threadIdx.x][1] = 2.0f * acc[3 * threadIdx.x + 1];
        dx[threadIdx.x][2] = 2.0f * acc[3 * threadIdx.x + 2];
    }
    c2r_presplit<M, NT>(s, 2 * B, tw);
    __syncthreads();
    auto sload = [s](int line, int i) { return s[line * LP + pad16(i)]; };
    auto sstore = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<M, 2 * B, NT, +1, C, kMaxRadix>(s, sload, sstore, tw, 2);
    // interleave, with the x-edge corrections
    const float c12 = g * (1.0f / 12.0f);
    for (int idx = threadIdx.x; idx < M * B; idx += NT) {
        const int b = idx / M;
        const int i = idx - b * M;
        const C fx = s[b * LP + pad16(i)];        // (Fx[2i], Fx[2i+1])
        const C fy = s[(B + b) * LP + pad16(i)];  // (Fy[2i], Fy[2i+1])
        float4 o = make_float4(fx.x, fy.x, fx.y, fy.y);
        if (i == 0) {  // x = 0, 1
            o.x += (-8.0f * dx[b][0] + dx[b][1]) * c12;
            o.z += dx[b][2] * c12;
        } else if (i == M - 1) {  // x = N-2, N-1
            o.x += dx[b][1] * c12;
            o.z += (dx[b][2] - 8.0f * dx[b][0]) * c12;
        }
        force[(size_t(y0 + b) * N) / 2 + i] = o;
    }
}

// y-edge corrections of Fy on rows 0, 1, N-2, N-1 from the three y-edge
// differences of every column (dy[j * N + x], j = D01, D02, D13).
__global__ void k_apply_edge_rows(const float* __restrict__ dy, float2* __restrict__ force, int N, float g) {
    allow_dependents();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    dy += size_t(blockIdx.y) * 3 * N;
    force += size_t(blockIdx.y) * N * N;
    const float c12 = g * (1.0f / 12.0f);
    const float d01 = dy[x], d02 = dy[N + x], d13 = dy[2 * N + x];
    force[x].y += (-8.0f * d01 + d02) * c12;
    force[size_t(N) + x].y += d13 * c12;
    force[size_t(N - 2) * N + x].y += d02 * c12;
    force[size_t(N - 1) * N + x].y += (d13 - 8.0f * d01) * c12;
}

// ---- filter build helpers ----------------------------------------------------------------
// Green's lattice G(i, j) = 1/r with minimum-image distances and 3.0 at
// r <= 0.5 (CosmosCuda.cuh:100-117), in FP64.
__global__ void k_green64(double* __restrict__ g, int N) {
    const int64_t NN = int64_t(N) * N;
    for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < NN; idx += int64_t(gridDim.x) * blockDim.x) {
        const int i = int(idx % N), j = int(idx / N);
        const double dx = double(i <= N / 2 ? i : i - N);
        const double dy = double(j <= N / 2 ? j : j - N);
        const double r = sqrt(dx * dx + dy * dy);
        g[idx] = r > 0.5 ? 1.0 / r : 3.0;
    }
}

// K = Ghat * W / (W^2 + 0.001) / N^2 on the quarter (kx, ky) in [0, N/2]^2.
__global__ void k_build_kq(const double* __restrict__ ghat, float* __restrict__ kq, int N, int cic) {
    const int M = N / 2;
    const int total = (M + 1) * (M + 1);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / (M + 1), ky = idx - kx * (M + 1);
        const double g = ghat[size_t(kx) * N + ky];
        const double w = cic ? cospi(double(kx) / N) * cospi(double(ky) / N) : 1.0;
        kq[idx] = float(g * w / (w * w + 0.001) / (double(N) * double(N)));
    }
}

// ---- host launchers ------------------------------------------------------------------------
template <class K>
static cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
}

template <int N>
static cudaError_t conv_passes_n(const float* rho, float2* spec, const float* kq, float* phi, const float2* tw,
                                 int batch, cudaStream_t st, float* clear) {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    k_rows_r2c<float, N, RS::B, RS::NT><<<dim3(N / RS::B, batch), RS::NT, RS::smem, st>>>(rho, spec, tw, clear);
    k_cols_conv<N, CS::B, CS::NT><<<dim3((N / 2) / CS::B, batch), CS::NT, CS::smem, st>>>(spec, kq, tw);
    k_rows_c2r<N, RS::B, RS::NT><<<dim3(N / RS::B, batch), RS::NT, RS::smem, st>>>(spec, phi, tw);
    return cudaGetLastError();
}

template <int N>
static cudaError_t filter_passes_n(const double* g, double2* spec64, double* ghat, const double2* tw64,
                                   cudaStream_t st) {
    using RS = RowShape<double, N>;
    using CS = ColShape<double, N>;
    cudaError_t e;
    if ((e = allow_smem(k_rows_r2c<double, N, RS::B, RS::NT>, RS::smem)) != cudaSuccess) return e;
    if ((e = allow_smem(k_cols_fwd_real64<N, CS::B, CS::NT>, CS::smem)) != cudaSuccess) return e;
    k_rows_r2c<double, N, RS::B, RS::NT><<<N / RS::B, RS::NT, RS::smem, st>>>(g, spec64, tw64, nullptr);
    k_cols_fwd_real64<N, CS::B, CS::NT><<<(N / 2) / CS::B, CS::NT, CS::smem, st>>>(spec64, ghat, tw64);
    return cudaGetLastError();
}

#define CPM_FOR_EACH_N(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192)

// Spectral-force shapes: the passes keep two lines per transform in shared
// memory (Fx and Fy, or phi_hat and phi_hat * iS), plus reduction scratch.
template <int N>
struct SpecShape {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    static constexpr int M = N / 2;
    static constexpr int RB0 = RS::B;
    static constexpr size_t row_bytes0 = 2 * size_t(RB0) * LinePad<M>::value * sizeof(float2);
    static constexpr int RB = row_bytes0 > 200 * 1024 ? RB0 / 2 : RB0;  // rows per CTA
    // Up to 512^2 one butterfly per thread per stage (2 RB lines; 64 registers
    // a thread), above that two (128 registers): measured 43 -> 39 us for the
    // 512^2 force passes, and 83 -> 86 us at 2048^2 the other way round.
    static constexpr int RNT0 = (N <= 512 ? 2 : 1) * RB * M / kMaxRadix;
    static constexpr int RNT = RNT0 < 64 ? 64 : (RNT0 > 1024 ? 1024 : RNT0);
    // two spectra per row, plus block_sum scratch: one slot per warp for each of the 3 * RB edge sums
    static constexpr size_t row_smem =
        2 * size_t(RB) * LinePad<M>::value * sizeof(float2) + size_t(RNT / 32) * 3 * RB * sizeof(float);
    // column pass threads of one lattice: one butterfly per thread in the
    // inverse transforms (2 B lines) up to CPM_COLS_FULL_MAX_N; batches of
    // lattices keep CS::NT (measured faster for the ensemble's 512^2 class)
    static constexpr int CNT = N <= CPM_COLS_FULL_MAX_N ? clamp_threads(2 * CS::B * N / kMaxRadix) : CS::NT;
    static constexpr size_t col_smem_for(int nt) {
        return 2 * size_t(CS::B) * LinePad<N>::value * sizeof(float2) + size_t(nt / 32) * 6 * 4;
    }
    static constexpr size_t col_smem = col_smem_for(CS::NT);
    static constexpr int ENT0 = M / kMaxRadix;
    static constexpr int ENT = ENT0 < 64 ? 64 : (ENT0 > 1024 ? 1024 : ENT0);  // edge-row C2R threads
    static constexpr size_t edge_smem = size_t(LinePad<M>::value) * sizeof(float2);
};

// The 3-row C2R of the y-edge differences only feeds the 4 boundary rows: it
// runs on the auxiliary stream, concurrent with the main C2R pass (fork/join
// with events, which CUDA-graph capture records as graph edges).
// The tensor-map (TMA) variants of the row and column passes serve lattices
// from kTmaMinN up (smaller lattices keep per-thread loads: their tiles are a
// few KB and their landing space would not fit beside the padded lines).
constexpr int kTmaMinN = 256;
// CPM_SPECTRAL_TMA=0 builds the per-thread-load passes only (for comparisons).
#ifndef CPM_SPECTRAL_TMA
#define CPM_SPECTRAL_TMA 1
#endif

template <int N>
static cudaError_t spectral_passes_n(const float* rho, float2* spec, float2* spec2, float2* edge, float* dy,
                                     const float* kq, float2* force, const float2* tw, float g, int batch,
                                     cudaStream_t st, cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join,
                                     const SpectralTc* tc, float* clear, const SpectralMaps* maps, int* status) {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    using SS = SpecShape<N>;
    const bool dependent = N >= kDependentMinN;
    const bool tma = CPM_SPECTRAL_TMA && N >= kTmaMinN && maps != nullptr && status != nullptr;
    cudaError_t e = cudaSuccess;
    bool cols_done = false;
    if constexpr (N >= kTmaMinN) {
        if (tma) {
            if ((e = launch_dependent(dependent, k_rows_r2c_tma<N, RS::B, RS::NT>, dim3(N / RS::B, batch),
                                      dim3(RS::NT), RS::smem + kTmaAlignPad, st, maps->rho, spec, tw, clear,
                                      status)) != cudaSuccess)
                return e;
            if (!tc) {
                if (batch == 1 && SS::CNT != CS::NT)
                    e = launch_dependent(dependent, k_cols_spectral_tma<N, CS::B, SS::CNT>, dim3(N / 2 / CS::B),
                                         dim3(SS::CNT), SS::col_smem_for(SS::CNT) + kTmaAlignPad, st, maps->spec,
                                         spec, spec2, edge, kq, tw, g, status);
                else
                    e = launch_dependent(dependent, k_cols_spectral_tma<N, CS::B, CS::NT>,
                                         dim3((N / 2) / CS::B, batch), dim3(CS::NT), SS::col_smem + kTmaAlignPad, st,
                                         maps->spec, spec, spec2, edge, kq, tw, g, status);
                if (e != cudaSuccess) return e;
                cols_done = true;
            }
        }
    }
    if (!tma &&
        (e = launch_dependent(dependent, k_rows_r2c<float, N, RS::B, RS::NT>, dim3(N / RS::B, batch), dim3(RS::NT),
                              RS::smem, st, rho, spec, tw, clear)) != cudaSuccess)
        return e;
    if (cols_done) {
    } else if (tc) {
        if ((e = launch_cols_spectral_tc(N, tc->bf16, spec, spec2, edge, kq, tw, tc->dft, g, tc->status,
                                         tc->skip_mma, batch, st)) != cudaSuccess)
            return e;
    } else if (batch == 1 && SS::CNT != CS::NT) {
        if ((e = launch_dependent(dependent, k_cols_spectral<N, CS::B, SS::CNT>, dim3(N / 2 / CS::B), dim3(SS::CNT),
                                  SS::col_smem_for(SS::CNT), st, spec, spec2, edge, kq, tw, g)) != cudaSuccess)
            return e;
    } else if ((e = launch_dependent(dependent, k_cols_spectral<N, CS::B, CS::NT>, dim3((N / 2) / CS::B, batch),
                                     dim3(CS::NT), SS::col_smem, st, spec, spec2, edge, kq, tw, g)) != cudaSuccess) {
        return e;
    }
    if ((e = cudaEventRecord(fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(aux, fork, 0)) != cudaSuccess) return e;
    k_rows_c2r<N, 1, SS::ENT, 4><<<dim3(3, batch), SS::ENT, SS::edge_smem, aux>>>(edge, dy, tw);
    if ((e = cudaEventRecord(join, aux)) != cudaSuccess) return e;
    if ((e = launch_dependent(dependent, k_rows_c2r_spectral<N, SS::RB, SS::RNT>, dim3(N / SS::RB, batch),
                              dim3(SS::RNT), SS::row_smem, st, spec, spec2, reinterpret_cast<float4*>(force), tw,
                              g)) != cudaSuccess)
        return e;
    if ((e = cudaStreamWaitEvent(st, join, 0)) != cudaSuccess) return e;
    k_apply_edge_rows<<<dim3((N + 255) / 256, batch), 256, 0, st>>>(dy, force, N, g);
    return cudaGetLastError();
}

template <int N>
static cudaError_t prepare_spectral_n() {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    using SS = SpecShape<N>;
    cudaError_t e;
    if constexpr (N >= kTmaMinN) {
        if ((e = allow_smem(k_rows_r2c_tma<N, RS::B, RS::NT>, RS::smem + kTmaAlignPad)) != cudaSuccess) return e;
        if ((e = allow_smem(k_cols_spectral_tma<N, CS::B, CS::NT>, SS::col_smem + kTmaAlignPad)) != cudaSuccess)
            return e;
        if ((e = allow_smem(k_cols_spectral_tma<N, CS::B, SS::CNT>, SS::col_smem_for(SS::CNT) + kTmaAlignPad)) !=
            cudaSuccess)
            return e;
    }
    if ((e = allow_smem(k_cols_spectral<N, CS::B, CS::NT>, SS::col_smem)) != cudaSuccess) return e;
    if ((e = allow_smem(k_cols_spectral<N, CS::B, SS::CNT>, SS::col_smem_for(SS::CNT))) != cudaSuccess) return e;
    if ((e = allow_smem(k_rows_c2r<N, 1, SS::ENT, 4>, SS::edge_smem)) != cudaSuccess) return e;
    return allow_smem(k_rows_c2r_spectral<N, SS::RB, SS::RNT>, SS::row_smem);
}

cudaError_t prepare_spectral_passes(int N) {
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return prepare_spectral_n<n>();
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

template <int N>
static cudaError_t spectral_maps_n(const float* rho, const float2* spec, int batch, SpectralMaps* maps) {
    if constexpr (N < kTmaMinN) {
        return cudaErrorNotSupported;
    } else {
        using RS = RowShape<float, N>;
        using CS = ColShape<float, N>;
        cudaError_t e = make_row_map(&maps->rho, rho, N, N, batch, RS::B);
        if (e == cudaSuccess) e = make_row_map(&maps->spec, spec, 2 * N, N / 2, batch, CS::B);
        return e;
    }
}

cudaError_t make_spectral_maps(int N, const float* rho, const float2* spec, int batch, SpectralMaps* maps) {
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return spectral_maps_n<n>(rho, spec, batch, maps);
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_spectral_force(int N, const float* rho, float2* spec, float2* spec2, float2* edge, float* dy,
                                  const float* kq, float2* force, const float2* tw, float g, cudaStream_t st,
                                  cudaStream_t aux, cudaEvent_t fork, cudaEvent_t join, int batch,
                                  const SpectralTc* tc, float* clear, const SpectralMaps* maps, int* status) {
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    if (tc && !tc_fft_supported(N)) return cudaErrorInvalidValue;
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return spectral_passes_n<n>(rho, spec, spec2, edge, dy, kq, force, tw, g, batch, st, aux, fork, join, tc, \
                                    clear, maps, status);
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

int spectral_launches_per_step() { return 5; }

template <int N>
static cudaError_t prepare_conv_n() {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    cudaError_t e;
    if ((e = allow_smem(k_rows_r2c<float, N, RS::B, RS::NT>, RS::smem)) != cudaSuccess) return e;
    if ((e = allow_smem(k_cols_conv<N, CS::B, CS::NT>, CS::smem)) != cudaSuccess) return e;
    return allow_smem(k_rows_c2r<N, RS::B, RS::NT>, RS::smem);
}

// Raises the dynamic shared-memory limit of the FFT kernels of lattice size N
// on the current device (called once per handle, outside stream capture).
cudaError_t prepare_conv_passes(int N) {
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return prepare_conv_n<n>();
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_conv_passes(int N, const float* rho, float2* spec, const float* kq, float* phi, const float2* tw,
                               cudaStream_t st, int batch, float* clear) {
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return conv_passes_n<n>(rho, spec, kq, phi, tw, batch, st, clear);
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

int conv_launches_per_step() { return 3; }

// Builds the twiddle tables (host, FP64 std::cos/std::sin) and the filter K.
int build_filter(int N, int cic, float* kq_dev, float2* tw_dev, cudaStream_t st) {
    std::vector<float2> twf(N);
    std::vector<double2> twd(N);
    for (int m = 0; m < N; ++m) {
        const double a = -2.0 * M_PI * double(m) / double(N);
        twd[m] = make_double2(std::cos(a), std::sin(a));
        twf[m] = make_float2(float(twd[m].x), float(twd[m].y));
    }
    CPM_CUDA(cudaMemcpyAsync(tw_dev, twf.data(), sizeof(float2) * N, cudaMemcpyHostToDevice, st));
    const size_t NN = size_t(N) * N;
    const int M = N / 2;
    double* g = nullptr;
    double2* spec64 = nullptr;
    double* ghat = nullptr;
    double2* tw64 = nullptr;
    int status = COSMOS_OK;
    auto cleanup = [&]() {
        cudaFreeAsync(g, st);
        cudaFreeAsync(spec64, st);
        cudaFreeAsync(ghat, st);
        cudaFreeAsync(tw64, st);
    };
    if (cudaMallocAsync(&g, sizeof(double) * NN, st) != cudaSuccess ||
        cudaMallocAsync(&spec64, sizeof(double2) * size_t(M) * N, st) != cudaSuccess ||
        cudaMallocAsync(&ghat, sizeof(double) * size_t(M + 1) * N, st) != cudaSuccess ||
        cudaMallocAsync(&tw64, sizeof(double2) * N, st) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return fail(COSMOS_ERR_NOMEM, "filter build: device allocation failed");
    }
    cudaError_t e = cudaMemcpyAsync(tw64, twd.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_green64<<<1024, 256, 0, st>>>(g, N);
        switch (N) {
#define CPM_CASE(n)                                            \
    case n:                                                    \
        e = filter_passes_n<n>(g, spec64, ghat, tw64, st);     \
        break;
            CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
            default:
                e = cudaErrorInvalidValue;
        }
    }
    if (e == cudaSuccess) {
        k_build_kq<<<1024, 256, 0, st>>>(ghat, kq_dev, N, cic);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) status = fail(COSMOS_ERR_CUDA, std::string("filter build: ") + cudaGetErrorString(e));
    cleanup();
    cudaStreamSynchronize(st);
    return status;
}

}  // namespace cpm
