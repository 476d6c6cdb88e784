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

#include "fft_passes.cuh"
#include "pm_internal.h"
#include "tma.cuh"

namespace cpm {

// ---- pass 1: rows, real -> half spectrum, transposed store (body: fft_passes.cuh) --------------
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
    r2c_rows<T, N, B, NT>(src, s, spec, tw, clear ? clear + size_t(blockIdx.y) * N * N : nullptr, y0);
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
    r2c_rows<float, N, B, NT>(src, s, spec, tw, clear ? clear + size_t(blockIdx.y) * N * N : nullptr, y0);
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
// B rows per CTA; the half spectrum is transposed: element (k, row) at
// spec[k * STRIDE + row].
template <int N, int B, int NT, int STRIDE = N>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N / 2>::value * sizeof(float2),
                                                 MinBlocks<NT>::value, 64>::value))
    k_rows_c2r(const float2* __restrict__ spec, float* __restrict__ out,
                                                 const float2* __restrict__ tw) {
    constexpr int M = N / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    spec += size_t(blockIdx.y) * M * STRIDE;        // M lines of STRIDE per lattice
    out += size_t(blockIdx.y) * gridDim.x * B * N;  // gridDim.x * B rows per lattice
    c2r_rows<N, B, NT, STRIDE>(reinterpret_cast<float2*>(smem_raw), spec, out, tw, int(blockIdx.x) * B);
}

// ---- spectral force (bodies: fft_passes.cuh) --------------------------------------------------
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

// Rows, spectral force: C2R of Fx and Fy with the x- and y-edge corrections
// (c2r_spectral_rows, fft_passes.cuh).
template <int N, int B, int NT>
__global__ void __launch_bounds__(NT, (FitBlocks<NT, size_t(B) * LinePad<N>::value * sizeof(float2),
                                                 CPM_C2R_SPECTRAL_MINB, (N <= CPM_C2R_FULL_MAX_N ? 64 : 128)>::value))
    k_rows_c2r_spectral(const float2* __restrict__ spec,
                                                             const float2* __restrict__ spec2,
                                                             const float2* __restrict__ edge,
                                                             float4* __restrict__ force,
                                                             const float2* __restrict__ tw, float g) {
    constexpr int M = N / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float dx[3 * B];
    dependency_wait();
    allow_dependents();
    const size_t lat = size_t(blockIdx.y) * M * N;
    c2r_spectral_rows<N, B, NT>(reinterpret_cast<float2*>(smem_raw), dx, spec + lat, spec2 + lat,
                                edge + size_t(blockIdx.y) * M * 4, force + lat, tw, g, int(blockIdx.x) * B);
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
    static constexpr size_t row_bytes0 = size_t(RB0) * LinePad<N>::value * sizeof(float2);
    static constexpr int RB = row_bytes0 > 200 * 1024 ? RB0 / 2 : RB0;  // rows per CTA
    // Up to 512^2 one butterfly per thread per stage (RB lines of N points; 64
    // registers a thread), above that two (128 registers): measured 43 -> 39 us
    // for the 512^2 force passes, and 83 -> 86 us at 2048^2 the other way round.
    static constexpr int RNT0 = (N <= CPM_C2R_FULL_MAX_N ? 2 : 1) * RB * M / kMaxRadix;
    static constexpr int RNT = RNT0 < 64 ? 64 : (RNT0 > 1024 ? 1024 : RNT0);
    // one N-point line per row (the two half spectra, then Z), plus block_sum
    // scratch: one slot per warp for each of the 3 * RB edge sums
    static constexpr size_t row_smem =
        size_t(RB) * LinePad<N>::value * sizeof(float2) + size_t(RNT / 32) * 3 * RB * sizeof(float);
    // column pass threads of one lattice: one butterfly per thread in the
    // inverse transforms (2 B lines) up to CPM_COLS_FULL_MAX_N; batches of
    // lattices keep CS::NT (measured faster for the ensemble's 512^2 class)
    static constexpr int CNT = N <= CPM_COLS_FULL_MAX_N ? clamp_threads(2 * CS::B * N / kMaxRadix) : CS::NT;
    static constexpr size_t col_smem_for(int nt) {
        return 2 * size_t(CS::B) * LinePad<N>::value * sizeof(float2) + size_t(nt / 32) * 6 * 4;
    }
    static constexpr size_t col_smem = col_smem_for(CS::NT);
    // the other column-pass shape (fft_shape = 1): one butterfly per thread from
    // 1024^2 up (twice CS::NT threads), two below (CS::NT threads)
    static constexpr int ACNT = N <= CPM_COLS_FULL_MAX_N ? CS::NT : clamp_threads(2 * CS::B * N / kMaxRadix);
};

// The tensor-map (TMA) variants of the row and column passes serve lattices
// from kTmaMinN up (smaller lattices keep per-thread loads: their tiles are a
// few KB and their landing space would not fit beside the padded lines).
constexpr int kTmaMinN = 256;
// CPM_SPECTRAL_TMA=0 builds the per-thread-load passes only (for comparisons).
#ifndef CPM_SPECTRAL_TMA
#define CPM_SPECTRAL_TMA 1
#endif

template <int N>
static cudaError_t spectral_passes_n(const float* rho, float2* spec, float2* spec2, float2* edge, const float* kq,
                                     float2* force, const float2* tw, float g, int batch, cudaStream_t st,
                                     const SpectralTc* tc, float* clear, const SpectralMaps* maps, int* status,
                                     int col_shape) {
    using RS = RowShape<float, N>;
    using CS = ColShape<float, N>;
    using SS = SpecShape<N>;
    // column-pass threads of a single lattice: the default shape, or the other one
    constexpr int CNT1 = SS::CNT, CNT2 = SS::ACNT;
    const bool alt = col_shape == 1 && batch == 1;
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
                if (alt)
                    e = launch_dependent(dependent, k_cols_spectral_tma<N, CS::B, CNT2>, dim3(N / 2 / CS::B),
                                         dim3(CNT2), SS::col_smem_for(CNT2) + kTmaAlignPad, st, maps->spec, spec,
                                         spec2, edge, kq, tw, g, status);
                else if (batch == 1 && CNT1 != CS::NT)
                    e = launch_dependent(dependent, k_cols_spectral_tma<N, CS::B, CNT1>, dim3(N / 2 / CS::B),
                                         dim3(CNT1), SS::col_smem_for(CNT1) + kTmaAlignPad, st, maps->spec,
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
    } else if (alt) {
        if ((e = launch_dependent(dependent, k_cols_spectral<N, CS::B, CNT2>, dim3(N / 2 / CS::B), dim3(CNT2),
                                  SS::col_smem_for(CNT2), st, spec, spec2, edge, kq, tw, g)) != cudaSuccess)
            return e;
    } else if (batch == 1 && SS::CNT != CS::NT) {
        if ((e = launch_dependent(dependent, k_cols_spectral<N, CS::B, SS::CNT>, dim3(N / 2 / CS::B), dim3(SS::CNT),
                                  SS::col_smem_for(SS::CNT), st, spec, spec2, edge, kq, tw, g)) != cudaSuccess)
            return e;
    } else if ((e = launch_dependent(dependent, k_cols_spectral<N, CS::B, CS::NT>, dim3((N / 2) / CS::B, batch),
                                     dim3(CS::NT), SS::col_smem, st, spec, spec2, edge, kq, tw, g)) != cudaSuccess) {
        return e;
    }
    return launch_dependent(dependent, k_rows_c2r_spectral<N, SS::RB, SS::RNT>, dim3(N / SS::RB, batch),
                            dim3(SS::RNT), SS::row_smem, st, spec, spec2, static_cast<const float2*>(edge),
                            reinterpret_cast<float4*>(force), tw, g);
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
        if ((e = allow_smem(k_cols_spectral_tma<N, CS::B, SS::ACNT>, SS::col_smem_for(SS::ACNT) + kTmaAlignPad)) !=
            cudaSuccess)
            return e;
    }
    if ((e = allow_smem(k_cols_spectral<N, CS::B, SS::ACNT>, SS::col_smem_for(SS::ACNT))) != cudaSuccess) return e;
    if ((e = allow_smem(k_cols_spectral<N, CS::B, CS::NT>, SS::col_smem)) != cudaSuccess) return e;
    if ((e = allow_smem(k_cols_spectral<N, CS::B, SS::CNT>, SS::col_smem_for(SS::CNT))) != cudaSuccess) return e;
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

cudaError_t launch_spectral_force(int N, const float* rho, float2* spec, float2* spec2, float2* edge, const float* kq,
                                  float2* force, const float2* tw, float g, cudaStream_t st, int batch,
                                  const SpectralTc* tc, float* clear, const SpectralMaps* maps, int* status,
                                  int col_shape) {
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    if (tc && !tc_fft_supported(N)) return cudaErrorInvalidValue;
    switch (N) {
#define CPM_CASE(n) \
    case n:         \
        return spectral_passes_n<n>(rho, spec, spec2, edge, kq, force, tw, g, batch, st, tc, clear, maps, status, \
                                    col_shape);
        CPM_FOR_EACH_N(CPM_CASE)
#undef CPM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

int spectral_launches_per_step() { return 3; }

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
