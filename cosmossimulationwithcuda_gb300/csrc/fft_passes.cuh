// Bodies of the FFT passes of the particle-mesh step, shared by the pass
// kernels (pm_fft.cu) and the persistent ensemble step (pm_ensemble_step.cu):
// launch shapes, the row R2C, the column pass of the spectral force, the C2R
// row passes and the edge corrections.  Each body works on one tile of one
// lattice (the caller offsets the lattice pointers) with NT threads.  The
// algorithm and the reference code it replaces are described in pm_fft.cu.
#pragma once

#include "fft_engine.cuh"

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
// Up to this lattice size the spectral C2R row pass runs one butterfly per
// thread per stage (twice the threads).
#ifndef CPM_C2R_FULL_MAX_N
#define CPM_C2R_FULL_MAX_N 512
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
// values z[n] = (x[2n], x[2n+1])), transformed in shared memory `s`; `spec`
// and `clear` (the lattice's density, or null) address one lattice.
template <class T, int N, int B, int NT, class Src>
__device__ __forceinline__ void r2c_rows(const Src& src, cplx_t<T>* s, cplx_t<T>* __restrict__ spec,
                                         const cplx_t<T>* __restrict__ tw, T* clear, int y0) {
    using C = cplx_t<T>;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<M>::value;
    auto dst = [s](int line, int i, C v) { s[line * LP + pad16(i)] = v; };
    fft_lines<M, B, NT, -1, C, kMaxRadix>(s, src, dst, tw, 2);
    if (clear) {  // the rows were read (fft_lines ends with a barrier): zero them for the next deposit
        C* z = reinterpret_cast<C*>(clear + size_t(y0) * N);
        for (int i = threadIdx.x; i < B * M; i += NT) z[i] = cmake<C>(T(0), T(0));
    }
    // X[k] = (Z[k] + conj Z[M-k])/2 - i/2 W^k (Z[k] - conj Z[M-k]),  W = exp(-2 pi i/N)
    // (unrolled: several twiddle loads and transposed stores in flight per
    // thread, measured -1 us per step at 2048^2)
#pragma unroll 4
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

// Body of the C2R row pass: B rows (from y0) of a half spectrum stored
// transposed, element (k, row) at spec[k * STRIDE + row], into real rows of
// `out`; spec / out address one lattice.
template <int N, int B, int NT, int STRIDE = N>
__device__ __forceinline__ void c2r_rows(float2* s, const float2* __restrict__ spec, float* __restrict__ out,
                                         const float2* __restrict__ tw, int y0) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<M>::value;
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

// ---- spectral force --------------------------------------------------------------------------
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
    // the filter and edge loops are unrolled so that several filter and
    // twiddle loads are in flight per thread (measured: -1.2 us per step at 2048^2)
#pragma unroll 4
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
#pragma unroll 4
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

// Body of the spectral C2R row pass: Fx = IFFT_x(i S(kx) g Phi) and
// Fy = IFFT_x(Psi) for B rows (from y0), with the x-edge corrections from
// Phi, written as interleaved (fx, fy).  Both are real, so one N-point
// complex inverse FFT of Z = X + i Y (X, Y the Hermitian spectra of Fx, Fy,
// extended to k in [0, N) by X[N-k] = conj X[k]) gives z = fx + i fy directly,
// the force's own (fx, fy) layout: no half-length pre-split and no
// interleaving pass.  spec / spec2 / edge / force address one lattice; s
// holds B padded lines of N points (row b: Phi in [0, M), Psi in [M, N)
// until Z replaces them) followed by the block_sum scratch (NT/32 * 3B
// floats); dx: 3B floats of shared scratch.  The y-edge corrections of rows
// 0, 1, N-2, N-1 enter their Fy spectra from the column pass's edge sums.
template <int N>
constexpr size_t c2r_spectral_line() { return size_t(LinePad<N>::value); }

template <int N, int B, int NT>
__device__ __forceinline__ void c2r_spectral_rows(float2* s, float* dx, const float2* __restrict__ spec,
                                                  const float2* __restrict__ spec2, const float2* __restrict__ edge,
                                                  float4* __restrict__ force, const float2* __restrict__ tw, float g,
                                                  int y0) {
    using C = float2;
    constexpr int M = N / 2;
    constexpr int LP = LinePad<N>::value;
    const float c12 = g * (1.0f / 12.0f);
    float* red = reinterpret_cast<float*>(s + B * LP);
#pragma unroll 4  // several transposed loads in flight per thread (measured: -2 us per step at 2048^2)
    for (int idx = threadIdx.x; idx < M * B; idx += NT) {
        const int k = idx / B;
        const int b = idx - k * B;
        s[b * LP + pad16(k)] = spec[size_t(k) * N + y0 + b];
        s[b * LP + pad16(M + k)] = spec2[size_t(k) * N + y0 + b];
    }
    __syncthreads();
    // One pass over the potential half spectra Phi: the x-edge differences
    //   D = Phi(M) ((-1)^a - (-1)^b) + 2 sum_{k=1}^{M-1} Re(Phi(k) w(k))
    // of every row, and the Fx spectrum i S(kx) g Phi in place (S(0) = S(N/2) = 0
    // empties the packed element 0).
    float acc[3 * B];
#pragma unroll
    for (int j = 0; j < 3 * B; ++j) acc[j] = 0.0f;
#pragma unroll 2
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
    // y-edge corrections of Fy on rows 0, 1, N-2, N-1, in Fourier space: there
    // the clamped stencil differs from the periodic one by
    //   c12 (a01 D01 + a02 D02 + a13 D13)(x),  (a01, a02, a13) = (-8, 1, 0),
    //   (0, 0, 1), (0, 1, 0), (-8, 0, 1) for y = 0, 1, N-2, N-1,
    // and the spectra over kx of the y-edge differences D are the column
    // pass's edge sums (edge[kx * 4 + j], j = D01, D02, D13, with the same
    // packing of kx = 0 and N/2 in element 0).  The row's inverse FFT is
    // linear, so adding them to the row's Fy spectrum Psi corrects Fy without
    // a separate transform of the edge lines.
    if (y0 <= 1 || y0 + B >= N - 1) {
        for (int b = 0; b < B; ++b) {
            const int y = y0 + b;
            float a01, a02, a13;
            if (y == 0) {
                a01 = -8.0f; a02 = 1.0f; a13 = 0.0f;
            } else if (y == 1) {
                a01 = 0.0f; a02 = 0.0f; a13 = 1.0f;
            } else if (y == N - 2) {
                a01 = 0.0f; a02 = 1.0f; a13 = 0.0f;
            } else if (y == N - 1) {
                a01 = -8.0f; a02 = 0.0f; a13 = 1.0f;
            } else {
                continue;
            }
            for (int k = threadIdx.x; k < M; k += NT) {
                const C e01 = edge[size_t(k) * 4 + 0], e02 = edge[size_t(k) * 4 + 1], e13 = edge[size_t(k) * 4 + 2];
                C* p = s + b * LP + pad16(M + k);
                p->x += c12 * (a01 * e01.x + a02 * e02.x + a13 * e13.x);
                p->y += c12 * (a01 * e01.y + a02 * e02.y + a13 * e13.y);
            }
        }
    }
    block_sum<NT, 3 * B>(acc, red);  // ends with a barrier: the Fx spectra are complete
    if (threadIdx.x < B) {
        dx[3 * threadIdx.x + 0] = 2.0f * acc[3 * threadIdx.x + 0];
        dx[3 * threadIdx.x + 1] = 2.0f * acc[3 * threadIdx.x + 1];
        dx[3 * threadIdx.x + 2] = 2.0f * acc[3 * threadIdx.x + 2];
    }
    // Z of every row, in place: the pair (k, M - k) reads X, Y at k, M - k
    // (elements k, M - k, M + k, N - k) and writes Z at k, N - k, M - k, M + k,
    // the same four elements, so no other thread's input is overwritten.
    // Element 0 of X and Y holds the packed real pair (X[0], X[M]).
    constexpr int H = M / 2 + 1;
    for (int idx = threadIdx.x; idx < H * B; idx += NT) {
        const int b = idx / H;
        const int k = idx - b * H;
        C* row = s + b * LP;
        if (k == 0) {
            const C x = row[0], y = row[pad16(M)];
            row[0] = cmake<C>(x.x, y.x);         // Z[0] = X[0] + i Y[0]
            row[pad16(M)] = cmake<C>(x.y, y.y);  // Z[M] = X[M] + i Y[M]
        } else {
            const int k2 = M - k;
            const C x1 = row[pad16(k)], y1 = row[pad16(M + k)];
            const C x2 = row[pad16(k2)], y2 = row[pad16(M + k2)];
            row[pad16(k)] = cmake<C>(x1.x - y1.y, x1.y + y1.x);          // Z[k] = X + iY
            row[pad16(N - k)] = cmake<C>(x1.x + y1.y, y1.x - x1.y);      // Z[N-k] = conj X + i conj Y
            if (k2 != k) {
                row[pad16(k2)] = cmake<C>(x2.x - y2.y, x2.y + y2.x);
                row[pad16(N - k2)] = cmake<C>(x2.x + y2.y, y2.x - x2.y);
            }
        }
    }
    __syncthreads();
    // z = fx + i fy, written straight from the last radix stage with the x-edge corrections
    float2* frow = reinterpret_cast<float2*>(force) + size_t(y0) * N;
    auto sload = [s](int line, int i) { return s[line * LP + pad16(i)]; };
    auto gstore = [frow, dx, c12](int line, int i, C v) {
        if (i <= 1 || i >= N - 2) {
            const float d01 = dx[3 * line + 0], d02 = dx[3 * line + 1], d13 = dx[3 * line + 2];
            v.x += (i == 0 ? -8.0f * d01 + d02 : i == 1 ? d13 : i == N - 2 ? d02 : d13 - 8.0f * d01) * c12;
        }
        frow[size_t(line) * N + i] = v;
    };
    fft_lines<N, B, NT, +1, C, kMaxRadix>(s, sload, gstore, tw, 1);
}

}  // namespace cpm
