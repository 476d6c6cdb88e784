// Batched shared-memory FFT engine (Stockham autosort, radix 2/4/8 stages).
//
// A CTA transforms B lines of L complex points that live in shared memory
// (line stride LinePad<L>).  Stage s (sub-transform length Ns so far, radix R)
// reads v[r] = a[j + r*L/R], multiplies by exp(DIR*2*pi*i*r*(j%Ns)/(Ns*R)),
// applies an R-point DFT in registers and writes v[r] to
// (j/Ns)*Ns*R + j%Ns + r*Ns; after the last stage the data is in natural
// order.  This is the Stockham formulation of Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors" (SC 2008).
// The radix plan is one radix-2 or radix-4 stage (when log2 L is not a
// multiple of 3) followed by radix-8 stages.
//
// The first stage may read from any source and the last stage may write to
// any destination (functors), so a pass can stream a line in from global
// memory and out to global memory without staging copies.
//
// Twiddles come from a table tw[m] = exp(-2*pi*i*m/Lt) of length Lt = L*stride
// computed on the host in double precision.
#pragma once

#include "pm_common.cuh"

namespace cpm {

// Padded shared-memory index: one spare element after every 16.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// Elements per padded line: L + L/16 + 1 (the +1 staggers consecutive lines
// across banks for the transposed accesses of the real-FFT passes).
template <int L>
struct LinePad {
    static constexpr int value = L + L / 16 + 1;
};

template <int L>
struct RadixPlan {
    static constexpr int log2L = (L <= 1) ? 0 : 1 + RadixPlan<(L >> 1)>::log2L;
    static constexpr int first = (log2L % 3 == 0) ? 8 : ((log2L % 3 == 1) ? 2 : 4);
};
template <>
struct RadixPlan<1> {
    static constexpr int log2L = 0;
    static constexpr int first = 1;
};

template <int DIR, class C>
__device__ __forceinline__ void dft2(C& a, C& b) {
    const C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int DIR, class C>
__device__ __forceinline__ void dft4(C& v0, C& v1, C& v2, C& v3) {
    const C t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3);
    const C t3 = cmul_i<DIR>(csub(v1, v3));
    v0 = cadd(t0, t2);
    v2 = csub(t0, t2);
    v1 = cadd(t1, t3);
    v3 = csub(t1, t3);
}

template <int DIR, class C>
__device__ __forceinline__ void dft8(C* v) {
    using R = decltype(C{}.x);
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    const R s = R(0.70710678118654752440);
    if (DIR < 0) {  // W8 = (s, -s), W8^3 = (-s, -s)
        o1 = cmake<C>(s * (o1.x + o1.y), s * (o1.y - o1.x));
        o3 = cmake<C>(s * (o3.y - o3.x), -s * (o3.x + o3.y));
    } else {        // conj: (s, s), (-s, s)
        o1 = cmake<C>(s * (o1.x - o1.y), s * (o1.x + o1.y));
        o3 = cmake<C>(-s * (o3.x + o3.y), s * (o3.x - o3.y));
    }
    o2 = cmul_i<DIR>(o2);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

template <int R, int DIR, class C>
__device__ __forceinline__ void dft_r(C* v) {
    if constexpr (R == 2) {
        dft2<DIR>(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4<DIR>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        dft8<DIR>(v);
    }
}

// One Stockham stage over B lines of length L with NT threads.
// load(line, i) -> C and store(line, i, C) address element i of a line.
template <int L, int R, int Ns, int B, int NT, int DIR, class C, class Load, class Store>
__device__ __forceinline__ void fft_stage(const Load& load, const Store& store, const C* __restrict__ tw,
                                          int tw_stride) {
    constexpr int LR = L / R;
    constexpr int NB = B * LR;  // butterflies in this stage
    constexpr int PER = (NB + NT - 1) / NT;
    C v[PER][R];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int bf = int(threadIdx.x) + q * NT;
        if ((NB % NT) == 0 || bf < NB) {
            const int line = bf / LR;
            const int j = bf - line * LR;
#pragma unroll
            for (int r = 0; r < R; ++r) v[q][r] = load(line, j + r * LR);
            if constexpr (Ns > 1) {
                // one table load per butterfly (w^1); the other powers by complex
                // multiplication in a tree of depth <= 3, so that a warp's twiddle
                // reads stay close to coalesced
                const int k = j % Ns;
                constexpr int step = L / (Ns * R);
                C w1 = tw[(k * step) * tw_stride];
                if (DIR > 0) w1.y = -w1.y;
                v[q][1] = cmul(v[q][1], w1);
                if constexpr (R >= 4) {
                    const C w2 = cmul(w1, w1);
                    const C w3 = cmul(w2, w1);
                    v[q][2] = cmul(v[q][2], w2);
                    v[q][3] = cmul(v[q][3], w3);
                    if constexpr (R == 8) {
                        const C w4 = cmul(w2, w2);
                        v[q][4] = cmul(v[q][4], w4);
                        v[q][5] = cmul(v[q][5], cmul(w4, w1));
                        v[q][6] = cmul(v[q][6], cmul(w4, w2));
                        v[q][7] = cmul(v[q][7], cmul(w4, w3));
                    }
                }
            }
            dft_r<R, DIR>(v[q]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int bf = int(threadIdx.x) + q * NT;
        if ((NB % NT) == 0 || bf < NB) {
            const int line = bf / LR;
            const int j = bf - line * LR;
            const int k = j % Ns;
            const int base = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) store(line, base + r * Ns, v[q][r]);
        }
    }
    __syncthreads();
}

// Recursive driver: stage with sub-length Ns, then the rest.
template <int L, int Ns, int B, int NT, int DIR, class C, class SrcLoad, class DstStore>
struct FftStages {
    static __device__ __forceinline__ void run(C* smem, const SrcLoad& src, const DstStore& dst,
                                               const C* __restrict__ tw, int tw_stride) {
        constexpr int R = (Ns == 1) ? RadixPlan<L>::first : 8;
        constexpr int LP = LinePad<L>::value;
        auto sload = [smem](int line, int i) { return smem[line * LP + pad16(i)]; };
        auto sstore = [smem](int line, int i, C v) { smem[line * LP + pad16(i)] = v; };
        constexpr bool first = (Ns == 1);
        constexpr bool last = (Ns * R == L);
        if constexpr (first && last) {
            fft_stage<L, R, Ns, B, NT, DIR, C>(src, dst, tw, tw_stride);
        } else if constexpr (first) {
            fft_stage<L, R, Ns, B, NT, DIR, C>(src, sstore, tw, tw_stride);
        } else if constexpr (last) {
            fft_stage<L, R, Ns, B, NT, DIR, C>(sload, dst, tw, tw_stride);
        } else {
            fft_stage<L, R, Ns, B, NT, DIR, C>(sload, sstore, tw, tw_stride);
        }
        if constexpr (!last) FftStages<L, Ns * R, B, NT, DIR, C, SrcLoad, DstStore>::run(smem, src, dst, tw, tw_stride);
    }
};

// Transform B lines: first stage reads through `src`, last stage writes through
// `dst`, intermediate stages use `smem` (B * LinePad<L> elements).
template <int L, int B, int NT, int DIR, class C, class SrcLoad, class DstStore>
__device__ __forceinline__ void fft_lines(C* smem, const SrcLoad& src, const DstStore& dst, const C* __restrict__ tw,
                                          int tw_stride) {
    FftStages<L, 1, B, NT, DIR, C, SrcLoad, DstStore>::run(smem, src, dst, tw, tw_stride);
}

}  // namespace cpm
