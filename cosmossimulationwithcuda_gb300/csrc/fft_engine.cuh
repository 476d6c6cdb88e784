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

// Elements per padded line: L + L/16 + stagger.  From 1024 points the
// stagger is 4: consecutive lines start a quarter of a bank row apart
// (4 float2 = 32 bytes), so that a warp that touches k = 0..32/B-1 of
// B = 2, 4 or 8 lines at once (the transposed loads and stores of the row
// passes) hits every bank twice: two wavefronts, the minimum for 256 bytes
// (a stagger of one element put four lines' elements on the same banks;
// measured -5% on the 2048^2 force passes).  Shorter lines keep a stagger of
// one (measured 2% faster at 512^2).
template <int L>
struct LinePad {
    static constexpr int value = L + L / 16 + (L >= 1024 ? 4 : 1);
};

template <int L>
struct Log2 {
    static constexpr int value = (L <= 1) ? 0 : 1 + Log2<(L >> 1)>::value;
};
template <>
struct Log2<1> {
    static constexpr int value = 0;
};

// Radix plan: one stage of radix 2^(log2 L mod log2 MAXR) (when nonzero),
// then radix-MAXR stages (MAXR = 8 or 16).
template <int L, int MAXR = 8>
struct RadixPlan {
    static constexpr int lr = MAXR == 16 ? 4 : 3;
    static constexpr int rem = Log2<L>::value % lr;
    static constexpr int first = rem == 0 ? MAXR : (1 << rem);
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

// 16-point DFT as 4 x 4: DFT4 over n1 (stride 4), twiddle W16^(n1 k2), DFT4
// over the other index; output in natural order.
template <int DIR, class C>
__device__ __forceinline__ void dft16(C* v) {
    using R = decltype(C{}.x);
    const R c1 = R(0.92387953251128675613), s1 = R(0.38268343236508977173), h = R(0.70710678118654752440);
    C u[4][4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        u[n][0] = v[n];
        u[n][1] = v[n + 4];
        u[n][2] = v[n + 8];
        u[n][3] = v[n + 12];
        dft4<DIR>(u[n][0], u[n][1], u[n][2], u[n][3]);
    }
    // twiddles W16^(n k) for n, k in 1..3; W16 = exp(DIR * 2 pi i / 16)
    const R sg = DIR < 0 ? R(-1) : R(1);
    const C w1 = cmake<C>(c1, sg * s1), w2 = cmake<C>(h, sg * h), w3 = cmake<C>(s1, sg * c1);
    const C w6 = cmake<C>(-h, sg * h), w9 = cmake<C>(-c1, -sg * s1);
    u[1][1] = cmul(u[1][1], w1);
    u[1][2] = cmul(u[1][2], w2);
    u[1][3] = cmul(u[1][3], w3);
    u[2][1] = cmul(u[2][1], w2);
    u[2][2] = cmul_i<DIR>(u[2][2]);
    u[2][3] = cmul(u[2][3], w6);
    u[3][1] = cmul(u[3][1], w3);
    u[3][2] = cmul(u[3][2], w6);
    u[3][3] = cmul(u[3][3], w9);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        C a = u[0][k], b = u[1][k], c = u[2][k], d = u[3][k];
        dft4<DIR>(a, b, c, d);
        v[k] = a;
        v[k + 4] = b;
        v[k + 8] = c;
        v[k + 12] = d;
    }
}

template <int R, int DIR, class C>
__device__ __forceinline__ void dft_r(C* v) {
    if constexpr (R == 2) {
        dft2<DIR>(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4<DIR>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        dft8<DIR>(v);
    } else if constexpr (R == 16) {
        dft16<DIR>(v);
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
                    if constexpr (R >= 8) {
                        const C w4 = cmul(w2, w2);
                        v[q][4] = cmul(v[q][4], w4);
                        v[q][5] = cmul(v[q][5], cmul(w4, w1));
                        v[q][6] = cmul(v[q][6], cmul(w4, w2));
                        v[q][7] = cmul(v[q][7], cmul(w4, w3));
                        if constexpr (R == 16) {
                            const C w8 = cmul(w4, w4);
                            const C w12 = cmul(w8, w4);
                            v[q][8] = cmul(v[q][8], w8);
                            v[q][9] = cmul(v[q][9], cmul(w8, w1));
                            v[q][10] = cmul(v[q][10], cmul(w8, w2));
                            v[q][11] = cmul(v[q][11], cmul(w8, w3));
                            v[q][12] = cmul(v[q][12], w12);
                            v[q][13] = cmul(v[q][13], cmul(w12, w1));
                            v[q][14] = cmul(v[q][14], cmul(w12, w2));
                            v[q][15] = cmul(v[q][15], cmul(w12, w3));
                        }
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
template <int L, int Ns, int B, int NT, int DIR, class C, class SrcLoad, class DstStore, int MAXR>
struct FftStages {
    static __device__ __forceinline__ void run(C* smem, const SrcLoad& src, const DstStore& dst,
                                               const C* __restrict__ tw, int tw_stride) {
        constexpr int R = (Ns == 1) ? RadixPlan<L, MAXR>::first : MAXR;
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
        if constexpr (!last)
            FftStages<L, Ns * R, B, NT, DIR, C, SrcLoad, DstStore, MAXR>::run(smem, src, dst, tw, tw_stride);
    }
};

// Transform B lines: first stage reads through `src`, last stage writes through
// `dst`, intermediate stages use `smem` (B * LinePad<L> elements).  MAXR is the
// largest radix (8 or 16): radix-16 halves the shared-memory round trips of
// radix-8 on long lines at the cost of more registers per thread.
template <int L, int B, int NT, int DIR, class C, int MAXR = 8, class SrcLoad, class DstStore>
__device__ __forceinline__ void fft_lines(C* smem, const SrcLoad& src, const DstStore& dst, const C* __restrict__ tw,
                                          int tw_stride) {
    FftStages<L, 1, B, NT, DIR, C, SrcLoad, DstStore, MAXR>::run(smem, src, dst, tw, tw_stride);
}

}  // namespace cpm
