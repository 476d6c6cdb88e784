// Per-particle and per-work-item bodies of the tile-ordered fused step
// (gather + update + deposit of the new positions), shared by the fused step
// kernels (pm_tiles.cu) and the persistent ensemble step
// (pm_ensemble_step.cu).  The design is described in pm_tiles.cu.
#pragma once

#include <cfloat>
#include <type_traits>

#include "pm_common.cuh"
#include "pm_internal.h"
#include "pm_particle_math.cuh"

namespace cpm {

constexpr int kFusedThreads = 256;
// Optional register limit: resident CTAs per SM the fused kernel must allow.
#ifdef CPM_FUSED_MIN_BLOCKS
#define CPM_FUSED_BOUNDS __launch_bounds__(kFusedThreads, CPM_FUSED_MIN_BLOCKS)
#else
#define CPM_FUSED_BOUNDS __launch_bounds__(kFusedThreads)
#endif

__host__ __device__ constexpr int win_y(int gran) { return (1 << gran) + 2 * kTileHalo + 1; }
__host__ __device__ constexpr int win_x(int gran) { return (win_y(gran) + 3) & ~3; }


// Window cells.  Each window cell is one lattice cell: a float2 force and a
// 32-bit fixed-point deposit accumulator.  Two paired forms are kept as
// compile-time options (measured slower, so off):
//   CPM_PAIR_GATHER=1   CIC force cells hold {f(x, y), f(x + 1, y)}: one
//                       16-byte load per stencil row instead of two 8-byte
//                       loads (the larger window leaves two CTAs per SM
//                       instead of three: fused kernel 0.175 -> 0.185 ms at
//                       20M particles / 2048^2);
//   CPM_PAIR_DEPOSIT=1  CIC deposit cells are 64-bit words whose low half
//                       collects the weight a particle puts on cell x and
//                       whose high half the weight on cell x + 1: one 64-bit
//                       integer atomic per stencil row instead of two 32-bit
//                       ones (cell x = low(x) + high(x - 1); each half is part
//                       of one cell's total, below 2^32, so no carry crosses
//                       halves and the sums are the same integers).  64-bit
//                       shared atomics are far slower than 32-bit ones here:
//                       0.175 -> 0.32 ms.
#ifndef CPM_PAIR_GATHER
#define CPM_PAIR_GATHER 0
#endif
#ifndef CPM_PAIR_DEPOSIT
#define CPM_PAIR_DEPOSIT 0
#endif
template <int CIC>
struct WinCell {
    using F = float2;
    using D = uint32_t;
};
template <>
struct WinCell<1> {
    using F = std::conditional_t<CPM_PAIR_GATHER != 0, float4, float2>;
    using D = std::conditional_t<CPM_PAIR_DEPOSIT != 0, unsigned long long, uint32_t>;
};
template <int CIC>
constexpr bool kPairGather = sizeof(typename WinCell<CIC>::F) == sizeof(float4);
template <int CIC>
constexpr bool kPairDeposit = sizeof(typename WinCell<CIC>::D) == sizeof(unsigned long long);

// Shared bytes of the two windows of a tile of edge 2^gran.
__host__ __device__ constexpr size_t window_bytes(int gran, int cic) {
    return size_t(win_y(gran)) * win_x(gran) *
           (cic ? sizeof(WinCell<1>::F) + sizeof(WinCell<1>::D) : sizeof(WinCell<0>::F) + sizeof(WinCell<0>::D));
}

template <int CIC>
struct Window {
    const typename WinCell<CIC>::F* f;  // staged force (nullptr: read the global field)
    typename WinCell<CIC>::D* d;        // fixed-point deposit window (nullptr: global float atomics)
    int x0, y0;
    float scale, heavy;
};

// The two windows carved from a 16-byte aligned shared block: force first.
template <int CIC, int GRAN>
struct WindowSmem {
    typename WinCell<CIC>::F* f;
    typename WinCell<CIC>::D* d;
    __device__ __forceinline__ explicit WindowSmem(void* base)
        : f(reinterpret_cast<typename WinCell<CIC>::F*>(base)),
          d(reinterpret_cast<typename WinCell<CIC>::D*>(f + win_y(GRAN) * win_x(GRAN))) {}
};

// Global deposits (particles outside their item's window, heavy particles,
// sparse items).  For an even cell column the two cells of a stencil row are
// one 8-byte aligned pair (N is even and the lattices start 8-byte aligned):
// one vector reduction per row instead of two scalar atomics.
#ifndef CPM_VEC_GLOBAL
#define CPM_VEC_GLOBAL 1
#endif
__device__ __forceinline__ void deposit_global(float* __restrict__ rho, int N, int nx, int ny, float a, float b,
                                               float c, float d, bool cic) {
    float* g = rho + size_t(nx) + size_t(ny) * N;
    if (cic) {
        if (CPM_VEC_GLOBAL && (nx & 1) == 0) {
            red_add_v2(g, a, b);
            red_add_v2(g + N, c, d);
        } else {
            atomicAdd(g, a);
            atomicAdd(g + 1, b);
            atomicAdd(g + N, c);
            atomicAdd(g + N + 1, d);
        }
    } else {
        atomicAdd(g, a);
    }
}

// One particle: gather, update, deposit of the new position.
template <int CIC, int WX, int WY>
__device__ __forceinline__ void step_particle(float& px, float& py, float& pxo, float& pyo, float pm,
                                              const Window<CIC>& w,
                                              const float2* __restrict__ force, float* __restrict__ rho, int N,
                                              float dt) {
    const int cx = int(px), cy = int(py);
    if (!active_cell(cx, cy, N)) return;
    const int lx = cx - w.x0, ly = cy - w.y0;
    float2 F;
    if constexpr (CIC != 0) {
        const CicWeights cw = cic_weights(px, py, cx, cy);
        if (w.f && unsigned(lx) < unsigned(WX - 1) && unsigned(ly) < unsigned(WY - 1)) {
            const auto* f = w.f + ly * WX + lx;
            if constexpr (kPairGather<CIC>) {
                const float4 r0 = f[0], r1 = f[WX];
                F = bilinear(cw, make_float2(r0.x, r0.y), make_float2(r0.z, r0.w), make_float2(r1.x, r1.y),
                             make_float2(r1.z, r1.w));
            } else {
                F = bilinear(cw, f[0], f[1], f[WX], f[WX + 1]);
            }
        } else {
            const size_t c = size_t(cx) + size_t(cy) * N;
            if (CPM_VEC_GLOBAL && (cx & 1) == 0) {  // the two cells of a row as one 16-byte aligned load
                const float4 r0 = __ldg(reinterpret_cast<const float4*>(force + c));
                const float4 r1 = __ldg(reinterpret_cast<const float4*>(force + c + N));
                F = bilinear(cw, make_float2(r0.x, r0.y), make_float2(r0.z, r0.w), make_float2(r1.x, r1.y),
                             make_float2(r1.z, r1.w));
            } else {
                F = bilinear(cw, __ldg(force + c), __ldg(force + c + 1), __ldg(force + c + N),
                             __ldg(force + c + N + 1));
            }
        }
    } else {
        F = (w.f && unsigned(lx) < unsigned(WX) && unsigned(ly) < unsigned(WY))
                ? w.f[ly * WX + lx]
                : __ldg(force + size_t(cx) + size_t(cy) * N);
    }
    verlet_wrap(px, py, pxo, pyo, F, dt, N);
    const int nx = int(px), ny = int(py);
    if (!active_cell(nx, ny, N)) return;
    const int mx = nx - w.x0, my = ny - w.y0;
    if constexpr (CIC != 0) {
        const CicWeights cw = cic_weights(px, py, nx, ny);
        const float a = __fmul_rn(cw.w00, pm), b = __fmul_rn(cw.w10, pm);
        const float c = __fmul_rn(cw.w01, pm), d = __fmul_rn(cw.w11, pm);
        if (w.d && pm <= w.heavy && unsigned(mx) < unsigned(WX - 1) && unsigned(my) < unsigned(WY - 1)) {
            auto* s = w.d + my * WX + mx;
            const uint32_t qa = __float2uint_rn(a * w.scale), qb = __float2uint_rn(b * w.scale);
            const uint32_t qc = __float2uint_rn(c * w.scale), qd = __float2uint_rn(d * w.scale);
            if constexpr (kPairDeposit<CIC>) {
                atomicAdd(s, (static_cast<unsigned long long>(qb) << 32) | qa);
                atomicAdd(s + WX, (static_cast<unsigned long long>(qd) << 32) | qc);
            } else {
                atomicAdd(s, qa);
                atomicAdd(s + 1, qb);
                atomicAdd(s + WX, qc);
                atomicAdd(s + WX + 1, qd);
            }
        } else {
            deposit_global(rho, N, nx, ny, a, b, c, d, true);
        }
    } else {
        if (w.d && pm <= w.heavy && unsigned(mx) < unsigned(WX) && unsigned(my) < unsigned(WY))
            atomicAdd(w.d + my * WX + mx, __float2uint_rn(pm * w.scale));
        else
            deposit_global(rho, N, nx, ny, pm, 0.f, 0.f, 0.f, false);
    }
}

template <int CIC, int WX, int WY>
__device__ __forceinline__ void step_range(const ParticleArrays& p, uint32_t b, uint32_t e, const Window<CIC>& w,
                                           const float2* __restrict__ force, float* __restrict__ rho, int N,
                                           float dt) {
    const uint32_t b4 = (b + 3u) & ~3u, e4 = e & ~3u;
    {  // ragged head / tail (or the whole range when it spans no full group)
        const uint32_t h_end = b4 < e ? b4 : e;
        const uint32_t t_beg = e4 > h_end ? e4 : h_end;
        const uint32_t nh = h_end - b, nt = e - t_beg;
        if (threadIdx.x < nh + nt) {
            const uint32_t i = threadIdx.x < nh ? b + threadIdx.x : t_beg + (threadIdx.x - nh);
            float px = p.x[i], py = p.y[i], pxo = p.xo[i], pyo = p.yo[i];
            step_particle<CIC, WX, WY>(px, py, pxo, pyo, p.m[i], w, force, rho, N, dt);
            p.x[i] = px;
            p.y[i] = py;
            p.xo[i] = pxo;
            p.yo[i] = pyo;
        }
    }
    if (b4 < e4) {
        float4* X = reinterpret_cast<float4*>(p.x);
        float4* Y = reinterpret_cast<float4*>(p.y);
        float4* XO = reinterpret_cast<float4*>(p.xo);
        float4* YO = reinterpret_cast<float4*>(p.yo);
        const float4* Mm = reinterpret_cast<const float4*>(p.m);
        for (uint32_t g = (b4 >> 2) + threadIdx.x; g < (e4 >> 2); g += kFusedThreads) {
            float4 x = __ldcs(X + g), y = __ldcs(Y + g), xo = __ldcs(XO + g), yo = __ldcs(YO + g);
            const float4 m = __ldcs(Mm + g);
            step_particle<CIC, WX, WY>(x.x, y.x, xo.x, yo.x, m.x, w, force, rho, N, dt);
            step_particle<CIC, WX, WY>(x.y, y.y, xo.y, yo.y, m.y, w, force, rho, N, dt);
            step_particle<CIC, WX, WY>(x.z, y.z, xo.z, yo.z, m.z, w, force, rho, N, dt);
            step_particle<CIC, WX, WY>(x.w, y.w, xo.w, yo.w, m.w, w, force, rho, N, dt);
            __stcs(X + g, x);
            __stcs(Y + g, y);
            __stcs(XO + g, xo);
            __stcs(YO + g, yo);
        }
    }
}


// Stage the force window of an item's tile (zero outside the lattice) and
// clear its deposit window; threads tid, tid + nthreads, ... of the caller.
template <int CIC, int GRAN>
__device__ __forceinline__ void stage_windows(const WorkItem& item, const float2* __restrict__ force, int N,
                                              const WindowSmem<CIC, GRAN>& win, int tid, int nthreads) {
    constexpr int WY = win_y(GRAN), WX = win_x(GRAN);
    for (int i = tid; i < WY * WX; i += nthreads) {
        const int r = i / WX, c = i - r * WX;
        const int gx = item.x0 + c, gy = item.y0 + r;
        const bool row_in = gy >= 0 && gy < N;
        const float2* frow = row_in ? force + size_t(gy) * N : force;
        const float2 f0 = row_in && gx >= 0 && gx < N ? __ldg(frow + gx) : make_float2(0.0f, 0.0f);
        if constexpr (kPairGather<CIC>) {
            const float2 f1 = row_in && gx + 1 >= 0 && gx + 1 < N ? __ldg(frow + gx + 1) : make_float2(0.0f, 0.0f);
            win.f[i] = make_float4(f0.x, f0.y, f1.x, f1.y);
        } else {
            win.f[i] = f0;
        }
        win.d[i] = 0u;
    }
}

// Flush an item's deposit window into the density: one 16-byte vector float
// reduction per group of four lattice cells, empty groups skipped.
template <int CIC, int GRAN>
__device__ __forceinline__ void flush_window(const WorkItem& item, float* __restrict__ rho, int N,
                                             const WindowSmem<CIC, GRAN>& win, int tid, int nthreads) {
    constexpr int WY = win_y(GRAN), WX = win_x(GRAN), W4 = WX / 4;
    const float inv = item.inv_scale;
    for (int i = tid; i < WY * W4; i += nthreads) {
        const int r = i / W4, c4 = i - r * W4;
        const int gy = item.y0 + r, gx = item.x0 + 4 * c4;
        if (gy < 0 || gy >= N || gx < 0 || gx >= N) continue;
        uint4 q;
        if constexpr (kPairDeposit<CIC>) {
            const unsigned long long* row = win.d + r * WX + 4 * c4;
            const ulonglong2 u0 = reinterpret_cast<const ulonglong2*>(row)[0];
            const ulonglong2 u1 = reinterpret_cast<const ulonglong2*>(row)[1];
            const uint32_t left = c4 > 0 ? uint32_t(row[-1] >> 32) : 0u;
            q = make_uint4(uint32_t(u0.x) + left, uint32_t(u0.y) + uint32_t(u0.x >> 32),
                           uint32_t(u1.x) + uint32_t(u0.y >> 32), uint32_t(u1.y) + uint32_t(u1.x >> 32));
        } else {
            q = reinterpret_cast<const uint4*>(win.d)[i];
        }
        if ((q.x | q.y | q.z | q.w) != 0u)
            red_add_v4(rho + size_t(gy) * N + gx, make_float4(__uint2float_rn(q.x) * inv, __uint2float_rn(q.y) * inv,
                                                              __uint2float_rn(q.z) * inv, __uint2float_rn(q.w) * inv));
    }
}

// One work item with kFusedThreads threads: stage the force window of the
// item's tile, step its particles (window gathers, fixed-point window
// deposits), flush the deposit window into the density; sparse items (fewer
// than kItemDirect particles) use global gathers and atomics.  force / rho
// address the item's lattice; win: the CTA's shared windows.
template <int CIC, int GRAN>
__device__ __forceinline__ void fused_item(const WorkItem& item, const ParticleArrays& p,
                                           const float2* __restrict__ force, float* __restrict__ rho, int N, float dt,
                                           const WindowSmem<CIC, GRAN>& win) {
    constexpr int WY = win_y(GRAN), WX = win_x(GRAN);
    if (item.end - item.begin < uint32_t(kItemDirect)) {
        // sparse tile: no windows, global gathers and atomics
        const Window<CIC> w{nullptr, nullptr, item.x0, item.y0, 1.0f, 0.0f};
        step_range<CIC, WX, WY>(p, item.begin, item.end, w, force, rho, N, dt);
        return;
    }
    stage_windows<CIC, GRAN>(item, force, N, win, int(threadIdx.x), kFusedThreads);
    __syncthreads();
    const Window<CIC> w{win.f, win.d, item.x0, item.y0, item.scale, item.heavy};
    step_range<CIC, WX, WY>(p, item.begin, item.end, w, force, rho, N, dt);
    __syncthreads();
    flush_window<CIC, GRAN>(item, rho, N, win, int(threadIdx.x), kFusedThreads);
    __syncthreads();
}

}  // namespace cpm
