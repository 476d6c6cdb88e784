// Per-particle and per-work-item bodies of the tile-ordered fused step
// (gather + update + deposit of the new positions), shared by the fused step
// kernels (pm_tiles.cu) and the persistent ensemble step
// (pm_ensemble_step.cu).  The design is described in pm_tiles.cu.
#pragma once

#include <cfloat>

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


struct Window {
    const float2* f;  // staged force (nullptr: read the global field)
    uint32_t* d;      // fixed-point deposit window (nullptr: global float atomics)
    int x0, y0;
    float scale, heavy;
};

__device__ __forceinline__ void deposit_global(float* __restrict__ rho, int N, int nx, int ny, float a, float b,
                                               float c, float d, bool cic) {
    float* g = rho + size_t(nx) + size_t(ny) * N;
    if (cic) {
        atomicAdd(g, a);
        atomicAdd(g + 1, b);
        atomicAdd(g + N, c);
        atomicAdd(g + N + 1, d);
    } else {
        atomicAdd(g, a);
    }
}

// One particle: gather, update, deposit of the new position.
template <int CIC, int WX, int WY>
__device__ __forceinline__ void step_particle(float& px, float& py, float& pxo, float& pyo, float pm, const Window& w,
                                              const float2* __restrict__ force, float* __restrict__ rho, int N,
                                              float dt) {
    const int cx = int(px), cy = int(py);
    if (!active_cell(cx, cy, N)) return;
    const int lx = cx - w.x0, ly = cy - w.y0;
    float2 F;
    if (CIC) {
        const CicWeights cw = cic_weights(px, py, cx, cy);
        if (w.f && unsigned(lx) < unsigned(WX - 1) && unsigned(ly) < unsigned(WY - 1)) {
            const float2* f = w.f + ly * WX + lx;
            F = bilinear(cw, f[0], f[1], f[WX], f[WX + 1]);
        } else {
            const size_t c = size_t(cx) + size_t(cy) * N;
            F = bilinear(cw, __ldg(force + c), __ldg(force + c + 1), __ldg(force + c + N), __ldg(force + c + N + 1));
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
    if (CIC) {
        const CicWeights cw = cic_weights(px, py, nx, ny);
        const float a = __fmul_rn(cw.w00, pm), b = __fmul_rn(cw.w10, pm);
        const float c = __fmul_rn(cw.w01, pm), d = __fmul_rn(cw.w11, pm);
        if (w.d && pm <= w.heavy && unsigned(mx) < unsigned(WX - 1) && unsigned(my) < unsigned(WY - 1)) {
            uint32_t* s = w.d + my * WX + mx;
            atomicAdd(s, __float2uint_rn(a * w.scale));
            atomicAdd(s + 1, __float2uint_rn(b * w.scale));
            atomicAdd(s + WX, __float2uint_rn(c * w.scale));
            atomicAdd(s + WX + 1, __float2uint_rn(d * w.scale));
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
__device__ __forceinline__ void step_range(const ParticleArrays& p, uint32_t b, uint32_t e, const Window& w,
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


// One work item with kFusedThreads threads: stage the force window of the
// item's tile, step its particles (window gathers, fixed-point window
// deposits), flush the deposit window into the density; sparse items (fewer
// than kItemDirect particles) use global gathers and atomics.  force / rho
// address the item's lattice; fwin / dwin: the CTA's shared windows.
template <int CIC, int GRAN>
__device__ __forceinline__ void fused_item(const WorkItem& item, const ParticleArrays& p,
                                           const float2* __restrict__ force, float* __restrict__ rho, int N, float dt,
                                           float2* fwin, uint32_t* dwin) {
    constexpr int WY = win_y(GRAN), WX = win_x(GRAN);
    if (item.end - item.begin < uint32_t(kItemDirect)) {
        // sparse tile: no windows, global gathers and atomics
        const Window w{nullptr, nullptr, item.x0, item.y0, 1.0f, 0.0f};
        step_range<CIC, WX, WY>(p, item.begin, item.end, w, force, rho, N, dt);
        return;
    }
    for (int i = threadIdx.x; i < WY * WX; i += kFusedThreads) {
        const int r = i / WX, c = i - r * WX;
        const int gx = item.x0 + c, gy = item.y0 + r;
        float2 f = make_float2(0.0f, 0.0f);
        if (gx >= 0 && gx < N && gy >= 0 && gy < N) f = __ldg(force + size_t(gy) * N + gx);
        fwin[i] = f;
        dwin[i] = 0u;
    }
    __syncthreads();
    const Window w{fwin, dwin, item.x0, item.y0, item.scale, item.heavy};
    step_range<CIC, WX, WY>(p, item.begin, item.end, w, force, rho, N, dt);
    __syncthreads();
    constexpr int W4 = WX / 4;
    const uint4* d4 = reinterpret_cast<const uint4*>(dwin);
    const float inv = item.inv_scale;
    for (int i = threadIdx.x; i < WY * W4; i += kFusedThreads) {
        const int r = i / W4, c4 = i - r * W4;
        const int gy = item.y0 + r, gx = item.x0 + 4 * c4;
        if (gy < 0 || gy >= N || gx < 0 || gx >= N) continue;
        const uint4 q = d4[i];
        if ((q.x | q.y | q.z | q.w) != 0u)
            red_add_v4(rho + size_t(gy) * N + gx,
                       make_float4(__uint2float_rn(q.x) * inv, __uint2float_rn(q.y) * inv,
                                   __uint2float_rn(q.z) * inv, __uint2float_rn(q.w) * inv));
    }
    __syncthreads();
}

}  // namespace cpm
