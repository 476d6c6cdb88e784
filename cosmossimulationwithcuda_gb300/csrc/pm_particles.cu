// Particle-side kernels of the particle-mesh step: deposit, gradient, gather +
// integrate, and the tile sort that orders the particle state.
//
// Reference semantics kept bit-for-bit in meaning (CosmosCuda.cuh):
//  - only the first 4*floor(P/4) particles take part (float4 walk, :239-242, :454);
//  - a particle is active when its cell (C truncation) lies in [1, N-1)^2
//    (:497 deposit, :257 gather); inactive particles are neither deposited
//    nor moved;
//  - CIC weights (1-fx)(1-fy), fx(1-fy), (1-fx)fy, fx fy on cells c, c+1,
//    c+N, c+N+1 (:498-511) for both deposit and gather (:263-278);
//  - position Verlet: x' = (2x - xOld) + dt*F*dt, wrap x' < 2 -> +(N-4),
//    x' > N-2 -> -(N-4), xOld' = pre-step x (unwrapped) (:286-303).
#include "pm_common.cuh"
#include "pm_internal.h"
#include "pm_particle_math.cuh"

namespace cpm {

namespace {

constexpr int kThreads = 256;

inline int stream_grid(int64_t work_items, int nsm) {
    const int64_t per_sm = 2048 / kThreads;
    int64_t g = (work_items + kThreads - 1) / kThreads;
    const int64_t cap = int64_t(nsm > 0 ? nsm : 152) * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return int(g);
}

__device__ __forceinline__ float comp(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

}  // namespace

// ---- deposit: global atomics (first step and fallback) -------------------------------------
__global__ void __launch_bounds__(kThreads) k_deposit_global(const float4* __restrict__ x, const float4* __restrict__ y,
                                                             const float4* __restrict__ m, int64_t ngroups,
                                                             float* __restrict__ rho, int N, int cic) {
    for (int64_t g = blockIdx.x * int64_t(kThreads) + threadIdx.x; g < ngroups; g += int64_t(gridDim.x) * kThreads) {
        const float4 xf = __ldcs(x + g);
        const float4 yf = __ldcs(y + g);
        const float4 mf = __ldcs(m + g);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float px = comp(xf, i), py = comp(yf, i), pm = comp(mf, i);
            const int cx = int(px), cy = int(py);
            if (!active_cell(cx, cy, N)) continue;
            float* c = rho + size_t(cx) + size_t(cy) * N;
            if (cic) {
                const float fx = px - float(cx), fy = py - float(cy);
                const float x1 = 1.0f - fx, y1 = 1.0f - fy;
                atomicAdd(c, (x1 * y1) * pm);
                atomicAdd(c + 1, (fx * y1) * pm);
                atomicAdd(c + N, (x1 * fy) * pm);
                atomicAdd(c + N + 1, (fx * fy) * pm);
            } else {
                atomicAdd(c, pm);
            }
        }
    }
}

cudaError_t launch_deposit_global(const ParticleArrays& p, int64_t P, float* rho, int N, int cic, int nsm,
                                  cudaStream_t st) {
    const int64_t ng = P / 4;
    if (ng > 0)
        k_deposit_global<<<stream_grid(ng, nsm), kThreads, 0, st>>>(
            reinterpret_cast<const float4*>(p.x), reinterpret_cast<const float4*>(p.y),
            reinterpret_cast<const float4*>(p.m), ng, rho, N, cic);
    return cudaGetLastError();
}

// ---- gradient: edge-clamped 4th-order difference (CosmosCuda.cuh:174-229) ------------------
__global__ void __launch_bounds__(kThreads) k_gradient(const float* __restrict__ phi, float2* __restrict__ force,
                                                       int N, int logN, float gmult) {
    const int64_t NN = int64_t(N) * N;
    phi += size_t(blockIdx.y) * NN;  // batch of lattices back to back
    force += size_t(blockIdx.y) * NN;
    for (int64_t idx = blockIdx.x * int64_t(kThreads) + threadIdx.x; idx < NN; idx += int64_t(gridDim.x) * kThreads) {
        const int cx = int(idx & (N - 1));
        const int cy = int(idx >> logN);
        const float c = __ldg(phi + idx);
        const float l = cx >= 1 ? __ldg(phi + idx - 1) : c;
        const float r = cx + 1 < N ? __ldg(phi + idx + 1) : c;
        const float t = cy >= 1 ? __ldg(phi + idx - N) : c;
        const float b = cy + 1 < N ? __ldg(phi + idx + N) : c;
        const float ll = cx >= 2 ? __ldg(phi + idx - 2) : c;
        const float rr = cx + 2 < N ? __ldg(phi + idx + 2) : c;
        const float tt = cy >= 2 ? __ldg(phi + idx - 2 * N) : c;
        const float bb = cy + 2 < N ? __ldg(phi + idx + 2 * N) : c;
        force[idx] = make_float2(diff4(ll, l, r, rr, gmult), diff4(tt, t, b, bb, gmult));
    }
}

cudaError_t launch_gradient(const float* phi, float2* force, int N, float gmult, cudaStream_t st, int batch) {
    if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
    const int64_t NN = int64_t(N) * N;
    int grid = int((NN + kThreads - 1) / kThreads);
    const int cap = (152 * 8 + batch - 1) / batch;
    if (grid > cap) grid = cap;
    k_gradient<<<dim3(grid, batch), kThreads, 0, st>>>(phi, force, N, ilog2(N), gmult);
    return cudaGetLastError();
}

// ---- gather + integrate ----------------------------------------------------------------------
// The operation order is fixed with explicit intrinsics (and mirrored by the
// FP32 oracle), so results are reproducible bit for bit:
//   F = fma(f11, w11, fma(f01, w01, fma(f10, w10, f00*w00)))
//   x' = fma(dt*F, dt, fma(2, x, -xOld))
__device__ __forceinline__ void gather_update(const float2* __restrict__ force, int N, int cic, float dt, float& px,
                                              float& py, float& pxo, float& pyo) {
    const int cx = int(px), cy = int(py);
    if (!active_cell(cx, cy, N)) return;
    const size_t c = size_t(cx) + size_t(cy) * N;
    float2 F;
    if (cic) {
        const CicWeights w = cic_weights(px, py, cx, cy);
        F = bilinear(w, __ldg(force + c), __ldg(force + c + 1), __ldg(force + c + N), __ldg(force + c + N + 1));
    } else {
        F = __ldg(force + c);
    }
    verlet_wrap(px, py, pxo, pyo, F, dt, N);
}

__global__ void __launch_bounds__(kThreads) k_integrate(const float2* __restrict__ force, float4* __restrict__ x,
                                                        float4* __restrict__ y, float4* __restrict__ xo,
                                                        float4* __restrict__ yo, int64_t ngroups, int N, int cic,
                                                        float dt) {
    for (int64_t g = blockIdx.x * int64_t(kThreads) + threadIdx.x; g < ngroups; g += int64_t(gridDim.x) * kThreads) {
        float4 X = __ldcs(x + g), Y = __ldcs(y + g), XO = __ldcs(xo + g), YO = __ldcs(yo + g);
        gather_update(force, N, cic, dt, X.x, Y.x, XO.x, YO.x);
        gather_update(force, N, cic, dt, X.y, Y.y, XO.y, YO.y);
        gather_update(force, N, cic, dt, X.z, Y.z, XO.z, YO.z);
        gather_update(force, N, cic, dt, X.w, Y.w, XO.w, YO.w);
        __stcs(x + g, X);
        __stcs(y + g, Y);
        __stcs(xo + g, XO);
        __stcs(yo + g, YO);
    }
}

cudaError_t launch_integrate(const float2* force, const ParticleArrays& p, int64_t P, int N, int cic, float dt,
                             int nsm, cudaStream_t st) {
    const int64_t ng = P / 4;
    if (ng > 0)
        k_integrate<<<stream_grid(ng, nsm), kThreads, 0, st>>>(
            force, reinterpret_cast<float4*>(p.x), reinterpret_cast<float4*>(p.y), reinterpret_cast<float4*>(p.xo),
            reinterpret_cast<float4*>(p.yo), ng, N, cic, dt);
    return cudaGetLastError();
}

// ---- sort keys ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_tile_keys(const float* __restrict__ x, const float* __restrict__ y,
                                                        int64_t P, int N, int gran, uint32_t* __restrict__ keys) {
    for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < P; i += int64_t(gridDim.x) * kThreads)
        keys[i] = tile_key(__ldg(x + i), __ldg(y + i), N, gran);
}

cudaError_t launch_tile_keys(const float* x, const float* y, int64_t P, int N, int gran, uint32_t* keys,
                             cudaStream_t st) {
    if (P > 0) k_tile_keys<<<stream_grid(P, 152), kThreads, 0, st>>>(x, y, P, N, gran, keys);
    return cudaGetLastError();
}

// Ensemble keys: slots [sim_off[s], sim_off[s+1]) belong to simulation s; the
// key is s * (T^2 + 1) + the tile key (T^2 = inactive), so one sort orders
// every simulation's segment by tile and keeps the segments in place.
__global__ void __launch_bounds__(kThreads) k_tile_keys_sims(const float* __restrict__ x, const float* __restrict__ y,
                                                             int64_t P, int N, int gran,
                                                             const int64_t* __restrict__ sim_off, int nsims,
                                                             uint32_t* __restrict__ keys) {
    const uint32_t T = uint32_t(N >> gran);
    const uint32_t stride = T * T + 1u;
    for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < P; i += int64_t(gridDim.x) * kThreads) {
        int lo = 0, hi = nsims;  // largest s with sim_off[s] <= i
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(sim_off + mid) <= i) lo = mid; else hi = mid;
        }
        keys[i] = uint32_t(lo) * stride + tile_key(__ldg(x + i), __ldg(y + i), N, gran);
    }
}

cudaError_t launch_tile_keys_sims(const float* x, const float* y, int64_t P, int N, int gran, const int64_t* sim_off,
                                  int nsims, uint32_t* keys, cudaStream_t st) {
    if (P > 0 && nsims > 0)
        k_tile_keys_sims<<<stream_grid(P, 152), kThreads, 0, st>>>(x, y, P, N, gran, sim_off, nsims, keys);
    return cudaGetLastError();
}

// ---- stable LSD radix sort (8-bit digits, reduce-then-scan) ------------------------------------
// Pass over digit `shift`:
//   upsweep   : CTA c counts the digits of its contiguous range -> counts[d*G + c]
//   scan      : exclusive scan of counts in (digit, CTA) order
//   downsweep : CTA c walks its range in tiles of 4096 in order; each warp
//               ranks its 512 keys stably (match_any peers + running per-warp
//               digit counts), warps are prefixed per digit, and keys/values
//               scatter to counts-offset + rank.
// Ranks follow input order inside a CTA and CTAs own increasing ranges, so the
// sort is stable.  No CTA waits on another.
constexpr int kRsThreads = 256;
constexpr int kRsIpt = 16;
constexpr int kRsTile = kRsThreads * kRsIpt;
constexpr int kRsWarps = kRsThreads / 32;

// CTAs per SM of the radix passes: the downsweep is register-limited to 3
// (80 registers), and a grid of exactly the resident CTAs runs as one wave
// (4 per SM at 111 registers ran as two waves of 2: 0.83 -> 0.68 ms per
// 20M-particle sort).
#ifndef CPM_RADIX_CTAS_PER_SM
#define CPM_RADIX_CTAS_PER_SM 3
#endif
int radix_grid(int64_t n, int nsm) {
    const int64_t tiles = (n + kRsTile - 1) / kRsTile;
    int64_t g = int64_t(CPM_RADIX_CTAS_PER_SM) * (nsm > 0 ? nsm : 152);
    if (g > tiles) g = tiles;
    if (g < 1) g = 1;
    return int(g);
}

// counts[256][grid] followed by the 256 digit totals
size_t radix_counts_elems(int grid) { return size_t(256) * grid + 256; }

__global__ void __launch_bounds__(kRsThreads) k_radix_upsweep(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                              int64_t tiles_per_cta, uint32_t* __restrict__ counts) {
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t lo = int64_t(blockIdx.x) * tiles_per_cta * kRsTile;
    int64_t hi = lo + tiles_per_cta * kRsTile;
    if (hi > n) hi = n;
    for (int64_t i = lo + threadIdx.x; i < hi; i += kRsThreads) atomicAdd(&hist[(__ldg(keys + i) >> shift) & 255u], 1u);
    __syncthreads();
    counts[size_t(threadIdx.x) * gridDim.x + blockIdx.x] = hist[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (256 threads); *total gets the sum.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += n;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    uint32_t wbase = 0, all = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t s = warp_sums[i];
        wbase += i < w ? s : 0u;
        all += s;
    }
    __syncthreads();
    *total = all;
    return wbase + incl - v;
}

// Row scan: CTA d scans counts[d][0..G) in place (exclusive) and writes the row
// total to digit_total[d].  The digit prefix is added in the downsweep.
__global__ void __launch_bounds__(kRsThreads) k_radix_scan_rows(uint32_t* __restrict__ counts, int G,
                                                                uint32_t* __restrict__ digit_total) {
    uint32_t* row = counts + size_t(blockIdx.x) * G;
    const int per = (G + kRsThreads - 1) / kRsThreads;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, G);
    uint32_t s = 0;
    for (int i = lo; i < hi; ++i) s += row[i];
    uint32_t tot;
    uint32_t run = block_exclusive_scan_256(s, &tot);
    for (int i = lo; i < hi; ++i) {
        const uint32_t c = row[i];
        row[i] = run;
        run += c;
    }
    if (threadIdx.x == 0) digit_total[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kRsThreads, CPM_RADIX_CTAS_PER_SM) k_radix_downsweep(const uint32_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ vin,
                                                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                int64_t n, int shift, int64_t tiles_per_cta,
                                                                const uint32_t* __restrict__ counts,
                                                                const uint32_t* __restrict__ digit_total) {
    __shared__ uint32_t run_off[256];
    __shared__ uint32_t tile_total[256];
    __shared__ uint32_t wcnt[kRsWarps][256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    {
        uint32_t all;
        const uint32_t digit_base = block_exclusive_scan_256(digit_total[tid], &all);
        run_off[tid] = digit_base + counts[size_t(tid) * gridDim.x + blockIdx.x];
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t t0 = int64_t(blockIdx.x) * tiles_per_cta;
    for (int64_t t = 0; t < tiles_per_cta; ++t) {
        const int64_t base = (t0 + t) * kRsTile;
        if (base >= n) break;
#pragma unroll
        for (int i = 0; i < kRsWarps; ++i) wcnt[i][tid] = 0;
        __syncthreads();
        uint32_t k[kRsIpt], v[kRsIpt], rank[kRsIpt];
#pragma unroll
        for (int i = 0; i < kRsIpt; ++i) {
            const int64_t e = base + int64_t(w) * 32 * kRsIpt + i * 32 + lane;
            const bool valid = e < n;
            k[i] = valid ? kin[e] : 0u;
            v[i] = valid ? vin[e] : 0u;
            const uint32_t dig = valid ? ((k[i] >> shift) & 255u) : 256u;
            const uint32_t peers = __match_any_sync(0xffffffffu, dig);
            uint32_t prior = 0;
            if (valid) prior = wcnt[w][dig];
            __syncwarp();
            if (valid && (__ffs(peers) - 1) == lane) wcnt[w][dig] = prior + __popc(peers);
            __syncwarp();
            rank[i] = valid ? prior + __popc(peers & lt_mask) : 0xffffffffu;
        }
        __syncthreads();
        {
            uint32_t s = 0;
#pragma unroll
            for (int i = 0; i < kRsWarps; ++i) {
                const uint32_t c = wcnt[i][tid];
                wcnt[i][tid] = s;
                s += c;
            }
            tile_total[tid] = s;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kRsIpt; ++i) {
            if (rank[i] != 0xffffffffu) {
                const uint32_t dig = (k[i] >> shift) & 255u;
                const uint32_t pos = run_off[dig] + wcnt[w][dig] + rank[i];
                kout[pos] = k[i];
                vout[pos] = v[i];
            }
        }
        __syncthreads();
        run_off[tid] += tile_total[tid];
        __syncthreads();
    }
}

cudaError_t launch_radix_sort(RadixScratch& s, int64_t n, int bits, int* result_buf, cudaStream_t st) {
    int cur = 0;
    if (n <= 0) {
        *result_buf = 0;
        return cudaSuccess;
    }
    const int64_t tiles = (n + kRsTile - 1) / kRsTile;
    const int64_t tpc = (tiles + s.grid - 1) / s.grid;
    uint32_t* digit_total = s.counts + size_t(256) * s.grid;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_upsweep<<<s.grid, kRsThreads, 0, st>>>(s.keys[cur], n, shift, tpc, s.counts);
        k_radix_scan_rows<<<256, kRsThreads, 0, st>>>(s.counts, s.grid, digit_total);
        k_radix_downsweep<<<s.grid, kRsThreads, 0, st>>>(s.keys[cur], s.vals[cur], s.keys[cur ^ 1], s.vals[cur ^ 1], n,
                                                        shift, tpc, s.counts, digit_total);
        cur ^= 1;
    }
    *result_buf = cur;
    return cudaGetLastError();
}

// ---- permutation helpers -----------------------------------------------------------------
__global__ void k_iota(uint32_t* __restrict__ v, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = uint32_t(i);
}

cudaError_t launch_iota(uint32_t* v, int64_t n, cudaStream_t st) {
    if (n > 0) k_iota<<<stream_grid(n, 152), kThreads, 0, st>>>(v, n);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(kThreads) k_permute(ParticleArrays src, ParticleArrays dst,
                                                      const uint32_t* __restrict__ perm, int64_t n) {
    // four destinations per thread: 24 independent gathers in flight
    const int64_t n4 = n / 4;
    for (int64_t q = blockIdx.x * int64_t(kThreads) + threadIdx.x; q < n4; q += int64_t(gridDim.x) * kThreads) {
        const uint4 p = __ldg(reinterpret_cast<const uint4*>(perm) + q);
        const uint32_t pp[4] = {p.x, p.y, p.z, p.w};
        float4 x, y, xo, yo, m;
        uint4 id;
        float* X = &x.x; float* Y = &y.x; float* XO = &xo.x; float* YO = &yo.x; float* Mm = &m.x;
        uint32_t* ID = &id.x;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            X[j] = __ldg(src.x + pp[j]);
            Y[j] = __ldg(src.y + pp[j]);
            XO[j] = __ldg(src.xo + pp[j]);
            YO[j] = __ldg(src.yo + pp[j]);
            Mm[j] = __ldg(src.m + pp[j]);
            ID[j] = __ldg(src.id + pp[j]);
        }
        reinterpret_cast<float4*>(dst.x)[q] = x;
        reinterpret_cast<float4*>(dst.y)[q] = y;
        reinterpret_cast<float4*>(dst.xo)[q] = xo;
        reinterpret_cast<float4*>(dst.yo)[q] = yo;
        reinterpret_cast<float4*>(dst.m)[q] = m;
        reinterpret_cast<uint4*>(dst.id)[q] = id;
    }
    for (int64_t i = n4 * 4 + blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(gridDim.x) * kThreads) {
        const uint32_t p = __ldg(perm + i);
        dst.x[i] = __ldg(src.x + p);
        dst.y[i] = __ldg(src.y + p);
        dst.xo[i] = __ldg(src.xo + p);
        dst.yo[i] = __ldg(src.yo + p);
        dst.m[i] = __ldg(src.m + p);
        dst.id[i] = __ldg(src.id + p);
    }
}

cudaError_t launch_permute(const ParticleArrays& src, const ParticleArrays& dst, const uint32_t* perm, int64_t n,
                           cudaStream_t st) {
    if (n > 0) k_permute<<<stream_grid(n, 152), kThreads, 0, st>>>(src, dst, perm, n);
    return cudaGetLastError();
}

__global__ void k_invert(const uint32_t* __restrict__ id, uint32_t* __restrict__ pos, int64_t n) {
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x)
        pos[id[s]] = uint32_t(s);
}

cudaError_t launch_invert(const uint32_t* id, uint32_t* pos, int64_t n, cudaStream_t st) {
    if (n > 0) k_invert<<<stream_grid(n, 152), kThreads, 0, st>>>(id, pos, n);
    return cudaGetLastError();
}

__global__ void k_gather_by_id(const float* __restrict__ in, const uint32_t* __restrict__ pos, int64_t offset,
                               int64_t count, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = in[pos[offset + i]];
}

cudaError_t launch_gather_by_id(const float* in, const uint32_t* pos, int64_t offset, int64_t count, float* out,
                                cudaStream_t st) {
    if (count > 0) k_gather_by_id<<<stream_grid(count, 152), kThreads, 0, st>>>(in, pos, offset, count, out);
    return cudaGetLastError();
}

__global__ void k_scatter_by_id(const float* __restrict__ in, const uint32_t* __restrict__ pos, int64_t offset,
                                int64_t count, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x)
        out[pos[offset + i]] = in[i];
}

cudaError_t launch_scatter_by_id(const float* in, const uint32_t* pos, int64_t offset, int64_t count, float* out,
                                 cudaStream_t st) {
    if (count > 0) k_scatter_by_id<<<stream_grid(count, 152), kThreads, 0, st>>>(in, pos, offset, count, out);
    return cudaGetLastError();
}

__global__ void k_unpermute(const float* __restrict__ in, const uint32_t* __restrict__ id, int64_t n,
                            float* __restrict__ out) {
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x)
        out[id[s]] = in[s];
}

cudaError_t launch_unpermute(const float* in, const uint32_t* id, int64_t n, float* out, cudaStream_t st) {
    if (n > 0) k_unpermute<<<stream_grid(n, 152), kThreads, 0, st>>>(in, id, n, out);
    return cudaGetLastError();
}

__global__ void k_fill(float* __restrict__ v, float value, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = value;
}

cudaError_t launch_fill(float* v, float value, int64_t n, cudaStream_t st) {
    if (n > 0) k_fill<<<stream_grid(n, 152), kThreads, 0, st>>>(v, value, n);
    return cudaGetLastError();
}

// ---- FP64 diagnostics ------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_diagnostics(ParticleArrays p, int64_t P, const float* __restrict__ phi,
                                                          int N, float dt, double* __restrict__ out) {
    double ke = 0.0, pe = 0.0, mx = 0.0, my = 0.0;
    const double inv_dt = 1.0 / double(dt);
    // The wrap moves x by N-4 but leaves xOld on the far side (the reference
    // keeps the pre-step position, CosmosCuda.cuh:288-301), so x - xOld of a
    // wrapped particle carries +-(N-4) from then on: take the displacement
    // modulo the wrap period.
    const double period = double(N) - 4.0, half = 0.5 * period;
    auto unwrap = [period, half](double d) { return d > half ? d - period : (d < -half ? d + period : d); };
    for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < P; i += int64_t(gridDim.x) * kThreads) {
        const float x = p.x[i], y = p.y[i];
        const int cx = int(x), cy = int(y);
        if (!active_cell(cx, cy, N)) continue;
        const double m = p.m[i];
        const double vx = unwrap(double(x) - double(p.xo[i])) * inv_dt;
        const double vy = unwrap(double(y) - double(p.yo[i])) * inv_dt;
        ke += 0.5 * m * (vx * vx + vy * vy);
        pe += 0.5 * m * double(phi[size_t(cx) + size_t(cy) * N]);
        mx += m * vx;
        my += m * vy;
    }
    for (int off = 16; off > 0; off >>= 1) {
        ke += __shfl_down_sync(0xffffffffu, ke, off);
        pe += __shfl_down_sync(0xffffffffu, pe, off);
        mx += __shfl_down_sync(0xffffffffu, mx, off);
        my += __shfl_down_sync(0xffffffffu, my, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, ke);
        atomicAdd(out + 1, pe);
        atomicAdd(out + 2, mx);
        atomicAdd(out + 3, my);
    }
}

cudaError_t launch_diagnostics(const ParticleArrays& p, int64_t P, const float* phi, int N, float dt, double* out,
                               cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, 4 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const int64_t Pq = (P / 4) * 4;
    if (Pq > 0) k_diagnostics<<<stream_grid(Pq, 152), kThreads, 0, st>>>(p, Pq, phi, N, dt, out);
    return cudaGetLastError();
}

}  // namespace cpm
