// Tile-ordered particle kernels: the fused gather + update + next-step deposit.
//
// After a sort the particle state is ordered by the Morton code of its
// (2^GRAN)^2-cell tile.  Each tile's slot range is cut into work items of at
// most kItemMax particles.  A CTA takes one item at a time and
//   1. stages the force field of the tile plus a kTileHalo-cell border (+1 for
//      the CIC corners) into shared memory,
//   2. streams the item's particles with 128-bit loads (x, y, xOld, yOld, m),
//      gathers the force from the window, applies the position-Verlet update
//      and wrap of the reference, and stores the new state,
//   3. deposits the NEW positions (the next step's density) into a shared
//      window of 32-bit fixed-point accumulators with native integer atomics,
//   4. flushes the window once into the global density with 16-byte vector
//      float reductions, skipping empty 4-cell groups.
// Particles that drifted outside the window since the last sort fall back to
// global loads / float atomics, so the result is correct for any drift.
// Items with fewer than kItemDirect particles (sparse tiles) skip the windows.
//
// Fixed point: an item's deposits are scaled by S = 2^k < 2^31 / M, M the
// summed mass of the item's (non-heavy) particles, so no window cell can
// overflow (a cell holds at most M * S plus half a unit of rounding per
// deposit, below 2^31 + 2^15 < 2^32); S is a power of two, so unit masses stay exact and the flush
// scales back exactly.  Particles heavier than M/128 deposit with global float
// atomics so that one heavy body cannot coarsen the resolution of the others.
// (Shared-memory float atomicAdd is a compare-and-swap loop on this
// architecture; integer atomicAdd is a single native operation.)
//
// Fusing step n's integrate with step n+1's deposit reads each particle once
// per step (20 B) and writes it once (16 B) instead of 12 + 32 B in two
// kernels; the reference does the deposit (CosmosCuda.cuh:446-595) and the
// gather (:231-312) as separate passes.
#include <cfloat>

#include "bulk_copy.cuh"
#include "tile_step.cuh"

namespace cpm {

namespace {

__device__ __forceinline__ uint32_t compact_bits(uint32_t v) {
    v &= 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0F0F0F0Fu;
    v = (v | (v >> 4)) & 0x00FF00FFu;
    v = (v | (v >> 8)) & 0x0000FFFFu;
    return v;
}

}  // namespace

// ---- work items from the sorted keys -------------------------------------------------------
// Tile ranges of the sorted keys: a tile's range starts where its key differs
// from the one before and ends where it differs from the one after.  One
// thread takes four consecutive keys with one 16-byte load (the key buffers
// are 16-byte aligned) plus the keys either side.
__global__ void k_tile_ranges(const uint32_t* __restrict__ keys, int64_t n, uint32_t ntiles,
                              uint32_t* __restrict__ tstart, uint32_t* __restrict__ tend) {
    constexpr uint32_t kNone = 0xFFFFFFFFu;  // no key: before the first one and after the last one
    const int64_t nq = (n + 3) / 4;
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < nq; q += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i0 = q * 4;
        uint32_t k[6];
        if (i0 + 4 <= n) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(keys) + q);
            k[1] = v.x;
            k[2] = v.y;
            k[3] = v.z;
            k[4] = v.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) k[1 + j] = i0 + j < n ? __ldg(keys + i0 + j) : kNone;
        }
        k[0] = i0 > 0 ? __ldg(keys + i0 - 1) : kNone;
        k[5] = i0 + 4 < n ? __ldg(keys + i0 + 4) : kNone;
#pragma unroll
        for (int j = 1; j <= 4; ++j) {
            const uint32_t key = k[j];
            if (key >= ntiles) continue;  // inactive particles, and the slots past n
            const uint32_t i = uint32_t(i0 + j - 1);
            if (k[j - 1] != key) tstart[key] = i;
            if (k[j + 1] != key) tend[key] = i + 1;
        }
    }
}

// One CTA: count the items of each tile, scan, write the items (tile order).
// Keys run over nsims blocks of `stride` = T^2 + 1 (the last one of each block
// holds the inactive particles, which get no items); the simulation index goes
// into WorkItem::sim.
__global__ void __launch_bounds__(1024) k_build_items(const uint32_t* __restrict__ tstart,
                                                      const uint32_t* __restrict__ tend, int ntiles, int stride,
                                                      int gran, int item_max, WorkItem* __restrict__ items,
                                                      uint32_t* __restrict__ n_items) {
    __shared__ uint32_t part[1024];
    const int seg = (ntiles + 1023) / 1024;
    const int lo = int(threadIdx.x) * seg;
    const int hi = min(lo + seg, ntiles);
    uint32_t cnt = 0;
    for (int t = lo; t < hi; ++t)
        if (t % stride != stride - 1) cnt += (tend[t] - tstart[t] + item_max - 1) / item_max;
    part[threadIdx.x] = cnt;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t base = part[threadIdx.x] - cnt;
    for (int t = lo; t < hi; ++t) {
        const int sim = t / stride, local = t - sim * stride;
        if (local == stride - 1) continue;  // inactive particles
        const uint32_t s = tstart[t], c = tend[t] - s;
        const uint32_t nch = (c + item_max - 1) / item_max;
        const int x0 = int(compact_bits(uint32_t(local)) << gran) - kTileHalo;
        const int y0 = int(compact_bits(uint32_t(local) >> 1) << gran) - kTileHalo;
        for (uint32_t j = 0; j < nch; ++j) {
            WorkItem w;
            w.x0 = x0;
            w.y0 = y0;
            w.begin = s + uint32_t((uint64_t(c) * j) / nch);
            w.end = s + uint32_t((uint64_t(c) * (j + 1)) / nch);
            w.scale = 1.0f;
            w.inv_scale = 1.0f;
            w.heavy = FLT_MAX;
            w.sim = uint32_t(sim);
            items[base++] = w;
        }
    }
    if (threadIdx.x == 1023) *n_items = part[1023];
}

__device__ __forceinline__ float block_sum_256(float v, float* red) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += red[i];
    return s;
}

// Deposit scale of each item: S = 2^k < 2^31 / M_light, with M_light the mass
// of the item's particles no heavier than 1/128 of the item's total mass.
__global__ void __launch_bounds__(256) k_item_scales(const float* __restrict__ m, WorkItem* __restrict__ items,
                                                     const uint32_t* __restrict__ n_items) {
    __shared__ float red[8];
    const uint32_t it = blockIdx.x;
    if (it >= *n_items) return;
    const uint32_t b = items[it].begin, e = items[it].end;
    float s = 0.0f;
    for (uint32_t i = b + threadIdx.x; i < e; i += 256) s += __ldg(m + i);
    const float total = block_sum_256(s, red);
    const float heavy = total / 128.0f;
    float sl = 0.0f;
    for (uint32_t i = b + threadIdx.x; i < e; i += 256) {
        const float mi = __ldg(m + i);
        sl += mi <= heavy ? mi : 0.0f;
    }
    const float light = block_sum_256(sl, red);
    if (threadIdx.x == 0) {
        int ex = 31;
        if (light > 0.0f) {
            int e2;
            frexpf(light * 1.001f, &e2);  // light < 2^e2
            ex = 31 - e2;
        }
        ex = ex > 120 ? 120 : (ex < -120 ? -120 : ex);
        items[it].scale = ldexpf(1.0f, ex);
        items[it].inv_scale = ldexpf(1.0f, -ex);
        items[it].heavy = heavy;
    }
}

// ---- the fused step kernel, tile windows ----------------------------------------------------
template <int CIC, int GRAN>
__global__ void CPM_FUSED_BOUNDS k_fused_tiles(const WorkItem* __restrict__ items,
                                                               const uint32_t* __restrict__ n_items_p,
                                                               ParticleArrays p, const float2* __restrict__ force,
                                                               float* __restrict__ rho, int N, float dt) {
    extern __shared__ float4 smem4[];
    const WindowSmem<CIC, GRAN> win(smem4);
    dependency_wait();
    allow_dependents();
    const uint32_t n_items = *n_items_p;
    const float2* const force0 = force;
    float* const rho0 = rho;
    for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
        const WorkItem item = items[it];
        fused_item<CIC, GRAN>(item, p, force0 + size_t(item.sim) * N * N, rho0 + size_t(item.sim) * N * N, N, dt,
                              win);
    }
}

// ---- the fused step kernel, tile windows, particles staged by bulk copies -----------------
// Same work as k_fused_tiles, with the particle arrays streamed into shared
// memory by the SM's bulk-copy engine instead of per-thread loads: one
// producer warp walks the CTA's work items in order and, per chunk of
// kBulkChunk particles (the 16-byte-aligned part of an item), copies the five
// arrays x, y, xOld, yOld, m into one of kBulkStages shared stages; eight
// consumer warps take one float4 group of each array per thread from the
// stage (conflict-free 16-byte shared loads), gather, update and deposit as
// before, and store the new state straight to global memory.  The copies of
// the next chunks (and of the next item's first chunks) are in flight while a
// chunk is computed, without holding registers, and the consumer warps of one
// CTA synchronise among themselves (named barrier) only around the windows.
// Waits are bounded: a timeout sets *status, the CTA stops issuing work,
// every warp keeps its barrier schedule with the work skipped, and the
// producer waits (bounded) for its copies in flight before the CTA exits.
// CPM_BULK_EVICT_FIRST=1 reads the particle chunks with an L2 evict-first
// policy (measured: 0.2602 -> 0.2617 ms per step at 20M / 2048^2, so off).
#ifndef CPM_BULK_EVICT_FIRST
#define CPM_BULK_EVICT_FIRST 0
#endif
constexpr int kBulkConsumers = 256;                    // 8 compute warps
constexpr int kBulkThreads = kBulkConsumers + 32;      // + 1 producer warp
constexpr int kBulkChunk = 4 * kBulkConsumers;         // particles per stage: one float4 group per thread
constexpr int kBulkStages = 2;
constexpr int kBulkArrays = 5;                         // x, y, xOld, yOld, m
constexpr size_t kBulkStageFloats = size_t(kBulkArrays) * kBulkChunk;

template <int CIC, int GRAN>
__global__ void __launch_bounds__(kBulkThreads) k_fused_tiles_bulk(const WorkItem* __restrict__ items,
                                                                  const uint32_t* __restrict__ n_items_p,
                                                                  ParticleArrays p, const float2* __restrict__ force,
                                                                  float* __restrict__ rho, int N, float dt,
                                                                  int* __restrict__ status, uint32_t tx_extra) {
    constexpr int WY = win_y(GRAN), WX = win_x(GRAN);
    extern __shared__ float4 smem4[];
    float* stages = reinterpret_cast<float*>(smem4);  // [stage][array][kBulkChunk]
    const WindowSmem<CIC, GRAN> win(stages + kBulkStages * kBulkStageFloats);
    __shared__ __align__(8) uint64_t full[kBulkStages], empty[kBulkStages];
    __shared__ volatile int abort_flag;
    const int tid = int(threadIdx.x), warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < kBulkStages; ++s) {
            bulk::mbar_init(&full[s], 1);
            bulk::mbar_init(&empty[s], kBulkConsumers / 32);
        }
        abort_flag = 0;
        bulk::fence_barrier_init();
    }
    __syncthreads();
    dependency_wait();
    allow_dependents();
    const uint32_t n_items = *n_items_p;

    if (warp == kBulkConsumers / 32) {  // ---- producer warp: one lane issues the copies ----
        if (lane != 0) return;
        float* const arr[kBulkArrays] = {p.x, p.y, p.xo, p.yo, p.m};
#if CPM_BULK_EVICT_FIRST
        const uint64_t policy = bulk::l2_evict_first_policy();
#endif
        uint32_t fills[kBulkStages] = {};
        uint32_t fill = 0;
        for (uint32_t it = blockIdx.x; it < n_items && !abort_flag; it += gridDim.x) {
            const WorkItem item = items[it];
            const uint32_t b4 = (item.begin + 3u) & ~3u, e4 = item.end & ~3u;
            for (uint32_t c = b4; c < e4 && !abort_flag; c += kBulkChunk, ++fill) {
                const uint32_t n = e4 - c < uint32_t(kBulkChunk) ? e4 - c : uint32_t(kBulkChunk);
                const int s = int(fill % kBulkStages);
                if (fills[s] > 0 && !bulk::wait(&empty[s], (fills[s] - 1u) & 1u)) {
                    abort_flag = 1;
                    atomicMax(status, 1);
                    break;
                }
                // tx_extra (a test hook, 0 otherwise) announces bytes that never arrive:
                // the waits on this stage run out with no copy left in flight
                bulk::arrive_expect_tx(&full[s], n * 4u * kBulkArrays + tx_extra);
                float* st = stages + size_t(s) * kBulkStageFloats;
#pragma unroll
                for (int a = 0; a < kBulkArrays; ++a)
#if CPM_BULK_EVICT_FIRST
                    bulk::copy_g2s_hint(st + a * kBulkChunk, arr[a] + c, n * 4u, &full[s], policy);
#else
                    bulk::copy_g2s(st + a * kBulkChunk, arr[a] + c, n * 4u, &full[s]);
#endif
                ++fills[s];
            }
        }
        // copies still in flight (only after a timeout) must land before the CTA's shared memory goes away
        for (int s = 0; s < kBulkStages; ++s)
            if (fills[s] > 0 && !bulk::wait(&full[s], (fills[s] - 1u) & 1u)) atomicMax(status, 2);
        return;
    }

    // ---- consumer warps ----
    const float2* const force0 = force;
    float* const rho0 = rho;
    uint32_t use = 0;
    for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
        const WorkItem item = items[it];
        force = force0 + size_t(item.sim) * N * N;
        rho = rho0 + size_t(item.sim) * N * N;
        const bool dense = item.end - item.begin >= uint32_t(kItemDirect);
        if (dense) {
            stage_windows<CIC, GRAN>(item, force, N, win, tid, kBulkConsumers);
            bulk::named_sync(kBulkConsumers);
        }
        const Window<CIC> w = dense ? Window<CIC>{win.f, win.d, item.x0, item.y0, item.scale, item.heavy}
                                    : Window<CIC>{nullptr, nullptr, item.x0, item.y0, 1.0f, 0.0f};
        const uint32_t b = item.begin, e = item.end;
        const uint32_t b4 = (b + 3u) & ~3u, e4 = e & ~3u;
        if (!abort_flag) {  // ragged head / tail (or the whole range when it spans no full group)
            const uint32_t h_end = b4 < e ? b4 : e;
            const uint32_t t_beg = e4 > h_end ? e4 : h_end;
            const uint32_t nh = h_end - b, nt = e - t_beg;
            if (uint32_t(tid) < nh + nt) {
                const uint32_t i = uint32_t(tid) < nh ? b + tid : t_beg + (tid - nh);
                float px = p.x[i], py = p.y[i], pxo = p.xo[i], pyo = p.yo[i];
                step_particle<CIC, WX, WY>(px, py, pxo, pyo, p.m[i], w, force, rho, N, dt);
                p.x[i] = px;
                p.y[i] = py;
                p.xo[i] = pxo;
                p.yo[i] = pyo;
            }
        }
        for (uint32_t c = b4; c < e4; c += kBulkChunk, ++use) {
            const uint32_t n = e4 - c < uint32_t(kBulkChunk) ? e4 - c : uint32_t(kBulkChunk);
            const int s = int(use % kBulkStages);
            bool ok = !abort_flag;
            if (ok && !bulk::wait(&full[s], (use / kBulkStages) & 1u)) {
                abort_flag = 1;
                atomicMax(status, 1);
                ok = false;
            }
            if (ok && uint32_t(4 * tid) < n) {
                const float4* st = reinterpret_cast<const float4*>(stages + size_t(s) * kBulkStageFloats);
                constexpr int A4 = kBulkChunk / 4;
                float4 x = st[tid], y = st[A4 + tid], xo = st[2 * A4 + tid], yo = st[3 * A4 + tid];
                const float4 m = st[4 * A4 + tid];
                step_particle<CIC, WX, WY>(x.x, y.x, xo.x, yo.x, m.x, w, force, rho, N, dt);
                step_particle<CIC, WX, WY>(x.y, y.y, xo.y, yo.y, m.y, w, force, rho, N, dt);
                step_particle<CIC, WX, WY>(x.z, y.z, xo.z, yo.z, m.z, w, force, rho, N, dt);
                step_particle<CIC, WX, WY>(x.w, y.w, xo.w, yo.w, m.w, w, force, rho, N, dt);
                const uint32_t g = (c >> 2) + uint32_t(tid);
                __stcs(reinterpret_cast<float4*>(p.x) + g, x);
                __stcs(reinterpret_cast<float4*>(p.y) + g, y);
                __stcs(reinterpret_cast<float4*>(p.xo) + g, xo);
                __stcs(reinterpret_cast<float4*>(p.yo) + g, yo);
            }
            __syncwarp();
            if (lane == 0) bulk::arrive(&empty[s]);
        }
        if (dense) {
            bulk::named_sync(kBulkConsumers);
            if (!abort_flag) flush_window<CIC, GRAN>(item, rho, N, win, tid, kBulkConsumers);
            bulk::named_sync(kBulkConsumers);
        }
    }
}

// ---- the fused step kernel, no tile order (global gathers and atomics) -----------------------
template <int CIC>
__global__ void __launch_bounds__(kFusedThreads) k_fused_global(ParticleArrays p, int64_t ngroups,
                                                                const float2* __restrict__ force,
                                                                float* __restrict__ rho, int N, float dt) {
    float4* X = reinterpret_cast<float4*>(p.x);
    float4* Y = reinterpret_cast<float4*>(p.y);
    float4* XO = reinterpret_cast<float4*>(p.xo);
    float4* YO = reinterpret_cast<float4*>(p.yo);
    const float4* Mm = reinterpret_cast<const float4*>(p.m);
    const Window<CIC> w{nullptr, nullptr, 0, 0, 1.0f, 0.0f};
    dependency_wait();
    for (int64_t g = blockIdx.x * int64_t(kFusedThreads) + threadIdx.x; g < ngroups;
         g += int64_t(gridDim.x) * kFusedThreads) {
        float4 x = __ldcs(X + g), y = __ldcs(Y + g), xo = __ldcs(XO + g), yo = __ldcs(YO + g);
        const float4 m = __ldcs(Mm + g);
        step_particle<CIC, 4, 4>(x.x, y.x, xo.x, yo.x, m.x, w, force, rho, N, dt);
        step_particle<CIC, 4, 4>(x.y, y.y, xo.y, yo.y, m.y, w, force, rho, N, dt);
        step_particle<CIC, 4, 4>(x.z, y.z, xo.z, yo.z, m.z, w, force, rho, N, dt);
        step_particle<CIC, 4, 4>(x.w, y.w, xo.w, yo.w, m.w, w, force, rho, N, dt);
        __stcs(X + g, x);
        __stcs(Y + g, y);
        __stcs(XO + g, xo);
        __stcs(YO + g, yo);
    }
}

// ---- host side -------------------------------------------------------------------------------
size_t tile_window_smem(int gran, int cic) { return window_bytes(gran, cic); }

int work_item_size(int64_t Pq, int nsm) {
    const int64_t want = 16 * int64_t(nsm > 0 ? nsm : 152);
    for (int s = kItemMax; s > kItemMin; s >>= 1)
        if (Pq / s >= want) return s;
    return kItemMin;
}

size_t max_work_items(int64_t Pq, int ntiles, int item_size) { return size_t(Pq / item_size) + size_t(ntiles) + 1; }

// The fused step kernel in use: particles staged by bulk copies (default), or
// loaded by each thread (CPM_FUSED_BULK=0).
#ifndef CPM_FUSED_BULK
#define CPM_FUSED_BULK 1
#endif
size_t fused_tiles_smem(int gran, int cic) {
    return (CPM_FUSED_BULK ? size_t(kBulkStages) * kBulkStageFloats * sizeof(float) : 0) + tile_window_smem(gran, cic);
}
constexpr int kFusedLaunchThreads = CPM_FUSED_BULK ? kBulkThreads : kFusedThreads;

template <int CIC, int GRAN>
static auto fused_kernel() {
#if CPM_FUSED_BULK
    return k_fused_tiles_bulk<CIC, GRAN>;
#else
    return k_fused_tiles<CIC, GRAN>;
#endif
}

cudaError_t prepare_tile_kernels(int gran, int cic, int nsm, int* grid) {
    cudaError_t e = cudaErrorInvalidValue;
    int per_sm = 0;
    const size_t smem = fused_tiles_smem(gran, cic);
#define CPM_TILES(C, G)                                                                                        \
    if (cic == C && gran == G) {                                                                               \
        e = cudaFuncSetAttribute(fused_kernel<C, G>(), cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)); \
        if (e == cudaSuccess)                                                                                  \
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_kernel<C, G>(), kFusedLaunchThreads, \
                                                              smem);                                           \
    }
    CPM_TILES(0, 4) CPM_TILES(0, 5) CPM_TILES(0, 6) CPM_TILES(1, 4) CPM_TILES(1, 5) CPM_TILES(1, 6)
#undef CPM_TILES
    if (e == cudaSuccess) *grid = nsm * (per_sm > 0 ? per_sm : 1);
    return e;
}

size_t tile_range_elems(int N, int gran, int nsims) {
    const size_t t = size_t(N >> gran);
    return (t * t + 1) * size_t(nsims);
}

cudaError_t launch_build_items(const uint32_t* sorted_keys, const float* m, int64_t Pq, int N, int gran,
                               uint32_t* tstart, uint32_t* tend, WorkItem* items, uint32_t* n_items, size_t max_items,
                               int item_size, cudaStream_t st, int nsims) {
    const int t = N >> gran;
    const int stride = t * t + 1;
    const uint32_t ntiles = uint32_t(tile_range_elems(N, gran, nsims));
    cudaError_t e = cudaMemsetAsync(tstart, 0, ntiles * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(tend, 0, ntiles * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (Pq > 0) {
        int64_t g = (Pq + 4 * 256 - 1) / (4 * 256);
        if (g > 4096) g = 4096;
        k_tile_ranges<<<int(g), 256, 0, st>>>(sorted_keys, Pq, ntiles, tstart, tend);
    }
    k_build_items<<<1, 1024, 0, st>>>(tstart, tend, int(ntiles), stride, gran, item_size, items, n_items);
    if (max_items > 0) k_item_scales<<<unsigned(max_items), 256, 0, st>>>(m, items, n_items);
    return cudaGetLastError();
}

cudaError_t launch_fused_tiles(const WorkItem* items, const uint32_t* n_items, const ParticleArrays& p,
                               const float2* force, float* rho, int N, int cic, float dt, int gran, int grid,
                               int* status, cudaStream_t st, uint32_t tx_extra) {
    const size_t smem = fused_tiles_smem(gran, cic);
#if CPM_FUSED_BULK
#define CPM_TILES(C, G)                                                                                      \
    if (cic == C && gran == G) {                                                                             \
        return launch_dependent(N >= kDependentMinN, k_fused_tiles_bulk<C, G>, dim3(grid),                    \
                                dim3(kBulkThreads), smem, st, items, n_items, p, force, rho, N, dt, status,  \
                                tx_extra);                                                                   \
    }
#else
    (void)status;
    (void)tx_extra;
#define CPM_TILES(C, G)                                                                                      \
    if (cic == C && gran == G) {                                                                             \
        return launch_dependent(N >= kDependentMinN, k_fused_tiles<C, G>, dim3(grid),                         \
                                dim3(kFusedThreads), smem, st, items, n_items, p, force, rho, N, dt);        \
    }
#endif
    CPM_TILES(0, 4) CPM_TILES(0, 5) CPM_TILES(0, 6) CPM_TILES(1, 4) CPM_TILES(1, 5) CPM_TILES(1, 6)
#undef CPM_TILES
    return cudaErrorInvalidValue;
}

cudaError_t launch_fused_global(const ParticleArrays& p, int64_t P, const float2* force, float* rho, int N, int cic,
                                float dt, int nsm, cudaStream_t st) {
    const int64_t ng = P / 4;
    if (ng <= 0) return cudaGetLastError();
    int64_t g = (ng + kFusedThreads - 1) / kFusedThreads;
    const int64_t cap = int64_t(nsm) * 8;
    if (g > cap) g = cap;
    return launch_dependent(N >= kDependentMinN, cic ? k_fused_global<1> : k_fused_global<0>, dim3(unsigned(g)),
                            dim3(kFusedThreads), 0, st, p, ng, force, rho, N, dt);
}

}  // namespace cpm
