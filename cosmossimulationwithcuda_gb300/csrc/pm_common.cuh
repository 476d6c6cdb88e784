// Shared device/host helpers of the cosmos_pm library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/cosmos_pm.h"

namespace cpm {

// ---- complex helpers, float2 / double2 ---------------------------------------
template <class T>
struct Cplx;
template <>
struct Cplx<float> {
    using type = float2;
};
template <>
struct Cplx<double> {
    using type = double2;
};
template <class T>
using cplx_t = typename Cplx<T>::type;

template <class C>
__device__ __forceinline__ C cmake(decltype(C{}.x) re, decltype(C{}.x) im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}
template <class C>
__device__ __forceinline__ C cadd(C a, C b) {
    return cmake<C>(a.x + b.x, a.y + b.y);
}
template <class C>
__device__ __forceinline__ C csub(C a, C b) {
    return cmake<C>(a.x - b.x, a.y - b.y);
}
template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
    return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class C>
__device__ __forceinline__ C cconj(C a) {
    return cmake<C>(a.x, -a.y);
}
template <class C>
__device__ __forceinline__ C cscale(C a, decltype(C{}.x) s) {
    return cmake<C>(a.x * s, a.y * s);
}

// Multiply by -i (DIR < 0) or +i (DIR > 0).
template <int DIR, class C>
__device__ __forceinline__ C cmul_i(C a) {
    return DIR < 0 ? cmake<C>(a.y, -a.x) : cmake<C>(-a.y, a.x);
}

// ---- Morton code of the cell (sort key) ---------------------------------------
__host__ __device__ __forceinline__ uint32_t spread_bits16(uint32_t v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// The reference's active window (CosmosCuda.cuh:497, :257): the cell of a
// particle (C truncation) must lie in [1, N-1) on both axes.
__host__ __device__ __forceinline__ bool active_cell(int cx, int cy, int N) {
    return cx >= 1 && cx < N - 1 && cy >= 1 && cy < N - 1;
}

__device__ __forceinline__ uint32_t tile_key(float x, float y, int N, int gran) {
    const int cx = int(x), cy = int(y);
    const uint32_t t = uint32_t(N) >> gran;
    if (!active_cell(cx, cy, N)) return t * t;
    return spread_bits16(uint32_t(cx) >> gran) | (spread_bits16(uint32_t(cy) >> gran) << 1);
}

inline int ilog2(int64_t v) {
    int l = 0;
    while ((int64_t(1) << l) < v) ++l;
    return l;
}

// ---- programmatic dependent launch ------------------------------------------------
// A kernel launched as a dependent may start while the kernel before it in
// the stream (or graph) finishes: its CTAs are placed as soon as the previous
// kernel's CTAs have all started and SM room frees up, and they block in
// dependency_wait() until that kernel has completed and its memory is
// visible.  Kernels call dependency_wait() before their first global access,
// so only the launch and CTA placement overlap; allow_dependents() lets the
// next kernel be placed before this one ends.  Without the launch attribute
// both are no-ops.  Measured per step: -6 us at 2048^2 (five kernels of 512
// to 1024 CTAs), +2.4 us at 512^2 (kernels of 128 CTAs), hence the lattice
// size from which the step's kernels launch as dependents.
constexpr int kDependentMinN = 1024;
__device__ __forceinline__ void dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
inline cudaError_t launch_dependent(bool dependent, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                    cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = dependent ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace cpm

// ---- host error plumbing ---------------------------------------------------------
#define CPM_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            return ::cpm::fail(COSMOS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                               \
    } while (0)

#define CPM_TRY(expr)              \
    do {                           \
        int s_ = (expr);           \
        if (s_ != COSMOS_OK) return s_; \
    } while (0)

namespace cpm {
// Records the message in a thread-local slot and returns the code.
int fail(int code, const std::string& msg);
const char* last_error_message();
}  // namespace cpm
