// Per-particle arithmetic of the step, shared by every kernel that gathers,
// updates or deposits, so that all paths produce identical bits.
//
// Reference (CosmosCuda.cuh):
//   weights  (1-fx)(1-fy), fx(1-fy), (1-fx)fy, fx fy   deposit :498-511, gather :267-278
//   update   x' = (2x - xOld) + dt*F*dt                  :286-287
//   wrap     x' < 2 -> += N-4 ; x' > N-2 -> -= N-4       :288-299
//   history  xOld' = x (pre-step, unwrapped)             :300-303
// The operation order is pinned with explicit intrinsics and mirrored by the
// FP32 oracle (oracle/cpu_pm.cpp, integrate_f32_exact).
#pragma once

#include "pm_common.cuh"

namespace cpm {

struct CicWeights {
    float w00, w10, w01, w11;
};

__device__ __forceinline__ CicWeights cic_weights(float px, float py, int cx, int cy) {
    const float fx = __fsub_rn(px, float(cx)), fy = __fsub_rn(py, float(cy));
    const float x1 = __fsub_rn(1.0f, fx), y1 = __fsub_rn(1.0f, fy);
    return {__fmul_rn(x1, y1), __fmul_rn(fx, y1), __fmul_rn(x1, fy), __fmul_rn(fx, fy)};
}

// F = fma(f11, w11, fma(f01, w01, fma(f10, w10, f00 * w00)))
__device__ __forceinline__ float2 bilinear(const CicWeights& w, float2 f00, float2 f10, float2 f01, float2 f11) {
    return make_float2(
        __fmaf_rn(f11.x, w.w11, __fmaf_rn(f01.x, w.w01, __fmaf_rn(f10.x, w.w10, __fmul_rn(f00.x, w.w00)))),
        __fmaf_rn(f11.y, w.w11, __fmaf_rn(f01.y, w.w01, __fmaf_rn(f10.y, w.w10, __fmul_rn(f00.y, w.w00)))));
}

// x' = fma(dt*F, dt, fma(2, x, -xOld)), then the reference wrap; xOld' = x.
__device__ __forceinline__ void verlet_wrap(float& px, float& py, float& pxo, float& pyo, float2 F, float dt, int N) {
    float nx = __fmaf_rn(__fmul_rn(dt, F.x), dt, __fmaf_rn(2.0f, px, -pxo));
    float ny = __fmaf_rn(__fmul_rn(dt, F.y), dt, __fmaf_rn(2.0f, py, -pyo));
    const float span = float(N) - 4.0f, hi = float(N) - 2.0f;
    if (nx < 2.0f) nx = __fadd_rn(nx, span);
    if (ny < 2.0f) ny = __fadd_rn(ny, span);
    if (nx > hi) nx = __fsub_rn(nx, span);
    if (ny > hi) ny = __fsub_rn(ny, span);
    pxo = px;
    pyo = py;
    px = nx;
    py = ny;
}

// The reference's 4th-order difference (CosmosCuda.cuh:183-226) with the
// operation order pinned: ((8r - rr) - 8l + ll) / 12 * g.  Out-of-range
// neighbours (outside [0, N)) are replaced by the centre value by the caller.
__device__ __forceinline__ float diff4(float ll, float l, float r, float rr, float g) {
    float t = __fmaf_rn(8.0f, r, -rr);
    t = __fmaf_rn(-8.0f, l, t);
    t = __fadd_rn(t, ll);
    return __fmul_rn(__fdiv_rn(t, 12.0f), g);
}

// Vector reduction of two floats into global memory (8-byte aligned address), sm_90+.
__device__ __forceinline__ void red_add_v2(float* addr, float a, float b) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(a), "f"(b) : "memory");
}

// Vector reduction into global memory (16-byte aligned address), sm_90+.
__device__ __forceinline__ void red_add_v4(float* addr, float4 v) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}

}  // namespace cpm
