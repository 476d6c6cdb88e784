// Render frame of the density, the reference's display chain as two kernels.
//
// Reference chain (CosmosCuda.cuh:1249-1256, run once per frame):
//   k_getRealComponentOfLattice  density lattice -> float frame      (:613-628)
//   k_calcBlurConvolution        BLUR_R x BLUR_R blur, zero outside   (:773-828),
//                                weights 1/(r+1) for r < (BLUR_R-1)/2, else 0 (:954-966)
//   k_resetMinMax, k_calcMinMax  frame min / max                      (:630-743)
//   k_smoothMinMax               running extremes across frames       (:744-755)
//   k_scaleWithMinMax            1.8 * ((v - min) / (max - min))^0.25  (:756-772)
// Kept semantics of the min / max pass: the maximum starts at FLT_MIN (not
// -FLT_MAX), and the reference's block reduction pads the lanes past its 24
// warps with 0.0, so the frame minimum is min(true minimum, 0) and the frame
// maximum max(true maximum, 0, FLT_MIN).  The running extremes start at
// (1e35, -1) (k_initSmoothMinMax, :744-747).
//
// Here: k_render_blur_minmax blurs a 32x32 tile per CTA from a shared-memory
// halo tile and reduces the tile's extremes into order-preserving integer keys
// with one atomic pair per CTA; the last CTA to finish folds them into the
// running extremes and re-arms the keys.  k_render_scale applies the power law.
// When the weight table is the identity (the default BLUR_R = 3: only the
// centre weight is nonzero) the blurred lattice equals the density, so
// k_render_minmax takes the extremes of the density and the blur is skipped.
#include <cfloat>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace cpm {

namespace {

constexpr int kTile = 32;

// Monotone float <-> uint32 key (for integer atomicMin / atomicMax).
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float funkey(uint32_t k) {
    return (k & 0x80000000u) ? __uint_as_float(k & 0x7FFFFFFFu) : __uint_as_float(~k);
}

}  // namespace

// Fold a CTA's (lo, hi) into the frame extremes: one atomic pair per CTA on
// order-preserving integer keys; the last CTA to finish folds the frame's
// extremes into the running extremes (k_smoothMinMax) and re-arms the keys.
// state: [0] min key, [1] max key, [2] finished-CTA counter (uint32);
// extremes: [0] running min, [1] running max (float).
__device__ __forceinline__ void fold_extremes(float lo, float hi, uint32_t* __restrict__ state,
                                              float* __restrict__ extremes) {
    for (int off = 16; off > 0; off >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    __shared__ float wlo[32], whi[32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) {
        wlo[threadIdx.x >> 5] = lo;
        whi[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < int(blockDim.x >> 5); ++w) {
            lo = fminf(lo, wlo[w]);
            hi = fmaxf(hi, whi[w]);
        }
        atomicMin(state + 0, fkey(lo));
        atomicMax(state + 1, fkey(hi));
        __threadfence();
        const uint32_t done = atomicAdd(state + 2, 1u);
        last = done == gridDim.x * gridDim.y - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const float fmin = funkey(atomicAdd(state + 0, 0u));
        const float fmax = funkey(atomicAdd(state + 1, 0u));
        if (extremes[0] > fmin) extremes[0] = fmin;  // k_smoothMinMax
        if (extremes[1] < fmax) extremes[1] = fmax;
        state[0] = 0xFFFFFFFFu;
        state[1] = 0u;
        state[2] = 0u;
    }
}

// Blur with an R x R weight table, one 32 x 32 tile per CTA from a shared
// halo tile, and the tile's extremes.
__global__ void __launch_bounds__(256) k_render_blur_minmax(const float* __restrict__ rho, float* __restrict__ blurred,
                                                            const float* __restrict__ kern, int R, int N, int T,
                                                            uint32_t* __restrict__ state, float* __restrict__ extremes) {
    extern __shared__ float tile[];
    __shared__ float wk[15 * 15];
    const int h = (R - 1) / 2;
    const int TW = T + 2 * h;
    const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
    for (int i = threadIdx.x; i < R * R; i += blockDim.x) wk[i] = __ldg(kern + i);
    for (int i = threadIdx.x; i < TW * TW; i += blockDim.x) {
        const int r = i / TW, c = i - r * TW;
        const int gx = x0 + c - h, gy = y0 + r - h;
        tile[i] = (gx >= 0 && gx < N && gy >= 0 && gy < N) ? __ldg(rho + size_t(gy) * N + gx) : 0.0f;
    }
    __syncthreads();
    float lo = 0.0f, hi = FLT_MIN;  // the reference's padding and initial maximum
    for (int i = threadIdx.x; i < T * T; i += blockDim.x) {
        const int ty = i / T, tx = i - ty * T;
        // two partial sums by column parity, rows outer: the reference's order
        float a0 = 0.0f, a1 = 0.0f;
        for (int iy = 0; iy < R; ++iy) {
            const float* row = tile + (ty + iy) * TW + tx;
            const float* kr = wk + iy * R;
            for (int ix = 0; ix < R; ix += 2) a0 = fmaf(row[ix], kr[ix], a0);
            for (int ix = 1; ix < R; ix += 2) a1 = fmaf(row[ix], kr[ix], a1);
        }
        const float acc = a0 + a1;
        blurred[size_t(y0 + ty) * N + x0 + tx] = acc;
        lo = fminf(lo, acc);
        hi = fmaxf(hi, acc);
    }
    fold_extremes(lo, hi, state, extremes);
}

// Extremes of an unblurred lattice (the weight table is the identity: with
// the default BLUR_R = 3 only the centre weight, 1, is nonzero, and the
// reference's sum 0 + x * 1 + sum of x * 0 is x itself).
__global__ void __launch_bounds__(512) k_render_minmax(const float4* __restrict__ src, int64_t n4,
                                                       uint32_t* __restrict__ state, float* __restrict__ extremes) {
    float lo = 0.0f, hi = FLT_MIN;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += int64_t(gridDim.x) * blockDim.x) {
        const float4 v = __ldg(src + i);
        lo = fminf(lo, fminf(fminf(v.x, v.y), fminf(v.z, v.w)));
        hi = fmaxf(hi, fmaxf(fmaxf(v.x, v.y), fmaxf(v.z, v.w)));
    }
    fold_extremes(lo, hi, state, extremes);
}

__global__ void k_render_scale(const float4* __restrict__ src, float4* __restrict__ frame,
                               const float* __restrict__ extremes, int64_t n4) {
    const float lo = extremes[0], hi = extremes[1];
    const float diff = hi - lo;
    // The reference is built with fast math, which turns its x / y and powf
    // into these two intrinsics.
    auto f = [lo, diff](float v) { return 1.8f * __powf(__fdividef(v - lo, diff), 0.25f); };
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n4; i += int64_t(gridDim.x) * blockDim.x) {
        const float4 v = __ldg(src + i);
        frame[i] = make_float4(f(v.x), f(v.y), f(v.z), f(v.w));
    }
}

// Blur weights of the reference (double r, float weight) for an odd R.
void render_weights(int R, float* w) {
    const int h = (R - 1) / 2;
    for (int iy = -h; iy <= h; ++iy)
        for (int ix = -h; ix <= h; ++ix) {
            const double r = sqrt(double(ix * ix + iy * iy));
            w[(ix + h) + (iy + h) * R] = r < h ? float(1.0 / (r + 1.0)) : 0.0f;
        }
}

cudaError_t render_init(uint32_t* state, float* extremes, cudaStream_t st) {
    const uint32_t s0[3] = {0xFFFFFFFFu, 0u, 0u};
    const float e0[2] = {1e35f, -1.0f};
    cudaError_t e = cudaMemcpyAsync(state, s0, sizeof(s0), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(extremes, e0, sizeof(e0), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

bool render_is_identity(int R, const float* w) {
    const int c = (R / 2) * R + R / 2;
    for (int i = 0; i < R * R; ++i)
        if (w[i] != (i == c ? 1.0f : 0.0f)) return false;
    return true;
}

cudaError_t launch_render(const float* rho, float* blurred, float* frame, const float* kern, int R, int N,
                          bool identity, uint32_t* state, float* extremes, cudaStream_t st) {
    const int64_t n4 = int64_t(N) * N / 4;
    const float* src = rho;
    if (identity) {
        int64_t g = (n4 + 511) / 512;
        if (g > 608) g = 608;
        k_render_minmax<<<int(g), 512, 0, st>>>(reinterpret_cast<const float4*>(rho), n4, state, extremes);
    } else {
        const int h = (R - 1) / 2;
        const int T = N < kTile ? N : kTile;  // N is a power of two
        const size_t smem = size_t(T + 2 * h) * (T + 2 * h) * sizeof(float);
        k_render_blur_minmax<<<dim3(N / T, N / T), 256, smem, st>>>(rho, blurred, kern, R, N, T, state, extremes);
        src = blurred;
    }
    int64_t g = (n4 + 255) / 256;
    if (g > 2432) g = 2432;
    k_render_scale<<<int(g), 256, 0, st>>>(reinterpret_cast<const float4*>(src), reinterpret_cast<float4*>(frame),
                                          extremes, n4);
    return cudaGetLastError();
}

}  // namespace cpm
