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

// state: [0] min key, [1] max key, [2] finished-CTA counter (uint32);
// extremes: [0] running min, [1] running max (float)
__global__ void __launch_bounds__(256) k_render_blur_minmax(const float* __restrict__ rho, float* __restrict__ blurred,
                                                            const float* __restrict__ kern, int R, int N, int T,
                                                            uint32_t* __restrict__ state, float* __restrict__ extremes) {
    extern __shared__ float tile[];
    const int h = (R - 1) / 2;
    const int TW = T + 2 * h;
    const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
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
            const float* kr = kern + iy * R;
            for (int ix = 0; ix < R; ix += 2) a0 = fmaf(row[ix], __ldg(kr + ix), a0);
            for (int ix = 1; ix < R; ix += 2) a1 = fmaf(row[ix], __ldg(kr + ix), a1);
        }
        const float acc = a0 + a1;
        blurred[size_t(y0 + ty) * N + x0 + tx] = acc;
        lo = fminf(lo, acc);
        hi = fmaxf(hi, acc);
    }
    for (int off = 16; off > 0; off >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    __shared__ float wlo[8], whi[8];
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

__global__ void k_render_scale(const float* __restrict__ blurred, float* __restrict__ frame,
                               const float* __restrict__ extremes, int64_t n) {
    const float lo = extremes[0], hi = extremes[1];
    const float diff = hi - lo;
    // The reference is built with fast math, which turns its x / y and powf
    // into these two intrinsics.
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        frame[i] = 1.8f * __powf(__fdividef(blurred[i] - lo, diff), 0.25f);
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

cudaError_t launch_render(const float* rho, float* blurred, float* frame, const float* kern, int R, int N,
                          uint32_t* state, float* extremes, cudaStream_t st) {
    const int h = (R - 1) / 2;
    const int T = N < kTile ? N : kTile;  // N is a power of two
    const size_t smem = size_t(T + 2 * h) * (T + 2 * h) * sizeof(float);
    k_render_blur_minmax<<<dim3(N / T, N / T), 256, smem, st>>>(rho, blurred, kern, R, N, T, state, extremes);
    const int64_t n = int64_t(N) * N;
    int64_t g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    k_render_scale<<<int(g), 256, 0, st>>>(blurred, frame, extremes, n);
    return cudaGetLastError();
}

}  // namespace cpm
