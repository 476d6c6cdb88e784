// Host-side launchers shared between the translation units of cosmos_pm.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cpm {

// pm_fft.cu
cudaError_t prepare_conv_passes(int N);
cudaError_t launch_conv_passes(int N, const float* rho, float2* spec, const float* kq, float* phi, const float2* tw,
                               cudaStream_t st);
int conv_launches_per_step();
int build_filter(int N, int cic, float* kq_dev, float2* tw_dev, cudaStream_t st);

// pm_particles.cu
struct ParticleArrays {
    float* x;
    float* y;
    float* xo;
    float* yo;
    float* m;
    uint32_t* id;
};

cudaError_t launch_deposit_global(const ParticleArrays& p, int64_t P, float* rho, int N, int cic, int nsm,
                                  cudaStream_t st);
cudaError_t launch_gradient(const float* phi, float2* force, int N, float gmult, cudaStream_t st);
cudaError_t launch_integrate(const float2* force, const ParticleArrays& p, int64_t P, int N, int cic, float dt,
                             int nsm, cudaStream_t st);
cudaError_t launch_tile_keys(const float* x, const float* y, int64_t P, int N, int gran, uint32_t* keys,
                             cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits of the key.
struct RadixScratch {
    uint32_t* keys[2];
    uint32_t* vals[2];
    uint32_t* counts;  // 256 * grid
    int grid;
};
size_t radix_counts_elems(int grid);
int radix_grid(int64_t n, int nsm);
// Sorts (keys[0], vals[0]) in place-ish; returns which buffer (0/1) holds the result.
cudaError_t launch_radix_sort(RadixScratch& s, int64_t n, int bits, int* result_buf, cudaStream_t st);

cudaError_t launch_iota(uint32_t* v, int64_t n, cudaStream_t st);
// dst.f[i] = src.f[perm[i]] for every array of the particle state.
cudaError_t launch_permute(const ParticleArrays& src, const ParticleArrays& dst, const uint32_t* perm, int64_t n,
                           cudaStream_t st);
// pos[id[s]] = s
cudaError_t launch_invert(const uint32_t* id, uint32_t* pos, int64_t n, cudaStream_t st);
// out[i] = in[pos[offset + i]] for i < count (gather by identity)
cudaError_t launch_gather_by_id(const float* in, const uint32_t* pos, int64_t offset, int64_t count, float* out,
                                cudaStream_t st);
// out[pos[offset + i]] = in[i] (scatter by identity)
cudaError_t launch_scatter_by_id(const float* in, const uint32_t* pos, int64_t offset, int64_t count, float* out,
                                 cudaStream_t st);
// out[id[s]] = in[s] for s < n (identity order from internal order)
cudaError_t launch_unpermute(const float* in, const uint32_t* id, int64_t n, float* out, cudaStream_t st);
cudaError_t launch_fill(float* v, float value, int64_t n, cudaStream_t st);

// FP64 diagnostics: out[0] = sum m v^2 / 2, out[1] = sum m phi / 2, out[2..3] = sum m v
cudaError_t launch_diagnostics(const ParticleArrays& p, int64_t P, const float* phi, int N, float dt, double* out,
                               cudaStream_t st);

}  // namespace cpm
