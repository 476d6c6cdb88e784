// Host-side launchers shared between the translation units of cosmos_pm.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cpm {

// pm_fft.cu
cudaError_t prepare_conv_passes(int N);
// batch: lattices of size N stored back to back, processed in one launch per pass
// clear: when not null (the density itself), the row pass zeroes each density
// row after reading it, ready for the next step's deposit.
cudaError_t launch_conv_passes(int N, const float* rho, float2* spec, const float* kq, float* phi, const float2* tw,
                               cudaStream_t st, int batch = 1, float* clear = nullptr);
int conv_launches_per_step();
int build_filter(int N, int cic, float* kq_dev, float2* tw_dev, cudaStream_t st);
// Spectral force: density -> force field (interleaved fx, fy) with the
// reference's clamped-edge stencil applied in Fourier space.  spec2: N*N/2
// float2; edge: (N/2)*4 float2; dy: 3*N float.
cudaError_t prepare_spectral_passes(int N);
// Tensor-core column pass (pm_fft_tc.cu): split-precision DFT stages.
struct SpectralTc {
    int bf16;         // 1: BF16 split, 0: FP16 split
    const void* dft;  // DFT matrix image (tc_dft_bytes(N) bytes, prepare_tc_columns)
    int* status;      // set to 1 when an MMA completion wait timed out
    int skip_mma;     // test hook: issue no MMA and no completion signal (the waits run out)
};
bool tc_fft_supported(int N);
size_t tc_dft_bytes(int N);
cudaError_t prepare_tc_columns(int N, int bf16, void* dft_dev, cudaStream_t st);
cudaError_t launch_cols_spectral_tc(int N, int bf16, float2* spec, float2* spec2, float2* edge, const float* kq,
                                    const float2* tw, const void* dft_dev, float g, int* status, int skip_mma,
                                    int batch, cudaStream_t st);
// pm_tma.cu: a row map (tma.cuh) of `rows` rows of `rowlen` floats for each
// of `batch` lattices stored back to back, loaded in boxes of `box_rows` rows.
cudaError_t make_row_map(CUtensorMap* map, const void* base, int rowlen, int rows, int batch, int box_rows);
// The row maps the spectral force's row and column passes load their tiles
// through: the density (rows of N floats) and the half spectrum's column lines
// (lines of N complex).  make_spectral_maps: cudaErrorNotSupported below
// 256^2 (those lattices keep per-thread loads).
struct SpectralMaps {
    CUtensorMap rho;
    CUtensorMap spec;
};
cudaError_t make_spectral_maps(int N, const float* rho, const float2* spec, int batch, SpectralMaps* maps);
// Test hook of the device allocations: true when this allocation must fail.
bool alloc_should_fail();
// edge: the column pass's y-edge sums (N/2 x 4 complex per lattice), which the
// C2R row pass adds to the Fy spectra of rows 0, 1, N-2, N-1;
// tc: the tensor-core column pass instead of the FP32 one (nullptr: FP32);
// maps + status: the row and column passes load their tiles through the
// tensor maps (from 256^2 up), and a load wait that runs out sets *status.
cudaError_t launch_spectral_force(int N, const float* rho, float2* spec, float2* spec2, float2* edge, const float* kq,
                                  float2* force, const float2* tw, float g, cudaStream_t st, int batch = 1,
                                  const SpectralTc* tc = nullptr, float* clear = nullptr,
                                  const SpectralMaps* maps = nullptr, int* status = nullptr, int col_shape = 0);
int spectral_launches_per_step();

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
cudaError_t launch_gradient(const float* phi, float2* force, int N, float gmult, cudaStream_t st, int batch = 1);
cudaError_t launch_integrate(const float2* force, const ParticleArrays& p, int64_t P, int N, int cic, float dt,
                             int nsm, cudaStream_t st);
cudaError_t launch_tile_keys(const float* x, const float* y, int64_t P, int N, int gran, uint32_t* keys,
                             cudaStream_t st);
// Ensemble keys: sim * (T^2 + 1) + tile key, slots [sim_off[s], sim_off[s+1]) in sim s.
cudaError_t launch_tile_keys_sims(const float* x, const float* y, int64_t P, int N, int gran, const int64_t* sim_off,
                                  int nsims, uint32_t* keys, cudaStream_t st);

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

// pm_tiles.cu -- tile-ordered fused gather + update + next-step deposit
#ifndef CPM_TILE_HALO
#define CPM_TILE_HALO 4
#endif
constexpr int kTileHalo = CPM_TILE_HALO;  // cells of drift tolerated around a tile's window
// Window origins stay on 4-cell boundaries (16-byte vector flushes of the density).
static_assert(kTileHalo % 4 == 0, "tile halo must be a multiple of 4 cells");
#ifndef CPM_ITEM_MAX
#define CPM_ITEM_MAX 8192
#endif
constexpr int kItemMax = CPM_ITEM_MAX;  // particles per work item, at most
constexpr int kItemMin = 2048;          // and at least (below the largest size)
#ifndef CPM_ITEM_DIRECT
#define CPM_ITEM_DIRECT 256
#endif
constexpr int kItemDirect = CPM_ITEM_DIRECT;  // items with fewer particles skip the shared windows
struct WorkItem {
    int x0, y0;           // window origin (cells): tile origin - kTileHalo
    uint32_t begin, end;  // slot range
    float scale;          // fixed-point scale of the deposit window (a power of two)
    float inv_scale;      // 1 / scale
    float heavy;          // particles heavier than this deposit with global float atomics
    uint32_t sim;         // lattice index within an ensemble (0 for one simulation)
};
// Elements of the tile-range arrays (tstart / tend) for nsims simulations.
size_t tile_range_elems(int N, int gran, int nsims);
size_t tile_window_smem(int gran, int cic);
// Work-item size for Pq particles: the largest of kItemMax, kItemMax / 2, ...
// that still gives about four items per resident CTA (16 per SM), so that the
// items of a smaller state still spread over the GPU; kItemMin below that.
int work_item_size(int64_t Pq, int nsm);
size_t max_work_items(int64_t Pq, int ntiles, int item_size);
cudaError_t prepare_tile_kernels(int gran, int cic, int nsm, int* grid);
// Builds the work items of the sorted state and their deposit scales (the
// masses of the sorted particles are read from `m`).
cudaError_t launch_build_items(const uint32_t* sorted_keys, const float* m, int64_t Pq, int N, int gran,
                               uint32_t* tstart, uint32_t* tend, WorkItem* items, uint32_t* n_items, size_t max_items,
                               int item_size, cudaStream_t st, int nsims = 1);
// status: a bounded wait of the kernel that ran out sets *status (1: a wait
// timed out; 2: copies were still in flight when the CTA gave up).
// tx_extra: test hook (0 in normal use): bytes announced per copy stage that
// never arrive, so the copy waits run out.
cudaError_t launch_fused_tiles(const WorkItem* items, const uint32_t* n_items, const ParticleArrays& p,
                               const float2* force, float* rho, int N, int cic, float dt, int gran, int grid,
                               int* status, cudaStream_t st, uint32_t tx_extra = 0);
cudaError_t launch_fused_global(const ParticleArrays& p, int64_t P, const float2* force, float* rho, int N, int cic,
                                float dt, int nsm, cudaStream_t st);

// pm_ensemble_step.cu -- the ensemble step as one persistent cooperative launch
constexpr int kEnsMaxClasses = 8;
struct EnsStepClass {  // one lattice class: nsims lattices of size N stored back to back
    int N, nsims;
    float* rho;
    float2 *spec, *spec2, *edge;
    const float* kq;
    float2* force;
    const float2* tw;
    const WorkItem* items;
    const uint32_t* n_items;
    ParticleArrays p;  // the class's current particle buffer
};
struct EnsStepArgs {
    int nclasses, cic;
    float g, dt;
    unsigned* barrier;  // grid-barrier arrival counter (zeroed by the launcher)
    int* status;        // 4: a grid barrier ran out of time
    int skip_arrive;    // test hook: CTA 0 does not arrive at the first barrier
    EnsStepClass cls[kEnsMaxClasses];
};
bool ensemble_step_supported(int N);
cudaError_t prepare_ensemble_step(int nsm, int* grid);
// args_dev: the step's arguments in device memory (read by every CTA);
// barrier: args_dev->barrier, zeroed on the stream before the launch.
cudaError_t launch_ensemble_step(const EnsStepArgs* args_dev, unsigned* barrier, int grid, cudaStream_t st);

// pm_ics.cu -- seeded initial conditions; particle i draws from (seed, first + i)
cudaError_t launch_generate(const cosmos_ic_params& p, int64_t count, int64_t first, int N, float dt, float* x,
                            float* y, float* xo, float* yo, float* m, cudaStream_t st);

// pm_render.cu -- display frame of the density (the reference's render chain)
void render_weights(int R, float* w);
bool render_is_identity(int R, const float* w);
cudaError_t render_init(uint32_t* state, float* extremes, cudaStream_t st);
cudaError_t launch_render(const float* rho, float* blurred, float* frame, const float* kern, int R, int N,
                          bool identity, uint32_t* state, float* extremes, cudaStream_t st);

}  // namespace cpm
