// The ensemble step as ONE persistent launch.
//
// The graph form of the ensemble step (pm_ensemble.cu) launches every pass of
// every lattice class as its own kernel node.  Here a single cooperative
// kernel, one CTA per resident slot, runs the whole step of all classes in
// four phases separated by grid-wide barriers:
//   phase 0  row R2C of every density lattice (zeroing each row behind it for
//            the deposit of phase 3)
//   phase 1  spectral column pass (forward FFT x K, y-edge sums, the two
//            inverse transforms) of every half-spectrum line block
//   phase 2  spectral C2R row pass of every row block (the y-edge sums enter
//            the Fy spectra of rows 0, 1, N-2, N-1)
//   phase 3  tile-ordered fused gather + update + deposit of every work item
// A phase's units (row blocks, line blocks, work items) of all classes are
// numbered consecutively and dealt to the CTAs round-robin.  The bodies are
// the ones of the per-pass kernels (fft_passes.cuh, tile_step.cuh), so each
// simulation takes the same step as in the graph form.
//
// Grid barrier: an arrival counter, zeroed before the launch, that every CTA
// increments once per barrier (release fence first) and then polls until all
// CTAs have arrived.  The poll is bounded in wall time (globaltimer) and in
// iterations; a barrier that runs out sets *status = 4 and the CTA returns, so
// every other CTA runs out at its next barrier and the launch ends with the
// status recorded instead of hanging.  A cooperative launch guarantees that
// all CTAs are resident, so a barrier that does not run out is complete.
//
// Supported lattice sizes: 128 to 1024 (one butterfly per thread in every
// FFT phase with 256 threads); other sizes keep the graph form.
#include "fft_passes.cuh"
#include "tile_step.cuh"

namespace cpm {

namespace {

constexpr int kEnsThreads = 256;  // = kFusedThreads (the fused-item body's stride)
static_assert(kEnsThreads == kFusedThreads, "fused-item body stride");
constexpr int kEnsGran = 5;       // tile edge of the classes the persistent step serves (N >= 64)

// Units per phase and lattice size, and the shared memory each body needs.
template <int N>
struct EnsShape {
    static constexpr int M = N / 2;
    static constexpr int RB = 4096 / M;    // R2C rows per unit: 4096 points
    static constexpr int CB = 2048 / N;    // column lines per unit
    static constexpr int QB = N >= 1024 ? 4 : 8;  // spectral C2R rows per unit
    static constexpr size_t r2c_smem = size_t(RB) * LinePad<M>::value * sizeof(float2);
    static constexpr size_t col_smem = 2 * size_t(CB) * LinePad<N>::value * sizeof(float2) + (kEnsThreads / 32) * 6 * 4;
    static constexpr size_t c2r_smem =
        size_t(QB) * LinePad<N>::value * sizeof(float2) + (kEnsThreads / 32) * 3 * QB * 4 + 3 * QB * 4;
    static constexpr size_t smem = r2c_smem > col_smem ? (r2c_smem > c2r_smem ? r2c_smem : c2r_smem)
                                                        : (col_smem > c2r_smem ? col_smem : c2r_smem);
};
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kEnsSmem =
    cmax(cmax(cmax(EnsShape<128>::smem, EnsShape<256>::smem), cmax(EnsShape<512>::smem, EnsShape<1024>::smem)),
         cmax(window_bytes(kEnsGran, 0), window_bytes(kEnsGran, 1)));

__device__ __forceinline__ uint64_t gtimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded grid barrier number `k` (0-based); false when it ran out.
__device__ __forceinline__ bool grid_barrier(unsigned* count, int k, int* status, bool skip_arrive) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (!skip_arrive) atomicAdd(count, 1u);
        const unsigned target = unsigned(k + 1) * gridDim.x;
        const uint64_t t0 = gtimer_ns();
        int good = 1;
        for (int it = 0;; ++it) {
            if (*reinterpret_cast<volatile unsigned*>(count) >= target) break;
            if (it > (1 << 24) || gtimer_ns() - t0 > 500000000ull) {
                good = 0;
                atomicMax(status, 4);
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <int N>
__device__ __forceinline__ int units_r2c(const EnsStepClass& c) { return c.nsims * (N / EnsShape<N>::RB); }
template <int N>
__device__ __forceinline__ int units_col(const EnsStepClass& c) { return c.nsims * ((N / 2) / EnsShape<N>::CB); }
template <int N>
__device__ __forceinline__ int units_c2r(const EnsStepClass& c) { return c.nsims * (N / EnsShape<N>::QB); }

template <int N>
__device__ __noinline__ void do_r2c(const EnsStepClass& c, int u, float2* s) {
    using S = EnsShape<N>;
    constexpr int per = N / S::RB;
    const int lat = u / per, y0 = (u - lat * per) * S::RB;
    const float* rho = c.rho + size_t(lat) * N * N;
    const float2* rows = reinterpret_cast<const float2*>(rho + size_t(y0) * N);
    auto src = [rows](int line, int i) { return rows[line * S::M + i]; };
    r2c_rows<float, N, S::RB, kEnsThreads>(src, s, c.spec + size_t(lat) * S::M * N, c.tw, c.rho + size_t(lat) * N * N,
                                           y0);
    __syncthreads();  // the shared lines are reused by the next unit
}

template <int N>
__device__ __noinline__ void do_col(const EnsStepClass& c, float g, int u, float2* s) {
    using S = EnsShape<N>;
    constexpr int per = S::M / S::CB;
    const int lat = u / per, kx0 = (u - lat * per) * S::CB;
    float2* spec = c.spec + size_t(lat) * S::M * N;
    float2* lines = spec + size_t(kx0) * N;
    auto gload = [lines](int line, int i) { return lines[size_t(line) * N + i]; };
    cols_spectral_lines<N, S::CB, kEnsThreads>(gload, s, lines, c.spec2 + size_t(lat) * S::M * N + size_t(kx0) * N,
                                               c.edge + size_t(lat) * S::M * 4, c.kq, c.tw, g, kx0);
    __syncthreads();
}

template <int N>
__device__ __noinline__ void do_c2r(const EnsStepClass& c, float g, int u, float2* s) {
    using S = EnsShape<N>;
    constexpr int per = N / S::QB;
    const int lat = u / per, r = u - lat * per;
    float* dx = reinterpret_cast<float*>(s + S::QB * LinePad<N>::value) + (kEnsThreads / 32) * 3 * S::QB;
    const size_t off = size_t(lat) * S::M * N;
    c2r_spectral_rows<N, S::QB, kEnsThreads>(s, dx, c.spec + off, c.spec2 + off, c.edge + size_t(lat) * S::M * 4,
                                             reinterpret_cast<float4*>(c.force) + off, c.tw, g, r * S::QB);
    __syncthreads();
}

#define CPM_ENS_DISPATCH(N_, CALL) \
    switch (N_) {                  \
        case 128: CALL(128); break; \
        case 256: CALL(256); break; \
        case 512: CALL(512); break; \
        case 1024: CALL(1024); break; \
        default: break;            \
    }

template <int N>
__device__ __forceinline__ int units_of(const EnsStepClass& c, int phase) {
    return phase == 0 ? units_r2c<N>(c) : phase == 1 ? units_col<N>(c) : units_c2r<N>(c);
}

__device__ __forceinline__ int phase_units(const EnsStepClass& c, int phase) {
    int n = 0;
#define CPM_U(n_) n = units_of<n_>(c, phase)
    CPM_ENS_DISPATCH(c.N, CPM_U)
#undef CPM_U
    return n;
}

// Runs unit `u` of class `c` in FFT phase `phase`.
__device__ __forceinline__ void run_unit(const EnsStepClass& c, int phase, int u, float g, float2* s) {
#define CPM_R(n_)                                  \
    if (phase == 0) do_r2c<n_>(c, u, s);           \
    else if (phase == 1) do_col<n_>(c, g, u, s);   \
    else do_c2r<n_>(c, g, u, s);
    CPM_ENS_DISPATCH(c.N, CPM_R)
#undef CPM_R
}

// The phases, and the FFT bodies of each lattice size, are separate
// non-inlined functions so that each gets its own register allocation
// (inlined into one body they exceeded the 128 registers of two CTAs per SM
// together and spilled).
__device__ __noinline__ void fft_phase(const EnsStepArgs& a, int phase, float2* s) {
    int base = 0;
    for (int ci = 0; ci < a.nclasses; ++ci) {
        const EnsStepClass& c = a.cls[ci];
        const int n = phase_units(c, phase);
        // this CTA's units of the class: global unit ids base .. base + n - 1
        int u = int(blockIdx.x) - base;
        if (u < 0) u += ((-u + int(gridDim.x) - 1) / int(gridDim.x)) * int(gridDim.x);
        for (; u < n; u += int(gridDim.x)) run_unit(c, phase, u, a.g, s);
        base += n;
    }
}

__device__ __noinline__ void fused_phase(const EnsStepArgs& a, float2* s) {
    uint32_t base = 0;
    for (int ci = 0; ci < a.nclasses; ++ci) {
        const EnsStepClass& c = a.cls[ci];
        const uint32_t n = *c.n_items;
        // this CTA's items of the class: global item ids base .. base + n - 1
        uint32_t it = blockIdx.x >= base ? blockIdx.x - base
                                         : blockIdx.x + ((base - blockIdx.x + gridDim.x - 1) / gridDim.x) * gridDim.x - base;
        for (; it < n; it += gridDim.x) {
            const WorkItem item = c.items[it];
            const float2* force = c.force + size_t(item.sim) * c.N * c.N;
            float* rho = c.rho + size_t(item.sim) * c.N * c.N;
            if (a.cic)
                fused_item<1, kEnsGran>(item, c.p, force, rho, c.N, a.dt, WindowSmem<1, kEnsGran>(s));
            else
                fused_item<0, kEnsGran>(item, c.p, force, rho, c.N, a.dt, WindowSmem<0, kEnsGran>(s));
        }
        base += n;
    }
}

__global__ void __launch_bounds__(kEnsThreads, 2) k_ensemble_step(const EnsStepArgs* __restrict__ args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    const EnsStepArgs& a = *args;
    for (int phase = 0; phase < 3; ++phase) {
        fft_phase(a, phase, s);
        if (!grid_barrier(a.barrier, phase, a.status, a.skip_arrive && phase == 0 && blockIdx.x == 0)) return;
    }
    fused_phase(a, s);  // phase 3
}

}  // namespace

bool ensemble_step_supported(int N) { return N == 128 || N == 256 || N == 512 || N == 1024; }

cudaError_t prepare_ensemble_step(int nsm, int* grid) {
    cudaError_t e = cudaFuncSetAttribute(k_ensemble_step, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kEnsSmem));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ensemble_step, kEnsThreads, kEnsSmem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    *grid = nsm * per_sm;
    return cudaSuccess;
}

cudaError_t launch_ensemble_step(const EnsStepArgs* args_dev, unsigned* barrier, int grid, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(barrier, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(kEnsThreads);
    cfg.dynamicSmemBytes = kEnsSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_ensemble_step, args_dev);
}

}  // namespace cpm
