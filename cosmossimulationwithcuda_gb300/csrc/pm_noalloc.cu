// Tile-key sort that allocates no device memory.
//
// For callers that cannot allocate device memory while they run -- a renderer
// or simulation host that only owns a fixed amount of device memory, code inside a
// custom allocator or memory-pool callback, or a real-time loop where an
// allocation may block on a device-wide synchronisation -- this entry point
// sorts caller-owned device positions with scratch that lives in a fixed,
// file-scope device array instead of in cudaMalloc'd buffers.
//
// The array is sized for kNoAllocMaxParticles particles (about 16.5 MB) and
// every GPU that loads this library keeps it until the process exits.  All
// calls on one device share it: two calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on the scratch and
// must be serialised by the caller.  The scratch keeps the last call's
// contents; nothing in it needs to start at zero (every pass writes all the
// counters it later reads).
#include <mutex>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace cpm {

namespace {

constexpr int64_t kNoAllocMaxParticles = COSMOS_NOALLOC_MAX_PARTICLES;
constexpr int kNoAllocMaxGrid = 512;
constexpr size_t kNoAllocCounts = size_t(256) * kNoAllocMaxGrid + 256;
constexpr size_t kNoAllocWords = 4 * size_t(kNoAllocMaxParticles) + kNoAllocCounts;

// keys[2] | vals[2] | radix counters
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};
int g_nsm[kMaxDevices] = {};

// Device address of the scratch array on the current device; the host-side
// symbol is only a stand-in for it.  Outside stream capture the address is
// looked up on every call (a device reset or a new primary context reloads the
// module and may move the array); under capture the address of the last
// uncaptured call on this device is used, so the first call on a device must
// come before any capture.
int scratch_for_current_device(cudaStream_t st, uint32_t** out, int* nsm) {
    int dev = -1;
    CPM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(COSMOS_ERR_INVALID, "device ordinal out of range");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CPM_CUDA(cudaStreamIsCapturing(st, &cs));
    std::lock_guard<std::mutex> lk(g_mu);
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(COSMOS_ERR_CUDA, std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
        int sms = 0;
        CPM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
        g_nsm[dev] = sms;
    } else if (!g_scratch_ptr[dev]) {
        return fail(COSMOS_ERR_STATE, "cosmos_tile_sort_noalloc: the first call on a device must come before any "
                                      "stream capture");
    }
    *out = g_scratch_ptr[dev];
    *nsm = g_nsm[dev];
    return COSMOS_OK;
}

}  // namespace

int tile_sort_noalloc(const float* x, const float* y, int64_t n, int N, int gran, uint32_t* perm, cudaStream_t st) {
    if (!x || !y || !perm) return fail(COSMOS_ERR_INVALID, "null device pointer");
    if (n < 0) return fail(COSMOS_ERR_INVALID, "negative particle count");
    if (n > kNoAllocMaxParticles)
        return fail(COSMOS_ERR_RANGE, "cosmos_tile_sort_noalloc: " + std::to_string(n) +
                                          " particles exceed the fixed scratch capacity of " +
                                          std::to_string(kNoAllocMaxParticles));
    if (N < 16 || N > 8192 || (N & (N - 1)) != 0)
        return fail(COSMOS_ERR_INVALID, "lattice_n must be a power of two in [16, 8192]");
    if (gran < 0 || gran > 13 || (N >> gran) < 1) return fail(COSMOS_ERR_INVALID, "granularity must satisfy 2^g <= N");
    if (n == 0) return COSMOS_OK;
    uint32_t* base = nullptr;
    int nsm = 0;
    CPM_TRY(scratch_for_current_device(st, &base, &nsm));
    RadixScratch rs{};
    rs.keys[0] = base;
    rs.keys[1] = base + kNoAllocMaxParticles;
    rs.vals[0] = base + 2 * kNoAllocMaxParticles;
    rs.vals[1] = base + 3 * kNoAllocMaxParticles;
    rs.counts = base + 4 * kNoAllocMaxParticles;
    rs.grid = radix_grid(n, nsm);
    if (rs.grid > kNoAllocMaxGrid) rs.grid = kNoAllocMaxGrid;
    const int T = N >> gran;
    const int bits = 2 * ilog2(T) + 1;
    CPM_CUDA(launch_tile_keys(x, y, n, N, gran, rs.keys[0], st));
    CPM_CUDA(launch_iota(rs.vals[0], n, st));
    int which = 0;
    CPM_CUDA(launch_radix_sort(rs, n, bits, &which, st));
    CPM_CUDA(cudaMemcpyAsync(perm, rs.vals[which], size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    return COSMOS_OK;
}

}  // namespace cpm

extern "C" int cosmos_tile_sort_noalloc(const float* x_dev, const float* y_dev, int64_t n, int32_t lattice_n,
                                        int32_t granularity, uint32_t* perm_dev, uint64_t stream) {
    return cpm::tile_sort_noalloc(x_dev, y_dev, n, lattice_n, granularity, perm_dev,
                                  reinterpret_cast<cudaStream_t>(stream));
}
