// C ABI of the cosmos_pm library: handle lifetime, particle I/O, the step
// sequence (direct launches or a replayed CUDA graph), asynchronous position
// readback, stage-level test hooks and diagnostics.
//
// Stands in for the Universe<K> class of CosmosCuda.cuh (constructor
// :881-1035, clear :1038-1069, step methods :1209-1300, worker loop
// :1318-1364, destructor :1396-1427) and its render chain (:1249-1256, kernels
// in pm_render.cu).  The frame ring and worker thread live in the C++ drop-in
// header (include/CosmosGB300.cuh); the multi-GPU exchange is not built.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace cpm {

static thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

const char* last_error_message() { return g_last_error.c_str(); }

// COSMOS_TEST_FAIL_ALLOC: allocations left before the one that fails (0: off).
static std::atomic<int64_t> g_fail_alloc_countdown{0};

bool alloc_should_fail() {
    int64_t c = g_fail_alloc_countdown.load();
    while (c > 0) {
        if (g_fail_alloc_countdown.compare_exchange_weak(c, c - 1)) return c == 1;
    }
    return false;
}

}  // namespace cpm

using cpm::ParticleArrays;

// Profiling event slots: [prologue deposit] [sort] fft | force | fused step | end
enum EvIdx { kEvPrologue = 0, kEvSort, kEvFft, kEvForce, kEvFused, kEvEnd, kNumEv };
// Entries of cosmos_pm_stage_times.
enum StageIdx { kTPrologue = 0, kTFft, kTForce, kTFused, kTSort, kNumTimes };

struct cosmos_pm {
    cosmos_pm_config cfg{};
    int N = 0, logN = 0, cic = 0, nsm = 0, device = 0;
    int64_t P = 0, Pq = 0, Palloc = 0;
    cudaStream_t stream = nullptr, copy_stream = nullptr;

    ParticleArrays buf[2]{};
    int cur = 0;
    bool identity_order = true;  // slot i holds identity i (no sort applied yet)
    uint32_t* pos = nullptr;     // identity -> slot, valid when pos_valid
    bool pos_valid = false;

    float* rho = nullptr;
    float2* spec = nullptr;
    float* phi = nullptr;
    float2* force = nullptr;
    float2* spec2 = nullptr;  // spectral mode: y-inverse of the Fy spectrum
    float2* edge = nullptr;   // spectral mode: y-edge differences per line kx
    void* tc_dft = nullptr;   // tensor-core modes: DFT matrix image
    int* tc_status = nullptr; // tensor-core modes: MMA wait timeout flag
    int* wait_status = nullptr;  // step kernels: a bounded copy wait (bulk / tensor-map loads) that ran out
    uint32_t copy_tx_extra = 0;  // test hook COSMOS_TEST_COPY_WAIT
    cpm::SpectralMaps maps{};    // spectral mode from 256^2 up: tensor maps of the row and column passes' tiles
    bool have_maps = false;
    cpm::SpectralTc tc{};
    float* kq = nullptr;
    float2* tw = nullptr;
    double* diag = nullptr;

    cpm::RadixScratch rs{};
    int gran = 5, sort_bits = 0, sort_interval = 0;
    int64_t steps_since_sort = 0;
    bool sort_due = false;

    // tile work items (valid after a sort, until the state is rewritten)
    uint32_t* tstart = nullptr;
    uint32_t* tend = nullptr;
    cpm::WorkItem* items = nullptr;
    uint32_t* n_items = nullptr;
    size_t max_items = 0;
    int item_size = cpm::kItemMax;  // particles per work item (work_item_size)
    bool items_valid = false;
    int tiles_grid = 0;
    bool density_valid = false;  // rho holds the density of the current positions

    float* stage[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaEvent_t stage_ready[2] = {nullptr, nullptr};
    cudaEvent_t stage_done[2] = {nullptr, nullptr};
    int stage_slot = 0;
    std::mutex ticket_mu;
    std::deque<std::pair<uint64_t, cudaEvent_t>> tickets;
    std::vector<cudaEvent_t> event_pool;
    uint64_t next_ticket = 1;

    bool profiling = false;
    cudaEvent_t ev[kNumEv] = {};
    // profiled graph steps: the stage events sit on a side branch of the graph
    cudaStream_t prof_stream = nullptr;
    cudaEvent_t prof_fork[kNumEv] = {};
    cudaEvent_t prof_join = nullptr;
    bool prof_forked = false;
    bool have_times = false;
    bool prof_sorted = false, prof_prologue = false;

    // display frames (allocated on the first render call)
    int blur_r = 3;
    bool render_identity = false;  // the weight table is the identity: no blur pass
    float* rkern = nullptr;
    float* blurred = nullptr;
    float* frame[2] = {nullptr, nullptr};
    uint32_t* rstate = nullptr;  // frame min / max keys + finished-CTA counter
    float* rext = nullptr;       // running min / max across frames
    cudaEvent_t frame_ready[2] = {nullptr, nullptr};
    cudaEvent_t frame_done[2] = {nullptr, nullptr};
    int frame_slot = 0;

    bool use_graph = true;
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [buffer parity][tiled]
    // kGraphSteps steps in one graph, for runs of steps without a sort
    cudaGraphExec_t graph_multi[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    // one step with the profiling events recorded between its stages (event nodes)
    cudaGraphExec_t graph_prof[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int64_t steps_taken = 0;  // steps advanced since creation (restored by a checkpoint load)
    int64_t kernels_enqueued = 0;  // kernel launches enqueued since creation (cosmos_pm_kernels_launched)

    std::string err;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};

int finish(cosmos_pm* h, int rc) {
    if (rc != COSMOS_OK && h) h->err = cpm::last_error_message();
    return rc;
}

template <class T>
int dalloc(T** p, size_t n) {
    if (n == 0) n = 1;
    if (cpm::alloc_should_fail()) {
        *p = nullptr;
        return cpm::fail(COSMOS_ERR_NOMEM, "device allocation of " + std::to_string(n * sizeof(T)) +
                                               " bytes failed (injected by COSMOS_TEST_FAIL_ALLOC)");
    }
    if (cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return cpm::fail(COSMOS_ERR_NOMEM, "device allocation of " + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    return COSMOS_OK;
}

ParticleArrays& state(cosmos_pm* h) { return h->buf[h->cur]; }

int sort_now(cosmos_pm* h);
int issue_ticket(cosmos_pm* h, uint64_t* ticket);

bool is_spectral(int mode) {
    return mode == COSMOS_FORCE_SPECTRAL || mode == COSMOS_FORCE_SPECTRAL_TC_FP16 ||
           mode == COSMOS_FORCE_SPECTRAL_TC_BF16;
}
bool is_tc(int mode) { return mode == COSMOS_FORCE_SPECTRAL_TC_FP16 || mode == COSMOS_FORCE_SPECTRAL_TC_BF16; }

// Profiling event i at the current point of stream st.  Direct launches: a
// plain record.  Under stream capture (a profiled graph step): an external
// event-record node on a side branch that depends on everything captured on
// st so far, so that the kernels of the step keep their own edges (and their
// programmatic, overlapping launches) and the event still marks the moment
// the work before it completed.  The side branch rejoins st at the end of
// the capture (join_profile_branch).
cudaError_t record_profile_event(cosmos_pm* h, int i, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusActive) return cudaEventRecord(h->ev[i], st);
    if ((e = cudaEventRecord(h->prof_fork[i], st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(h->prof_stream, h->prof_fork[i], 0)) != cudaSuccess) return e;
    h->prof_forked = true;
    return cudaEventRecordWithFlags(h->ev[i], h->prof_stream, cudaEventRecordExternal);
}

cudaError_t join_profile_branch(cosmos_pm* h, cudaStream_t st) {
    if (!h->prof_forked) return cudaSuccess;
    h->prof_forked = false;
    const cudaError_t e = cudaEventRecord(h->prof_join, h->prof_stream);
    return e != cudaSuccess ? e : cudaStreamWaitEvent(st, h->prof_join, 0);
}

// clear_rho: zero the density behind the row pass (the step clears it for the deposit that follows).
int launch_spectral(cosmos_pm* h, cudaStream_t st, bool clear_rho = false) {
    CPM_CUDA(cpm::launch_spectral_force(h->N, h->rho, h->spec, h->spec2, h->edge, h->kq, h->force, h->tw,
                                        h->cfg.gravity_multiplier, st, 1,
                                        is_tc(h->cfg.force_mode) ? &h->tc : nullptr, clear_rho ? h->rho : nullptr,
                                        h->have_maps ? &h->maps : nullptr, h->wait_status, h->cfg.fft_shape));
    return COSMOS_OK;
}

// Density -> force field.  Gradient mode: FFT convolution to the potential,
// then the reference's edge-clamped stencil.  Spectral mode: the stencil is
// applied in Fourier space (no potential field is written).  The profiling
// event between the two halves marks the start of the force pass.
// Kernels of one step: the force passes (the row pass clears the density) and
// the fused step kernel.
int step_launches(const cosmos_pm* h) {
    const int force = is_spectral(h->cfg.force_mode) ? cpm::spectral_launches_per_step()
                                                     : cpm::conv_launches_per_step() + 1;
    return force + 1;
}

// Kernels of one re-sort: keys, identities, 3 per radix pass, permutation,
// tile ranges, work items, item scales.
int sort_launches(const cosmos_pm* h) { return 2 + 3 * ((h->sort_bits + 7) / 8) + 4; }

// Force of the density in rho; rho is zeroed behind the row pass, ready for the deposit.
int enqueue_force(cosmos_pm* h, cudaStream_t st, bool profile) {
    const float g = h->cfg.gravity_multiplier;
    if (is_spectral(h->cfg.force_mode)) {
        CPM_TRY(launch_spectral(h, st, true));
        if (profile) CPM_CUDA(record_profile_event(h, kEvForce, st));
    } else {
        CPM_CUDA(cpm::launch_conv_passes(h->N, h->rho, h->spec, h->kq, h->phi, h->tw, st, 1, h->rho));
        if (profile) CPM_CUDA(record_profile_event(h, kEvForce, st));
        CPM_CUDA(cpm::launch_gradient(h->phi, h->force, h->N, g, st));
    }
    return COSMOS_OK;
}

// One step's kernels on stream st (buffer parity `cur`), assuming rho holds the
// density of the current positions:
//   FFT convolution rho -> phi, gradient phi -> force (the row pass clears rho
//   as it reads it), fused gather + update + deposit of the new positions into rho.
int enqueue_step_body(cosmos_pm* h, cudaStream_t st, bool profile) {
    ParticleArrays& p = state(h);
    auto rec = [&](int i) -> int {
        if (profile) CPM_CUDA(record_profile_event(h, i, st));
        return COSMOS_OK;
    };
    CPM_TRY(rec(kEvFft));
    CPM_TRY(enqueue_force(h, st, profile));
    CPM_TRY(rec(kEvFused));
    if (h->items_valid)
        CPM_CUDA(cpm::launch_fused_tiles(h->items, h->n_items, p, h->force, h->rho, h->N, h->cic, h->cfg.dt, h->gran,
                                         h->tiles_grid, h->wait_status, st, h->copy_tx_extra));
    else
        CPM_CUDA(cpm::launch_fused_global(p, h->P, h->force, h->rho, h->N, h->cic, h->cfg.dt, h->nsm, st));
    CPM_TRY(rec(kEvEnd));
    return COSMOS_OK;
}

// Density of the current positions (first step after the state was written).
int enqueue_prologue(cosmos_pm* h, cudaStream_t st) {
    CPM_CUDA(cudaMemsetAsync(h->rho, 0, size_t(h->N) * h->N * sizeof(float), st));
    CPM_CUDA(cpm::launch_deposit_global(state(h), h->P, h->rho, h->N, h->cic, h->nsm, st));
    h->density_valid = true;
    return COSMOS_OK;
}

// Invalidate what depends on the particle state after a host-side rewrite.
void state_rewritten(cosmos_pm* h) {
    h->sort_due = true;
    h->items_valid = false;
    h->density_valid = false;
}

// The step body `steps` times (1 or kGraphSteps) as one graph, cached per
// buffer parity and tiling; profile: one step with the stage events recorded
// as event nodes of the graph.
int get_graph(cosmos_pm* h, cudaGraphExec_t* out, int steps = 1, bool profile = false) {
    cudaGraphExec_t& g =
        (profile ? h->graph_prof : steps == 1 ? h->graph : h->graph_multi)[h->cur][h->items_valid ? 1 : 0];
    if (!g) {
        cudaGraph_t graph = nullptr;
        CPM_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = COSMOS_OK;
        for (int i = 0; i < steps && rc == COSMOS_OK; ++i) rc = enqueue_step_body(h, h->stream, profile);
        if (rc == COSMOS_OK && join_profile_branch(h, h->stream) != cudaSuccess)
            rc = cpm::fail(COSMOS_ERR_CUDA, "profile branch join");
        const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        if (rc != COSMOS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cpm::fail(COSMOS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        const cudaError_t ie = cudaGraphInstantiate(&g, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            g = nullptr;
            return cpm::fail(COSMOS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
    }
    *out = g;
    return COSMOS_OK;
}

int enqueue_step(cosmos_pm* h) {
    bool sorted = false, prologue = false;
    if (h->profiling) CPM_CUDA(cudaEventRecord(h->ev[kEvPrologue], h->stream));
    if (!h->density_valid) {
        CPM_TRY(enqueue_prologue(h, h->stream));
        h->kernels_enqueued += 1;
        prologue = true;
    }
    if (h->profiling) CPM_CUDA(cudaEventRecord(h->ev[kEvSort], h->stream));
    if (h->sort_interval > 0 && (h->sort_due || h->steps_since_sort >= h->sort_interval)) {
        CPM_TRY(sort_now(h));
        h->kernels_enqueued += sort_launches(h);
        sorted = true;
    }
    if (h->profiling) {
        if (h->use_graph) {  // the step as it runs (graph-launched), events between its stages
            cudaGraphExec_t g = nullptr;
            CPM_TRY(get_graph(h, &g, 1, true));
            CPM_CUDA(cudaGraphLaunch(g, h->stream));
        } else {
            CPM_TRY(enqueue_step_body(h, h->stream, true));
        }
        h->have_times = true;
        h->prof_sorted = sorted;
        h->prof_prologue = prologue;
    } else if (h->use_graph) {
        cudaGraphExec_t g = nullptr;
        CPM_TRY(get_graph(h, &g));
        CPM_CUDA(cudaGraphLaunch(g, h->stream));
    } else {
        CPM_TRY(enqueue_step_body(h, h->stream, false));
    }
    ++h->steps_since_sort;
    ++h->steps_taken;
    h->kernels_enqueued += step_launches(h);
    return COSMOS_OK;
}

// kGraphSteps steps as one graph launch when none of them sorts, profiles or
// needs the prologue: the kernels of consecutive steps then follow one
// another inside the graph (as programmatic dependents from 1024^2 up).
constexpr int kGraphSteps = 4;
bool can_enqueue_multi(const cosmos_pm* h, int remaining) {
    if (!h->use_graph || h->profiling || !h->density_valid || remaining < kGraphSteps) return false;
    if (h->sort_interval > 0 && (h->sort_due || h->steps_since_sort + kGraphSteps > h->sort_interval)) return false;
    return true;
}

int enqueue_multi(cosmos_pm* h) {
    cudaGraphExec_t g = nullptr;
    CPM_TRY(get_graph(h, &g, kGraphSteps));
    CPM_CUDA(cudaGraphLaunch(g, h->stream));
    h->steps_since_sort += kGraphSteps;
    h->steps_taken += kGraphSteps;
    h->kernels_enqueued += int64_t(kGraphSteps) * step_launches(h);
    return COSMOS_OK;
}

// Stable sort of the first Pq slots by tile key; trailing P % 4 particles keep
// their slots (the step never touches them, like the reference).
int sort_now(cosmos_pm* h) {
    cudaStream_t st = h->stream;
    ParticleArrays& src = h->buf[h->cur];
    ParticleArrays& dst = h->buf[h->cur ^ 1];
    CPM_CUDA(cpm::launch_tile_keys(src.x, src.y, h->Pq, h->N, h->gran, h->rs.keys[0], st));
    CPM_CUDA(cpm::launch_iota(h->rs.vals[0], h->P, st));
    int which = 0;
    CPM_CUDA(cpm::launch_radix_sort(h->rs, h->Pq, h->sort_bits, &which, st));
    if (which != 0 && h->P > h->Pq)  // trailing identities ride along unsorted
        CPM_CUDA(cudaMemcpyAsync(h->rs.vals[which] + h->Pq, h->rs.vals[0] + h->Pq, (h->P - h->Pq) * sizeof(uint32_t),
                                 cudaMemcpyDeviceToDevice, st));
    CPM_CUDA(cpm::launch_permute(src, dst, h->rs.vals[which], h->P, st));
    CPM_CUDA(cpm::launch_build_items(h->rs.keys[which], dst.m, h->Pq, h->N, h->gran, h->tstart, h->tend, h->items,
                                     h->n_items, h->max_items, h->item_size, st));
    h->cur ^= 1;
    h->identity_order = false;
    h->pos_valid = false;
    h->steps_since_sort = 0;
    h->sort_due = false;
    h->items_valid = true;
    return COSMOS_OK;
}

int ensure_pos(cosmos_pm* h) {
    if (h->identity_order || h->pos_valid) return COSMOS_OK;
    CPM_CUDA(cpm::launch_invert(state(h).id, h->pos, h->P, h->stream));
    h->pos_valid = true;
    return COSMOS_OK;
}

int check_range(cosmos_pm* h, int64_t count, int64_t offset) {
    if (count < 0 || offset < 0 || offset + count > h->P)
        return cpm::fail(COSMOS_ERR_RANGE, "particle range [" + std::to_string(offset) + ", " +
                                               std::to_string(offset + count) + ") outside [0, " + std::to_string(h->P) +
                                               ")");
    return COSMOS_OK;
}

// Tile order pays off when a tile holds enough particles to amortise its
// window staging: sort every 32 steps when the mean occupancy of the
// 32x32-cell tiles is at least 256 particles.  (On the 20M-particle disk the
// fused kernel's time is flat over a 32-step cycle for the first ~500 steps;
// later the fast particles of the dense centre leave the 4-cell window halo
// and it grows from 0.15 to 0.22 ms between two sorts.  A 16-step cadence, or
// an 8-cell halo, keeps it flatter but costs as much in sorts or in window
// staging: the mean step time stays within 1% of this setting.)
int default_sort_interval(int64_t P, int N) {
    const double tiles = double(N / 32 > 0 ? N / 32 : 1) * double(N / 32 > 0 ? N / 32 : 1);
    return double(P) / tiles >= 256.0 ? 32 : 0;
}

void destroy_all(cosmos_pm* h) {
    DeviceGuard g(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    for (auto& b : h->buf) {
        cudaFree(b.x);
        cudaFree(b.y);
        cudaFree(b.xo);
        cudaFree(b.yo);
        cudaFree(b.m);
        cudaFree(b.id);
    }
    cudaFree(h->pos);
    cudaFree(h->rho);
    cudaFree(h->spec);
    cudaFree(h->phi);
    cudaFree(h->force);
    cudaFree(h->spec2);
    cudaFree(h->edge);
    cudaFree(h->tc_dft);
    cudaFree(h->tc_status);
    cudaFree(h->wait_status);
    cudaFree(h->kq);
    cudaFree(h->tw);
    cudaFree(h->diag);
    for (int i = 0; i < 2; ++i) {
        cudaFree(h->rs.keys[i]);
        cudaFree(h->rs.vals[i]);
        cudaFree(h->stage[i][0]);
        cudaFree(h->stage[i][1]);
        if (h->stage_ready[i]) cudaEventDestroy(h->stage_ready[i]);
        if (h->stage_done[i]) cudaEventDestroy(h->stage_done[i]);
        for (int j = 0; j < 2; ++j) {
            if (h->graph[i][j]) cudaGraphExecDestroy(h->graph[i][j]);
            if (h->graph_multi[i][j]) cudaGraphExecDestroy(h->graph_multi[i][j]);
            if (h->graph_prof[i][j]) cudaGraphExecDestroy(h->graph_prof[i][j]);
        }
    }
    cudaFree(h->rs.counts);
    cudaFree(h->rkern);
    cudaFree(h->blurred);
    cudaFree(h->rstate);
    cudaFree(h->rext);
    for (int i = 0; i < 2; ++i) {
        cudaFree(h->frame[i]);
        if (h->frame_ready[i]) cudaEventDestroy(h->frame_ready[i]);
        if (h->frame_done[i]) cudaEventDestroy(h->frame_done[i]);
    }
    cudaFree(h->tstart);
    cudaFree(h->tend);
    cudaFree(h->items);
    cudaFree(h->n_items);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : h->prof_fork)
        if (e) cudaEventDestroy(e);
    if (h->prof_join) cudaEventDestroy(h->prof_join);
    if (h->prof_stream) cudaStreamDestroy(h->prof_stream);
    for (auto& t : h->tickets) cudaEventDestroy(t.second);
    for (auto e : h->event_pool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
}

int create_impl(const cosmos_pm_config* cfg, cosmos_pm** out) {
    if (!cfg || !out) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *out = nullptr;
    const int N = cfg->lattice_n;
    if (N < 16 || N > 8192 || (N & (N - 1)) != 0)
        return cpm::fail(COSMOS_ERR_INVALID, "lattice_n must be a power of two in [16, 8192]");
    if (cfg->deposit != COSMOS_DEPOSIT_NGP && cfg->deposit != COSMOS_DEPOSIT_CIC)
        return cpm::fail(COSMOS_ERR_INVALID, "deposit must be COSMOS_DEPOSIT_NGP or COSMOS_DEPOSIT_CIC");
    if (cfg->num_particles < 0 || cfg->num_particles > int64_t(0xFFFFFFF0u))
        return cpm::fail(COSMOS_ERR_INVALID, "num_particles must be in [0, 2^32 - 16]");
    if (!std::isfinite(cfg->dt) || !std::isfinite(cfg->gravity_multiplier))
        return cpm::fail(COSMOS_ERR_INVALID, "dt and gravity_multiplier must be finite");
    if (cfg->force_mode != COSMOS_FORCE_GRADIENT && !is_spectral(cfg->force_mode))
        return cpm::fail(COSMOS_ERR_INVALID, "force_mode must be one of the COSMOS_FORCE_* modes");
    if (is_tc(cfg->force_mode) && !cpm::tc_fft_supported(N))
        return cpm::fail(COSMOS_ERR_INVALID, "the tensor-core force modes support lattice_n 1024, 2048 and 4096");
    if (cfg->sort_granularity != -1 &&
        (cfg->sort_granularity < 4 || cfg->sort_granularity > 6 || (N >> cfg->sort_granularity) < 1))
        return cpm::fail(COSMOS_ERR_INVALID, "sort_granularity must be -1 (default) or 4..6 with 2^g <= N");
    if (cfg->blur_r != 0 && (cfg->blur_r < 1 || cfg->blur_r > 15 || cfg->blur_r % 2 == 0))
        return cpm::fail(COSMOS_ERR_INVALID, "blur_r must be 0 (default 3) or odd in [1, 15]");
    if (cfg->item_size != 0 && cfg->item_size != 2048 && cfg->item_size != 4096 && cfg->item_size != 8192)
        return cpm::fail(COSMOS_ERR_INVALID, "item_size must be 0 (default), 2048, 4096 or 8192");
    if (cfg->fused_ctas_per_sm < 0 || cfg->fused_ctas_per_sm > 32)
        return cpm::fail(COSMOS_ERR_INVALID, "fused_ctas_per_sm must be in [0, 32]");
    if (cfg->fft_shape != 0 && cfg->fft_shape != 1) return cpm::fail(COSMOS_ERR_INVALID, "fft_shape must be 0 or 1");
    int ndev = 0;
    CPM_CUDA(cudaGetDeviceCount(&ndev));
    if (cfg->device < 0 || cfg->device >= ndev) return cpm::fail(COSMOS_ERR_INVALID, "device ordinal out of range");

    cosmos_pm* h = new cosmos_pm;
    h->cfg = *cfg;
    h->N = N;
    h->logN = cpm::ilog2(N);
    h->cic = cfg->deposit == COSMOS_DEPOSIT_CIC;
    h->device = cfg->device;
    h->P = cfg->num_particles;
    h->Pq = (h->P / 4) * 4;
    h->Palloc = ((h->P + 3) / 4) * 4;
    h->use_graph = cfg->use_graph != 0;
    h->blur_r = cfg->blur_r != 0 ? cfg->blur_r : 3;
    h->gran = cfg->sort_granularity >= 0 ? cfg->sort_granularity : (N >= 64 ? 5 : 4);
    {
        const int T = N >> h->gran;
        h->sort_bits = 2 * cpm::ilog2(T) + 1;
    }
    h->sort_interval = cfg->sort_interval >= 0 ? cfg->sort_interval : default_sort_interval(h->P, N);

    DeviceGuard guard(h->device);
    auto bail = [&](int rc) {
        destroy_all(h);
        delete h;
        return rc;
    };
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "device query"));
    h->nsm = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "stream creation"));
    for (auto& e : h->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "event creation"));
    for (auto& e : h->prof_fork)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(cpm::fail(COSMOS_ERR_CUDA, "event creation"));
    if (cudaEventCreateWithFlags(&h->prof_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->prof_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "profiling stream"));
    for (int i = 0; i < 2; ++i) {
        if (cudaEventCreateWithFlags(&h->stage_ready[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->stage_done[i], cudaEventDisableTiming) != cudaSuccess)
            return bail(cpm::fail(COSMOS_ERR_CUDA, "event creation"));
    }
    const size_t NN = size_t(N) * N;
    const size_t Pa = size_t(h->Palloc);
    int rc = COSMOS_OK;
    for (int b = 0; b < 2 && rc == COSMOS_OK; ++b) {
        ParticleArrays& a = h->buf[b];
        if ((rc = dalloc(&a.x, Pa)) || (rc = dalloc(&a.y, Pa)) || (rc = dalloc(&a.xo, Pa)) ||
            (rc = dalloc(&a.yo, Pa)) || (rc = dalloc(&a.m, Pa)) || (rc = dalloc(&a.id, Pa)))
            break;
    }
    if (rc == COSMOS_OK) {
        h->rs.grid = cpm::radix_grid(h->Pq, h->nsm);
        if ((rc = dalloc(&h->pos, Pa)) || (rc = dalloc(&h->rho, NN)) || (rc = dalloc(&h->spec, NN / 2)) ||
            (rc = dalloc(&h->phi, NN)) || (rc = dalloc(&h->force, NN)) ||
            (rc = dalloc(&h->kq, size_t(N / 2 + 1) * (N / 2 + 1))) || (rc = dalloc(&h->tw, size_t(N))) ||
            (rc = dalloc(&h->diag, 4)) || (rc = dalloc(&h->rs.keys[0], Pa)) || (rc = dalloc(&h->rs.keys[1], Pa)) ||
            (rc = dalloc(&h->rs.vals[0], Pa)) || (rc = dalloc(&h->rs.vals[1], Pa)) ||
            (rc = dalloc(&h->rs.counts, cpm::radix_counts_elems(h->rs.grid))))
            ;
    }
    const int ntiles = (N >> h->gran) * (N >> h->gran);
    h->item_size = cfg->item_size ? cfg->item_size : cpm::work_item_size(h->Pq, h->nsm);
    h->max_items = cpm::max_work_items(h->Pq, ntiles, h->item_size);
    if (rc == COSMOS_OK) {
        const size_t nranges = cpm::tile_range_elems(N, h->gran, 1);
        if ((rc = dalloc(&h->tstart, nranges)) || (rc = dalloc(&h->tend, nranges)) ||
            (rc = dalloc(&h->items, h->max_items)) || (rc = dalloc(&h->n_items, 1)) ||
            (rc = dalloc(&h->wait_status, 1)))
            ;
    }
    if (rc != COSMOS_OK) return bail(rc);
    if (cudaMemsetAsync(h->n_items, 0, sizeof(uint32_t), h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->wait_status, 0, sizeof(int), h->stream) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "memset"));
    if (cpm::prepare_tile_kernels(h->gran, h->cic, h->nsm, &h->tiles_grid) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "tile kernel attributes"));
    if (cfg->fused_ctas_per_sm > 0 && h->tiles_grid > h->nsm * cfg->fused_ctas_per_sm)
        h->tiles_grid = h->nsm * cfg->fused_ctas_per_sm;
    // zero state; identities; filter
    for (int b = 0; b < 2; ++b) {
        ParticleArrays& a = h->buf[b];
        for (float* f : {a.x, a.y, a.xo, a.yo, a.m})
            if (cudaMemsetAsync(f, 0, Pa * sizeof(float), h->stream) != cudaSuccess)
                return bail(cpm::fail(COSMOS_ERR_CUDA, "memset"));
    }
    if (cpm::launch_iota(h->buf[0].id, h->Palloc, h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->rho, 0, NN * sizeof(float), h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->phi, 0, NN * sizeof(float), h->stream) != cudaSuccess ||
        cudaMemsetAsync(h->force, 0, NN * sizeof(float2), h->stream) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "initialisation"));
    if (cpm::prepare_conv_passes(N) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "kernel attributes"));
    if (is_spectral(cfg->force_mode)) {
        if ((rc = dalloc(&h->spec2, NN / 2)) || (rc = dalloc(&h->edge, size_t(N / 2) * 4))) return bail(rc);
        if (is_tc(cfg->force_mode)) {
            const int bf16 = cfg->force_mode == COSMOS_FORCE_SPECTRAL_TC_BF16;
            if ((rc = dalloc(reinterpret_cast<unsigned char**>(&h->tc_dft), cpm::tc_dft_bytes(N))) ||
                (rc = dalloc(&h->tc_status, 1)))
                return bail(rc);
            if (cudaMemsetAsync(h->tc_status, 0, sizeof(int), h->stream) != cudaSuccess ||
                cpm::prepare_tc_columns(N, bf16, h->tc_dft, h->stream) != cudaSuccess)
                return bail(cpm::fail(COSMOS_ERR_CUDA, "tensor-core column pass setup"));
            h->tc = cpm::SpectralTc{bf16, h->tc_dft, h->tc_status};
        }
        if (cpm::prepare_spectral_passes(N) != cudaSuccess)
            return bail(cpm::fail(COSMOS_ERR_CUDA, "spectral kernel attributes"));
        if (N >= 256) {  // tiles of the row and column passes arrive by tensor-map loads
            const cudaError_t me = cpm::make_spectral_maps(N, h->rho, h->spec, 1, &h->maps);
            if (me != cudaSuccess)
                return bail(cpm::fail(COSMOS_ERR_CUDA, std::string("tensor maps: ") + cudaGetErrorString(me)));
            h->have_maps = true;
        }
    }
    if ((rc = cpm::build_filter(N, h->cic, h->kq, h->tw, h->stream)) != COSMOS_OK) return bail(rc);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "create sync"));
    *out = h;
    return COSMOS_OK;
}

int set_particles_impl(cosmos_pm* h, const float* x, const float* y, const float* xo, const float* yo, const float* m,
                       int64_t count, int64_t offset) {
    CPM_TRY(check_range(h, count, offset));
    if (count == 0) return COSMOS_OK;
    if (!x || !y) return cpm::fail(COSMOS_ERR_INVALID, "x and y are required");
    cudaStream_t st = h->stream;
    ParticleArrays& p = state(h);
    const size_t bytes = size_t(count) * sizeof(float);
    const float* srcs[5] = {x, y, xo ? xo : x, yo ? yo : y, m};
    float* dsts[5] = {p.x, p.y, p.xo, p.yo, p.m};
    if (h->identity_order) {
        for (int i = 0; i < 5; ++i)
            if (srcs[i]) CPM_CUDA(cudaMemcpyAsync(dsts[i] + offset, srcs[i], bytes, cudaMemcpyHostToDevice, st));
    } else {
        CPM_TRY(ensure_pos(h));
        float* tmp = nullptr;
        if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) {
            cudaGetLastError();
            return cpm::fail(COSMOS_ERR_NOMEM, "staging allocation");
        }
        for (int i = 0; i < 5; ++i) {
            if (!srcs[i]) continue;
            CPM_CUDA(cudaMemcpyAsync(tmp, srcs[i], bytes, cudaMemcpyHostToDevice, st));
            CPM_CUDA(cpm::launch_scatter_by_id(tmp, h->pos, offset, count, dsts[i], st));
        }
        CPM_CUDA(cudaFreeAsync(tmp, st));
    }
    CPM_CUDA(cudaStreamSynchronize(st));
    state_rewritten(h);
    return COSMOS_OK;
}

int get_particles_impl(cosmos_pm* h, float* x, float* y, float* xo, float* yo, float* m, int64_t count,
                       int64_t offset);

// ---- checkpoints: header + the five particle arrays in identity order ----
struct CheckpointHeader {
    char magic[8];  // "COSMOSPM"
    uint32_t version;
    int32_t lattice_n, deposit, force_mode;
    int64_t num_particles;
    float dt, gravity_multiplier;
    int64_t steps;
    uint64_t checksum;  // FNV-1a over the array bytes
};
constexpr uint32_t kCheckpointVersion = 1;

uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 0x100000001B3ull;
    return h;
}

int checkpoint_save_impl(cosmos_pm* h, const char* path) {
    if (!path) return cpm::fail(COSMOS_ERR_INVALID, "null path");
    const size_t P = size_t(h->P);
    std::vector<float> a(P * 5);
    CPM_TRY(get_particles_impl(h, a.data(), a.data() + P, a.data() + 2 * P, a.data() + 3 * P, a.data() + 4 * P,
                               h->P, 0));
    CheckpointHeader hd{};
    std::memcpy(hd.magic, "COSMOSPM", 8);
    hd.version = kCheckpointVersion;
    hd.lattice_n = h->N;
    hd.deposit = h->cfg.deposit;
    hd.force_mode = h->cfg.force_mode;
    hd.num_particles = h->P;
    hd.dt = h->cfg.dt;
    hd.gravity_multiplier = h->cfg.gravity_multiplier;
    hd.steps = h->steps_taken;
    hd.checksum = fnv1a(0xCBF29CE484222325ull, a.data(), a.size() * sizeof(float));
    FILE* f = std::fopen(path, "wb");
    if (!f) return cpm::fail(COSMOS_ERR_INVALID, std::string("cannot open ") + path + " for writing");
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
                    std::fwrite(a.data(), sizeof(float), a.size(), f) == a.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return cpm::fail(COSMOS_ERR_INVALID, std::string("writing ") + path + " failed");
    return COSMOS_OK;
}

int checkpoint_load_impl(cosmos_pm* h, const char* path) {
    if (!path) return cpm::fail(COSMOS_ERR_INVALID, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return cpm::fail(COSMOS_ERR_INVALID, std::string("cannot open ") + path);
    CheckpointHeader hd{};
    const size_t P = size_t(h->P);
    std::vector<float> a(P * 5);
    const bool got_header = std::fread(&hd, sizeof(hd), 1, f) == 1;
    const bool got_data = got_header && std::fread(a.data(), sizeof(float), a.size(), f) == a.size();
    const bool at_end = got_data && std::fgetc(f) == EOF;
    std::fclose(f);
    if (!got_header || std::memcmp(hd.magic, "COSMOSPM", 8) != 0 || hd.version != kCheckpointVersion)
        return cpm::fail(COSMOS_ERR_INVALID, std::string(path) + " is not a cosmos_pm checkpoint");
    if (hd.lattice_n != h->N || hd.num_particles != h->P || hd.deposit != h->cfg.deposit ||
        hd.dt != h->cfg.dt || hd.gravity_multiplier != h->cfg.gravity_multiplier)
        return cpm::fail(COSMOS_ERR_INVALID, "checkpoint made with a different lattice, particle count, deposit, "
                                             "time step or gravity multiplier");
    if (!got_data || !at_end) return cpm::fail(COSMOS_ERR_INVALID, std::string(path) + " is truncated or too long");
    if (fnv1a(0xCBF29CE484222325ull, a.data(), a.size() * sizeof(float)) != hd.checksum)
        return cpm::fail(COSMOS_ERR_INVALID, std::string(path) + ": checksum mismatch");
    CPM_TRY(set_particles_impl(h, a.data(), a.data() + P, a.data() + 2 * P, a.data() + 3 * P, a.data() + 4 * P,
                               h->P, 0));
    h->steps_taken = hd.steps;
    return COSMOS_OK;
}

int generate_impl(cosmos_pm* h, const cosmos_ic_params* ic, int64_t count, int64_t offset) {
    if (!ic) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    CPM_TRY(check_range(h, count, offset));
    if (ic->kind < COSMOS_IC_UNIFORM || ic->kind > COSMOS_IC_RING_DISK)
        return cpm::fail(COSMOS_ERR_INVALID, "unknown initial-condition kind");
    if (ic->kind == COSMOS_IC_RING_DISK && ic->total_particles <= 0)
        return cpm::fail(COSMOS_ERR_INVALID, "RING_DISK needs total_particles > 0");
    if (ic->kind != COSMOS_IC_UNIFORM && !(ic->scale > 0.0f))
        return cpm::fail(COSMOS_ERR_INVALID, "scale must be positive");
    if (count == 0) return COSMOS_OK;
    cudaStream_t st = h->stream;
    float* tmp = nullptr;
    if (cudaMallocAsync(&tmp, size_t(count) * 5 * sizeof(float), st) != cudaSuccess) {
        cudaGetLastError();
        return cpm::fail(COSMOS_ERR_NOMEM, "generation buffer");
    }
    float* g[5] = {tmp, tmp + count, tmp + 2 * count, tmp + 3 * count, tmp + 4 * count};
    int rc = COSMOS_OK;
    auto body = [&]() -> int {
        CPM_CUDA(cpm::launch_generate(*ic, count, offset, h->N, h->cfg.dt, g[0], g[1], g[2], g[3], g[4], st));
        ParticleArrays& p = state(h);
        float* dsts[5] = {p.x, p.y, p.xo, p.yo, p.m};
        if (h->identity_order) {
            for (int i = 0; i < 5; ++i)
                CPM_CUDA(cudaMemcpyAsync(dsts[i] + offset, g[i], size_t(count) * sizeof(float), cudaMemcpyDeviceToDevice,
                                         st));
        } else {
            CPM_TRY(ensure_pos(h));
            for (int i = 0; i < 5; ++i) CPM_CUDA(cpm::launch_scatter_by_id(g[i], h->pos, offset, count, dsts[i], st));
        }
        return COSMOS_OK;
    };
    rc = body();
    cudaFreeAsync(tmp, st);
    if (rc != COSMOS_OK) return rc;
    CPM_CUDA(cudaStreamSynchronize(st));
    state_rewritten(h);
    return COSMOS_OK;
}

int get_particles_impl(cosmos_pm* h, float* x, float* y, float* xo, float* yo, float* m, int64_t count,
                       int64_t offset) {
    CPM_TRY(check_range(h, count, offset));
    if (count == 0) return COSMOS_OK;
    cudaStream_t st = h->stream;
    ParticleArrays& p = state(h);
    const size_t bytes = size_t(count) * sizeof(float);
    float* dsts[5] = {x, y, xo, yo, m};
    const float* srcs[5] = {p.x, p.y, p.xo, p.yo, p.m};
    if (h->identity_order) {
        for (int i = 0; i < 5; ++i)
            if (dsts[i]) CPM_CUDA(cudaMemcpyAsync(dsts[i], srcs[i] + offset, bytes, cudaMemcpyDeviceToHost, st));
    } else {
        CPM_TRY(ensure_pos(h));
        float* tmp = nullptr;
        if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) {
            cudaGetLastError();
            return cpm::fail(COSMOS_ERR_NOMEM, "staging allocation");
        }
        for (int i = 0; i < 5; ++i) {
            if (!dsts[i]) continue;
            CPM_CUDA(cpm::launch_gather_by_id(srcs[i], h->pos, offset, count, tmp, st));
            CPM_CUDA(cudaMemcpyAsync(dsts[i], tmp, bytes, cudaMemcpyDeviceToHost, st));
            CPM_CUDA(cudaStreamSynchronize(st));
        }
        CPM_CUDA(cudaFreeAsync(tmp, st));
    }
    CPM_CUDA(cudaStreamSynchronize(st));
    return COSMOS_OK;
}

int positions_async_impl(cosmos_pm* h, float* hx, float* hy, int ordered, uint64_t* ticket) {
    if (!hx || !hy || !ticket) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    const int s = h->stage_slot;
    h->stage_slot ^= 1;
    cudaStream_t st = h->stream;
    const size_t bytes = size_t(h->P) * sizeof(float);
    if (!h->stage[s][0]) {
        CPM_TRY(dalloc(&h->stage[s][0], size_t(h->Palloc)));
        CPM_TRY(dalloc(&h->stage[s][1], size_t(h->Palloc)));
    }
    // the previous readback from this staging slot must have left the device
    CPM_CUDA(cudaStreamWaitEvent(st, h->stage_done[s], 0));
    ParticleArrays& p = state(h);
    if (ordered && !h->identity_order) {
        CPM_CUDA(cpm::launch_unpermute(p.x, p.id, h->P, h->stage[s][0], st));
        CPM_CUDA(cpm::launch_unpermute(p.y, p.id, h->P, h->stage[s][1], st));
    } else {
        CPM_CUDA(cudaMemcpyAsync(h->stage[s][0], p.x, bytes, cudaMemcpyDeviceToDevice, st));
        CPM_CUDA(cudaMemcpyAsync(h->stage[s][1], p.y, bytes, cudaMemcpyDeviceToDevice, st));
    }
    CPM_CUDA(cudaEventRecord(h->stage_ready[s], st));
    CPM_CUDA(cudaStreamWaitEvent(h->copy_stream, h->stage_ready[s], 0));
    CPM_CUDA(cudaMemcpyAsync(hx, h->stage[s][0], bytes, cudaMemcpyDeviceToHost, h->copy_stream));
    CPM_CUDA(cudaMemcpyAsync(hy, h->stage[s][1], bytes, cudaMemcpyDeviceToHost, h->copy_stream));
    CPM_CUDA(cudaEventRecord(h->stage_done[s], h->copy_stream));
    return issue_ticket(h, ticket);
}

// A ticket for everything enqueued on the copy stream so far.
int issue_ticket(cosmos_pm* h, uint64_t* ticket) {
    cudaEvent_t ev = nullptr;
    {
        std::lock_guard<std::mutex> lk(h->ticket_mu);
        if (!h->event_pool.empty()) {
            ev = h->event_pool.back();
            h->event_pool.pop_back();
        }
    }
    if (!ev) CPM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CPM_CUDA(cudaEventRecord(ev, h->copy_stream));
    std::lock_guard<std::mutex> lk(h->ticket_mu);
    *ticket = h->next_ticket++;
    h->tickets.emplace_back(*ticket, ev);
    return COSMOS_OK;
}

// Render buffers, blur weights and the running extremes, on first use.
int ensure_render(cosmos_pm* h) {
    if (h->rkern) return COSMOS_OK;
    const size_t NN = size_t(h->N) * h->N;
    const int R = h->blur_r;
    int rc = COSMOS_OK;
    if ((rc = dalloc(&h->blurred, NN)) || (rc = dalloc(&h->frame[0], NN)) || (rc = dalloc(&h->frame[1], NN)) ||
        (rc = dalloc(&h->rstate, 3)) || (rc = dalloc(&h->rext, 2)))
        return rc;
    for (int i = 0; i < 2; ++i) {
        CPM_CUDA(cudaEventCreateWithFlags(&h->frame_ready[i], cudaEventDisableTiming));
        CPM_CUDA(cudaEventCreateWithFlags(&h->frame_done[i], cudaEventDisableTiming));
    }
    std::vector<float> w(size_t(R) * R);
    cpm::render_weights(R, w.data());
    h->render_identity = cpm::render_is_identity(R, w.data());
    float* k = nullptr;
    if ((rc = dalloc(&k, w.size()))) return rc;
    if (cudaMemcpy(k, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(k);
        return cpm::fail(COSMOS_ERR_CUDA, "blur weights upload");
    }
    CPM_CUDA(cpm::render_init(h->rstate, h->rext, h->stream));
    h->rkern = k;
    return COSMOS_OK;
}

// Render the density of the current positions into device frame slot s.
int enqueue_render(cosmos_pm* h, int s) {
    CPM_TRY(ensure_render(h));
    if (!h->density_valid) {
        CPM_TRY(enqueue_prologue(h, h->stream));
        h->kernels_enqueued += 1;
    }
    CPM_CUDA(cpm::launch_render(h->rho, h->blurred, h->frame[s], h->rkern, h->blur_r, h->N, h->render_identity,
                                h->rstate, h->rext, h->stream));
    h->kernels_enqueued += 2;  // extremes (with the blur when there is one), power-law scale
    return COSMOS_OK;
}

int render_frame_impl(cosmos_pm* h, float* host) {
    if (!host) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    CPM_TRY(ensure_render(h));
    const int s = h->frame_slot;
    h->frame_slot ^= 1;
    CPM_CUDA(cudaStreamWaitEvent(h->stream, h->frame_done[s], 0));
    CPM_TRY(enqueue_render(h, s));
    CPM_CUDA(cudaMemcpyAsync(host, h->frame[s], size_t(h->N) * h->N * sizeof(float), cudaMemcpyDeviceToHost,
                             h->stream));
    CPM_CUDA(cudaEventRecord(h->frame_done[s], h->stream));
    CPM_CUDA(cudaStreamSynchronize(h->stream));
    return COSMOS_OK;
}

int frame_async_impl(cosmos_pm* h, float* host, uint64_t* ticket) {
    if (!host || !ticket) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    CPM_TRY(ensure_render(h));
    const int s = h->frame_slot;
    h->frame_slot ^= 1;
    // the previous copy out of this slot must have left the device
    CPM_CUDA(cudaStreamWaitEvent(h->stream, h->frame_done[s], 0));
    CPM_TRY(enqueue_render(h, s));
    CPM_CUDA(cudaEventRecord(h->frame_ready[s], h->stream));
    CPM_CUDA(cudaStreamWaitEvent(h->copy_stream, h->frame_ready[s], 0));
    CPM_CUDA(cudaMemcpyAsync(host, h->frame[s], size_t(h->N) * h->N * sizeof(float), cudaMemcpyDeviceToHost,
                             h->copy_stream));
    CPM_CUDA(cudaEventRecord(h->frame_done[s], h->copy_stream));
    return issue_ticket(h, ticket);
}

// Returns the event of a ticket still outstanding, or nullptr if it completed.
int ticket_query(cosmos_pm* h, uint64_t ticket, bool wait, int32_t* done) {
    cudaEvent_t ev = nullptr;
    {
        std::lock_guard<std::mutex> lk(h->ticket_mu);
        if (ticket == 0 || ticket >= h->next_ticket) return cpm::fail(COSMOS_ERR_INVALID, "unknown ticket");
        for (auto& t : h->tickets)
            if (t.first == ticket) ev = t.second;
    }
    if (!ev) {  // retired earlier
        *done = 1;
        return COSMOS_OK;
    }
    cudaError_t e = wait ? cudaEventSynchronize(ev) : cudaEventQuery(ev);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return COSMOS_OK;
    }
    if (e != cudaSuccess) return cpm::fail(COSMOS_ERR_CUDA, std::string("ticket: ") + cudaGetErrorString(e));
    *done = 1;
    // retire this and every older ticket (same stream, completed in order)
    std::lock_guard<std::mutex> lk(h->ticket_mu);
    while (!h->tickets.empty() && h->tickets.front().first <= ticket) {
        h->event_pool.push_back(h->tickets.front().second);
        h->tickets.pop_front();
    }
    return COSMOS_OK;
}

}  // namespace

// ================================= C ABI ============================================
extern "C" {

void cosmos_pm_default_config(cosmos_pm_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->lattice_n = 2048;
    c->deposit = COSMOS_DEPOSIT_CIC;
    c->dt = 1e-3f;
    c->gravity_multiplier = 1.0f;
    c->num_particles = 0;
    c->device = 0;
    c->force_mode = COSMOS_FORCE_GRADIENT;
    c->sort_interval = -1;
    c->sort_granularity = -1;
    c->use_graph = 1;
    c->blur_r = 3;
}

int cosmos_pm_create(const cosmos_pm_config* cfg, cosmos_pm** out) { return create_impl(cfg, out); }

int cosmos_pm_destroy(cosmos_pm* h) {
    if (!h) return COSMOS_OK;
    destroy_all(h);
    delete h;
    return COSMOS_OK;
}

int cosmos_pm_set_particles(cosmos_pm* h, const float* x, const float* y, const float* xo, const float* yo,
                            const float* m, int64_t count, int64_t offset) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, set_particles_impl(h, x, y, xo, yo, m, count, offset));
}

int cosmos_pm_generate(cosmos_pm* h, const cosmos_ic_params* ic, int64_t count, int64_t offset) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, generate_impl(h, ic, count, offset));
}

int cosmos_pm_get_particles(cosmos_pm* h, float* x, float* y, float* xo, float* yo, float* m, int64_t count,
                            int64_t offset) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, get_particles_impl(h, x, y, xo, yo, m, count, offset));
}

int cosmos_pm_clear(cosmos_pm* h) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        ParticleArrays& p = state(h);
        for (float* f : {p.x, p.y, p.xo, p.yo}) CPM_CUDA(cpm::launch_fill(f, -10.0f, h->P, h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        state_rewritten(h);
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_step(cosmos_pm* h, int32_t nsteps) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    if (nsteps < 0) return finish(h, cpm::fail(COSMOS_ERR_INVALID, "nsteps < 0"));
    DeviceGuard g(h->device);
    for (int i = 0; i < nsteps;) {
        const bool multi = can_enqueue_multi(h, nsteps - i);
        const int rc = multi ? enqueue_multi(h) : enqueue_step(h);
        if (rc != COSMOS_OK) return finish(h, rc);
        i += multi ? kGraphSteps : 1;
    }
    return COSMOS_OK;
}

int cosmos_pm_synchronize(cosmos_pm* h) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->copy_stream));
        {  // a copy wait of a step kernel that gave up
            int st = 0;
            CPM_CUDA(cudaMemcpy(&st, h->wait_status, sizeof(int), cudaMemcpyDeviceToHost));
            if (st) {
                CPM_CUDA(cudaMemset(h->wait_status, 0, sizeof(int)));
                return cpm::fail(COSMOS_ERR_TIMEOUT,
                                 st == 3 ? "a tensor-map load destination was off the 128-byte grid (tile skipped)"
                                         : "a step kernel's copy wait (bulk or tensor-map load) timed out");
            }
        }
        if (h->tc_status) {  // a tensor-core completion wait that gave up
            int st = 0;
            CPM_CUDA(cudaMemcpy(&st, h->tc_status, sizeof(int), cudaMemcpyDeviceToHost));
            if (st) {
                CPM_CUDA(cudaMemset(h->tc_status, 0, sizeof(int)));
                return cpm::fail(COSMOS_ERR_TIMEOUT,
                                 st >= 2 ? "tensor-core column pass: an MMA completion wait timed out twice; the "
                                           "CTA's tensor memory was left allocated"
                                         : "tensor-core column pass: an MMA completion wait timed out");
            }
        }
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_get_positions_async(cosmos_pm* h, float* hx, float* hy, int32_t ordered, uint64_t* ticket) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, positions_async_impl(h, hx, hy, ordered, ticket));
}

int cosmos_pm_render_frame(cosmos_pm* h, float* host_frame) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, render_frame_impl(h, host_frame));
}

int cosmos_pm_get_frame_async(cosmos_pm* h, float* host_frame, uint64_t* ticket) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, frame_async_impl(h, host_frame, ticket));
}

int cosmos_pm_poll(cosmos_pm* h, uint64_t ticket, int32_t* done) {
    if (!h || !done) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    return ticket_query(h, ticket, false, done);
}

int cosmos_pm_wait(cosmos_pm* h, uint64_t ticket) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    int32_t done = 0;
    return finish(h, ticket_query(h, ticket, true, &done));
}

int cosmos_pm_run_stage(cosmos_pm* h, int32_t stage_id) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        cudaStream_t st = h->stream;
        ParticleArrays& p = state(h);
        switch (stage_id) {
            case COSMOS_STAGE_DEPOSIT:
                CPM_CUDA(cudaMemsetAsync(h->rho, 0, size_t(h->N) * h->N * sizeof(float), st));
                CPM_CUDA(cpm::launch_deposit_global(p, h->P, h->rho, h->N, h->cic, h->nsm, st));
                h->density_valid = true;
                break;
            case COSMOS_STAGE_POTENTIAL:
                CPM_CUDA(cpm::launch_conv_passes(h->N, h->rho, h->spec, h->kq, h->phi, h->tw, st));
                break;
            case COSMOS_STAGE_FORCE:
                // gradient mode: from the potential field; spectral modes: from the density
                if (is_spectral(h->cfg.force_mode))
                    CPM_TRY(launch_spectral(h, st));
                else
                    CPM_CUDA(cpm::launch_gradient(h->phi, h->force, h->N, h->cfg.gravity_multiplier, st));
                break;
            case COSMOS_STAGE_INTEGRATE:
                CPM_CUDA(cpm::launch_integrate(h->force, p, h->P, h->N, h->cic, h->cfg.dt, h->nsm, st));
                h->density_valid = false;  // positions moved; the density is stale
                ++h->steps_taken;
                break;
            default:
                return cpm::fail(COSMOS_ERR_INVALID, "unknown stage");
        }
        CPM_CUDA(cudaStreamSynchronize(st));
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_get_field(cosmos_pm* h, int32_t field, float* host) {
    if (!h || !host) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        const size_t NN = size_t(h->N) * h->N;
        const void* src = nullptr;
        size_t bytes = NN * sizeof(float);
        if (field == COSMOS_FIELD_DENSITY) src = h->rho;
        else if (field == COSMOS_FIELD_POTENTIAL) src = h->phi;
        else if (field == COSMOS_FIELD_FORCE) { src = h->force; bytes *= 2; }
        else return cpm::fail(COSMOS_ERR_INVALID, "unknown field");
        CPM_CUDA(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_set_field(cosmos_pm* h, int32_t field, const float* host) {
    if (!h || !host) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        const size_t NN = size_t(h->N) * h->N;
        void* dst = nullptr;
        size_t bytes = NN * sizeof(float);
        if (field == COSMOS_FIELD_DENSITY) dst = h->rho;
        else if (field == COSMOS_FIELD_POTENTIAL) dst = h->phi;
        else if (field == COSMOS_FIELD_FORCE) { dst = h->force; bytes *= 2; }
        else return cpm::fail(COSMOS_ERR_INVALID, "unknown field");
        CPM_CUDA(cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        if (field == COSMOS_FIELD_DENSITY) h->density_valid = true;  // the caller supplies the density
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_sort(cosmos_pm* h, uint32_t* perm) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        CPM_TRY(sort_now(h));
        if (perm)
            CPM_CUDA(cudaMemcpyAsync(perm, state(h).id, size_t(h->P) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                     h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_tile_keys(cosmos_pm* h, const float* x, const float* y, int64_t count, int32_t gran, uint32_t* keys) {
    if (!h || !x || !y || !keys) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        if (count <= 0) return COSMOS_OK;
        if (gran < 0 || (h->N >> gran) < 1 || gran > 13) return cpm::fail(COSMOS_ERR_INVALID, "granularity");
        cudaStream_t st = h->stream;
        float *dx = nullptr, *dy = nullptr;
        uint32_t* dk = nullptr;
        if (cudaMallocAsync(&dx, count * sizeof(float), st) != cudaSuccess ||
            cudaMallocAsync(&dy, count * sizeof(float), st) != cudaSuccess ||
            cudaMallocAsync(&dk, count * sizeof(uint32_t), st) != cudaSuccess) {
            cudaGetLastError();
            cudaFreeAsync(dx, st);
            cudaFreeAsync(dy, st);
            cudaFreeAsync(dk, st);
            return cpm::fail(COSMOS_ERR_NOMEM, "staging allocation");
        }
        CPM_CUDA(cudaMemcpyAsync(dx, x, count * sizeof(float), cudaMemcpyHostToDevice, st));
        CPM_CUDA(cudaMemcpyAsync(dy, y, count * sizeof(float), cudaMemcpyHostToDevice, st));
        CPM_CUDA(cpm::launch_tile_keys(dx, dy, count, h->N, gran, dk, st));
        CPM_CUDA(cudaMemcpyAsync(keys, dk, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CPM_CUDA(cudaFreeAsync(dx, st));
        CPM_CUDA(cudaFreeAsync(dy, st));
        CPM_CUDA(cudaFreeAsync(dk, st));
        CPM_CUDA(cudaStreamSynchronize(st));
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_diagnostics(cosmos_pm* h, double* ke, double* pe, double* px, double* py) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        double out[4];
        CPM_CUDA(cpm::launch_diagnostics(state(h), h->P, h->phi, h->N, h->cfg.dt, h->diag, h->stream));
        CPM_CUDA(cudaMemcpyAsync(out, h->diag, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
        CPM_CUDA(cudaStreamSynchronize(h->stream));
        if (ke) *ke = out[0];
        if (pe) *pe = out[1];
        if (px) *px = out[2];
        if (py) *py = out[3];
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_set_profiling(cosmos_pm* h, int32_t enabled) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    h->profiling = enabled != 0;
    h->have_times = false;
    return COSMOS_OK;
}

int cosmos_pm_stage_times(cosmos_pm* h, float* times, int32_t* n) {
    if (!h || !times || !n) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(h->device);
    auto impl = [&]() -> int {
        if (!h->have_times) return cpm::fail(COSMOS_ERR_STATE, "no profiled step yet");
        CPM_CUDA(cudaEventSynchronize(h->ev[kEvEnd]));
        // entries: prologue deposit, fft convolution (3 passes), force, fused step, sort
        float t[kNumTimes] = {0};
        if (h->prof_prologue) CPM_CUDA(cudaEventElapsedTime(&t[kTPrologue], h->ev[kEvPrologue], h->ev[kEvSort]));
        if (h->prof_sorted) CPM_CUDA(cudaEventElapsedTime(&t[kTSort], h->ev[kEvSort], h->ev[kEvFft]));
        CPM_CUDA(cudaEventElapsedTime(&t[kTFft], h->ev[kEvFft], h->ev[kEvForce]));
        CPM_CUDA(cudaEventElapsedTime(&t[kTForce], h->ev[kEvForce], h->ev[kEvFused]));
        CPM_CUDA(cudaEventElapsedTime(&t[kTFused], h->ev[kEvFused], h->ev[kEvEnd]));
        const int cnt = *n < kNumTimes ? *n : kNumTimes;
        for (int i = 0; i < cnt; ++i) times[i] = t[i];
        *n = cnt;
        return COSMOS_OK;
    };
    return finish(h, impl());
}

int cosmos_pm_stream(cosmos_pm* h, uint64_t* stream) {
    if (!h || !stream) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *stream = reinterpret_cast<uint64_t>(h->stream);
    return COSMOS_OK;
}

int cosmos_pm_launches_per_step(cosmos_pm* h, int32_t* launches) {
    if (!h || !launches) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *launches = step_launches(h);
    return COSMOS_OK;
}

int cosmos_pm_kernels_launched(cosmos_pm* h, int64_t* launches) {
    if (!h || !launches) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *launches = h->kernels_enqueued;
    return COSMOS_OK;
}

int cosmos_pm_checkpoint_save(cosmos_pm* h, const char* path) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, checkpoint_save_impl(h, path));
}

int cosmos_pm_checkpoint_load(cosmos_pm* h, const char* path) {
    if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(h->device);
    return finish(h, checkpoint_load_impl(h, path));
}

int cosmos_pm_steps_taken(cosmos_pm* h, int64_t* steps) {
    if (!h || !steps) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *steps = h->steps_taken;
    return COSMOS_OK;
}

int cosmos_pm_test_hook(cosmos_pm* h, int32_t hook, int64_t value) {
    switch (hook) {
        case COSMOS_TEST_FAIL_ALLOC:
            cpm::g_fail_alloc_countdown.store(value > 0 ? value : 0);
            return COSMOS_OK;
        case COSMOS_TEST_TC_SKIP_MMA:
        case COSMOS_TEST_COPY_WAIT: {
            if (!h) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
            if (hook == COSMOS_TEST_TC_SKIP_MMA && !is_tc(h->cfg.force_mode))
                return finish(h, cpm::fail(COSMOS_ERR_STATE, "not a tensor-core force mode"));
            DeviceGuard g(h->device);
            cudaStreamSynchronize(h->stream);
            if (hook == COSMOS_TEST_TC_SKIP_MMA)
                h->tc.skip_mma = value != 0;
            else
                h->copy_tx_extra = value != 0 ? 16u : 0u;
            for (auto* set : {&h->graph, &h->graph_multi, &h->graph_prof})  // captured steps hold the old argument
                for (auto& row : *set)
                    for (auto& gr : row)
                        if (gr) {
                            cudaGraphExecDestroy(gr);
                            gr = nullptr;
                        }
            return COSMOS_OK;
        }
        default:
            return cpm::fail(COSMOS_ERR_INVALID, "unknown test hook");
    }
}

int cosmos_pm_host_alloc(int64_t bytes, void** out) {
    if (!out) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *out = nullptr;
    if (bytes <= 0) return cpm::fail(COSMOS_ERR_INVALID, "bytes must be positive");
    if (cudaMallocHost(out, size_t(bytes)) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return cpm::fail(COSMOS_ERR_NOMEM, "page-locked allocation of " + std::to_string(bytes) + " bytes failed");
    }
    return COSMOS_OK;
}

int cosmos_pm_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) return cpm::fail(COSMOS_ERR_CUDA, "cudaFreeHost");
    return COSMOS_OK;
}

const char* cosmos_pm_last_error(cosmos_pm* h) {
    if (h) return h->err.c_str();
    return cpm::last_error_message();
}

const char* cosmos_pm_version(void) { return "0.1.0"; }

}  // extern "C"
