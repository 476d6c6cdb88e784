// Ensemble of independent particle-mesh simulations on one GPU
// (include/cosmos_ensemble.h).
//
// Simulations are grouped by lattice size N into classes.  A class stores its
// simulations back to back: one particle state (segments of P_s particles,
// 16-byte aligned), S_N lattices of each field, one filter and twiddle table.
// Every pass of the step covers the whole class in one launch:
//   force passes   the FFT kernels with gridDim.y = S_N (pm_fft.cu batches)
//   fused step     k_fused_tiles over the class's work items; an item carries
//                  its simulation index and addresses that lattice
//   tile sort      keys sim * (T^2 + 1) + tile, one stable radix sort per
//                  class, so each simulation's segment stays in place
// The classes run on their own streams, forked from and joined back into the
// ensemble stream, and the whole step is captured as one CUDA graph.
//
// The reference has no ensemble (one Universe<K> per process,
// CosmosCuda.cuh:830-1428); each simulation here takes the step of a
// cosmos_pm handle with the same configuration and the tile path.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cosmos_ensemble.h"
#include "pm_common.cuh"
#include "pm_internal.h"

using cpm::ParticleArrays;

namespace {

struct EnsClass {
    int N = 0, gran = 5, nsims = 0, sort_bits = 0, tiles_grid = 0;
    std::vector<int> sims;      // global simulation indices, in segment order
    std::vector<int64_t> off;   // segment offsets (nsims + 1)
    int64_t P = 0;
    int64_t* off_dev = nullptr;
    ParticleArrays buf[2]{};
    int cur = 0;
    bool identity_order = true;
    uint32_t* pos = nullptr;
    bool pos_valid = false;
    float* rho = nullptr;
    float2* spec = nullptr;
    float* phi = nullptr;
    float2* force = nullptr;
    float2* spec2 = nullptr;
    float2* edge = nullptr;
    float* kq = nullptr;
    float2* tw = nullptr;
    cpm::RadixScratch rs{};
    uint32_t *tstart = nullptr, *tend = nullptr, *n_items = nullptr;
    int* status = nullptr;  // step kernels: a bounded copy wait (bulk / tensor-map loads) that ran out
    cpm::SpectralMaps maps{};
    bool have_maps = false;
    cpm::WorkItem* items = nullptr;
    size_t max_items = 0;
    int item_size = cpm::kItemMax;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

}  // namespace

struct cosmos_ensemble {
    cosmos_ensemble_config cfg{};
    int device = 0, nsm = 0, cic = 0, sort_interval = 32;
    std::vector<EnsClass> classes;
    std::vector<std::pair<int, int>> where;  // sim -> (class, local index)
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr;
    int item_size = cpm::kItemMax;  // work-item size of every class (the classes run concurrently)
    bool density_valid = false, sort_due = true;
    int64_t steps_since_sort = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // by buffer parity (all classes flip together)
    // persistent step: grid size, barrier counter and status word, test hook
    int persistent_grid = 0;
    unsigned* barrier = nullptr;
    int* pstatus = nullptr;
    int skip_arrive = 0;
    cpm::EnsStepArgs* pargs = nullptr;  // device: the step's arguments for buffer parity 0 and 1
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

int finish(cosmos_ensemble* e, int rc) {
    if (rc != COSMOS_OK && e) e->err = cpm::last_error_message();
    return rc;
}

template <class T>
int dalloc(T** p, size_t n) {
    if (n == 0) n = 1;
    if (cpm::alloc_should_fail()) {
        *p = nullptr;
        return cpm::fail(COSMOS_ERR_NOMEM, "device allocation failed (injected by COSMOS_TEST_FAIL_ALLOC)");
    }
    if (cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return cpm::fail(COSMOS_ERR_NOMEM, "device allocation of " + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    return COSMOS_OK;
}

ParticleArrays segment(const ParticleArrays& a, int64_t off) {
    return ParticleArrays{a.x + off, a.y + off, a.xo + off, a.yo + off, a.m + off, a.id + off};
}

int bits_for(uint64_t max_key) {
    int b = 1;
    while ((uint64_t(1) << b) <= max_key) ++b;
    return b;
}

void destroy_class(EnsClass& c) {
    for (auto& b : c.buf)
        for (void* p : {(void*)b.x, (void*)b.y, (void*)b.xo, (void*)b.yo, (void*)b.m, (void*)b.id}) cudaFree(p);
    for (void* p : {(void*)c.off_dev, (void*)c.pos, (void*)c.rho, (void*)c.spec, (void*)c.phi, (void*)c.force,
                    (void*)c.spec2, (void*)c.edge, (void*)c.kq, (void*)c.tw, (void*)c.rs.keys[0],
                    (void*)c.rs.keys[1], (void*)c.rs.vals[0], (void*)c.rs.vals[1], (void*)c.rs.counts,
                    (void*)c.tstart, (void*)c.tend, (void*)c.n_items, (void*)c.items, (void*)c.status})
        cudaFree(p);
    if (c.done) cudaEventDestroy(c.done);
    if (c.stream) cudaStreamDestroy(c.stream);
}

void destroy_all(cosmos_ensemble* e) {
    DeviceGuard g(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto& c : e->classes) {
        if (c.stream) cudaStreamSynchronize(c.stream);
    }
    for (auto& gr : e->graph)
        if (gr) cudaGraphExecDestroy(gr);
    for (auto& c : e->classes) destroy_class(c);
    cudaFree(e->barrier);
    cudaFree(e->pstatus);
    cudaFree(e->pargs);
    if (e->start) cudaEventDestroy(e->start);
    if (e->stream) cudaStreamDestroy(e->stream);
}

int alloc_class(cosmos_ensemble* e, EnsClass& c) {
    const size_t NN = size_t(c.N) * c.N;
    const size_t S = size_t(c.nsims);
    const size_t Pa = size_t(c.P);
    int rc = COSMOS_OK;
    for (auto& b : c.buf)
        if ((rc = dalloc(&b.x, Pa)) || (rc = dalloc(&b.y, Pa)) || (rc = dalloc(&b.xo, Pa)) || (rc = dalloc(&b.yo, Pa)) ||
            (rc = dalloc(&b.m, Pa)) || (rc = dalloc(&b.id, Pa)))
            return rc;
    c.rs.grid = cpm::radix_grid(c.P, e->nsm);
    const size_t nranges = cpm::tile_range_elems(c.N, c.gran, c.nsims);
    c.item_size = e->item_size;
    c.max_items = cpm::max_work_items(c.P, int(nranges), c.item_size);
    if ((rc = dalloc(&c.off_dev, S + 1)) || (rc = dalloc(&c.pos, Pa)) || (rc = dalloc(&c.rho, S * NN)) ||
        (rc = dalloc(&c.spec, S * NN / 2)) || (rc = dalloc(&c.force, S * NN)) ||
        (rc = dalloc(&c.kq, size_t(c.N / 2 + 1) * (c.N / 2 + 1))) || (rc = dalloc(&c.tw, size_t(c.N))) ||
        (rc = dalloc(&c.rs.keys[0], Pa)) || (rc = dalloc(&c.rs.keys[1], Pa)) || (rc = dalloc(&c.rs.vals[0], Pa)) ||
        (rc = dalloc(&c.rs.vals[1], Pa)) || (rc = dalloc(&c.rs.counts, cpm::radix_counts_elems(c.rs.grid))) ||
        (rc = dalloc(&c.tstart, nranges)) || (rc = dalloc(&c.tend, nranges)) || (rc = dalloc(&c.n_items, 1)) ||
        (rc = dalloc(&c.items, c.max_items)) || (rc = dalloc(&c.status, 1)))
        return rc;
    if (e->cfg.force_mode == COSMOS_FORCE_SPECTRAL) {
        if ((rc = dalloc(&c.spec2, S * NN / 2)) || (rc = dalloc(&c.edge, S * size_t(c.N / 2) * 4)))
            return rc;
    } else if ((rc = dalloc(&c.phi, S * NN))) {
        return rc;
    }
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming) != cudaSuccess)
        return cpm::fail(COSMOS_ERR_CUDA, "class streams / events");
    cudaStream_t st = e->stream;
    CPM_CUDA(cudaMemcpyAsync(c.off_dev, c.off.data(), (S + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    for (auto& b : c.buf)
        for (float* f : {b.x, b.y, b.xo, b.yo, b.m}) CPM_CUDA(cudaMemsetAsync(f, 0, Pa * sizeof(float), st));
    CPM_CUDA(cpm::launch_iota(c.buf[0].id, c.P, st));
    CPM_CUDA(cudaMemsetAsync(c.rho, 0, S * NN * sizeof(float), st));
    CPM_CUDA(cudaMemsetAsync(c.force, 0, S * NN * sizeof(float2), st));
    CPM_CUDA(cudaMemsetAsync(c.n_items, 0, sizeof(uint32_t), st));
    CPM_CUDA(cudaMemsetAsync(c.status, 0, sizeof(int), st));
    CPM_CUDA(cpm::prepare_conv_passes(c.N));
    if (e->cfg.force_mode == COSMOS_FORCE_SPECTRAL) {
        CPM_CUDA(cpm::prepare_spectral_passes(c.N));
        if (c.N >= 256) {  // the class's lattices as one batch of tensor-map tiles
            CPM_CUDA(cpm::make_spectral_maps(c.N, c.rho, c.spec, c.nsims, &c.maps));
            c.have_maps = true;
        }
    }
    CPM_CUDA(cpm::prepare_tile_kernels(c.gran, e->cic, e->nsm, &c.tiles_grid));
    CPM_TRY(cpm::build_filter(c.N, e->cic, c.kq, c.tw, st));
    const uint64_t T = uint64_t(c.N >> c.gran);
    c.sort_bits = bits_for(uint64_t(c.nsims) * (T * T + 1) - 1);
    return COSMOS_OK;
}

// The persistent step's arguments for both buffer parities (every class
// flips its particle buffers together at a sort), in device memory.
int upload_step_args(cosmos_ensemble* e) {
    cpm::EnsStepArgs a[2] = {};
    for (int parity = 0; parity < 2; ++parity) {
        cpm::EnsStepArgs& x = a[parity];
        x.nclasses = int(e->classes.size());
        x.cic = e->cic;
        x.g = e->cfg.gravity_multiplier;
        x.dt = e->cfg.dt;
        x.barrier = e->barrier;
        x.status = e->pstatus;
        x.skip_arrive = e->skip_arrive;
        for (int i = 0; i < x.nclasses; ++i) {
            EnsClass& c = e->classes[i];
            x.cls[i] = cpm::EnsStepClass{c.N,    c.nsims, c.rho, c.spec,  c.spec2,  c.edge,
                                         c.kq,   c.force, c.tw,  c.items, c.n_items, c.buf[parity]};
        }
    }
    CPM_CUDA(cudaMemcpy(e->pargs, a, sizeof(a), cudaMemcpyHostToDevice));
    return COSMOS_OK;
}

int create_impl(const cosmos_ensemble_config* cfg, const int32_t* ns, const int64_t* ps, cosmos_ensemble** out) {
    if (!cfg || !ns || !ps || !out) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *out = nullptr;
    const int S = cfg->num_sims;
    if (S < 1 || S > 4096) return cpm::fail(COSMOS_ERR_INVALID, "num_sims must be in [1, 4096]");
    if (cfg->deposit != COSMOS_DEPOSIT_NGP && cfg->deposit != COSMOS_DEPOSIT_CIC)
        return cpm::fail(COSMOS_ERR_INVALID, "deposit must be COSMOS_DEPOSIT_NGP or COSMOS_DEPOSIT_CIC");
    if (cfg->force_mode != COSMOS_FORCE_GRADIENT && cfg->force_mode != COSMOS_FORCE_SPECTRAL)
        return cpm::fail(COSMOS_ERR_INVALID, "force_mode must be COSMOS_FORCE_GRADIENT or COSMOS_FORCE_SPECTRAL");
    if (!std::isfinite(cfg->dt) || !std::isfinite(cfg->gravity_multiplier))
        return cpm::fail(COSMOS_ERR_INVALID, "dt and gravity_multiplier must be finite");
    std::map<int, std::vector<int>> by_n;
    for (int s = 0; s < S; ++s) {
        const int N = ns[s];
        if (N < 16 || N > 8192 || (N & (N - 1)) != 0)
            return cpm::fail(COSMOS_ERR_INVALID, "lattice_n[" + std::to_string(s) + "] must be a power of two in [16, 8192]");
        if (ps[s] < 0 || ps[s] % 4 != 0)
            return cpm::fail(COSMOS_ERR_INVALID, "num_particles[" + std::to_string(s) + "] must be a non-negative multiple of 4");
        by_n[N].push_back(s);
    }
    int ndev = 0;
    CPM_CUDA(cudaGetDeviceCount(&ndev));
    if (cfg->device < 0 || cfg->device >= ndev) return cpm::fail(COSMOS_ERR_INVALID, "device ordinal out of range");

    cosmos_ensemble* e = new cosmos_ensemble;
    e->cfg = *cfg;
    e->device = cfg->device;
    e->cic = cfg->deposit == COSMOS_DEPOSIT_CIC;
    e->sort_interval = cfg->sort_interval > 0 ? cfg->sort_interval : 32;
    e->where.resize(S);
    DeviceGuard guard(e->device);
    auto bail = [&](int rc) {
        destroy_all(e);
        delete e;
        return rc;
    };
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, e->device) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "device query"));
    e->nsm = prop.multiProcessorCount;
    int64_t total_particles = 0;
    for (int s = 0; s < S; ++s) total_particles += ps[s];
    e->item_size = cpm::work_item_size(total_particles, e->nsm);
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->start, cudaEventDisableTiming) != cudaSuccess)
        return bail(cpm::fail(COSMOS_ERR_CUDA, "stream creation"));
    e->classes.resize(by_n.size());
    int ci = 0;
    for (auto& kv : by_n) {
        EnsClass& c = e->classes[ci];
        c.N = kv.first;
        c.gran = c.N >= 64 ? 5 : 4;
        c.sims = kv.second;
        c.nsims = int(c.sims.size());
        if (uint64_t(c.nsims) * (uint64_t(c.N >> c.gran) * (c.N >> c.gran) + 1) > 0xFFFFFFFFull)
            return bail(cpm::fail(COSMOS_ERR_INVALID, "too many simulations of one lattice size for 32-bit keys"));
        c.off.assign(c.nsims + 1, 0);
        for (int j = 0; j < c.nsims; ++j) {
            c.off[j + 1] = c.off[j] + ps[c.sims[j]];
            e->where[c.sims[j]] = {ci, j};
        }
        c.P = c.off[c.nsims];
        if (c.P > int64_t(0xFFFFFFF0u)) return bail(cpm::fail(COSMOS_ERR_INVALID, "too many particles in one lattice class"));
        const int rc = alloc_class(e, c);
        if (rc != COSMOS_OK) return bail(rc);
        ++ci;
    }
    if (cfg->persistent_step) {
        if (cfg->force_mode != COSMOS_FORCE_SPECTRAL || e->classes.size() > size_t(cpm::kEnsMaxClasses))
            return bail(cpm::fail(COSMOS_ERR_INVALID, "persistent_step needs the spectral force and at most 8 lattice sizes"));
        for (auto& c : e->classes)
            if (!cpm::ensemble_step_supported(c.N))
                return bail(cpm::fail(COSMOS_ERR_INVALID, "persistent_step supports lattices of 128 to 1024"));
        int rc = COSMOS_OK;
        if ((rc = dalloc(&e->barrier, 1)) || (rc = dalloc(&e->pstatus, 1)) || (rc = dalloc(&e->pargs, 2)))
            return bail(rc);
        if (cudaMemsetAsync(e->pstatus, 0, sizeof(int), e->stream) != cudaSuccess ||
            cpm::prepare_ensemble_step(e->nsm, &e->persistent_grid) != cudaSuccess)
            return bail(cpm::fail(COSMOS_ERR_CUDA, "persistent step setup"));
        if ((rc = upload_step_args(e)) != COSMOS_OK) return bail(rc);
    }
    if (cudaStreamSynchronize(e->stream) != cudaSuccess) return bail(cpm::fail(COSMOS_ERR_CUDA, "create sync"));
    *out = e;
    return COSMOS_OK;
}

// ---- the step ---------------------------------------------------------------------------------
int class_sort(cosmos_ensemble* e, EnsClass& c, cudaStream_t st) {
    ParticleArrays& src = c.buf[c.cur];
    ParticleArrays& dst = c.buf[c.cur ^ 1];
    CPM_CUDA(cpm::launch_tile_keys_sims(src.x, src.y, c.P, c.N, c.gran, c.off_dev, c.nsims, c.rs.keys[0], st));
    CPM_CUDA(cpm::launch_iota(c.rs.vals[0], c.P, st));
    int which = 0;
    CPM_CUDA(cpm::launch_radix_sort(c.rs, c.P, c.sort_bits, &which, st));
    CPM_CUDA(cpm::launch_permute(src, dst, c.rs.vals[which], c.P, st));
    CPM_CUDA(cpm::launch_build_items(c.rs.keys[which], dst.m, c.P, c.N, c.gran, c.tstart, c.tend, c.items, c.n_items,
                                     c.max_items, c.item_size, st, c.nsims));
    c.cur ^= 1;
    c.identity_order = false;
    c.pos_valid = false;
    (void)e;
    return COSMOS_OK;
}

// Density of the current positions, one deposit launch per simulation.
int class_prologue(cosmos_ensemble* e, EnsClass& c, cudaStream_t st) {
    const size_t NN = size_t(c.N) * c.N;
    CPM_CUDA(cudaMemsetAsync(c.rho, 0, size_t(c.nsims) * NN * sizeof(float), st));
    for (int j = 0; j < c.nsims; ++j)
        CPM_CUDA(cpm::launch_deposit_global(segment(c.buf[c.cur], c.off[j]), c.off[j + 1] - c.off[j],
                                            c.rho + size_t(j) * NN, c.N, e->cic, e->nsm, st));
    return COSMOS_OK;
}

// Force passes, density clear and fused step of one class on its stream.
int class_body(cosmos_ensemble* e, EnsClass& c) {
    cudaStream_t st = c.stream;
    const size_t NN = size_t(c.N) * c.N;
    const float g = e->cfg.gravity_multiplier;
    if (e->cfg.force_mode == COSMOS_FORCE_SPECTRAL) {
        CPM_CUDA(cpm::launch_spectral_force(c.N, c.rho, c.spec, c.spec2, c.edge, c.kq, c.force, c.tw, g, st, c.nsims,
                                            nullptr, nullptr,
                                            c.have_maps ? &c.maps : nullptr, c.status));
    } else {
        CPM_CUDA(cpm::launch_conv_passes(c.N, c.rho, c.spec, c.kq, c.phi, c.tw, st, c.nsims));
        CPM_CUDA(cpm::launch_gradient(c.phi, c.force, c.N, g, st, c.nsims));
    }
    CPM_CUDA(cudaMemsetAsync(c.rho, 0, size_t(c.nsims) * NN * sizeof(float), st));
    CPM_CUDA(cpm::launch_fused_tiles(c.items, c.n_items, c.buf[c.cur], c.force, c.rho, c.N, e->cic, e->cfg.dt, c.gran,
                                     c.tiles_grid, c.status, st));
    return COSMOS_OK;
}

// The step of every class as one persistent launch (pm_ensemble_step.cu),
// with the arguments of the current buffer parity (upload_step_args).
int step_body_persistent(cosmos_ensemble* e) {
    const int parity = e->classes.empty() ? 0 : e->classes[0].cur;
    CPM_CUDA(cpm::launch_ensemble_step(e->pargs + parity, e->barrier, e->persistent_grid, e->stream));
    return COSMOS_OK;
}

// All classes: fork from the ensemble stream, run concurrently, join back.
int step_body(cosmos_ensemble* e) {
    if (e->cfg.persistent_step) return step_body_persistent(e);
    CPM_CUDA(cudaEventRecord(e->start, e->stream));
    for (auto& c : e->classes) {
        CPM_CUDA(cudaStreamWaitEvent(c.stream, e->start, 0));
        CPM_TRY(class_body(e, c));
        CPM_CUDA(cudaEventRecord(c.done, c.stream));
    }
    for (auto& c : e->classes) CPM_CUDA(cudaStreamWaitEvent(e->stream, c.done, 0));
    return COSMOS_OK;
}

int get_graph(cosmos_ensemble* e, cudaGraphExec_t* out) {
    cudaGraphExec_t& g = e->graph[e->classes.empty() ? 0 : e->classes[0].cur];
    if (!g) {
        cudaGraph_t graph = nullptr;
        CPM_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = step_body(e);
        const cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
        if (rc != COSMOS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return cpm::fail(COSMOS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
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

int enqueue_step(cosmos_ensemble* e) {
    if (!e->density_valid) {
        for (auto& c : e->classes) CPM_TRY(class_prologue(e, c, e->stream));
        e->density_valid = true;
    }
    if (e->sort_due || e->steps_since_sort >= e->sort_interval) {
        for (auto& c : e->classes) CPM_TRY(class_sort(e, c, e->stream));
        e->sort_due = false;
        e->steps_since_sort = 0;
    }
    if (e->cfg.use_graph) {
        cudaGraphExec_t g = nullptr;
        CPM_TRY(get_graph(e, &g));
        CPM_CUDA(cudaGraphLaunch(g, e->stream));
    } else {
        CPM_TRY(step_body(e));
    }
    ++e->steps_since_sort;
    return COSMOS_OK;
}

// ---- particle I/O --------------------------------------------------------------------------------
int locate(cosmos_ensemble* e, int32_t sim, int64_t count, int64_t offset, EnsClass** cls, int64_t* base) {
    if (sim < 0 || sim >= int32_t(e->where.size())) return cpm::fail(COSMOS_ERR_RANGE, "simulation index out of range");
    EnsClass& c = e->classes[e->where[sim].first];
    const int j = e->where[sim].second;
    const int64_t Ps = c.off[j + 1] - c.off[j];
    if (count < 0 || offset < 0 || offset + count > Ps)
        return cpm::fail(COSMOS_ERR_RANGE, "particle range outside [0, " + std::to_string(Ps) + ")");
    *cls = &c;
    *base = c.off[j] + offset;
    return COSMOS_OK;
}

int ensure_pos(EnsClass& c, cudaStream_t st) {
    if (c.identity_order || c.pos_valid) return COSMOS_OK;
    CPM_CUDA(cpm::launch_invert(c.buf[c.cur].id, c.pos, c.P, st));
    c.pos_valid = true;
    return COSMOS_OK;
}

int set_impl(cosmos_ensemble* e, int32_t sim, const float* x, const float* y, const float* xo, const float* yo,
             const float* m, int64_t count, int64_t offset) {
    EnsClass* c = nullptr;
    int64_t base = 0;
    CPM_TRY(locate(e, sim, count, offset, &c, &base));
    if (count == 0) return COSMOS_OK;
    if (!x || !y) return cpm::fail(COSMOS_ERR_INVALID, "x and y are required");
    cudaStream_t st = e->stream;
    CPM_CUDA(cudaStreamSynchronize(st));
    ParticleArrays& p = c->buf[c->cur];
    const size_t bytes = size_t(count) * sizeof(float);
    const float* srcs[5] = {x, y, xo ? xo : x, yo ? yo : y, m};
    float* dsts[5] = {p.x, p.y, p.xo, p.yo, p.m};
    if (c->identity_order) {
        for (int i = 0; i < 5; ++i)
            if (srcs[i]) CPM_CUDA(cudaMemcpyAsync(dsts[i] + base, srcs[i], bytes, cudaMemcpyHostToDevice, st));
    } else {
        CPM_TRY(ensure_pos(*c, st));
        float* tmp = nullptr;
        if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) {
            cudaGetLastError();
            return cpm::fail(COSMOS_ERR_NOMEM, "staging allocation");
        }
        for (int i = 0; i < 5; ++i) {
            if (!srcs[i]) continue;
            CPM_CUDA(cudaMemcpyAsync(tmp, srcs[i], bytes, cudaMemcpyHostToDevice, st));
            CPM_CUDA(cpm::launch_scatter_by_id(tmp, c->pos, base, count, dsts[i], st));
        }
        CPM_CUDA(cudaFreeAsync(tmp, st));
    }
    CPM_CUDA(cudaStreamSynchronize(st));
    e->density_valid = false;
    e->sort_due = true;
    return COSMOS_OK;
}

int get_impl(cosmos_ensemble* e, int32_t sim, float* x, float* y, float* xo, float* yo, float* m, int64_t count,
             int64_t offset) {
    EnsClass* c = nullptr;
    int64_t base = 0;
    CPM_TRY(locate(e, sim, count, offset, &c, &base));
    if (count == 0) return COSMOS_OK;
    cudaStream_t st = e->stream;
    const ParticleArrays& p = c->buf[c->cur];
    const size_t bytes = size_t(count) * sizeof(float);
    float* dsts[5] = {x, y, xo, yo, m};
    const float* srcs[5] = {p.x, p.y, p.xo, p.yo, p.m};
    if (c->identity_order) {
        for (int i = 0; i < 5; ++i)
            if (dsts[i]) CPM_CUDA(cudaMemcpyAsync(dsts[i], srcs[i] + base, bytes, cudaMemcpyDeviceToHost, st));
    } else {
        CPM_TRY(ensure_pos(*c, st));
        float* tmp = nullptr;
        if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) {
            cudaGetLastError();
            return cpm::fail(COSMOS_ERR_NOMEM, "staging allocation");
        }
        for (int i = 0; i < 5; ++i) {
            if (!dsts[i]) continue;
            CPM_CUDA(cpm::launch_gather_by_id(srcs[i], c->pos, base, count, tmp, st));
            CPM_CUDA(cudaMemcpyAsync(dsts[i], tmp, bytes, cudaMemcpyDeviceToHost, st));
            CPM_CUDA(cudaStreamSynchronize(st));
        }
        CPM_CUDA(cudaFreeAsync(tmp, st));
    }
    CPM_CUDA(cudaStreamSynchronize(st));
    return COSMOS_OK;
}

}  // namespace

// ================================= C ABI ============================================
extern "C" {

void cosmos_ensemble_default_config(cosmos_ensemble_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->deposit = COSMOS_DEPOSIT_CIC;
    c->dt = 1e-3f;
    c->gravity_multiplier = 1.0f;
    c->force_mode = COSMOS_FORCE_SPECTRAL;
    c->sort_interval = 32;
    c->use_graph = 1;
}

int cosmos_ensemble_create(const cosmos_ensemble_config* cfg, const int32_t* lattice_n, const int64_t* num_particles,
                           cosmos_ensemble** out) {
    return create_impl(cfg, lattice_n, num_particles, out);
}

int cosmos_ensemble_destroy(cosmos_ensemble* e) {
    if (!e) return COSMOS_OK;
    destroy_all(e);
    delete e;
    return COSMOS_OK;
}

int cosmos_ensemble_set_particles(cosmos_ensemble* e, int32_t sim, const float* x, const float* y, const float* xo,
                                  const float* yo, const float* m, int64_t count, int64_t offset) {
    if (!e) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(e->device);
    return finish(e, set_impl(e, sim, x, y, xo, yo, m, count, offset));
}

int cosmos_ensemble_get_particles(cosmos_ensemble* e, int32_t sim, float* x, float* y, float* xo, float* yo, float* m,
                                  int64_t count, int64_t offset) {
    if (!e) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(e->device);
    return finish(e, get_impl(e, sim, x, y, xo, yo, m, count, offset));
}

int cosmos_ensemble_step(cosmos_ensemble* e, int32_t nsteps) {
    if (!e) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    if (nsteps < 0) return finish(e, cpm::fail(COSMOS_ERR_INVALID, "nsteps < 0"));
    DeviceGuard g(e->device);
    for (int i = 0; i < nsteps; ++i) {
        const int rc = enqueue_step(e);
        if (rc != COSMOS_OK) return finish(e, rc);
    }
    return COSMOS_OK;
}

int cosmos_ensemble_synchronize(cosmos_ensemble* e) {
    if (!e) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    DeviceGuard g(e->device);
    auto impl = [&]() -> int {
        CPM_CUDA(cudaStreamSynchronize(e->stream));
        if (e->pstatus) {  // a grid barrier of the persistent step that ran out
            int st = 0;
            CPM_CUDA(cudaMemcpy(&st, e->pstatus, sizeof(int), cudaMemcpyDeviceToHost));
            if (st) {
                CPM_CUDA(cudaMemset(e->pstatus, 0, sizeof(int)));
                return cpm::fail(COSMOS_ERR_TIMEOUT, "persistent ensemble step: a grid barrier wait timed out");
            }
        }
        for (auto& c : e->classes) {  // a copy wait of a step kernel that gave up
            int st = 0;
            CPM_CUDA(cudaMemcpy(&st, c.status, sizeof(int), cudaMemcpyDeviceToHost));
            if (st) {
                CPM_CUDA(cudaMemset(c.status, 0, sizeof(int)));
                return cpm::fail(COSMOS_ERR_TIMEOUT,
                                 st == 3 ? "a tensor-map load destination was off the 128-byte grid (tile skipped)"
                                         : "a step kernel's copy wait (bulk or tensor-map load) timed out");
            }
        }
        return COSMOS_OK;
    };
    return finish(e, impl());
}

int cosmos_ensemble_get_field(cosmos_ensemble* e, int32_t sim, int32_t field, float* host) {
    if (!e || !host) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    DeviceGuard g(e->device);
    auto impl = [&]() -> int {
        EnsClass* c = nullptr;
        int64_t base = 0;
        CPM_TRY(locate(e, sim, 0, 0, &c, &base));
        const int j = e->where[sim].second;
        const size_t NN = size_t(c->N) * c->N;
        const void* src = nullptr;
        size_t bytes = NN * sizeof(float);
        if (field == COSMOS_FIELD_DENSITY) {
            src = c->rho + j * NN;
        } else if (field == COSMOS_FIELD_POTENTIAL) {
            if (!c->phi) return cpm::fail(COSMOS_ERR_STATE, "no potential field in spectral force mode");
            src = c->phi + j * NN;
        } else if (field == COSMOS_FIELD_FORCE) {
            src = c->force + j * NN;
            bytes *= 2;
        } else {
            return cpm::fail(COSMOS_ERR_INVALID, "unknown field");
        }
        CPM_CUDA(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, e->stream));
        CPM_CUDA(cudaStreamSynchronize(e->stream));
        return COSMOS_OK;
    };
    return finish(e, impl());
}

int cosmos_ensemble_launches_per_step(cosmos_ensemble* e, int32_t* launches) {
    if (!e || !launches) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    const int force = e->cfg.force_mode == COSMOS_FORCE_SPECTRAL ? cpm::spectral_launches_per_step()
                                                                 : cpm::conv_launches_per_step() + 1;
    *launches = e->cfg.persistent_step ? 1 : int32_t(e->classes.size()) * (force + 1);
    return COSMOS_OK;
}

int cosmos_ensemble_test_barrier(cosmos_ensemble* e, int32_t value) {
    if (!e) return cpm::fail(COSMOS_ERR_INVALID, "null handle");
    if (!e->cfg.persistent_step) return finish(e, cpm::fail(COSMOS_ERR_STATE, "not a persistent-step ensemble"));
    DeviceGuard g(e->device);
    cudaStreamSynchronize(e->stream);
    e->skip_arrive = value != 0;
    return finish(e, upload_step_args(e));
}

int cosmos_ensemble_stream(cosmos_ensemble* e, uint64_t* stream) {
    if (!e || !stream) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    *stream = reinterpret_cast<uint64_t>(e->stream);
    return COSMOS_OK;
}

const char* cosmos_ensemble_last_error(cosmos_ensemble* e) {
    if (e) return e->err.c_str();
    return cpm::last_error_message();
}

}  // extern "C"
