// Autotuner of the step's launch shapes (cosmos_pm_autotune, include/cosmos_pm.h).
//
// The fused step kernel stages a tile's force window and deposit window in
// shared memory, so its speed depends on the tile edge (the sort key
// granularity), on how far particles drift from their tile between re-sorts
// (the sort cadence; the sort itself costs about three fused steps), on the
// size of its work items and on how many CTAs share an SM; the spectral
// column pass has two launch shapes (one or two radix-16 butterflies per
// thread).  The best choice depends on the lattice, the particle count and
// how clustered the state is, so it is measured on the caller's own state:
// every candidate runs on a temporary handle, graph-launched, timed with CUDA
// events on the handle's stream.  The library's defaults are timed first; the
// search is coordinate-wise: tile edge x cadence, then the work-item size, the
// fused kernel's CTAs per SM and the column-pass shape, each with the best of
// the ones before, and a candidate is taken only when it is more than 1.5%
// faster than the best so far.  Results are
// cached in a plain text file, one line per key:
//     v2 N=<n> logP2=<2*log2(P) rounded> deposit=<0|1> force=<mode> gpu=<name>|
//         <gran> <interval> <item_size> <ctas_per_sm> <fft_shape> <ms>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace {

std::mutex g_cache_mu;

std::string cache_key(const cosmos_pm_config& c, const char* gpu) {
    const int logp2 = c.num_particles > 0 ? int(std::lround(2.0 * std::log2(double(c.num_particles)))) : 0;
    std::ostringstream k;
    k << "v2 N=" << c.lattice_n << " logP2=" << logp2 << " deposit=" << c.deposit << " force=" << c.force_mode
      << " gpu=" << gpu;
    return k.str();
}

// The tuned fields of a configuration, as one cache record.
struct Choice {
    int gran = 5, interval = 32, item = 0, ctas = 0, fft = 0;
    float ms = 0.0f;
};

void apply(const Choice& ch, cosmos_pm_config* c) {
    c->sort_granularity = ch.gran;
    c->sort_interval = ch.interval;
    c->item_size = ch.item;
    c->fused_ctas_per_sm = ch.ctas;
    c->fft_shape = ch.fft;
}

bool cache_lookup(const char* path, const std::string& key, Choice* out) {
    if (!path) return false;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ifstream f(path);
    std::string line;
    bool hit = false;
    while (std::getline(f, line)) {  // the last entry of a key wins
        const size_t bar = line.rfind('|');
        if (bar == std::string::npos || line.compare(0, bar, key) != 0 || bar != key.size()) continue;
        std::istringstream v(line.substr(bar + 1));
        Choice c;
        if (v >> c.gran >> c.interval >> c.item >> c.ctas >> c.fft >> c.ms) {
            *out = c;
            hit = true;
        }
    }
    return hit;
}

void cache_store(const char* path, const std::string& key, const Choice& c) {
    if (!path) return;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ofstream f(path, std::ios::app);
    f << key << '|' << c.gran << ' ' << c.interval << ' ' << c.item << ' ' << c.ctas << ' ' << c.fft << ' ' << c.ms
      << '\n';
}

// Steps per second of one candidate: warm-up (prologue + first sort + graph
// capture), then `steps` timed steps.
int time_candidate(const cosmos_pm_config& cfg, const float* x, const float* y, const float* xo, const float* yo,
                   const float* m, int steps, float* ms_per_step) {
    cosmos_pm* h = nullptr;
    int rc = cosmos_pm_create(&cfg, &h);
    if (rc != COSMOS_OK) return rc;
    cudaEvent_t a = nullptr, b = nullptr;
    auto done = [&](int r) {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
        cosmos_pm_destroy(h);
        return r;
    };
    uint64_t s = 0;
    if ((rc = cosmos_pm_set_particles(h, x, y, xo, yo, m, cfg.num_particles, 0)) != COSMOS_OK ||
        (rc = cosmos_pm_step(h, 3)) != COSMOS_OK || (rc = cosmos_pm_synchronize(h)) != COSMOS_OK ||
        (rc = cosmos_pm_stream(h, &s)) != COSMOS_OK)
        return done(rc);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
        return done(cpm::fail(COSMOS_ERR_CUDA, "autotune events"));
    if (cudaEventRecord(a, st) != cudaSuccess) return done(cpm::fail(COSMOS_ERR_CUDA, "autotune event record"));
    if ((rc = cosmos_pm_step(h, steps)) != COSMOS_OK) return done(rc);
    if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess)
        return done(cpm::fail(COSMOS_ERR_CUDA, "autotune event wait"));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return done(cpm::fail(COSMOS_ERR_CUDA, "autotune timing"));
    *ms_per_step = ms / float(steps);
    return done(COSMOS_OK);
}

}  // namespace

extern "C" int cosmos_pm_autotune(const cosmos_pm_config* base, const float* x, const float* y, const float* xo,
                                  const float* yo, const float* m, int32_t steps, const char* cache_path,
                                  cosmos_pm_config* best, float* best_ms) {
    if (!base || !x || !y || !best || !best_ms) return cpm::fail(COSMOS_ERR_INVALID, "null argument");
    if (steps < 1) return cpm::fail(COSMOS_ERR_INVALID, "steps must be >= 1");
    cudaDeviceProp prop;
    CPM_CUDA(cudaGetDeviceProperties(&prop, base->device));
    std::string gpu(prop.name);
    for (char& ch : gpu)
        if (ch == '|' || ch == '\n') ch = '_';
    const std::string key = cache_key(*base, gpu.c_str());
    *best = *base;
    Choice cur;
    if (cache_lookup(cache_path, key, &cur)) {
        apply(cur, best);
        *best_ms = cur.ms;
        return COSMOS_OK;
    }
    bool any = false;
    // A candidate replaces the best so far only when it is faster by more than
    // kMargin: differences below that are within the run-to-run spread of a
    // timing window and would not hold on a longer run.
    constexpr float kMargin = 0.015f;
    // times `ch`; keeps it when faster; false on a hard error in *rc
    auto trial = [&](const Choice& ch, int* rc) -> bool {
        cosmos_pm_config c = *base;
        apply(ch, &c);
        float ms = 0.0f;
        *rc = time_candidate(c, x, y, xo, yo, m, steps, &ms);
        if (*rc == COSMOS_ERR_NOMEM || *rc == COSMOS_ERR_INVALID) {  // a candidate that does not fit or apply
            *rc = COSMOS_OK;
            return true;
        }
        if (*rc != COSMOS_OK) return false;
        if (!any || ms < cur.ms * (1.0f - kMargin)) {
            cur = ch;
            cur.ms = ms;
            any = true;
        }
        return true;
    };
    int rc = COSMOS_OK;
    {  // the library's defaults first: the reference every candidate has to beat
        Choice def;
        def.gran = base->sort_granularity;
        def.interval = base->sort_interval;
        if (!trial(def, &rc)) return rc;
    }
    // 1. tile edge x sort cadence (the other fields at their defaults)
    const int grans[] = {4, 5, 6};
    const int intervals[] = {8, 16, 24, 32, 48, 64, 0};
    for (int gr : grans) {
        if ((base->lattice_n >> gr) < 1) continue;
        for (int itv : intervals) {
            if (itv == 0 && gr != grans[0]) continue;  // "never sort" ignores the tile edge
            Choice ch;
            ch.gran = gr;
            ch.interval = itv;
            if (!trial(ch, &rc)) return rc;
        }
    }
    if (!any) return cpm::fail(COSMOS_ERR_NOMEM, "autotune: no candidate fits on the device");
    // 2-4. work-item size, fused-kernel CTAs per SM, column-pass shape (tile order only)
    if (cur.interval != 0) {
        for (int item : {2048, 4096, 8192}) {
            Choice ch = cur;
            ch.item = item;
            if (!trial(ch, &rc)) return rc;
        }
        for (int ctas : {2, 3}) {
            Choice ch = cur;
            ch.ctas = ctas;
            if (!trial(ch, &rc)) return rc;
        }
    }
    if (base->force_mode != COSMOS_FORCE_GRADIENT) {
        Choice ch = cur;
        ch.fft = 1;
        if (!trial(ch, &rc)) return rc;
    }
    apply(cur, best);
    *best_ms = cur.ms;
    cache_store(cache_path, key, cur);
    return COSMOS_OK;
}
