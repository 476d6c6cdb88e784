// Autotuner of the particle sort (cosmos_pm_autotune, include/cosmos_pm.h).
//
// The fused step kernel stages a tile's force window and deposit window in
// shared memory, so its speed depends on the tile edge (the sort key
// granularity) and on how far particles drift from their tile between
// re-sorts (the sort cadence); the sort itself costs about three fused steps.
// The best pair depends on the lattice, the particle count and how clustered
// the state is, so it is measured on the caller's own state: every candidate
// runs on a temporary handle, graph-launched, timed with CUDA events on the
// handle's stream.  Results are cached in a plain text file, one line per key:
//     N=<n> logP2=<2*log2(P) rounded> deposit=<0|1> force=<0|1> gpu=<name>|<gran> <interval> <ms>
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
    k << "N=" << c.lattice_n << " logP2=" << logp2 << " deposit=" << c.deposit << " force=" << c.force_mode
      << " gpu=" << gpu;
    return k.str();
}

bool cache_lookup(const char* path, const std::string& key, int* gran, int* interval, float* ms) {
    if (!path) return false;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ifstream f(path);
    std::string line;
    bool hit = false;
    while (std::getline(f, line)) {  // the last entry of a key wins
        const size_t bar = line.rfind('|');
        if (bar == std::string::npos || line.compare(0, bar, key) != 0 || bar != key.size()) continue;
        std::istringstream v(line.substr(bar + 1));
        int g = 0, i = 0;
        float t = 0.0f;
        if (v >> g >> i >> t) {
            *gran = g;
            *interval = i;
            *ms = t;
            hit = true;
        }
    }
    return hit;
}

void cache_store(const char* path, const std::string& key, int gran, int interval, float ms) {
    if (!path) return;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ofstream f(path, std::ios::app);
    f << key << '|' << gran << ' ' << interval << ' ' << ms << '\n';
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
    int g = 0, iv = 0;
    float t = 0.0f;
    if (cache_lookup(cache_path, key, &g, &iv, &t)) {
        best->sort_granularity = g;
        best->sort_interval = iv;
        *best_ms = t;
        return COSMOS_OK;
    }
    const int grans[] = {4, 5, 6};
    const int intervals[] = {8, 16, 24, 32, 48, 64, 0};
    float best_t = 0.0f;
    bool any = false;
    for (int gr : grans) {
        if ((base->lattice_n >> gr) < 1) continue;
        for (int itv : intervals) {
            cosmos_pm_config c = *base;
            c.sort_granularity = gr;
            c.sort_interval = itv;
            if (itv == 0 && gr != grans[0]) continue;  // "never sort" ignores the tile edge
            float ms = 0.0f;
            const int rc = time_candidate(c, x, y, xo, yo, m, steps, &ms);
            if (rc == COSMOS_ERR_NOMEM) continue;  // a candidate that does not fit is skipped
            if (rc != COSMOS_OK) return rc;
            if (!any || ms < best_t) {
                best_t = ms;
                *best = c;
                any = true;
            }
        }
    }
    if (!any) return cpm::fail(COSMOS_ERR_NOMEM, "autotune: no candidate fits on the device");
    *best_ms = best_t;
    cache_store(cache_path, key, best->sort_granularity, best->sort_interval, best_t);
    return COSMOS_OK;
}
