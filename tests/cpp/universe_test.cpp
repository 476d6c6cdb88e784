// Drives the Universe<K> drop-in (include/CosmosGB300.cuh) the way the
// reference's main.cu drives Universe<K> of CosmosCuda.cuh: clear, two
// galaxies on a collision course with central black holes, the frame worker,
// popFrame, nBodyStop.  Built and run by tests/test_gpu_universe.py; prints
// one line "PASS {json}" or "FAIL <reason>".
//
//   universe_test <lowAccuracy 0|1>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#define __OVERRIDE_CONSTANTS__
namespace OVERRIDE_CONSTANTS {
constexpr int THREADS = 768;
constexpr int NUM_CUDA_DEVICES = 1;
constexpr int N = 256;
constexpr float dt = 50.0f;
constexpr float gravityMultiplier = 1.0f;
constexpr int MAX_FRAMES_BUFFERED = 4;
constexpr int BLUR_R = 3;
}  // namespace OVERRIDE_CONSTANTS
#define COSMOS_GB300_THROW
#include "CosmosGB300.cuh"

namespace {

constexpr int K = 2;
constexpr int kParticles = 200000;
constexpr int kPerGalaxy = 100000;

#define REQUIRE(cond, what)                                  \
    do {                                                     \
        if (!(cond)) {                                       \
            std::printf("FAIL %s (line %d)\n", what, __LINE__); \
            return 1;                                        \
        }                                                    \
    } while (0)

// main.cu's collision scenario, scaled to the lattice
void collision(Universe<K>& u) {
    u.clear();
    u.addGalaxy(kPerGalaxy, 0.25f, 0.25f, 0.005f, 1.0f, 0.2f, 0.000025f, 0.000025f, true);
    u.addGalaxy(kPerGalaxy, 0.75f, 0.75f, 0.005f, 1.0f, 0.2f, -0.00005f, -0.00005f, true);
}

bool frame_ok(const std::vector<float>& f, float* fmax) {
    float mx = 0.0f;
    for (float v : f) {
        if (!std::isfinite(v) || v < 0.0f || v > 1.8f * 1.0001f) return false;
        mx = v > mx ? v : mx;
    }
    *fmax = mx;
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    const bool lowAccuracy = argc > 1 && std::string(argv[1]) == "1";
    const int dev[1] = {0};
    const float perf[1] = {1.0f};
    try {
        Universe<K> u(kParticles, dev, perf, lowAccuracy, 1234);
        REQUIRE(u.getLatticeSize() == 256, "lattice size");
        std::vector<float> x0, y0;
        u.getParticles(x0, y0);
        for (int i = 0; i < kParticles; ++i)
            REQUIRE(x0[i] >= 0.01f * 256 && x0[i] < 0.99f * 256 + 1e-3f && y0[i] >= 0.01f * 256, "uniform fill");

        // the counter sits at the end after construction: addGalaxy without
        // clear() adds nothing (the reference's behaviour) and wraps it
        u.addGalaxy(1000, 0.5f, 0.5f);
        std::vector<float> x1, y1;
        u.getParticles(x1, y1);
        REQUIRE(x1 == x0 && y1 == y0, "addGalaxy after construction changes nothing");

        collision(u);
        u.getParticles(x1, y1);
        int bad = 0;
        for (int i = 0; i < kParticles; ++i) {
            const float cx = i < kPerGalaxy ? 64.0f : 192.0f;
            const float r = std::hypot(x1[i] - cx, y1[i] - cx);
            if (r > 0.2f * 256 * 1.0001f) ++bad;
        }
        REQUIRE(bad == 0, "galaxy radii");
        REQUIRE(x1[kPerGalaxy - 1] == 64.0f && y1[kPerGalaxy - 1] == 64.0f, "first black hole at the centre");
        REQUIRE(x1[kParticles - 1] == 192.0f, "second black hole at the centre");

        // the same seed and calls give the same galaxies
        {
            Universe<K> twin(kParticles, dev, perf, lowAccuracy, 1234);
            collision(twin);
            std::vector<float> x2, y2;
            twin.getParticles(x2, y2);
            REQUIRE(x2 == x1 && y2 == y1, "seeded fill repeats");

            // the first frame the worker delivers is the frame of the density
            // at the start of the interval's last step
            twin.nBodyStartGeneratingFrames();
            bool ready = false;
            auto t0 = std::chrono::steady_clock::now();
            std::vector<float> first;
            while (std::chrono::steady_clock::now() - t0 < std::chrono::seconds(30)) {
                std::vector<float>& f = twin.popFrame(ready);
                if (ready) {
                    first = f;
                    break;
                }
                std::this_thread::sleep_for(std::chrono::milliseconds(1));
            }
            twin.nBodyStop();
            REQUIRE(!first.empty(), "first frame arrives");

            Universe<K> manual(kParticles, dev, perf, lowAccuracy, 1234);
            collision(manual);
            std::vector<float> want(size_t(256) * 256), later(size_t(256) * 256);
            REQUIRE(cosmos_pm_step(manual.handle(), K - 1) == COSMOS_OK, "manual steps");
            REQUIRE(cosmos_pm_render_frame(manual.handle(), want.data()) == COSMOS_OK, "manual frame");
            REQUIRE(cosmos_pm_step(manual.handle(), 1) == COSMOS_OK, "manual step");
            REQUIRE(cosmos_pm_render_frame(manual.handle(), later.data()) == COSMOS_OK, "manual later frame");
            // Float atomics may reorder the last bits of a density cell, which
            // can move a particle across a cell edge one step later, and the
            // frame's fourth root magnifies a lone particle in an empty cell:
            // compare typical pixels, and against the frame one step later.
            std::vector<double> d_want(want.size()), d_later(want.size());
            for (size_t i = 0; i < want.size(); ++i) {
                d_want[i] = std::fabs(double(want[i]) - first[i]);
                d_later[i] = std::fabs(double(later[i]) - first[i]);
            }
            auto median = [](std::vector<double> v) {
                std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
                return v[v.size() / 2];
            };
            double mean_want = 0.0, mean_later = 0.0;
            for (size_t i = 0; i < want.size(); ++i) {
                mean_want += d_want[i];
                mean_later += d_later[i];
            }
            REQUIRE(median(d_want) <= 1e-5, "worker frame timing matches step(K-1) + render");
            REQUIRE(mean_want < 0.2 * mean_later, "worker frame is not the frame one step later");
        }

        // run the worker, read frames as they come
        u.nBodyStartGeneratingFrames();
        int got = 0;
        float fmax = 0.0f;
        auto t0 = std::chrono::steady_clock::now();
        while (got < 20 && std::chrono::steady_clock::now() - t0 < std::chrono::seconds(60)) {
            bool ready = false;
            std::vector<float>& f = u.popFrame(ready);
            if (!ready) {
                std::this_thread::sleep_for(std::chrono::milliseconds(1));
                continue;
            }
            REQUIRE(f.size() == size_t(256) * 256, "frame size");
            REQUIRE(frame_ok(f, &fmax), "frame values in [0, 1.8]");
            REQUIRE(fmax > 0.1f, "frame not blank");
            ++got;
        }
        REQUIRE(got == 20, "20 frames within 60 s");

        // without popping, the ring holds at most MAX_FRAMES_BUFFERED - 1 frames
        std::this_thread::sleep_for(std::chrono::milliseconds(500));
        u.nBodyStop();
        int pending = 0;
        for (;;) {
            bool ready = false;
            u.popFrame(ready);
            if (!ready) break;
            ++pending;
        }
        REQUIRE(pending <= Constants::MAX_FRAMES_BUFFERED - 1, "ring capacity");
        REQUIRE(pending >= 1, "frames kept while not popped");

        // adding a galaxy while the worker runs is safe (the mouse-click path)
        u.nBodyStartGeneratingFrames();
        u.addGalaxy(20000, 0.5f, 0.5f, 0.005f, 1.0f, 0.15f, 0.0f, 0.0f, true);
        std::this_thread::sleep_for(std::chrono::milliseconds(200));
        u.nBodyStop();

        std::vector<float> x3, y3;
        u.getParticles(x3, y3);
        int moved = 0, finite = 0;
        for (int i = 0; i < kParticles; ++i) {
            finite += std::isfinite(x3[i]) && std::isfinite(y3[i]);
            moved += x3[i] != x1[i];
        }
        REQUIRE(finite == kParticles, "positions finite");
        REQUIRE(moved > kParticles / 2, "particles moved");
        std::printf("PASS {\"frames\": %d, \"pending\": %d, \"moved\": %d, \"low_accuracy\": %d}\n", got, pending,
                    moved, int(lowAccuracy));
    } catch (const std::exception& e) {
        std::printf("FAIL exception: %s\n", e.what());
        return 1;
    }
    return 0;
}
