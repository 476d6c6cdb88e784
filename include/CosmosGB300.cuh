// CosmosGB300.cuh -- drop-in for the Universe<K> class of
// tugrul512bit/CosmosSimulationWithCuda (CosmosCuda.cuh:830-1428), on top of
// the cosmos_pm C ABI (cosmos_pm.h, libcosmos_pm.so).
//
// A program written against CosmosCuda.cuh switches by replacing
//     #include "CosmosCuda.cuh"
// with
//     #include "CosmosGB300.cuh"
// and linking -lcosmos_pm.  The same compile-time constants apply (the
// Constants namespace, with the __OVERRIDE_CONSTANTS__ / OVERRIDE_CONSTANTS
// hook of CosmosCuda.cuh:29-74), and the class keeps the reference's public
// members with their argument meaning:
//     Universe(particles, cudaDevices, devicePerformances, lowAccuracy)  :881-1035
//     clear()                                                            :1037-1069
//     addGalaxy(n, cx, cy, angularVelocity, massPerParticle, radius,
//               comVx, comVy, blackHole)                                 :1071-1175
//     getLatticeSize()                                                   :1313-1315
//     nBodyStartGeneratingFrames()                                       :1317-1358
//     popFrame(ready)                                                    :1360-1375
//     nBodyStop()                                                        :1376-1390
//     ~Universe()                                                        :1396-1427
// Differences, all on purpose:
//  - one GPU per Universe: NUM_CUDA_DEVICES must be 1 (the multi-GPU lattice
//    broadcast of the reference is not part of this library);
//  - the random fills of the constructor and addGalaxy run on the device
//    (cosmos_pm_generate, counter-based and seeded: seed() below) instead of
//    on host threads with std::random_device, so runs repeat on any machine;
//    the formulas are the reference's;
//  - errors print "GPUassert: <message>" and exit like the reference's
//    gpuErrchk (CosmosCuda.cuh:19-27), or throw std::runtime_error when
//    COSMOS_GB300_THROW is defined;
//  - the force is taken in the spectral mode of the library: the reference's
//    edge-clamped 4th-order stencil applied in Fourier space, within 1e-6 of
//    an FP64 evaluation (the reference's own FP32 lattice gradient sits near
//    1e-4); define COSMOS_GB300_GRADIENT_FORCE before the include for the
//    reference's lattice gradient instead.
// Frames follow the reference's timing: the frame of a render interval shows
// the density deposited at the start of the interval's last step.
#ifndef COSMOS_GB300_CUH
#define COSMOS_GB300_CUH

#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "cosmos_pm.h"

#ifndef __OVERRIDE_CONSTANTS__
namespace Constants {
constexpr int THREADS = 768;  // kept for source compatibility; the library sizes its own launches
constexpr int NUM_CUDA_DEVICES = 1;
constexpr int N = 2048;
constexpr double MATH_PI = 3.14159265358979323846;
constexpr float dt = 50.0f;
constexpr float gravityMultiplier = 1.0f;
constexpr int MAX_FRAMES_BUFFERED = 40;
constexpr int BLUR_R = 3;
constexpr int BLUR_HALF_R = (BLUR_R - 1) / 2;
}  // namespace Constants
#else
namespace Constants {
constexpr int THREADS = OVERRIDE_CONSTANTS::THREADS;
constexpr int NUM_CUDA_DEVICES = OVERRIDE_CONSTANTS::NUM_CUDA_DEVICES;
constexpr int N = OVERRIDE_CONSTANTS::N;
constexpr double MATH_PI = 3.14159265358979323846;
constexpr float dt = OVERRIDE_CONSTANTS::dt;
constexpr float gravityMultiplier = OVERRIDE_CONSTANTS::gravityMultiplier;
constexpr int MAX_FRAMES_BUFFERED = OVERRIDE_CONSTANTS::MAX_FRAMES_BUFFERED;
constexpr int BLUR_R = OVERRIDE_CONSTANTS::BLUR_R;
constexpr int BLUR_HALF_R = (BLUR_R - 1) / 2;
}  // namespace Constants
#endif

namespace cosmos_gb300_detail {
[[noreturn]] inline void die(const std::string& what) {
#ifdef COSMOS_GB300_THROW
    throw std::runtime_error(what);
#else
    std::fprintf(stderr, "GPUassert: %s\n", what.c_str());
    std::exit(1);
#endif
}
inline void check(int rc, cosmos_pm* h, const char* call) {
    if (rc != COSMOS_OK) die(std::string(call) + ": " + cosmos_pm_last_error(h));
}
}  // namespace cosmos_gb300_detail

template <int NUM_TIME_STEPS_PER_RENDER>
struct Universe {
    static_assert(Constants::NUM_CUDA_DEVICES == 1, "CosmosGB300: one GPU per Universe (NUM_CUDA_DEVICES = 1)");
    static_assert(NUM_TIME_STEPS_PER_RENDER >= 1, "at least one time step per render");
    static_assert(Constants::N >= 16 && Constants::N <= 8192 && (Constants::N & (Constants::N - 1)) == 0,
                  "N must be a power of two in [16, 8192]");
    static_assert(Constants::MAX_FRAMES_BUFFERED >= 2, "MAX_FRAMES_BUFFERED must be at least 2");

   private:
    int particleCounter = 0;
    int totalNumParticles = 0;
    cosmos_pm* sim = nullptr;
    float* frame_h = nullptr;  // page-locked
    uint64_t rng_seed = 0x5eedULL;
    uint64_t rng_calls = 0;

    std::mutex simLock;  // one host thread in the library at a time
    std::mutex lock;     // frame queue
    std::vector<std::vector<float>> frames;
    std::thread worker;
    int pushCtr = 0;
    int popCtr = 0;
    bool working = false;

    void check(int rc, const char* call) { cosmos_gb300_detail::check(rc, sim, call); }

    // Each random fill is one call of the device generator with its own seed
    // (Universe seed + fill counter); particle i draws from (seed, i).
    void generate(cosmos_ic_params ic, int count, int offset) {
        if (count <= 0) return;
        ic.seed = rng_seed + 0x9E3779B97F4A7C15ull * (++rng_calls);
        std::lock_guard<std::mutex> g(simLock);
        check(cosmos_pm_generate(sim, &ic, count, offset), "cosmos_pm_generate");
    }

    void pushFrame(const float* frame) {  // CosmosCuda.cuh:1302-1308
        std::lock_guard<std::mutex> lg(lock);
        if (pushCtr < popCtr + Constants::MAX_FRAMES_BUFFERED - 1) {
            std::memcpy(frames[pushCtr % Constants::MAX_FRAMES_BUFFERED].data(), frame,
                        sizeof(float) * size_t(Constants::N) * Constants::N);
            pushCtr++;
        }
    }

   public:
    Universe(int particles, const int (&cudaDevices)[Constants::NUM_CUDA_DEVICES],
             const float (&devicePerformances)[Constants::NUM_CUDA_DEVICES], bool lowAccuracy,
             uint64_t seed = 0x5eedULL)
        : rng_seed(seed) {
        (void)devicePerformances;  // one device: its share is 1
        if (particles < 0) cosmos_gb300_detail::die("particles < 0");
        totalNumParticles = particles;
        cosmos_pm_config cfg;
        cosmos_pm_default_config(&cfg);
        cfg.lattice_n = Constants::N;
        cfg.deposit = lowAccuracy ? COSMOS_DEPOSIT_NGP : COSMOS_DEPOSIT_CIC;
        cfg.dt = Constants::dt;
        cfg.gravity_multiplier = Constants::gravityMultiplier;
        cfg.num_particles = particles;
        cfg.device = cudaDevices[0];
        cfg.blur_r = Constants::BLUR_R;
#ifdef COSMOS_GB300_GRADIENT_FORCE
        cfg.force_mode = COSMOS_FORCE_GRADIENT;
#else
        cfg.force_mode = COSMOS_FORCE_SPECTRAL;
#endif
        check(cosmos_pm_create(&cfg, &sim), "cosmos_pm_create");
        void* p = nullptr;
        check(cosmos_pm_host_alloc(int64_t(sizeof(float)) * Constants::N * Constants::N, &p), "cosmos_pm_host_alloc");
        frame_h = static_cast<float*>(p);
        // uniform fill of [0.01 N, 0.99 N), at rest, equal masses 1/particles (:929-950)
        cosmos_ic_params ic{};
        ic.kind = COSMOS_IC_UNIFORM;
        ic.center_x = ic.center_y = 0.5f * Constants::N;
        ic.scale = 0.49f * Constants::N;
        ic.mass = 1.0f;
        ic.g = Constants::gravityMultiplier;
        generate(ic, particles, 0);
        // the reference leaves the counter at the end: the next addGalaxy
        // without clear() adds nothing and wraps the counter to 0 (:967, :1171-1173)
        particleCounter = particles;
    }

    Universe(const Universe&) = delete;
    Universe& operator=(const Universe&) = delete;

    // Moves all particles out of the simulation area (:1037-1069).
    void clear() {
        {
            std::lock_guard<std::mutex> g(simLock);
            check(cosmos_pm_clear(sim), "cosmos_pm_clear");
        }
        particleCounter = 0;
    }

    // Adds a galaxy of n particles centred at (cx, cy) in normalised
    // coordinates: the reference's ring-disk formulas (:1071-1175), drawn on
    // the device (COSMOS_IC_RING_DISK).
    void addGalaxy(int n, float normalizedCenterX = 0.5f, float normalizedCenterY = 0.5f,
                   float angularVelocity = 1.0f, float massPerParticle = 1.0f, float normalizedRadius = 0.3f,
                   float centerOfMassVelocityX = 0.0f, float centerOfMassVelocityY = 0.0f, bool blackHole = false) {
        const int start = particleCounter;
        const int maxCount = (particleCounter + n < totalNumParticles) ? particleCounter + n : totalNumParticles;
        const int count = maxCount - start;
        cosmos_ic_params ic{};
        ic.kind = COSMOS_IC_RING_DISK;
        ic.black_hole = blackHole ? 1 : 0;
        ic.center_x = normalizedCenterX;
        ic.center_y = normalizedCenterY;
        ic.scale = normalizedRadius;
        ic.mass = massPerParticle;
        ic.bulk_vx = centerOfMassVelocityX;
        ic.bulk_vy = centerOfMassVelocityY;
        ic.spin = angularVelocity;
        ic.g = Constants::gravityMultiplier;
        ic.total_particles = totalNumParticles;
        generate(ic, count, start);
        particleCounter = maxCount;
        if (particleCounter >= totalNumParticles) particleCounter = 0;
    }

    constexpr int getLatticeSize() { return Constants::N; }

    // Starts the worker thread: NUM_TIME_STEPS_PER_RENDER steps per frame,
    // frames pushed into a ring of MAX_FRAMES_BUFFERED (:1317-1358).
    void nBodyStartGeneratingFrames() {
        {
            std::lock_guard<std::mutex> lg(lock);
            if (working) return;
            pushCtr = 0;
            popCtr = 0;
            frames.assign(Constants::MAX_FRAMES_BUFFERED, std::vector<float>(size_t(Constants::N) * Constants::N));
            working = true;
        }
        worker = std::thread([this]() {
            while (true) {
                uint64_t ticket = 0;
                {
                    std::lock_guard<std::mutex> g(simLock);
                    // the reference renders the density deposited at the start of
                    // the interval's last step
                    if (NUM_TIME_STEPS_PER_RENDER > 1)
                        check(cosmos_pm_step(sim, NUM_TIME_STEPS_PER_RENDER - 1), "cosmos_pm_step");
                    check(cosmos_pm_get_frame_async(sim, frame_h, &ticket), "cosmos_pm_get_frame_async");
                    check(cosmos_pm_step(sim, 1), "cosmos_pm_step");
                    check(cosmos_pm_wait(sim, ticket), "cosmos_pm_wait");
                }
                pushFrame(frame_h);
                bool keep;
                {
                    std::lock_guard<std::mutex> lg(lock);
                    keep = working;
                }
                if (!keep) break;
            }
        });
    }

    // Returns the oldest unread frame (N*N floats, 0..1.8) and sets ready, or
    // sets ready = false and returns the last frame (:1360-1375).
    std::vector<float>& popFrame(bool& ready) {
        static std::vector<float> result(size_t(Constants::N) * Constants::N);
        std::lock_guard<std::mutex> lg(lock);
        if (popCtr < pushCtr) {
            result.swap(frames[popCtr % Constants::MAX_FRAMES_BUFFERED]);
            popCtr++;
            ready = true;
        } else {
            ready = false;
        }
        return result;
    }

    // Stops the worker after its current frame (:1376-1390).
    void nBodyStop() {
        {
            std::lock_guard<std::mutex> lg(lock);
            working = false;
        }
        if (worker.joinable()) worker.join();
    }

    // Extensions (not in the reference): the seed of the random fills, the
    // library handle (for the rest of the C ABI), and the particle state.
    void seed(uint64_t s) {
        rng_seed = s;
        rng_calls = 0;
    }
    cosmos_pm* handle() { return sim; }
    void getParticles(std::vector<float>& px, std::vector<float>& py) {
        px.resize(totalNumParticles);
        py.resize(totalNumParticles);
        std::lock_guard<std::mutex> g(simLock);
        check(cosmos_pm_get_particles(sim, px.data(), py.data(), nullptr, nullptr, nullptr, totalNumParticles, 0),
              "cosmos_pm_get_particles");
    }

    ~Universe() {
        nBodyStop();
        if (frame_h) cosmos_pm_host_free(frame_h);
        cosmos_pm_destroy(sim);
    }
};

#endif  // COSMOS_GB300_CUH
