/*
 * cosmos_pm.h -- C ABI of the GB300 particle-mesh gravity step.
 *
 * Drop-in for the hot path of tugrul512bit/CosmosSimulationWithCuda
 * (CosmosCuda.cuh): the simulation class Universe<K> owns a particle state
 * (x, y, xOld, yOld, m), builds the 1/r Green's filter once, and advances the
 * state with the particle-mesh step
 *     deposit (NGP / CIC) -> 2-D FFT convolution -> gradient -> gather + update.
 * Every entry point below replaces one part of that class; the comment on each
 * names the reference code it stands for.
 *
 * Conventions
 *  - Plain C types only: host pointers, sizes in elements, int status codes.
 *  - Every function returns COSMOS_OK (0) or a negative COSMOS_ERR_* code and
 *    never exits the process (the reference calls exit() on any CUDA error,
 *    CosmosCuda.cuh:19-27).  cosmos_pm_last_error() gives a message.
 *  - The library owns all device memory of a handle; the caller owns every
 *    host buffer it passes.
 *  - One host thread per handle at a time, except cosmos_pm_poll(), which may
 *    be called from any thread.
 *  - Particle identity: particle i is the i-th element of the arrays given to
 *    cosmos_pm_set_particles().  The library may keep particles in a different
 *    order internally (sorted by lattice tile); every get/set call below
 *    addresses particles by identity unless it says otherwise.
 *  - Like the reference, only the first 4*floor(P/4) particles take part in
 *    the step (it walks float4 groups, CosmosCuda.cuh:239-242, 454-471).
 */
#ifndef COSMOS_PM_H
#define COSMOS_PM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define COSMOS_OK 0
#define COSMOS_ERR_INVALID -1   /* bad argument or configuration */
#define COSMOS_ERR_CUDA -2      /* a CUDA runtime call failed */
#define COSMOS_ERR_NOMEM -3     /* device or pinned allocation failed */
#define COSMOS_ERR_RANGE -4     /* offset/count outside the particle range */
#define COSMOS_ERR_TIMEOUT -5   /* a bounded device-side wait gave up */
#define COSMOS_ERR_STATE -6     /* call not valid in the handle's current state */

/* ---- configuration -------------------------------------------------------- */
/* Mass assignment: NGP = the reference's lowAccuracy=true, CIC = false
 * (CosmosCuda.cuh:890, deposit :507-515, gather :262-284). */
#define COSMOS_DEPOSIT_NGP 0
#define COSMOS_DEPOSIT_CIC 1

/* Force evaluation.
 *  GRADIENT: potential on the lattice, then the reference's edge-clamped
 *            4th-order difference (CosmosCuda.cuh:174-229).
 *  SPECTRAL: the same difference stencil applied in Fourier space with the
 *            reference's edge clamping restored at the border cells; the
 *            force comes out of the inverse FFT directly instead of being
 *            differenced from an FP32 potential (about 100x smaller error
 *            against FP64 at the same memory traffic). */
#define COSMOS_FORCE_GRADIENT 0
#define COSMOS_FORCE_SPECTRAL 1
/* SPECTRAL with the column FFTs (3 of the step's 5 length-N transforms) on
 * the tensor cores: each transform is a four-step FFT whose two DFT stages
 * are tcgen05 GEMMs on split 16-bit operands (high part + rounding of the
 * remainder, three products accumulated in FP32).  FP16 split (range-scaled)
 * or BF16 split.  N = 1024, 2048 or 4096 only. */
#define COSMOS_FORCE_SPECTRAL_TC_FP16 2
#define COSMOS_FORCE_SPECTRAL_TC_BF16 3

typedef struct cosmos_pm_config {
    int32_t lattice_n;          /* N: power of two, 16..8192   (Constants::N, CosmosCuda.cuh:38) */
    int32_t deposit;            /* COSMOS_DEPOSIT_NGP / _CIC   (Universe ctor lowAccuracy, :881,890) */
    float dt;                   /* time step                   (Constants::dt, :43) */
    float gravity_multiplier;   /* force multiplier            (Constants::gravityMultiplier, :45) */
    int64_t num_particles;      /* P                           (Universe ctor `particles`, :881) */
    int32_t device;             /* CUDA device ordinal         (cudaDevices[0], :881,970) */
    int32_t force_mode;         /* COSMOS_FORCE_*  (0 = reference-faithful gradient) */
    int32_t sort_interval;      /* steps between particle re-sorts; 0 = never sort,
                                   -1 = library default for this lattice/particle count */
    int32_t sort_granularity;   /* log2 of the tile edge (cells) used as sort key; -1 = default */
    int32_t use_graph;          /* 1 = replay each step from a captured CUDA graph */
    int32_t blur_r;             /* render blur width, odd, 1..15 (Constants::BLUR_R, :49); 0 = 3 */
    /* Launch shapes (no counterpart in the reference, whose shapes are
     * compile-time constants, CosmosCuda.cuh:29-74); 0 = library default.
     * cosmos_pm_autotune picks them. */
    int32_t item_size;          /* particles per work item of the fused step kernel: 2048, 4096 or
                                   8192; 0 = chosen from the particle count */
    int32_t fused_ctas_per_sm;  /* resident CTAs per SM of the fused step kernel's grid; 0 = as many
                                   as fit */
    int32_t fft_shape;          /* spectral modes: 0 = default column-pass shape, 1 = the other
                                   shape (one radix-16 butterfly per thread per stage instead of two
                                   from 1024^2 up, two instead of one below) */
    int32_t reserved[3];
} cosmos_pm_config;

typedef struct cosmos_pm cosmos_pm; /* opaque handle (one Universe) */

/* Fill *cfg with defaults: N=2048, CIC, dt=1e-3, gravity 1, P=0, device 0,
 * gradient force, library-default sorting, graphs on. */
void cosmos_pm_default_config(cosmos_pm_config* cfg);

/* Create a simulation: allocates the particle state (zeroed), the lattices and
 * the filter, and builds the filter in FP64 on the device.  Replaces the
 * Universe constructor's allocation and filter build (CosmosCuda.cuh:969-1034);
 * the constructor's random particle fill is not part of it (use
 * cosmos_pm_set_particles with seeded data). */
int cosmos_pm_create(const cosmos_pm_config* cfg, cosmos_pm** out);

/* Release everything.  Replaces ~Universe (CosmosCuda.cuh:1396-1427). */
int cosmos_pm_destroy(cosmos_pm* h);

/* Copy `count` particles from host arrays into identities [offset, offset+count).
 * Any of x_old, y_old may be NULL (then they are set equal to x, y: zero
 * velocity); m may be NULL (masses unchanged).  Synchronous.  Replaces the
 * host-to-device uploads of the constructor and of addGalaxy
 * (CosmosCuda.cuh:1012-1016, 1151-1155). */
int cosmos_pm_set_particles(cosmos_pm* h, const float* x, const float* y, const float* x_old,
                            const float* y_old, const float* m, int64_t count, int64_t offset);

/* Copy particles [offset, offset+count) (by identity) to host arrays; any
 * pointer may be NULL to skip that array.  Synchronous. */
int cosmos_pm_get_particles(cosmos_pm* h, float* x, float* y, float* x_old, float* y_old, float* m,
                            int64_t count, int64_t offset);

/* Park every particle at (-10, -10) with xOld = x, so none is deposited or
 * moved.  Replaces Universe::clear (CosmosCuda.cuh:1038-1069). */
int cosmos_pm_clear(cosmos_pm* h);

/* Enqueue `nsteps` particle-mesh steps on the handle's stream and return
 * without waiting.  One step = scatterMassOnLattice, calcLatticeFft2D,
 * multiplyLatticeFilterElementwise, calcLatticeIfft2D, multiSampleForces
 * (CosmosCuda.cuh:1209-1300, loop :1336-1342). */
int cosmos_pm_step(cosmos_pm* h, int32_t nsteps);

/* Wait until every enqueued step and copy of the handle has finished. */
int cosmos_pm_synchronize(cosmos_pm* h);

/* Asynchronous readback of the positions after the last enqueued step into
 * host_x, host_y (P floats each; page-locked memory gives a truly
 * asynchronous copy).  ordered=1 delivers particle identities in order;
 * ordered=0 delivers the library's internal order (cheaper; enough for a
 * renderer).  The step stream does not wait for the copy.  Returns a ticket
 * for cosmos_pm_poll / cosmos_pm_wait.  New API: the reference has no
 * position readback (it renders a density frame, CosmosCuda.cuh:1343-1351). */
int cosmos_pm_get_positions_async(cosmos_pm* h, float* host_x, float* host_y, int32_t ordered,
                                  uint64_t* ticket);

/* Render a display frame of the current density (the density of the
 * particles' current positions) into host_frame (N*N floats), with the
 * reference's render chain: BLUR_R blur, frame min / max folded into running
 * extremes, 1.8 * ((v - min) / (max - min))^0.25 (CosmosCuda.cuh:1249-1256,
 * kernels :613-828).  Synchronous. */
int cosmos_pm_render_frame(cosmos_pm* h, float* host_frame);

/* The same frame, asynchronously: rendered on the step stream after the last
 * enqueued step and copied to host_frame (page-locked for a truly
 * asynchronous copy) on the copy stream.  Replaces the worker's frame push
 * (CosmosCuda.cuh:1343-1351, pushFrame :1302-1308). */
int cosmos_pm_get_frame_async(cosmos_pm* h, float* host_frame, uint64_t* ticket);

/* *done = 1 when the copy behind `ticket` has landed in host memory. */
int cosmos_pm_poll(cosmos_pm* h, uint64_t ticket, int32_t* done);

/* Block until the copy behind `ticket` has landed. */
int cosmos_pm_wait(cosmos_pm* h, uint64_t ticket);

/* ---- seeded initial conditions on the device --------------------------------
 * Replaces the host fills of the constructor (CosmosCuda.cuh:929-950) and of
 * addGalaxy (:1071-1116), which draw from std::random_device.  Particle i of
 * a generated set draws from a counter-based stream keyed by (seed, i), with
 * i the particle's identity, and every float operation is a separately
 * rounded float32 operation, so the result is reproducible bit for bit (on
 * any GPU and by the float32 restatement in the test oracle).  Positions and
 * velocities of identity i depend only on (seed, i) and the parameters; the
 * per-particle mass is `mass` over the call's count. */
#define COSMOS_IC_UNIFORM 0    /* square of half-width scale, Gaussian velocities */
#define COSMOS_IC_EXP_DISK 1   /* exponential disk, circular speeds from the enclosed mass */
#define COSMOS_IC_PLUMMER 2    /* projected Plummer sphere, circular speeds */
#define COSMOS_IC_RING_DISK 3  /* the reference's addGalaxy ring disk */
typedef struct cosmos_ic_params {
    int32_t kind;             /* COSMOS_IC_* */
    int32_t black_hole;       /* RING_DISK: the last particle is a heavy body at the centre */
    uint64_t seed;
    float center_x, center_y; /* cells; RING_DISK: fractions of N (normalizedCenterX/Y) */
    float scale;              /* UNIFORM half-width, EXP_DISK scale length, PLUMMER radius a (cells);
                                 RING_DISK normalizedRadius */
    float rmax;               /* EXP_DISK / PLUMMER truncation radius (cells); <= 0: none */
    float mass;               /* total mass of the generated particles; RING_DISK massPerParticle */
    float mass_sigma;         /* lognormal spread of the masses (0: equal); not RING_DISK */
    float bulk_vx, bulk_vy;   /* bulk velocity (cells per unit time);
                                 RING_DISK centerOfMassVelocityX/Y */
    float spin;               /* EXP_DISK / PLUMMER rotation sense (+1, -1, 0); RING_DISK angularVelocity */
    float dispersion;         /* UNIFORM velocity sigma; EXP_DISK / PLUMMER sigma per axis as a
                                 fraction of the circular speed */
    float g;                  /* gravity multiplier of the circular speeds */
    int32_t pad;
    int64_t total_particles;  /* RING_DISK: the reference's totalNumParticles (mass divisor) */
    int32_t reserved[4];
} cosmos_ic_params;

/* Generate `count` particles of one family into identities [offset,
 * offset+count) on the device (synchronous).  xOld = x - v dt with the
 * handle's dt (RING_DISK: the reference's xOld formula). */
int cosmos_pm_generate(cosmos_pm* h, const cosmos_ic_params* ic, int64_t count, int64_t offset);

/* ---- stage-level access (test hooks; the reference's private step methods) */
#define COSMOS_FIELD_DENSITY 0   /* N*N float: accumulator_d after deposit (:1242) */
#define COSMOS_FIELD_POTENTIAL 1 /* N*N float: latticeShifted_d (:1297) */
#define COSMOS_FIELD_FORCE 2     /* N*N*2 float (fx, fy): latticeShiftedForceXY_d (:1298) */

/* Run one stage of the step on the current state.
 *  COSMOS_STAGE_DEPOSIT   : density from the particles   (scatterMassOnLattice, :1209-1264)
 *  COSMOS_STAGE_POTENTIAL : potential from the density   (:1265-1297, FFT conv + shift)
 *  COSMOS_STAGE_FORCE     : force field from the density or potential (:1298)
 *  COSMOS_STAGE_INTEGRATE : gather + update from the force field (:1299) */
#define COSMOS_STAGE_DEPOSIT 0
#define COSMOS_STAGE_POTENTIAL 1
#define COSMOS_STAGE_FORCE 2
#define COSMOS_STAGE_INTEGRATE 3
int cosmos_pm_run_stage(cosmos_pm* h, int32_t stage);

/* Copy a lattice field to / from the host (synchronous). */
int cosmos_pm_get_field(cosmos_pm* h, int32_t field, float* host);
int cosmos_pm_set_field(cosmos_pm* h, int32_t field, const float* host);

/* Sort the particles by lattice tile now (stable by identity order within a
 * tile) and write the resulting internal order: perm[i] = identity of the
 * particle in internal slot i.  perm may be NULL. */
int cosmos_pm_sort(cosmos_pm* h, uint32_t* perm);

/* Tile keys the sort uses, computed on the device from host positions: for
 * testing the key function bit-exactly.  keys: count uint32. */
int cosmos_pm_tile_keys(cosmos_pm* h, const float* x, const float* y, int64_t count, int32_t granularity,
                        uint32_t* keys);

/* FP64 diagnostics: kinetic energy sum(m v^2)/2 with v = (x - xOld)/dt, the
 * displacement taken modulo the wrap period N-4 (a wrapped particle's xOld
 * stays on the far side), the momentum sum(m v), over active particles, and
 * sum(m phi(x))/2 sampled from the potential field (NGP sample; run
 * COSMOS_STAGE_DEPOSIT and COSMOS_STAGE_POTENTIAL first for the current
 * positions).  With force = +grad(phi), the total energy is kinetic minus
 * that sum.  No counterpart in the reference. */
int cosmos_pm_diagnostics(cosmos_pm* h, double* kinetic, double* potential, double* momentum_x,
                          double* momentum_y);

/* Per-stage device time of the last step run with profiling on (ms), for
 * benchmarks: times[i] in the order prologue deposit (first step after the
 * state was written, else 0), FFT passes (spectral mode: all force passes),
 * stencil (gradient mode), fused gather + update + deposit, tile sort (0 when
 * the step did not sort).  A profiled step runs as one step per graph launch
 * (direct launches when graphs are off) with events recorded between its
 * stages, on a side branch of the graph so that the step's kernels keep
 * their overlapping (programmatic) launches: a stage time is the time from
 * the completion of the stage before to the completion of this one.  The
 * prologue and the sort run before the step as direct launches.
 * *n = capacity on entry, entries written on return. */
int cosmos_pm_set_profiling(cosmos_pm* h, int32_t enabled);
int cosmos_pm_stage_times(cosmos_pm* h, float* times, int32_t* n);

/* The cudaStream_t the handle enqueues on (as an integer), for callers that
 * record their own events around cosmos_pm_step. */
int cosmos_pm_stream(cosmos_pm* h, uint64_t* stream);

/* Number of kernel launches one step enqueues (for launch accounting). */
int cosmos_pm_launches_per_step(cosmos_pm* h, int32_t* launches);

/* Kernels the handle has enqueued since creation: every step's kernels, the
 * re-sorts, the first-step deposits and the frame renders (for launch
 * accounting over a region: read it before and after). */
int cosmos_pm_kernels_launched(cosmos_pm* h, int64_t* launches);

/* ---- autotuning -----------------------------------------------------------
 * No counterpart in the reference (its launch shapes are compile-time
 * constants, CosmosCuda.cuh:29-74).  Measures, on the caller's own particle
 * state, the tile edge of the particle sort (sort_granularity 4, 5, 6: 16, 32,
 * 64 cells) x the re-sort cadence (sort_interval 8, 16, 24, 32, 48, 64, or
 * never), then with the best of those the work-item size of the fused step
 * kernel (item_size 2048, 4096, 8192), its CTAs per SM (fused_ctas_per_sm 2,
 * 3 or as many as fit) and, in the spectral modes, the column-pass shape
 * (fft_shape 0, 1): each candidate runs on a temporary handle from the same
 * host state, `steps` graph-launched steps timed with CUDA events after a
 * warm-up that includes its first sort.  The library's defaults are timed
 * first and a candidate is taken only when it is more than 1.5% faster than
 * the best so far.  *best = *base with the chosen fields; *best_ms = its time
 * per step (amortising the sorts).
 * cache_path (may be NULL): a text file of earlier results keyed by lattice
 * size, particle count (half-octave bucket), deposit, force mode and GPU
 * name; a hit returns the cached choice without running, a miss appends the
 * new result.  The handle memory of one candidate at a time is allocated. */
int cosmos_pm_autotune(const cosmos_pm_config* base, const float* x, const float* y, const float* x_old,
                       const float* y_old, const float* m, int32_t steps, const char* cache_path,
                       cosmos_pm_config* best, float* best_ms);

/* ---- tile sort without device allocation ---------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run (a host that owns a fixed amount of device memory, code inside
 * an allocator or memory-pool callback, a real-time loop where cudaMalloc may
 * stall on a device-wide synchronisation): writes to perm_dev the stable sort
 * permutation (perm[i] = index of the i-th particle in tile-key order, the
 * keys of cosmos_pm_tile_keys) of n device-resident positions.  It calls no
 * cudaMalloc / cudaFree: its scratch is a fixed device array of about 16.5 MB
 * that every GPU loading this library keeps until the process exits, sized
 * for COSMOS_NOALLOC_MAX_PARTICLES particles; larger n returns
 * COSMOS_ERR_RANGE.  All n particles are ordered (cosmos_pm_sort orders
 * the first 4*floor(P/4) of a handle and leaves the rest in place, so the two
 * agree only when n is a multiple of 4).  Work is enqueued on `stream` (a
 * cudaStream_t as an integer, 0 = legacy default stream) and not waited for.
 * A call outside stream capture looks up the scratch address on the current
 * device (so a device reset between calls is harmless); a call under capture
 * uses the address found by the last uncaptured call, so the first call on a
 * device must come before any stream capture (COSMOS_ERR_STATE otherwise).
 * All calls on a device share the scratch, so calls whose work overlaps on
 * the GPU race; serialise them. */
#define COSMOS_NOALLOC_MAX_PARTICLES (1 << 20)
int cosmos_tile_sort_noalloc(const float* x_dev, const float* y_dev, int64_t n, int32_t lattice_n,
                             int32_t granularity, uint32_t* perm_dev, uint64_t stream);

/* ---- checkpoint / resume ----------------------------------------------------
 * No counterpart in the reference.  A checkpoint is a header (lattice size,
 * deposit, force mode, particle count, dt, gravity multiplier, steps taken,
 * FNV-1a checksum) followed by x, y, xOld, yOld, m in identity order.  Loading
 * requires the same lattice size, particle count, deposit, dt and gravity
 * multiplier (COSMOS_ERR_INVALID otherwise, and for a truncated or corrupted
 * file) and restores the step counter.  Synchronous. */
int cosmos_pm_checkpoint_save(cosmos_pm* h, const char* path);
int cosmos_pm_checkpoint_load(cosmos_pm* h, const char* path);
/* Steps advanced since creation (or since the loaded checkpoint's). */
int cosmos_pm_steps_taken(cosmos_pm* h, int64_t* steps);

/* ---- test hooks (failure injection without a GPU fault) ----------------------
 * COSMOS_TEST_FAIL_ALLOC:  the value-th device allocation from now, in any
 *                          handle, fails with COSMOS_ERR_NOMEM (0: off); h may
 *                          be NULL.
 * COSMOS_TEST_TC_SKIP_MMA: (tensor-core force modes) the column pass issues no
 *                          MMA and no completion signal while value != 0, so
 *                          its bounded waits run out: the next
 *                          cosmos_pm_synchronize returns COSMOS_ERR_TIMEOUT and
 *                          the handle stays usable.
 * COSMOS_TEST_COPY_WAIT:   while value != 0, the fused step kernel announces
 *                          16 bytes more per particle-copy stage than it
 *                          copies, so its bounded copy waits run out (no copy
 *                          is left in flight): the next cosmos_pm_synchronize
 *                          returns COSMOS_ERR_TIMEOUT and the handle stays
 *                          usable (the step that gave up is incomplete). */
#define COSMOS_TEST_FAIL_ALLOC 1
#define COSMOS_TEST_TC_SKIP_MMA 2
#define COSMOS_TEST_COPY_WAIT 3
int cosmos_pm_test_hook(cosmos_pm* h, int32_t hook, int64_t value);

/* Page-locked host memory for the asynchronous readbacks (the reference's
 * cudaMallocHost of frame_h, CosmosCuda.cuh:928-929).  *out = NULL on failure. */
int cosmos_pm_host_alloc(int64_t bytes, void** out);
int cosmos_pm_host_free(void* p);

/* Message of the last error on this handle (or the last create failure when
 * h is NULL).  The string stays valid until the next call on the handle. */
const char* cosmos_pm_last_error(cosmos_pm* h);

/* Library version, e.g. "0.1.0". */
const char* cosmos_pm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* COSMOS_PM_H */
