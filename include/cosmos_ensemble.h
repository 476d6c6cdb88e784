/*
 * cosmos_ensemble.h -- many independent particle-mesh simulations on one GPU.
 *
 * No counterpart in the reference, which runs one Universe<K> per process
 * (CosmosCuda.cuh:830-1428).  An ensemble holds S simulations with their own
 * lattice size N_s and particle count P_s (one time step, deposit mode,
 * gravity multiplier and force mode for all) and advances all of them with
 * one CUDA-graph launch per step: simulations of the same N are stored back
 * to back and every pass of the step (the FFT passes, the force, the fused
 * gather + update + deposit) covers all of them in one kernel launch; the
 * lattice sizes run concurrently on their own streams inside the graph.
 * With persistent_step = 1 the step of all simulations is instead one
 * persistent kernel launch (its phases separated by grid barriers).
 * Each simulation follows exactly the step of a cosmos_pm handle with the
 * same configuration (the same kernels, tile-sorted).
 *
 * Conventions as in cosmos_pm.h (status codes, host buffers owned by the
 * caller, one host thread per handle).  Additional rule: every P_s must be a
 * multiple of 4 (the reference only steps 4*floor(P/4) particles; the
 * ensemble keeps each simulation's segment 16-byte aligned).
 */
#ifndef COSMOS_ENSEMBLE_H
#define COSMOS_ENSEMBLE_H

#include <stdint.h>

#include "cosmos_pm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cosmos_ensemble_config {
    int32_t num_sims;          /* S, 1..4096 */
    int32_t deposit;           /* COSMOS_DEPOSIT_NGP / _CIC, all simulations */
    float dt;                  /* time step, all simulations */
    float gravity_multiplier;  /* force multiplier, all simulations */
    int32_t device;            /* CUDA device ordinal */
    int32_t force_mode;        /* COSMOS_FORCE_GRADIENT / _SPECTRAL */
    int32_t sort_interval;     /* steps between tile re-sorts; <= 0: 32 */
    int32_t use_graph;         /* 1 = one captured CUDA graph per step */
    int32_t persistent_step;   /* 1 = the whole step of all simulations as ONE persistent
                                  cooperative kernel launch (phases separated by bounded
                                  grid barriers; spectral force, lattices 128..1024 and at
                                  most 8 lattice sizes; create fails otherwise); 0 = one
                                  kernel launch per pass and lattice size */
    int32_t reserved[7];
} cosmos_ensemble_config;

typedef struct cosmos_ensemble cosmos_ensemble;

/* Defaults: S = 0 (set it), CIC, dt = 1e-3, gravity 1, device 0, spectral
 * force, sort every 32 steps, graphs on. */
void cosmos_ensemble_default_config(cosmos_ensemble_config* cfg);

/* lattice_n[s]: power of two in [16, 8192]; num_particles[s]: multiple of 4,
 * >= 0.  Particles start zeroed (at rest at the origin, outside the active
 * window).  Builds one filter per distinct N. */
int cosmos_ensemble_create(const cosmos_ensemble_config* cfg, const int32_t* lattice_n,
                           const int64_t* num_particles, cosmos_ensemble** out);
int cosmos_ensemble_destroy(cosmos_ensemble* e);

/* Particles [offset, offset+count) of simulation `sim`, by identity (as
 * cosmos_pm_set_particles / cosmos_pm_get_particles).  Synchronous. */
int cosmos_ensemble_set_particles(cosmos_ensemble* e, int32_t sim, const float* x, const float* y,
                                  const float* x_old, const float* y_old, const float* m, int64_t count,
                                  int64_t offset);
int cosmos_ensemble_get_particles(cosmos_ensemble* e, int32_t sim, float* x, float* y, float* x_old,
                                  float* y_old, float* m, int64_t count, int64_t offset);

/* Enqueue nsteps steps of every simulation; returns without waiting. */
int cosmos_ensemble_step(cosmos_ensemble* e, int32_t nsteps);
int cosmos_ensemble_synchronize(cosmos_ensemble* e);

/* A lattice field of simulation `sim` (COSMOS_FIELD_*; the potential only in
 * gradient mode).  Synchronous. */
int cosmos_ensemble_get_field(cosmos_ensemble* e, int32_t sim, int32_t field, float* host);

/* Kernel launches per step (all simulations) and the stream the steps run
 * on (a cudaStream_t as an integer). */
int cosmos_ensemble_launches_per_step(cosmos_ensemble* e, int32_t* launches);
int cosmos_ensemble_stream(cosmos_ensemble* e, uint64_t* stream);

/* Test hook (persistent step): while value != 0 one CTA skips its arrival at
 * the first grid barrier, so every barrier wait runs out; the next
 * cosmos_ensemble_synchronize returns COSMOS_ERR_TIMEOUT and the handle stays
 * usable (the step that gave up is incomplete). */
int cosmos_ensemble_test_barrier(cosmos_ensemble* e, int32_t value);

/* Message of the last error on this handle (or the last create failure when
 * e is NULL). */
const char* cosmos_ensemble_last_error(cosmos_ensemble* e);

#ifdef __cplusplus
}
#endif
#endif /* COSMOS_ENSEMBLE_H */
