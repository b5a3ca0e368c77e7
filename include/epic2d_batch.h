/* epic2d_batch.h — many independent runs advanced together, every phase of a
 * step one launch for all of them (no counterpart in the reference, which runs
 * one simulation per process).
 *
 * The runs' grids are laid end to end in one node space (run r's node (i, j)
 * at node_off[r] + i*ny_r + j) and each species of all runs shares one
 * particle array (a particle's stored cell is its node in that space, so it
 * carries its run).  The deposit, finalisation, E-field, push, rewind, cell
 * sort and the spectral mixed-precision solve (one batched GEMM schedule for
 * all runs' transforms, with a per-run stopping test) each run as one launch
 * over the whole batch; a step is captured as a CUDA graph.  The arithmetic
 * per run is the single-run mixed form's, so a run gives the same particles
 * and potential, bit for bit, in a batch as alone (epic_run with the same
 * sort_every, loaded by epic_load_particles_device with the same seed).
 *
 * Electron-neutral MCC (runs submitted with collisions) is one launch sequence
 * for all colliding runs: every electron uses its own run's parameters, with
 * Philox draws keyed by its position in the batch's array and its run's seed,
 * so a colliding run is statistically, not bitwise, the run alone; runs
 * without collisions stay bitwise equal to their single runs.
 *
 * An autotuner picks, when the batch is built, the GEMM tile (16, 32, or 64
 * register-blocked) for each lattice-size class by timing them on the
 * batch's own transforms; the choice does not change results.
 *
 * Runs must use the mixed form with CIC deposition and the same number of
 * species (species k plays the same role in every run; MCC needs electrons as
 * species 0 and ions as species 1); the colliding runs share one gas density.
 * Lattices with a side of 512 or more unknowns run alone (a single run solves
 * them by FFT passes where their sides allow, so a batch could not equal it).
 * A run's emitters (its request's [Emitters]) inject first in every step with
 * the run alone's draws, and get room for the request's `steps` steps of
 * injections (past it epic_batch_run returns EPIC_ERR_CAPACITY).  A run with
 * conductors (its request's [Grids]) is loaded by the host loader, as
 * epic_load_particles with load_seed; its SOR solves get the rho override and
 * the push erases the particles that end inside them.
 * Walls may be periodic, reflective or absorbing, mixed within a batch; with
 * an absorbing run or conductors in the batch the push erases particles in order
 * (as a single run) and the deposit and the MCC's selection run as their own
 * passes. */
#ifndef EPIC2D_BATCH_H
#define EPIC2D_BATCH_H

#include "epic2d_serve.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct epic_batch epic_batch;

/* Builds a batch on the current device from nruns requests (configuration,
 * species, collisions, load_seed, conductors and emitters of each; steps sizes
 * the room for a run's injections; arrival is ignored). */
epic_status epic_batch_create(const epic_request* runs, int nruns, int sort_every, epic_batch** out);
void epic_batch_destroy(epic_batch* b);
/* Loads every run on the device (its load_seed) and computes its initial field
 * and rewind (src/main.cpp:366-382). */
epic_status epic_batch_initial_field(epic_batch* b);
/* Advances every run by `steps` steps (use_graph: replay a captured step). */
epic_status epic_batch_run(epic_batch* b, int steps, int use_graph);
/* Run `run`'s particles of `species` as {x, y, vx, vy, vz} records, or a grid
 * (EPIC_GRID_PHI / EPIC_GRID_RHO) in the run's own nx*ny layout. */
epic_status epic_batch_get_particles(epic_batch* b, int run, int species, double* out, int64_t capacity,
                                     int64_t* n);
epic_status epic_batch_get_grid(epic_batch* b, int run, int which, double* out);
epic_status epic_batch_num_particles(epic_batch* b, int64_t* total);
/* Cross sections of the colliding runs (epic_set_log_cross_sections), needed
 * before the first step of a batch with collisions. */
epic_status epic_batch_set_log_cross_sections(epic_batch* b, const double* ela, const double* exc, const double* ion,
                                              int64_t n, double e_min, double e_max);
/* The autotuner's choices: GEMM tile per size class (max(R, C) <= 48, <= 96,
 * <= 160, larger). */
epic_status epic_batch_tuning(epic_batch* b, int tiles[4]);
/* The autotuner's launch shapes of the particle passes, chosen when the
 * particles are loaded (epic_batch_initial_field) by timing a sample of them:
 * shapes = {push threads per CTA, push CTAs, deposit threads per CTA, deposit
 * CTAs}; push_ms (5) and deposit_ms (6), when not NULL, receive the sample's
 * time per launch of each shape tried (push: 128 and 256 threads with every
 * CTA resident, 256 with 1 and 2 CTAs per SM, 128 with 3; deposit: 128 and
 * 256 at full occupancy, 256 with 4, 8 and 16 CTAs per SM, 128 with 8); a
 * shape replaces the default (push: 256 resident; deposit: 256 with 8 per SM)
 * only when it is at least 5 % faster on the sample.  No shape changes
 * results. */
epic_status epic_batch_particle_tuning(epic_batch* b, int shapes[4], float push_ms[5], float deposit_ms[6]);
/* Per-phase timing of directly launched steps (epic_batch_run with
 * use_graph = 0), as epic_set_profiling / epic_get_profile for one run:
 * phases 0 deposit, 1 finalisation + rho, 2 Poisson solve, 3 E-field, 4 push,
 * 5 MCC, 6 cell sort; get_profile waits for the stream, returns accumulated
 * milliseconds and counts and resets them. */
epic_status epic_batch_set_profiling(epic_batch* b, int enable);
epic_status epic_batch_get_profile(epic_batch* b, double ms[7], int64_t counts[7]);
void* epic_batch_stream(epic_batch* b);

#ifdef __cplusplus
}
#endif
#endif
