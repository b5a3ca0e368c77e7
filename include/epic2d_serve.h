/* epic2d_serve.h — continuous-batching serving loop over GPU-resident runs
 * (no counterpart in the reference, which runs one simulation per process).
 *
 * Requests — each a complete PIC run: configuration, species, step count,
 * collisions on/off, loader seed, arrival time — are held until they arrive,
 * then admitted in arrival order while the estimated device bytes of all
 * admitted runs stay within the budget and fewer than max_inflight runs are
 * resident.  An admitted run is created on the GPU, loaded on the device
 * (epic_load_particles_device), given its initial field, and advanced in
 * chunks of chunk_steps steps replayed from captured graphs on its own
 * stream, so the chunks of all resident runs overlap on the device.  A
 * finished run is digested (epic_digest), its energies are recorded, and its
 * memory returns to the budget for the next arrivals.  Runs whose Poisson
 * solve uses a grid-wide barrier (FP64 PCG or red-black SOR, or the mixed
 * form under gssolver with dx != dy) are admitted only when nothing else is resident,
 * and nothing else is admitted while they run.  Every kernel of a run is
 * deterministic, so its result is bit-identical alone and in a mix.
 *
 * One scheduler thread drives the device; the calls below may come from any
 * thread. */
#ifndef EPIC2D_SERVE_H
#define EPIC2D_SERVE_H

#include "epic2d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct epic_server epic_server;

enum { EPIC_REQUEST_MAX_CONDUCTORS = 8, EPIC_REQUEST_MAX_EMITTERS = 8 };

typedef struct {
  epic_config cfg;
  epic_species_desc species[8];
  int num_species;
  int steps;
  int collisions;       /* MCC every step (species 0 against the gas, ions into species 1) */
  uint64_t load_seed;   /* Philox seed of the device loader */
  double arrival_s;     /* arrival, seconds after epic_server_start */
  /* The deck's [Grids] and [Emitters] (epic_conductors_from_ini,
   * epic_emitters_from_ini).  A run with conductors is loaded on the host
   * (epic_load_particles with load_seed), whose loader keeps particles out of
   * them; a run with emitters gets the room its injections need. */
  int num_conductors;
  epic_conductor conductors[EPIC_REQUEST_MAX_CONDUCTORS];
  int num_emitters;
  epic_emitter emitters[EPIC_REQUEST_MAX_EMITTERS];
} epic_request;

typedef struct {
  int64_t id;
  int status;           /* epic_status of the run (EPIC_ERR_BUDGET: it can never fit the budget) */
  double arrival_s, admit_s, finish_s;
  int64_t particle_steps;  /* initial particles x steps */
  int64_t bytes;           /* admission estimate */
  uint64_t digest[2];      /* epic_digest at the end */
  double kinetic_energy;   /* sum over species and components of Compute_KE (norm species 0) */
  double potential_energy; /* Compute_PE (norm species 0) */
} epic_result;

typedef struct {
  int64_t submitted, completed, failed;
  double p50_latency_s, p99_latency_s, mean_latency_s, max_latency_s;
  double makespan_s;          /* first arrival to last completion */
  double particle_steps_per_s;
  int64_t peak_bytes;         /* largest total estimate resident at once */
  int peak_inflight;
} epic_server_stats;

/* Estimated device bytes of one run (grids, particles, sort, MCC and loader
 * scratch), used for admission. */
int64_t epic_estimate_bytes(const epic_config* cfg, const epic_species_desc* species, int num_species,
                            int collisions);

epic_status epic_server_create(int64_t hbm_budget_bytes, int max_inflight, int chunk_steps, epic_server** out);
void epic_server_destroy(epic_server* srv);
/* Cross sections for every request with collisions (epic_set_log_cross_sections). */
epic_status epic_server_set_log_cross_sections(epic_server* srv, const double* ela, const double* exc,
                                               const double* ion, int64_t n, double e_min, double e_max);
epic_status epic_server_submit(epic_server* srv, const epic_request* req, int64_t* id);
/* Starts the clock and the scheduler thread. */
epic_status epic_server_start(epic_server* srv);
/* Waits until every submitted request has finished (EPIC_ERR_TIMEOUT after timeout_s). */
epic_status epic_server_wait(epic_server* srv, double timeout_s);
epic_status epic_server_result(epic_server* srv, int64_t id, epic_result* out);
epic_status epic_server_get_stats(epic_server* srv, epic_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif
