/* eqserve: continuous-batching request loop over the eqfield trap solver.
 *
 * No counterpart in the reference (eQ steps one fixed simulation per MPI rank,
 * src/simulation.cpp:415-520).  A request is one trap simulation (one species, or
 * the sender/receiver pair of eqf_couple_species) run for a number of steps.
 * Requests are admitted in arrival order while the device-memory budget allows
 * (eqf_footprint_estimate), grouped into cohorts -- one eqfield batch each, on its
 * own CUDA stream, holding requests of one class (multigrid depth and Krylov
 * method): the oldest waiting request and the later ones of its class -- and
 * cohorts step concurrently, so requests that arrive while
 * others run are admitted as memory frees up and their steps overlap on the
 * device.  A request whose steps are done is read out and frozen (its cohort
 * stops computing it); a cohort is released when all its requests are done.
 * Every trap's field and solver state stays resident on the device for the
 * whole request.  Since cohorts are class-pure and every trap's arithmetic is
 * independent of the others in its batch, a request's result is the same, bit
 * for bit, alone and in any mix.
 *
 * Single-threaded: all calls on one server from one host thread.  Every call
 * returns EQF_OK (0) or a negative EQF_ERR_* code (eqfield.h) with eqs_last_error. */
#ifndef EQSERVE_H
#define EQSERVE_H

#include <stdint.h>

#include "eqfield.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct eqs_server eqs_server;

typedef struct eqs_config {
  eqf_solver_opts opts;     /* cohort solver options (graphs and adaptive sweeps forced on) */
  int64_t hbm_budget;       /* device bytes the server's cohorts may hold */
  int32_t max_cohorts;      /* cohorts stepping concurrently (one stream each) */
  int32_t max_cohort_traps; /* traps per cohort */
  int32_t min_batch;        /* form a cohort once this many requests wait ... */
  double max_wait_ms;       /* ... or the oldest has waited this long, or the GPU idles */
  int32_t steps_in_flight;  /* steps queued ahead per cohort */
  int32_t reuse_slots;      /* 1 (default): admit waiting requests into the slots of
                               finished ones in a resident cohort (eqf_replace_traps)
                               when their grids fit; 0: only into new cohorts */
} eqs_config;

typedef struct eqs_request {
  eqf_trap_params species[2]; /* species 1 and (n_species = 2) species 2, same mesh */
  int32_t n_species;          /* 1 or 2 */
  int64_t n_cells;
  const double* xy;           /* 2 * n_cells cell centres */
  const double* s;            /* n_cells source rates (species 1 production) */
  const int32_t* sender;      /* n_cells sender flags (2 species only) */
  double vmax, K, uptake;     /* sender/receiver law (2 species only) */
  int32_t steps;              /* >= 1 */
  int32_t want_nodal;         /* also return the final nodal field(s) */
} eqs_request;

typedef struct eqs_result_info {
  double t_submit, t_admit, t_done; /* seconds since the server was created */
  int32_t steps;
  int32_t status;                   /* EQF_OK, or the error the request ended with */
  int64_t n_nodes, n_cells;
  int32_t n_species;
  int32_t cohort;                   /* id of the cohort that ran it */
} eqs_result_info;

typedef struct eqs_stats {
  int64_t submitted, admitted, completed, failed, cohorts;
  int64_t pending, running;
  double dof_steps;                 /* completed work: nodes x species x steps */
  double busy_s;                    /* wall time with at least one cohort running */
  double step_ms_p50, step_ms_p99, step_ms_p999; /* cohort step latency (CUDA events) */
  int64_t step_samples;
  int64_t bytes_in_use, bytes_peak;
  double admit_s;                   /* host seconds spent forming cohorts (incl. releases) */
  double launch_s;                  /* host seconds spent queueing cohort steps */
  double release_s;                 /* host seconds spent releasing retired cohorts */
  double first_step_s;              /* of launch_s: queueing each cohort's first step
                                       (its one-time set-up: cell index, graph capture) */
  double readout_s;                 /* of launch_s: queueing finished requests' readouts
                                       and freezes */
  int64_t slot_admitted;            /* of admitted: into the free slots of a resident
                                       cohort */
  double fill_s;                    /* host seconds spent admitting into free slots */
  int64_t fills;                    /* slot admissions (each one eqf_replace_traps) */
  double refill_step_s;             /* of launch_s: queueing the first step after a
                                       fill (cell index and step graph rebuilt) */
} eqs_stats;

int eqs_default_config(eqs_config* cfg);
int eqs_create(const eqs_config* cfg, eqs_server** out);
int eqs_destroy(eqs_server* s);
const char* eqs_last_error(const eqs_server* s);

/* Copies the request's inputs and queues it; *id >= 0.  A request larger than the
 * whole budget is refused with EQF_ERR_TOO_LARGE. */
int eqs_submit(eqs_server* s, const eqs_request* r, int64_t* id);

/* Non-blocking progress: retire finished steps and requests, release finished
 * cohorts, admit waiting requests into a new cohort, queue further steps. */
int eqs_progress(eqs_server* s);

/* Ids of requests finished since the last call (each reported once). */
int eqs_take_done(eqs_server* s, int64_t* ids, int32_t cap, int32_t* n);

/* Copies a finished request's per-cell concentrations (n_species * n_cells,
 * species-major) and, when it asked for them, its nodal fields (n_species *
 * n_nodes), then forgets the request.  cells / nodal may be NULL. */
int eqs_result(eqs_server* s, int64_t id, double* cells, double* nodal, eqs_result_info* info);

int eqs_get_stats(eqs_server* s, eqs_stats* st);

/* Runs eqs_progress until no request is pending or running. */
int eqs_drain(eqs_server* s);

#ifdef __cplusplus
}
#endif

#endif /* EQSERVE_H */
