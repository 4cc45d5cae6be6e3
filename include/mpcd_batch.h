/*
 * mpcd_batch.h - many independent MPCD + microswimmer boxes ("replicas")
 * advanced together on one GPU, in split precision.
 *
 * The reference runs one box per process (src/main.cpp:117-148,
 * Simulation::run, src/simulation.cpp:59-156); a batch runs many such
 * boxes of different sizes and swimmer sizes at once: every MPC step is one
 * launch per stage for all replicas (cell maps, fluid collide + stream + bin)
 * plus one cluster launch per MD layout size, captured in CUDA graphs.  Each
 * replica's physics is the single-box split-precision step of mpcd_gpu.h
 * (MPCD_FP32), with the same random-number keys (its seed, its step counter,
 * its own cell indices): a replica's trajectory is the one it would have run
 * alone, up to the order of float additions into its cell sums.
 *
 * Lifecycle of a replica: mpcd_batch_add -> setters (as for one engine) ->
 * mpcd_batch_admit (device ranges, upload, binning) -> mpcd_batch_set_steps
 * -> mpcd_batch_run ... -> getters -> mpcd_batch_remove.  Replicas can be
 * admitted and removed between runs; device memory is reserved once, at
 * mpcd_batch_create, from the capacities given there.
 *
 * All calls from one host thread per batch.  Status codes as mpcd_gpu.h.
 */
#ifndef MPCD_BATCH_H
#define MPCD_BATCH_H

#include "mpcd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpcd_batch mpcd_batch;

typedef struct {
  int device;
  int max_replicas;      /* replica slots */
  long max_particles;    /* fluid particles over all resident replicas */
  long max_cells;        /* cells over all resident replicas */
  long max_slots;        /* MD bead slots (helpers and padding included) */
  long max_springs;      /* one-sided springs */
  long max_halo;         /* halo entries of the MD tiles */
  int max_cilia;
  long max_bonds;        /* beat rest-length entries (rodlength per cilium) */
  int md_lanes;          /* MD layout: threads per bead slot (1 or 2; 0: 2) */
  int md_tile;           /* MD layout: slots per CTA (0: 512 / md_lanes) */
  int sort_interval;     /* MPC steps between counting sorts (0: 25) */
  int sorts_per_graph;   /* sort periods captured in one CUDA graph (0: 4) */
} mpcd_batch_params;

/* launch configuration chosen by mpcd_batch_autotune (or set by hand) */
typedef struct {
  int fluid_threads, fluid_blocks;   /* blocks 0: one per page up to 8 per SM; threads 0: the fluid pass
                                        staged through shared memory by bulk copies (TMA) */
  int cell_threads, cell_blocks;
  int sort_interval;
} mpcd_batch_tuning;

int mpcd_batch_create(const mpcd_batch_params* p, mpcd_batch** out);
int mpcd_batch_destroy(mpcd_batch* b);
const char* mpcd_batch_last_error(const mpcd_batch* b);

/* a new replica slot; p->precision must be MPCD_FP32, p->walls MPCD_WALLS_NONE */
int mpcd_batch_add(mpcd_batch* b, const mpcd_params* p, int* replica);
/* a new replica holding a copy of a single-box engine's state: its
 * parameters (precision and walls as for mpcd_batch_add), fluid, grid shift,
 * time, step counter, beads, springs and cilia.  The engine is not changed. */
int mpcd_batch_add_engine(mpcd_batch* b, mpcd_engine* h, int* replica);
/* setters before admission, with the meaning of the mpcd_gpu.h setters */
int mpcd_batch_set_fluid(mpcd_batch* b, int r, long n, const double* pos, const double* vel);
int mpcd_batch_set_shift(mpcd_batch* b, int r, const double* a3);
int mpcd_batch_set_time(mpcd_batch* b, int r, double globalt);
int mpcd_batch_set_beads(mpcd_batch* b, int r, long nb, const double* pos, const double* vel, const int* moves);
int mpcd_batch_set_springs(mpcd_batch* b, int r, long ns, const int* target, const int* other, const int* kind,
                           const int* ref, const double* rest, const double* k);
int mpcd_batch_set_cilia(mpcd_batch* b, int r, int nc, const mpcd_cilium* cilia, const double* newlength,
                         const double* oldlength);
/* device bytes the replica will hold once admitted (fluid, cells, MD) */
int mpcd_batch_footprint(mpcd_batch* b, int r, long long* bytes);
/* the same estimate from the sizes alone: fluid particles, cells, beads,
 * springs, cilia, bond-table entries */
long long mpcd_batch_estimate(const mpcd_batch* b, long nf, long ncell, long nb, long nsprings, int ncilia,
                              long nbonds);
/* plans the replica's MD, takes its device ranges, uploads and bins it;
 * MPCD_EINVAL (nothing changed) when a capacity is exhausted */
int mpcd_batch_admit(mpcd_batch* b, int r);
/* steps the replica runs from now on (it idles once they are done) */
int mpcd_batch_set_steps(mpcd_batch* b, int r, long long nsteps);
/* nsteps MPC steps of every replica with steps left */
int mpcd_batch_run(mpcd_batch* b, int nsteps);
/* One MPC step of every replica with steps left, in which replica r takes
 * the grid shift, Gamma variates and rotation axes of `inj` (mpcd_inject of
 * mpcd_gpu.h, indexed by r's own cells; virt must be NULL) instead of its
 * generator's: the replica-batch counterpart of mpcd_step(h, inj), used to
 * run a replica against the reference's recorded randomness.  Launched
 * without graphs; waits for the step.  MPCD_EDEVICE when an injected Gamma is
 * missing for a thermostatted cell. */
int mpcd_batch_step_inject(mpcd_batch* b, int r, const mpcd_inject* inj);
/* like run, timed with CUDA events on the batch's stream: total device ms */
int mpcd_batch_timed_run(mpcd_batch* b, int nsteps, double* total_ms);
int mpcd_batch_sync(mpcd_batch* b);
/* steps done and left, simulation time, and the replica's device error bits */
int mpcd_batch_status(mpcd_batch* b, int r, long long* steps_done, long long* steps_left, double* globalt,
                      unsigned* err_bits);
int mpcd_batch_get_fluid(mpcd_batch* b, int r, long n, double* pos, double* vel);
int mpcd_batch_get_beads(mpcd_batch* b, int r, long nb, double* pos, double* vel);
int mpcd_batch_get_shift(mpcd_batch* b, int r, double* a3);
/* per cilium [midpnt, tstroke] and the bond tables (any may be NULL), as mpcd_get_cilia */
int mpcd_batch_get_cilia(mpcd_batch* b, int r, int nc, double* state2, double* newlength, double* oldlength);
/* collisions the replica has done (the step counter that keys its random
 * numbers), before admission: a replica rebuilt from another's state
 * continues that one's random sequence */
int mpcd_batch_set_step_count(mpcd_batch* b, int r, long long steps_done);
int mpcd_batch_observables(mpcd_batch* b, int r, mpcd_obs* out);
/* frees the replica's device ranges and its slot */
int mpcd_batch_remove(mpcd_batch* b, int r);
int mpcd_batch_resident(const mpcd_batch* b);

/* re-plans every swimmer's MD with another cluster layout (threads per
 * slot, slots per CTA); nothing changes when a swimmer does not fit */
int mpcd_batch_set_md_layout(mpcd_batch* b, int lanes, int tile);
int mpcd_batch_get_md_layout(const mpcd_batch* b, int* lanes, int* tile);
/* times candidate configurations (MD layout, fluid and cell launch shapes,
 * sort interval) on `trial_steps` real steps each (the replicas advance;
 * results do not depend on the configuration) and keeps the fastest */
int mpcd_batch_autotune(mpcd_batch* b, int trial_steps, mpcd_batch_tuning* chosen);
int mpcd_batch_set_tuning(mpcd_batch* b, const mpcd_batch_tuning* t);
int mpcd_batch_get_tuning(const mpcd_batch* b, mpcd_batch_tuning* t);
/* nsteps steps launched stage by stage without graphs, each stage bracketed
 * by CUDA events and the MD after the fluid pass (not beside it): device ms
 * per step of out[0] prologue + cell maps, out[1] fluid collide + stream +
 * bin, out[2] MD of all swimmers, out[3] counting sorts (amortised) */
int mpcd_batch_stage_times(mpcd_batch* b, int nsteps, double* out4);
/* kernels launched so far (graph launches count their kernels) */
long long mpcd_batch_launch_count(const mpcd_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* MPCD_BATCH_H */
