/*
 * mpcd_server.h - continuous batching of swimmer runs on one GPU.
 *
 * A request is a sim.cfg (the reference's input, src/main.cpp:48-98) plus a
 * number of MPC steps and a seed.  The server builds each request's system on
 * the host (preparation threads), admits it into a replica batch
 * (mpcd_batch.h) as soon as its device footprint fits the budget and the
 * batch's capacities, runs every resident request in the batch's shared
 * launches, and retires requests as they finish (their result stays on the
 * host), so requests that arrive while others run join the running batch.
 * A request's physics does not depend on what else is resident: its random
 * numbers are keyed by its own seed and step counter (mpcd_batch.h).
 *
 * Admission is first come, first served with look-ahead: a request that does
 * not fit yet lets later, smaller requests in.  Times are seconds since the
 * server started.  Thread-safe: any host thread may submit and wait.
 */
#ifndef MPCD_SERVER_H
#define MPCD_SERVER_H

#include "mpcd_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpcd_server mpcd_server;

typedef struct {
  mpcd_batch_params batch;  /* capacities of the device batch; its MD layout must hold the largest swimmer */
  long long budget_bytes;   /* admission limit on the sum of resident footprints (0: capacities only) */
  int chunk_steps;          /* MPC steps per scheduling round (0: 25) */
  int keep_fluid;           /* 1: a finished request keeps its fluid state for mpcd_server_result_fluid */
  int lookahead;            /* queued requests considered per round (0: 16) */
  int prep_threads;         /* host threads building requests from their cfg (0: 2) */
  double preempt_wait_s;    /* > 0: when the oldest waiting request has waited this long, the
                               resident request with the most steps left (more than it needs) is
                               pre-empted (0: never) */
} mpcd_server_params;

#define MPCD_REQ_QUEUED 0
#define MPCD_REQ_RESIDENT 1
#define MPCD_REQ_DONE 2
#define MPCD_REQ_FAILED 3

typedef struct {
  long long id;
  int state;               /* MPCD_REQ_* */
  long long steps;         /* MPC steps run */
  double t_submit, t_admit, t_done;
  long long nfluid, nbeads;
  long long footprint;     /* device bytes while resident */
  mpcd_obs obs;            /* observables at completion */
  unsigned err_bits;       /* device check bits of the replica */
  int preemptions;         /* times it was pre-empted */
} mpcd_request_info;

typedef struct {
  long long submitted, completed, failed, resident, queued;
  double p50_s, p99_s, mean_s, max_s; /* completion latency (submit -> done) of completed requests */
  double particle_steps;              /* (fluid + beads) x steps of completed requests */
  double busy_s;                      /* wall time with at least one request resident */
  double throughput;                  /* particle_steps / busy_s */
  long long peak_resident_bytes;
  int peak_resident;
  long long gpu_launches;
  long long preemptions;
} mpcd_server_stats;

int mpcd_server_create(const mpcd_server_params* p, mpcd_server** out);
/* stops the server; queued and resident requests are dropped */
int mpcd_server_destroy(mpcd_server* s);
const char* mpcd_server_last_error(const mpcd_server* s);
int mpcd_server_submit(mpcd_server* s, const char* cfg_text, long long nsteps, unsigned long long seed,
                       long long* id);
int mpcd_server_info(mpcd_server* s, long long id, mpcd_request_info* out);
/* waits until the request is done or failed (MPCD_ESTATE after timeout_s) */
int mpcd_server_wait(mpcd_server* s, long long id, double timeout_s, mpcd_request_info* out);
/* waits until every submitted request is done or failed */
int mpcd_server_drain(mpcd_server* s, double timeout_s);
int mpcd_server_result_beads(mpcd_server* s, long long id, long nb, double* pos, double* vel);
int mpcd_server_result_fluid(mpcd_server* s, long long id, long n, double* pos, double* vel);
int mpcd_server_get_stats(mpcd_server* s, mpcd_server_stats* out);
/* Pre-empts a resident request at the end of the current round: its state
 * (fluid, beads, cilia beat state, grid shift, time, step counter) is read
 * back to the host, its device ranges are freed, and it waits at the head of
 * the queue; admitted again, it resumes from that state with the same random
 * sequence, so its result is that of an uninterrupted run up to the order of
 * float additions into cell sums (its dissipated energy counts from the
 * resumption).  MPCD_ESTATE if it is not resident. */
int mpcd_server_preempt(mpcd_server* s, long long id);
/* why a request failed ("" otherwise); valid until the server is destroyed */
const char* mpcd_server_request_error(mpcd_server* s, long long id);

#ifdef __cplusplus
}
#endif

#endif /* MPCD_SERVER_H */
