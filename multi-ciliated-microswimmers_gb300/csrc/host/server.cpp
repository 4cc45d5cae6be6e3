// Continuous batching of swimmer runs (include/mpcd_server.h).
//
// Three parties:
//  - callers submit requests (any thread) and wait for results;
//  - preparation threads build each request's system on the host from its
//    sim.cfg (objects, springs, fluid: the reference's Simulation
//    constructor, src/simulation.cpp:19-35, without an engine) and estimates
//    its device footprint;
//  - the device thread owns the replica batch: between scheduling rounds it
//    admits prepared requests that fit, runs one round of `chunk_steps` MPC
//    steps of every resident request in the batch's shared launches, and
//    retires the requests whose steps are done (observables, beads and,
//    when asked, the fluid go back to the host; the device ranges are freed).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "libconfig_lite.hpp"
#include "mpcd_server.h"
#include "objects.hpp"

namespace {

struct Request {
  long long id = 0;
  std::string cfg;
  long long nsteps = 0;
  unsigned long long seed = 0;
  int state = MPCD_REQ_QUEUED;
  double t_submit = 0, t_admit = -1, t_done = -1;
  std::string error;
  // prepared on the host
  std::unique_ptr<cilia::HostSystem> sys;
  long nbeads = 0, nfluid = 0;
  long long footprint = 0;
  int replica = -1;
  // pre-emption: the host system keeps the springs and cilia layout while the
  // request is resident; a pre-empted request's state is read back into it
  long long steps_offset = 0;  // collisions done before the current admission
  int preemptions = 0;
  bool preempt_flag = false;
  // results
  mpcd_obs obs{};
  unsigned err = 0;
  long long steps_done = 0;
  std::vector<double> bpos, bvel, fpos, fvel;
};

using ReqPtr = std::shared_ptr<Request>;

}  // namespace

struct mpcd_server {
  mpcd_server_params p{};
  mpcd_batch* batch = nullptr;
  std::string error;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_prep, cv_ready, cv_done;
  std::map<long long, ReqPtr> all;
  std::deque<ReqPtr> to_prep, ready;
  std::vector<ReqPtr> resident;
  bool stop = false;
  long long next_id = 1;
  std::vector<std::thread> prep_threads;
  std::thread dev_thread;
  // statistics (device thread writes, callers read under mu)
  long long resident_bytes = 0, peak_bytes = 0;
  int peak_resident = 0;
  long long preemptions = 0;
  double busy_s = 0.0;
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

void prepare(mpcd_server* s, const ReqPtr& q) {
  libconfig::Config c;
  c.readString(q->cfg.c_str());
  cilia::SimOptions so;
  so.host_only = 1;
  so.precision = MPCD_FP32;
  so.read_files = 0;
  so.seed = q->seed;
  cilia::Simulation sim(c.getRoot(), so);
  q->sys.reset(new cilia::HostSystem(std::move(sim.host)));
  q->nbeads = sim.nbeads;
  q->nfluid = (long)q->sys->fpos.size() / 3;
  const long ncell = (long)q->sys->p.sizes[0] * q->sys->p.sizes[1] * q->sys->p.sizes[2];
  q->footprint = mpcd_batch_estimate(s->batch, q->nfluid, ncell, q->nbeads, (long)q->sys->springs.size(),
                                     (int)q->sys->cilia.size(), (long)q->sys->newlen.size());
}

void prep_loop(mpcd_server* s) {
  for (;;) {
    ReqPtr q;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_prep.wait(lk, [&] { return s->stop || !s->to_prep.empty(); });
      if (s->stop) return;
      q = s->to_prep.front();
      s->to_prep.pop_front();
    }
    std::string err;
    try {
      prepare(s, q);
    } catch (const libconfig::ParseException& e) {
      err = std::string("cfg parse error at line ") + std::to_string(e.getLine()) + ": " + e.getError();
    } catch (const libconfig::SettingException& e) {
      err = std::string("cfg setting error: ") + e.getPath();
    } catch (const std::exception& e) {
      err = e.what();
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (!err.empty()) {
      q->state = MPCD_REQ_FAILED;
      q->error = err;
      q->t_done = s->now();
      s->cv_done.notify_all();
    } else if (s->p.budget_bytes > 0 && q->footprint > s->p.budget_bytes) {
      q->state = MPCD_REQ_FAILED;
      q->error = "request footprint exceeds the device budget";
      q->sys.reset();
      q->t_done = s->now();
      s->cv_done.notify_all();
    } else {
      s->ready.push_back(q);
      s->cv_ready.notify_all();
    }
  }
}

// moves ready requests into the batch while they fit (device thread only)
void admit_ready(mpcd_server* s) {
  std::vector<ReqPtr> cand;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const int la = s->p.lookahead > 0 ? s->p.lookahead : 16;
    for (size_t k = 0; k < s->ready.size() && (int)cand.size() < la; ++k) cand.push_back(s->ready[k]);
  }
  for (const ReqPtr& q : cand) {
    if (s->p.budget_bytes > 0 && s->resident_bytes + q->footprint > s->p.budget_bytes) continue;
    int r = -1;
    std::string err;
    bool fits = false;
    try {
      cilia::add_to_batch(s->batch, *q->sys, q->nbeads, &r);
      if (q->steps_offset > 0 && mpcd_batch_set_step_count(s->batch, r, q->steps_offset) != MPCD_OK)
        throw std::runtime_error(mpcd_batch_last_error(s->batch));
      if (mpcd_batch_admit(s->batch, r) == MPCD_OK) {
        fits = mpcd_batch_set_steps(s->batch, r, q->nsteps - q->steps_offset) == MPCD_OK;
        if (!fits) err = mpcd_batch_last_error(s->batch);
      } else {
        err = mpcd_batch_last_error(s->batch);
      }
      if (!fits) mpcd_batch_remove(s->batch, r);
    } catch (const std::exception& e) {
      err = e.what();
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (fits) {
      q->replica = r;
      q->state = MPCD_REQ_RESIDENT;
      if (q->t_admit < 0) q->t_admit = s->now();
      // the fluid's host copy is not needed while resident (a pre-emption reads it back)
      std::vector<double>().swap(q->sys->fpos);
      std::vector<double>().swap(q->sys->fvel);
      s->resident.push_back(q);
      s->resident_bytes += q->footprint;
      s->peak_bytes = std::max(s->peak_bytes, s->resident_bytes);
      s->peak_resident = std::max(s->peak_resident, (int)s->resident.size());
      s->ready.erase(std::find(s->ready.begin(), s->ready.end(), q));
    } else if (s->resident.empty()) {
      // it does not fit into an empty batch: it never will
      q->state = MPCD_REQ_FAILED;
      q->error = "request does not fit the batch capacities: " + err;
      q->sys.reset();
      q->t_done = s->now();
      s->ready.erase(std::find(s->ready.begin(), s->ready.end(), q));
      s->cv_done.notify_all();
    }
  }
}

// Pre-emption policy (mpcd_server_params.preempt_wait_s): when the oldest
// ready request has waited longer than that and is still not resident, the
// resident request with the most steps left (more than the waiting one
// needs) is pre-empted at the end of the round, so that a short request does
// not wait behind long ones for the whole of their runs.
void choose_preemption(mpcd_server* s) {
  if (s->p.preempt_wait_s <= 0) return;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->ready.empty() || s->resident.empty()) return;
  const ReqPtr& head = s->ready.front();
  if (s->now() - head->t_submit < s->p.preempt_wait_s) return;
  for (const ReqPtr& q : s->resident)
    if (q->preempt_flag) return;  // one at a time
  ReqPtr victim;
  long long most = head->nsteps - head->steps_offset;
  for (const ReqPtr& q : s->resident) {
    const long long left = q->nsteps - q->steps_done;
    if (left > most) {
      most = left;
      victim = q;
    }
  }
  if (victim) victim->preempt_flag = true;
}

// Reads a resident request's state back into its host system, frees its
// replica and puts it at the head of the ready queue; it resumes from that
// state (and its step counter, so its random sequence continues) when it is
// admitted again.  The dissipated energy restarts from zero at resumption.
void preempt(mpcd_server* s, const ReqPtr& q) {
  cilia::HostSystem& h = *q->sys;
  long long done = 0, left = 0;
  double t = 0;
  unsigned err = 0;
  bool ok = mpcd_batch_status(s->batch, q->replica, &done, &left, &t, &err) == MPCD_OK && !err;
  if (ok && q->nfluid > 0) {
    h.fpos.resize(3 * q->nfluid);
    h.fvel.resize(3 * q->nfluid);
    ok = mpcd_batch_get_fluid(s->batch, q->replica, q->nfluid, h.fpos.data(), h.fvel.data()) == MPCD_OK;
  }
  if (ok && q->nbeads > 0) {
    ok = mpcd_batch_get_beads(s->batch, q->replica, q->nbeads, h.bpos.data(), h.bvel.data()) == MPCD_OK;
    std::vector<double> st(2 * h.cilia.size());
    ok = ok && mpcd_batch_get_cilia(s->batch, q->replica, (int)h.cilia.size(), st.data(), h.newlen.data(),
                                    h.oldlen.data()) == MPCD_OK;
    for (size_t c = 0; ok && c < h.cilia.size(); ++c) {
      h.cilia[c].midpnt = st[2 * c];
      h.cilia[c].tstroke = st[2 * c + 1];
    }
  }
  ok = ok && mpcd_batch_get_shift(s->batch, q->replica, h.a) == MPCD_OK;
  if (!ok) return;  // left resident; it finishes normally
  h.globalt = t;
  mpcd_batch_remove(s->batch, q->replica);
  std::lock_guard<std::mutex> lk(s->mu);
  q->replica = -1;
  q->steps_offset = done;
  q->steps_done = done;
  q->preempt_flag = false;
  q->preemptions++;
  s->preemptions++;
  q->state = MPCD_REQ_QUEUED;
  s->resident_bytes -= q->footprint;
  s->resident.erase(std::find(s->resident.begin(), s->resident.end(), q));
  // right behind the oldest waiting request (the one the room is made for),
  // ahead of everything else
  s->ready.insert(s->ready.empty() ? s->ready.begin() : s->ready.begin() + 1, q);
}

void retire(mpcd_server* s, const ReqPtr& q, long long steps, unsigned err) {
  mpcd_obs o{};
  const int rc_obs = mpcd_batch_observables(s->batch, q->replica, &o);
  std::vector<double> bp, bv, fp, fv;
  if (q->nbeads > 0) {
    bp.resize(3 * q->nbeads);
    bv.resize(3 * q->nbeads);
    mpcd_batch_get_beads(s->batch, q->replica, q->nbeads, bp.data(), bv.data());
  }
  if (s->p.keep_fluid && q->nfluid > 0) {
    fp.resize(3 * q->nfluid);
    fv.resize(3 * q->nfluid);
    mpcd_batch_get_fluid(s->batch, q->replica, q->nfluid, fp.data(), fv.data());
  }
  mpcd_batch_remove(s->batch, q->replica);
  std::lock_guard<std::mutex> lk(s->mu);
  q->obs = o;
  q->err = err;
  q->steps_done = steps;
  q->bpos.swap(bp);
  q->bvel.swap(bv);
  q->fpos.swap(fp);
  q->fvel.swap(fv);
  q->state = (err || rc_obs != MPCD_OK) ? MPCD_REQ_FAILED : MPCD_REQ_DONE;
  if (q->state == MPCD_REQ_FAILED) q->error = "device check failed for this request";
  q->t_done = s->now();
  q->sys.reset();
  s->resident_bytes -= q->footprint;
  s->resident.erase(std::find(s->resident.begin(), s->resident.end(), q));
  s->cv_done.notify_all();
}

void dev_loop(mpcd_server* s) {
  const int chunk = s->p.chunk_steps > 0 ? s->p.chunk_steps : 25;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) return;
      if (s->resident.empty() && s->ready.empty()) {
        s->cv_ready.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    const double t_round = s->now();
    admit_ready(s);
    std::vector<ReqPtr> res;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      res = s->resident;
    }
    if (res.empty()) continue;
    if (mpcd_batch_run(s->batch, chunk) != MPCD_OK || mpcd_batch_sync(s->batch) != MPCD_OK) {
      std::lock_guard<std::mutex> lk(s->mu);
      s->error = std::string("batch run failed: ") + mpcd_batch_last_error(s->batch);
      for (const ReqPtr& q : res) {
        q->state = MPCD_REQ_FAILED;
        q->error = s->error;
        q->t_done = s->now();
      }
      s->resident.clear();
      s->cv_done.notify_all();
      s->stop = true;
      return;
    }
    choose_preemption(s);
    for (const ReqPtr& q : res) {
      long long done = 0, left = 0;
      double t = 0;
      unsigned err = 0;
      if (mpcd_batch_status(s->batch, q->replica, &done, &left, &t, &err) != MPCD_OK) err |= 0x80000000u;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        q->steps_done = done;
      }
      if (left == 0 || err)
        retire(s, q, done, err);
      else if (q->preempt_flag)
        preempt(s, q);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->busy_s += s->now() - t_round;
  }
}

void fill_info(const Request& q, mpcd_request_info* o) {
  std::memset(o, 0, sizeof *o);
  o->id = q.id;
  o->state = q.state;
  o->steps = q.steps_done;
  o->t_submit = q.t_submit;
  o->t_admit = q.t_admit;
  o->t_done = q.t_done;
  o->nfluid = q.nfluid;
  o->nbeads = q.nbeads;
  o->footprint = q.footprint;
  o->obs = q.obs;
  o->err_bits = q.err;
  o->preemptions = q.preemptions;
}

}  // namespace

extern "C" {

int mpcd_server_create(const mpcd_server_params* p, mpcd_server** out) {
  if (!p || !out) return MPCD_EINVAL;
  *out = nullptr;
  std::unique_ptr<mpcd_server> s(new mpcd_server());
  s->p = *p;
  s->t0 = std::chrono::steady_clock::now();
  int rc = mpcd_batch_create(&s->p.batch, &s->batch);
  if (rc) return rc;
  const int np = s->p.prep_threads > 0 ? std::min(s->p.prep_threads, 16) : 2;
  for (int k = 0; k < np; ++k) s->prep_threads.emplace_back(prep_loop, s.get());
  s->dev_thread = std::thread(dev_loop, s.get());
  *out = s.release();
  return MPCD_OK;
}

int mpcd_server_destroy(mpcd_server* s) {
  if (!s) return MPCD_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_prep.notify_all();
  s->cv_ready.notify_all();
  for (auto& t : s->prep_threads)
    if (t.joinable()) t.join();
  if (s->dev_thread.joinable()) s->dev_thread.join();
  mpcd_batch_destroy(s->batch);
  delete s;
  return MPCD_OK;
}

const char* mpcd_server_last_error(const mpcd_server* s) { return s ? s->error.c_str() : "null server"; }

int mpcd_server_submit(mpcd_server* s, const char* cfg_text, long long nsteps, unsigned long long seed,
                       long long* id) {
  if (!s || !cfg_text || nsteps < 0 || !id) return MPCD_EINVAL;
  ReqPtr q(new Request());
  q->cfg = cfg_text;
  q->nsteps = nsteps;
  q->seed = seed;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return MPCD_ESTATE;
    q->id = s->next_id++;
    q->t_submit = s->now();
    s->all[q->id] = q;
    s->to_prep.push_back(q);
  }
  s->cv_prep.notify_one();
  *id = q->id;
  return MPCD_OK;
}

int mpcd_server_info(mpcd_server* s, long long id, mpcd_request_info* out) {
  if (!s || !out) return MPCD_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return MPCD_EINVAL;
  fill_info(*it->second, out);
  return MPCD_OK;
}

int mpcd_server_wait(mpcd_server* s, long long id, double timeout_s, mpcd_request_info* out) {
  if (!s) return MPCD_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return MPCD_EINVAL;
  ReqPtr q = it->second;
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    return q->state == MPCD_REQ_DONE || q->state == MPCD_REQ_FAILED || s->stop;
  });
  if (out) fill_info(*q, out);
  if (!ok) return MPCD_ESTATE;
  if (q->state == MPCD_REQ_FAILED) {
    s->error = q->error;
    return MPCD_EDEVICE;
  }
  return MPCD_OK;
}

int mpcd_server_drain(mpcd_server* s, double timeout_s) {
  if (!s) return MPCD_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
    if (s->stop) return true;
    for (auto& kv : s->all)
      if (kv.second->state != MPCD_REQ_DONE && kv.second->state != MPCD_REQ_FAILED) return false;
    return true;
  });
  return ok ? MPCD_OK : MPCD_ESTATE;
}

int mpcd_server_result_beads(mpcd_server* s, long long id, long nb, double* pos, double* vel) {
  if (!s) return MPCD_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end() || it->second->state != MPCD_REQ_DONE || nb != it->second->nbeads) return MPCD_EINVAL;
  const Request& q = *it->second;
  if (pos && nb) std::memcpy(pos, q.bpos.data(), 3 * nb * sizeof(double));
  if (vel && nb) std::memcpy(vel, q.bvel.data(), 3 * nb * sizeof(double));
  return MPCD_OK;
}

int mpcd_server_result_fluid(mpcd_server* s, long long id, long n, double* pos, double* vel) {
  if (!s) return MPCD_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end() || it->second->state != MPCD_REQ_DONE || n != it->second->nfluid ||
      (long)it->second->fpos.size() != 3 * n)
    return MPCD_EINVAL;
  const Request& q = *it->second;
  if (pos && n) std::memcpy(pos, q.fpos.data(), 3 * n * sizeof(double));
  if (vel && n) std::memcpy(vel, q.fvel.data(), 3 * n * sizeof(double));
  return MPCD_OK;
}

const char* mpcd_server_request_error(mpcd_server* s, long long id) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return "unknown request";
  return it->second->error.c_str();
}

int mpcd_server_get_stats(mpcd_server* s, mpcd_server_stats* out) {
  if (!s || !out) return MPCD_EINVAL;
  std::memset(out, 0, sizeof *out);
  std::vector<double> lat;
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto& kv : s->all) {
    const Request& q = *kv.second;
    out->submitted++;
    if (q.state == MPCD_REQ_DONE) {
      out->completed++;
      lat.push_back(q.t_done - q.t_submit);
      out->particle_steps += (double)(q.nfluid + q.nbeads) * (double)q.steps_done;
    } else if (q.state == MPCD_REQ_FAILED) {
      out->failed++;
    } else if (q.state == MPCD_REQ_RESIDENT) {
      out->resident++;
    } else {
      out->queued++;
    }
  }
  if (!lat.empty()) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double f) {
      const double x = f * (lat.size() - 1);
      const size_t i = (size_t)x;
      const double w = x - i;
      return i + 1 < lat.size() ? lat[i] * (1 - w) + lat[i + 1] * w : lat[i];
    };
    out->p50_s = pct(0.5);
    out->p99_s = pct(0.99);
    out->max_s = lat.back();
    double m = 0;
    for (double x : lat) m += x;
    out->mean_s = m / lat.size();
  }
  out->busy_s = s->busy_s;
  out->throughput = s->busy_s > 0 ? out->particle_steps / s->busy_s : 0.0;
  out->peak_resident_bytes = s->peak_bytes;
  out->peak_resident = s->peak_resident;
  out->gpu_launches = mpcd_batch_launch_count(s->batch);
  out->preemptions = s->preemptions;
  return MPCD_OK;
}

int mpcd_server_preempt(mpcd_server* s, long long id) {
  if (!s) return MPCD_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return MPCD_EINVAL;
  if (it->second->state != MPCD_REQ_RESIDENT) return MPCD_ESTATE;
  it->second->preempt_flag = true;
  return MPCD_OK;
}

}  // extern "C"
