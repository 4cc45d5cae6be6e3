// C ABI of the replica batch (include/mpcd_batch.h).
//
// Host side: capacities reserved at creation, first-fit range allocators for
// every per-replica array, page tables, MD plans rebased into the shared MD
// arrays, and CUDA graphs of whole sort periods.  One step of the batch is
//   prologue -> cell_params -> { fluid_step | MD launches (one per cluster
//   size, each on its own stream) } -> next step
// so the memory-bound fluid pass and the latency-bound MD chains of all
// swimmers overlap on the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/mpcd_batch.h"
#include "batch_internal.h"
#include "engine_export.h"
#include "md_plan.h"

using namespace mpcd;

namespace {

// first-fit allocator of [offset, offset + n) ranges out of [0, cap)
class RangeAlloc {
 public:
  void reset(long cap) {
    cap_ = cap;
    free_.clear();
    if (cap > 0) free_[0] = cap;
  }
  long alloc(long n) {
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const long off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        return off;
      }
    }
    return -1;
  }
  void release(long off, long n) {
    if (n <= 0 || off < 0) return;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  long largest() const {
    long m = 0;
    for (auto& f : free_) m = std::max(m, f.second);
    return m;
  }

 private:
  long cap_ = 0;
  std::map<long, long> free_;
};

inline float bits_to_float(uint32_t u) {
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
}
inline uint32_t float_to_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, sizeof u);
  return u;
}

// wrap an unwrapped coordinate into cell index + offset in [0,1)
inline void wrap_coord(double x, int L, int& i, double& o) {
  double xw = x - std::floor(x / L) * L;
  if (xw >= L) xw -= L;
  if (xw < 0) xw += L;
  double fi = std::floor(xw);
  i = (int)fi;
  o = xw - fi;
  if (i >= L) i -= L;
  if (o >= 1.0) {
    o = 0.0;
    i = (i + 1) % L;
  }
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc((void**)p, (count > 0 ? count : 1) * sizeof(T));
}

struct Replica {
  bool used = false, admitted = false;
  mpcd_params p{};
  int nsub = 0;
  long ncell = 0;
  // staged host data
  std::vector<double> fpos, fvel;
  long nf = 0;
  double a[3] = {0.5, 0.5, 0.5};
  double globalt = 0.0;
  long long steps = 0;  // collisions done before admission
  long nb = 0;
  std::vector<double> bpos, bvel;
  std::vector<int> bmoves;
  std::vector<int> sp_t, sp_o, sp_k, sp_r;
  std::vector<double> sp_rest, sp_kk;
  std::vector<mpcd_cilium> cil;
  std::vector<double> newlen, oldlen;
  MDPlan plan;
  // device ranges
  long page0 = -1, npages = 0;    // fluid pages
  long cpage0 = -1, ncpages = 0;  // cell pages
  long tile0 = -1, ntiles_alloc = 0;
  long sp0 = -1, nsp = 0, h0 = -1, nh = 0, c0 = -1, nc = 0, b0 = -1, nbond = 0;
};

struct MDLaunch {
  int ctiles = 0, hmax = 0, nsp_max = 0, nbond_max = 0, nbuf = 2;
  int offset = 0, count = 0;  // into the device list of replica indices
};

}  // namespace

struct mpcd_batch {
  mpcd_batch_params p{};
  std::string error;
  cudaStream_t s0 = nullptr;
  cudaStream_t smd[kMaxClusterTiles] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kMaxClusterTiles] = {};
  int T = 512, lanes = 2;
  long part_cap = 0, cell_cap = 0, tile_cap = 0;
  long slot_cap = 0, tile_arr_cap = 0;  // MD slots; entries of the per-tile arrays (any layout)
  long npart_pages = 0, ncell_pages = 0;
  // device tables
  BatchRep* d_rep = nullptr;
  BatchStep* d_step = nullptr;
  BatchState* d_state = nullptr;
  int* d_part_page_rep = nullptr;
  int* d_cell_page_rep = nullptr;
  int* d_tile_rep = nullptr;
  int* d_md_reps = nullptr;
  double* d_obs = nullptr;
  // fluid (two buffers: the counting sort scatters from one into the other)
  BatchFluid fl[2] = {};
  int cur = 0;
  BatchCells cells{};
  uint32_t *d_count = nullptr, *d_start = nullptr, *d_rank = nullptr, *d_blocksums = nullptr;
  MDState md;
  // host mirrors
  std::vector<BatchRep> rep;
  std::vector<int> part_page_rep, cell_page_rep, tile_rep;
  std::vector<Replica> reps;
  RangeAlloc a_part, a_cell, a_tile, a_sp, a_halo, a_cil, a_bond;
  // MD launch plan and graphs
  std::vector<MDLaunch> launches;
  bool graphs_dirty = true;
  cudaGraphExec_t g_chunk[2] = {nullptr, nullptr};
  cudaGraphExec_t g_step[2] = {nullptr, nullptr};
  int chunk_steps = 0;
  long since_sort = 0;
  mpcd_batch_tuning tune{256, 0, 256, 0, 25};
  long long launches_total = 0;
  int kernels_per_step = 0, kernels_per_sort = 0;
  void* flush = nullptr;
};

namespace {

int fail(mpcd_batch* b, int code, const std::string& msg) {
  if (b) b->error = msg;
  return code;
}

int cuda_fail(mpcd_batch* b, cudaError_t e, const char* what) {
  return fail(b, e == cudaErrorMemoryAllocation ? MPCD_ENOMEM : MPCD_ECUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define BK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(b, e_, #call); \
  } while (0)

BatchTables tables(mpcd_batch* b) {
  BatchTables t;
  t.rep = b->d_rep;
  t.step = b->d_step;
  t.state = b->d_state;
  t.part_page_rep = b->d_part_page_rep;
  t.cell_page_rep = b->d_cell_page_rep;
  t.npart_pages = b->npart_pages;
  t.ncell_pages = b->ncell_pages;
  t.nrep = b->p.max_replicas;
  return t;
}

Replica* get_rep(mpcd_batch* b, int r) {
  if (!b || r < 0 || r >= (int)b->reps.size() || !b->reps[r].used) return nullptr;
  cudaSetDevice(b->p.device);  // the calling thread may not have the batch's device current
  return &b->reps[r];
}

void shift_from_counter(uint64_t seed, uint64_t step, double* a) {
  u32x4 q = draw4(seed, step, kStreamShift, 0u, 0u);
  a[0] = u01_dbl(q.x);
  a[1] = u01_dbl(q.y);
  a[2] = u01_dbl(q.z);
}

void free_all(mpcd_batch* b) {
  for (int par = 0; par < 2; ++par) {
    if (b->g_chunk[par]) cudaGraphExecDestroy(b->g_chunk[par]);
    if (b->g_step[par]) cudaGraphExecDestroy(b->g_step[par]);
    b->g_chunk[par] = b->g_step[par] = nullptr;
    cudaFree(b->fl[par].id);
    cudaFree(b->fl[par].pos);
    cudaFree(b->fl[par].vel);
  }
  cudaFree(b->d_rep);
  cudaFree(b->d_step);
  cudaFree(b->d_state);
  cudaFree(b->d_part_page_rep);
  cudaFree(b->d_cell_page_rep);
  cudaFree(b->d_tile_rep);
  cudaFree(b->d_md_reps);
  cudaFree(b->d_obs);
  cudaFree(b->cells.sum);
  cudaFree(b->cells.cnt);
  cudaFree(b->cells.par);
  cudaFree(b->d_count);
  cudaFree(b->d_start);
  cudaFree(b->d_rank);
  cudaFree(b->d_blocksums);
  MDState& m = b->md;
  cudaFree(m.x[0]);
  cudaFree(m.y[0]);
  cudaFree(m.z[0]);
  cudaFree(m.vx);
  cudaFree(m.vy);
  cudaFree(m.vz);
  cudaFree(m.moves);
  cudaFree(m.prim);
  cudaFree(m.nhelp);
  cudaFree(m.tile_help);
  cudaFree(m.tile_react);
  cudaFree(m.sp_start);
  cudaFree(m.sp_other);
  cudaFree(m.sp_local);
  cudaFree(m.halo);
  cudaFree(m.halo_start);
  cudaFree(m.diag);
  cudaFree(m.sp_kind);
  cudaFree(m.sp_ref);
  cudaFree(m.sp_rest);
  cudaFree(m.sp_m2k);
  cudaFree(m.cil);
  cudaFree(m.midpnt);
  cudaFree(m.tstroke);
  cudaFree(m.newlen);
  cudaFree(m.oldlen);
  cudaFree(m.tile_cil);
  cudaFree(b->flush);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  for (int g = 0; g < kMaxClusterTiles; ++g) {
    if (b->ev_join[g]) cudaEventDestroy(b->ev_join[g]);
    if (b->smd[g]) cudaStreamDestroy(b->smd[g]);
  }
  if (b->s0) cudaStreamDestroy(b->s0);
}

// MD launches: replicas grouped by tile count; a group is split where the
// union of its members' shared-memory layouts would not fit one CTA
int plan_launches(mpcd_batch* b) {
  std::vector<int> list;
  b->launches.clear();
  // position buffers for a launch layout: 2 if that fits, else 1; 0 if neither
  auto buffers = [&](const MDLaunch& L) {
    for (int nbuf = 2; nbuf >= 1; --nbuf)
      if (md_cluster_batch_feasible(b->lanes, b->T, L.ctiles,
                                    md_cluster_batch_smem(b->T, L.hmax, L.nsp_max, L.nbond_max, nbuf)))
        return nbuf;
    return 0;
  };
  for (int c = 1; c <= kMaxClusterTiles; ++c) {
    MDLaunch cur;
    for (int r = 0; r < (int)b->reps.size(); ++r) {
      const Replica& R = b->reps[r];
      if (!R.admitted || R.nb == 0 || R.plan.ntiles != c) continue;
      MDLaunch nxt = cur;
      nxt.ctiles = c;
      nxt.hmax = std::max(cur.hmax, R.plan.hmax);
      nxt.nsp_max = std::max(cur.nsp_max, R.plan.cl_nsp_max);
      nxt.nbond_max = std::max(cur.nbond_max, R.plan.cl_nbond_max);
      nxt.nbuf = buffers(nxt);
      if (cur.count > 0 && nxt.nbuf < cur.nbuf) {  // would shrink or break the layout: new launch
        b->launches.push_back(cur);
        nxt = MDLaunch{};
        nxt.ctiles = c;
        nxt.hmax = R.plan.hmax;
        nxt.nsp_max = R.plan.cl_nsp_max;
        nxt.nbond_max = R.plan.cl_nbond_max;
        nxt.nbuf = buffers(nxt);
        nxt.offset = (int)list.size();
        nxt.count = 0;
      } else if (cur.count == 0) {
        nxt.offset = (int)list.size();
      }
      if (nxt.nbuf == 0) return fail(b, MPCD_EINVAL, "an admitted swimmer's MD layout does not fit on the device");
      list.push_back(r);
      nxt.count += 1;
      cur = nxt;
    }
    if (cur.count > 0) b->launches.push_back(cur);
  }
  if (!list.empty())
    BK(cudaMemcpyAsync(b->d_md_reps, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, b->s0));
  return MPCD_OK;
}

// enqueue one step (prologue, cell maps, fluid | MD) on s0 with MD forked off
int enqueue_step(mpcd_batch* b, int par, const BatchTables& t) {
  int n = 0;
  n += launch_batch_prologue(t, b->s0);
  n += launch_batch_cell_params(t, b->cells, b->tune.cell_threads, b->tune.cell_blocks, b->s0);
  const int nl = (int)b->launches.size();
  if (nl > 0) {
    BK(cudaEventRecord(b->ev_fork, b->s0));
    for (int k = 0; k < nl; ++k) {
      cudaStream_t s = b->smd[k % kMaxClusterTiles];
      if (k < kMaxClusterTiles) BK(cudaStreamWaitEvent(s, b->ev_fork, 0));
      const MDLaunch& L = b->launches[k];
      cudaError_t st = cudaSuccess;
      n += launch_md_cluster_batch(b->md, t, b->cells, b->d_md_reps + L.offset, L.count, L.ctiles, L.hmax, L.nsp_max,
                                   L.nbond_max, L.nbuf, s, &st);
      if (st != cudaSuccess) return cuda_fail(b, st, "batch MD launch");
    }
  }
  n += launch_batch_fluid_step(t, b->fl[par], b->cells, b->tune.fluid_threads, b->tune.fluid_blocks, b->s0);
  for (int k = 0; k < std::min(nl, (int)kMaxClusterTiles); ++k) {
    BK(cudaEventRecord(b->ev_join[k], b->smd[k]));
    BK(cudaStreamWaitEvent(b->s0, b->ev_join[k], 0));
  }
  b->kernels_per_step = n;
  return MPCD_OK;
}

int enqueue_sort(mpcd_batch* b, int par) {
  const BatchTables t = tables(b);
  b->kernels_per_sort = launch_batch_sort(t, b->fl[par], b->fl[par ^ 1], b->d_count, b->d_start, b->d_rank,
                                          b->d_blocksums, b->cell_cap, b->s0);
  return MPCD_OK;
}

int capture(mpcd_batch* b, int par, int nsteps, bool sorts, cudaGraphExec_t* out) {
  if (*out) {
    cudaGraphExecDestroy(*out);
    *out = nullptr;
  }
  BK(cudaStreamBeginCapture(b->s0, cudaStreamCaptureModeThreadLocal));
  int rc = MPCD_OK;
  int p = par;
  for (int k = 0; k < nsteps && rc == MPCD_OK; ++k) {
    rc = enqueue_step(b, p, tables(b));
    if (rc == MPCD_OK && sorts && (k + 1) % b->tune.sort_interval == 0) {
      rc = enqueue_sort(b, p);
      p ^= 1;
    }
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->s0, &g);
  if (rc != MPCD_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(b, e, "graph capture");
  e = cudaGraphInstantiate(out, g, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(b, e, "graph instantiate");
  return MPCD_OK;
}

int rebuild_graphs(mpcd_batch* b) {
  if (!b->graphs_dirty) return MPCD_OK;
  int rc = plan_launches(b);
  if (rc) return rc;
  const int per = std::max(1, b->p.sorts_per_graph);
  b->chunk_steps = b->tune.sort_interval * per;
  for (int par = 0; par < 2; ++par) {
    rc = capture(b, par, b->chunk_steps, true, &b->g_chunk[par]);
    if (rc) return rc;
    rc = capture(b, par, 1, false, &b->g_step[par]);
    if (rc) return rc;
  }
  b->graphs_dirty = false;
  return MPCD_OK;
}

int run_steps(mpcd_batch* b, int nsteps) {
  int rc = rebuild_graphs(b);
  if (rc) return rc;
  const int K = b->tune.sort_interval;
  const int per = std::max(1, b->p.sorts_per_graph);
  while (nsteps > 0) {
    if (b->since_sort == 0 && nsteps >= b->chunk_steps) {
      BK(cudaGraphLaunch(b->g_chunk[b->cur], b->s0));
      b->launches_total += (long long)b->chunk_steps * b->kernels_per_step + (long long)per * b->kernels_per_sort;
      if (per & 1) b->cur ^= 1;
      nsteps -= b->chunk_steps;
      continue;
    }
    BK(cudaGraphLaunch(b->g_step[b->cur], b->s0));
    b->launches_total += b->kernels_per_step;
    --nsteps;
    if (++b->since_sort >= K) {
      enqueue_sort(b, b->cur);
      b->launches_total += b->kernels_per_sort;
      b->cur ^= 1;
      b->since_sort = 0;
    }
  }
  BK(cudaGetLastError());
  return MPCD_OK;
}

int upload_tables(mpcd_batch* b) {
  BK(cudaMemcpyAsync(b->d_rep, b->rep.data(), b->rep.size() * sizeof(BatchRep), cudaMemcpyHostToDevice, b->s0));
  return MPCD_OK;
}

template <typename T>
int put_range(mpcd_batch* b, T* dst, long off, const T* src, long n) {
  if (n <= 0) return MPCD_OK;
  BK(cudaMemcpyAsync(dst + off, src, n * sizeof(T), cudaMemcpyHostToDevice, b->s0));
  return MPCD_OK;
}

void release_ranges(mpcd_batch* b, Replica& R) {
  if (R.page0 >= 0) b->a_part.release(R.page0, R.npages);
  if (R.cpage0 >= 0) b->a_cell.release(R.cpage0, R.ncpages);
  if (R.tile0 >= 0) b->a_tile.release(R.tile0, R.ntiles_alloc);
  if (R.sp0 >= 0) b->a_sp.release(R.sp0, R.nsp);
  if (R.h0 >= 0) b->a_halo.release(R.h0, R.nh);
  if (R.c0 >= 0) b->a_cil.release(R.c0, R.nc);
  if (R.b0 >= 0) b->a_bond.release(R.b0, R.nbond);
  R.page0 = R.cpage0 = R.tile0 = R.sp0 = R.h0 = R.c0 = R.b0 = -1;
  R.npages = R.ncpages = R.ntiles_alloc = R.nsp = R.nh = R.nc = R.nbond = 0;
}

std::string plan_replica(mpcd_batch* b, Replica& R) {
  if (R.nb == 0) {
    R.plan = MDPlan{};
    return "";
  }
  MDInput in;
  in.nb = R.nb;
  in.bpos = R.bpos.data();
  in.bvel = R.bvel.data();
  in.bmoves = R.bmoves.data();
  in.nsp = (long)R.sp_t.size();
  in.sp_t = R.sp_t.data();
  in.sp_o = R.sp_o.data();
  in.sp_k = R.sp_k.data();
  in.sp_r = R.sp_r.data();
  in.sp_rest = R.sp_rest.data();
  in.sp_kk = R.sp_kk.data();
  in.ncil = (int)R.cil.size();
  in.cil = R.cil.data();
  in.nbond = (long)R.newlen.size();
  in.newlen = R.newlen.data();
  in.oldlen = R.oldlen.data();
  in.split = 1;
  MDForce f;
  f.lanes = b->lanes;
  f.tile = b->T;
  std::string why = plan_md(in, f, true, false, 1, R.plan);
  if (!why.empty()) return why;
  bool fits = false;
  for (int nbuf = 2; nbuf >= 1 && !fits; --nbuf)
    fits = md_cluster_batch_feasible(b->lanes, b->T, R.plan.ntiles,
                                     md_cluster_batch_smem(b->T, R.plan.hmax, R.plan.cl_nsp_max,
                                                           R.plan.cl_nbond_max, nbuf));
  if (!fits) return "the replica's MD cluster does not fit on the device with this layout";
  return "";
}

// uploads replica r's planned MD into its ranges of the shared arrays,
// rebasing the plan's box-local slot, spring, halo, cilium and bond indices
int upload_md(mpcd_batch* b, int r, Replica& R) {
  const MDPlan& pl = R.plan;
  MDState& m = b->md;
  if (pl.ntiles > 0) {
    const long sb = R.tile0 * (long)b->T;
    const long ns = pl.nslots;
    int rc;
    if ((rc = put_range(b, m.x[0], sb, pl.X.data(), ns))) return rc;
    if ((rc = put_range(b, m.y[0], sb, pl.Y.data(), ns))) return rc;
    if ((rc = put_range(b, m.z[0], sb, pl.Z.data(), ns))) return rc;
    if ((rc = put_range(b, m.vx, sb, pl.VX.data(), ns))) return rc;
    if ((rc = put_range(b, m.vy, sb, pl.VY.data(), ns))) return rc;
    if ((rc = put_range(b, m.vz, sb, pl.VZ.data(), ns))) return rc;
    if ((rc = put_range(b, m.moves, sb, pl.mv.data(), ns))) return rc;
    std::vector<int> v(ns + 1);
    for (long k = 0; k < ns; ++k) v[k] = pl.prim[k] + (int)sb;
    if ((rc = put_range(b, m.prim, sb, v.data(), ns))) return rc;
    if ((rc = put_range(b, m.nhelp, sb, pl.nhelp.data(), ns))) return rc;
    for (long k = 0; k <= ns; ++k) v[k] = pl.start[k] + (int)R.sp0;
    if ((rc = put_range(b, m.sp_start, sb, v.data(), ns + 1))) return rc;
    const long nt = pl.ntiles;
    if ((rc = put_range(b, m.tile_help, R.tile0, pl.thelp.data(), nt))) return rc;
    if ((rc = put_range(b, m.tile_react, R.tile0, pl.tile_react.data(), nt))) return rc;
    std::vector<int> tv(nt + 1);
    for (long t = 0; t <= nt; ++t) tv[t] = pl.hstart[t] + (int)std::max(R.h0, 0L);
    if ((rc = put_range(b, m.halo_start, R.tile0, tv.data(), nt + 1))) return rc;
    for (long t = 0; t <= nt; ++t) tv[t] = pl.tcil[t] + (int)std::max(R.c0, 0L);
    if ((rc = put_range(b, m.tile_cil, R.tile0, tv.data(), nt + 1))) return rc;
    if (R.nsp > 0) {
      std::vector<int> so(R.nsp), sr(R.nsp);
      for (long k = 0; k < R.nsp; ++k) {
        so[k] = pl.so[k] + (int)sb;
        sr[k] = (pl.sk[k] & 3) >= 2 ? pl.sr[k] + (int)R.b0 : pl.sr[k];
      }
      if ((rc = put_range(b, m.sp_other, R.sp0, so.data(), R.nsp))) return rc;
      if ((rc = put_range(b, m.sp_local, R.sp0, pl.sl.data(), R.nsp))) return rc;
      if ((rc = put_range(b, m.sp_kind, R.sp0, pl.sk.data(), R.nsp))) return rc;
      if ((rc = put_range(b, m.sp_ref, R.sp0, sr.data(), R.nsp))) return rc;
      if ((rc = put_range(b, m.sp_rest, R.sp0, pl.srest.data(), R.nsp))) return rc;
      if ((rc = put_range(b, m.sp_m2k, R.sp0, pl.sm2k.data(), R.nsp))) return rc;
    }
    if (R.nh > 0) {
      std::vector<int> hv(R.nh);
      for (long k = 0; k < R.nh; ++k) hv[k] = pl.halo[k] + (int)sb;
      if ((rc = put_range(b, m.halo, R.h0, hv.data(), R.nh))) return rc;
    }
    if (R.nc > 0) {
      std::vector<CiliumDev> cd = pl.cd;
      for (auto& c : cd) {
        c.slot0 += (int)sb;
        c.bond_base += (int)R.b0;
      }
      if ((rc = put_range(b, m.cil, R.c0, cd.data(), R.nc))) return rc;
      if ((rc = put_range(b, m.midpnt, R.c0, pl.mid.data(), R.nc))) return rc;
      if ((rc = put_range(b, m.tstroke, R.c0, pl.ts.data(), R.nc))) return rc;
    }
    if (R.nbond > 0) {
      if ((rc = put_range(b, m.newlen, R.b0, pl.newlen.data(), R.nbond))) return rc;
      if ((rc = put_range(b, m.oldlen, R.b0, pl.oldlen.data(), R.nbond))) return rc;
      if ((rc = put_range(b, m.diag, R.b0, pl.diag.data(), R.nbond))) return rc;
    }
    for (long t = 0; t < nt; ++t) b->tile_rep[R.tile0 + t] = r;
    b->tile_rep[R.tile0 + nt] = -1;  // spare tile
    if ((rc = put_range(b, b->d_tile_rep, R.tile0, b->tile_rep.data() + R.tile0, nt + 1))) return rc;
  }
  return MPCD_OK;
}

// copies replica r's bead state, beat state and bond tables from the device
// into its host description (R.bpos, R.bvel, R.cil, R.newlen, R.oldlen)
int pull_md_state(mpcd_batch* b, Replica& R) {
  const MDPlan& pl = R.plan;
  if (R.nb == 0 || pl.ntiles == 0) return MPCD_OK;
  const long sb = R.tile0 * (long)b->T, ns = pl.nslots;
  std::vector<double> X(ns), Y(ns), Z(ns), VX(ns), VY(ns), VZ(ns);
  const MDState& m = b->md;
  BK(cudaMemcpyAsync(X.data(), m.x[0] + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(Y.data(), m.y[0] + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(Z.data(), m.z[0] + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(VX.data(), m.vx + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(VY.data(), m.vy + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(VZ.data(), m.vz + sb, ns * 8, cudaMemcpyDeviceToHost, b->s0));
  std::vector<double> mid(R.nc), ts(R.nc);
  if (R.nc > 0) {
    BK(cudaMemcpyAsync(mid.data(), m.midpnt + R.c0, R.nc * 8, cudaMemcpyDeviceToHost, b->s0));
    BK(cudaMemcpyAsync(ts.data(), m.tstroke + R.c0, R.nc * 8, cudaMemcpyDeviceToHost, b->s0));
  }
  if (R.nbond > 0) {
    BK(cudaMemcpyAsync(R.newlen.data(), m.newlen + R.b0, R.nbond * 8, cudaMemcpyDeviceToHost, b->s0));
    BK(cudaMemcpyAsync(R.oldlen.data(), m.oldlen + R.b0, R.nbond * 8, cudaMemcpyDeviceToHost, b->s0));
  }
  BK(cudaStreamSynchronize(b->s0));
  for (long k = 0; k < R.nb; ++k) {
    const int sl = pl.slot_of[k];
    R.bpos[3 * k] = X[sl];
    R.bpos[3 * k + 1] = Y[sl];
    R.bpos[3 * k + 2] = Z[sl];
    R.bvel[3 * k] = VX[sl];
    R.bvel[3 * k + 1] = VY[sl];
    R.bvel[3 * k + 2] = VZ[sl];
  }
  for (long c = 0; c < R.nc; ++c) {
    R.cil[c].midpnt = mid[c];
    R.cil[c].tstroke = ts[c];
  }
  return MPCD_OK;
}

// takes the MD ranges of a planned replica (all or nothing)
bool take_md_ranges(mpcd_batch* b, Replica& R) {
  const MDPlan& pl = R.plan;
  R.ntiles_alloc = pl.ntiles > 0 ? pl.ntiles + 1 : 0;
  R.nsp = pl.nsp_kept();
  R.nh = (long)pl.halo.size();
  R.nc = (long)pl.cd.size();
  R.nbond = (long)pl.newlen.size();
  bool ok = true;
  auto take = [&](RangeAlloc& a, long n, long& off) {
    off = n > 0 ? a.alloc(n) : -1;
    if (n > 0 && off < 0) ok = false;
  };
  take(b->a_tile, R.ntiles_alloc, R.tile0);
  take(b->a_sp, R.nsp, R.sp0);
  take(b->a_halo, R.nh, R.h0);
  take(b->a_cil, R.nc, R.c0);
  take(b->a_bond, R.nbond, R.b0);
  return ok;
}

}  // namespace

extern "C" {

int mpcd_batch_create(const mpcd_batch_params* params, mpcd_batch** out) {
  if (!params || !out) return MPCD_EINVAL;
  *out = nullptr;
  mpcd_batch_params p = *params;
  if (p.max_replicas <= 0 || p.max_particles < 0 || p.max_cells <= 0 || p.max_slots < 0 || p.max_springs < 0 ||
      p.max_halo < 0 || p.max_cilia < 0 || p.max_bonds < 0)
    return MPCD_EINVAL;
  if (p.md_lanes == 0) p.md_lanes = 2;
  if (p.md_lanes != 1 && p.md_lanes != 2) return MPCD_EINVAL;
  if (p.md_tile == 0) p.md_tile = 512 / p.md_lanes;
  if (p.md_tile < 32 || p.md_tile % 32 || p.md_tile * p.md_lanes > 1024) return MPCD_EINVAL;
  if (p.sort_interval <= 0) p.sort_interval = 25;
  if (p.sorts_per_graph <= 0) p.sorts_per_graph = 4;
  mpcd_batch* b = new (std::nothrow) mpcd_batch();
  if (!b) return MPCD_ENOMEM;
  b->p = p;
  b->T = p.md_tile;
  b->lanes = p.md_lanes;
  b->tune.sort_interval = p.sort_interval;
  auto bail = [&](cudaError_t e, const char* what) {
    fprintf(stderr, "mpcd_batch_create: %s: %s\n", what, cudaGetErrorString(e));
    free_all(b);
    delete b;
    return e == cudaErrorMemoryAllocation ? MPCD_ENOMEM : MPCD_ECUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(p.device)) != cudaSuccess) return bail(e, "cudaSetDevice");
  if ((e = cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  for (int g = 0; g < kMaxClusterTiles; ++g) {
    // the MD chains are latency-bound: their CTAs take SMs before the fluid pass's
    if ((e = cudaStreamCreateWithPriority(&b->smd[g], cudaStreamNonBlocking, prio_greatest)) != cudaSuccess)
      return bail(e, "stream");
    if ((e = cudaEventCreateWithFlags(&b->ev_join[g], cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
  }
  if ((e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
  b->npart_pages = (p.max_particles + kPartPage - 1) / kPartPage;
  b->ncell_pages = (p.max_cells + kCellPage - 1) / kCellPage;
  b->part_cap = b->npart_pages * kPartPage;
  b->cell_cap = b->ncell_pages * kCellPage;
  // slots for the beads plus one spare tile per replica (for the smallest tile size)
  const long nslots = ((p.max_slots + 31) / 32 + 32L * p.max_replicas) * 32L;
  b->slot_cap = nslots;
  b->tile_cap = nslots / b->T;
  b->tile_arr_cap = nslots / 32 + 1;
  const int R = p.max_replicas;
  if ((e = dalloc(&b->d_rep, R)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_step, R)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_state, R)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_obs, 8 * (size_t)R)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_md_reps, R)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_part_page_rep, b->npart_pages)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_cell_page_rep, b->ncell_pages)) != cudaSuccess) return bail(e, "alloc tables");
  if ((e = dalloc(&b->d_tile_rep, b->tile_arr_cap)) != cudaSuccess) return bail(e, "alloc tables");
  for (int par = 0; par < 2; ++par) {
    if ((e = dalloc(&b->fl[par].id, b->part_cap)) != cudaSuccess) return bail(e, "alloc fluid");
    if ((e = dalloc(&b->fl[par].pos, b->part_cap)) != cudaSuccess) return bail(e, "alloc fluid");
    if ((e = dalloc(&b->fl[par].vel, b->part_cap)) != cudaSuccess) return bail(e, "alloc fluid");
  }
  if ((e = dalloc(&b->cells.sum, b->cell_cap)) != cudaSuccess) return bail(e, "alloc cells");
  if ((e = dalloc(&b->cells.cnt, b->cell_cap)) != cudaSuccess) return bail(e, "alloc cells");
  if ((e = dalloc(&b->cells.par, 2 * b->cell_cap)) != cudaSuccess) return bail(e, "alloc cells");
  if ((e = dalloc(&b->d_count, b->cell_cap)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&b->d_start, b->cell_cap)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&b->d_rank, b->part_cap)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&b->d_blocksums, b->cell_cap / 1024 + 2)) != cudaSuccess) return bail(e, "alloc sort");
  MDState& m = b->md;
  m.tile = b->T;
  m.ntiles = (int)b->tile_cap;
  m.nslots = (int)nslots;
  m.split = 1;
  m.cluster = 1;
  m.cl_lanes = b->lanes;
  if ((e = dalloc(&m.x[0], nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.y[0], nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.z[0], nslots)) != cudaSuccess) return bail(e, "alloc MD");
  m.x[1] = m.x[0];
  m.y[1] = m.y[0];
  m.z[1] = m.z[0];
  if ((e = dalloc(&m.vx, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.vy, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.vz, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.moves, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.prim, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.nhelp, nslots)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_start, nslots + 1)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.tile_help, b->tile_arr_cap)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.tile_react, b->tile_arr_cap)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.tile_cil, b->tile_arr_cap + 1)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.halo_start, b->tile_arr_cap + 1)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_other, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_local, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_kind, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_ref, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_rest, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.sp_m2k, p.max_springs)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.halo, p.max_halo)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.cil, p.max_cilia)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.midpnt, p.max_cilia)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.tstroke, p.max_cilia)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.newlen, p.max_bonds)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.oldlen, p.max_bonds)) != cudaSuccess) return bail(e, "alloc MD");
  if ((e = dalloc(&m.diag, p.max_bonds)) != cudaSuccess) return bail(e, "alloc MD");
  m.ncil = p.max_cilia;
  // every slot starts empty, every page and tile free
  b->rep.assign(R, BatchRep{});
  b->part_page_rep.assign(b->npart_pages, -1);
  b->cell_page_rep.assign(b->ncell_pages, -1);
  b->tile_rep.assign(b->tile_arr_cap, -1);
  b->reps.assign(R, Replica{});
  {
    std::vector<int> neg(nslots, -1);
    if ((e = cudaMemcpy(m.moves, neg.data(), nslots * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail(e, "init MD");
  }
  if ((e = cudaMemset(m.tile_help, 0, b->tile_arr_cap * sizeof(int))) != cudaSuccess) return bail(e, "init MD");
  if ((e = cudaMemset(b->cells.sum, 0, b->cell_cap * sizeof(float4))) != cudaSuccess) return bail(e, "init cells");
  if ((e = cudaMemset(b->cells.cnt, 0, b->cell_cap * sizeof(uint32_t))) != cudaSuccess) return bail(e, "init cells");
  if ((e = cudaMemset(b->d_state, 0, R * sizeof(BatchState))) != cudaSuccess) return bail(e, "init tables");
  if ((e = cudaMemset(b->d_step, 0, R * sizeof(BatchStep))) != cudaSuccess) return bail(e, "init tables");
  if ((e = cudaMemcpy(b->d_rep, b->rep.data(), R * sizeof(BatchRep), cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(e, "init tables");
  if ((e = cudaMemcpy(b->d_part_page_rep, b->part_page_rep.data(), b->npart_pages * sizeof(int),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(e, "init tables");
  if ((e = cudaMemcpy(b->d_cell_page_rep, b->cell_page_rep.data(), b->ncell_pages * sizeof(int),
                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(e, "init tables");
  if ((e = cudaMemcpy(b->d_tile_rep, b->tile_rep.data(), b->tile_arr_cap * sizeof(int), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return bail(e, "init tables");
  b->a_part.reset(b->npart_pages);
  b->a_cell.reset(b->ncell_pages);
  b->a_tile.reset(b->tile_cap);
  b->a_sp.reset(p.max_springs);
  b->a_halo.reset(p.max_halo);
  b->a_cil.reset(p.max_cilia);
  b->a_bond.reset(p.max_bonds);
  *out = b;
  return MPCD_OK;
}

int mpcd_batch_destroy(mpcd_batch* b) {
  if (!b) return MPCD_OK;
  if (b->s0) cudaStreamSynchronize(b->s0);
  free_all(b);
  delete b;
  return MPCD_OK;
}

const char* mpcd_batch_last_error(const mpcd_batch* b) { return b ? b->error.c_str() : "null batch"; }

int mpcd_batch_add(mpcd_batch* b, const mpcd_params* params, int* replica) {
  if (!b || !params || !replica) return fail(b, MPCD_EINVAL, "add: bad arguments");
  const mpcd_params& p = *params;
  for (int q = 0; q < 3; ++q)
    if (p.sizes[q] < 2 || p.sizes[q] > 1024) return fail(b, MPCD_EINVAL, "add: box edge outside 2..1024");
  if (!(p.tstep > 0) || !(p.ststep > 0) || !(p.bead_mass > 0)) return fail(b, MPCD_EINVAL, "add: bad step sizes");
  if (p.precision != MPCD_FP32) return fail(b, MPCD_EINVAL, "add: a batch runs split precision (MPCD_FP32)");
  if (p.walls != MPCD_WALLS_NONE) return fail(b, MPCD_EINVAL, "add: walls are not supported in a batch");
  const int nsub = (int)((p.tstep + 0.00000001) / p.ststep);
  if (nsub < 1 || nsub > 511) return fail(b, MPCD_EINVAL, "add: 1 .. 511 MD substeps per MPC step");
  int r = -1;
  for (int k = 0; k < (int)b->reps.size(); ++k)
    if (!b->reps[k].used) {
      r = k;
      break;
    }
  if (r < 0) return fail(b, MPCD_EINVAL, "add: no free replica slot");
  Replica& R = b->reps[r];
  R = Replica{};
  R.used = true;
  R.p = p;
  R.nsub = nsub;
  R.ncell = (long)p.sizes[0] * p.sizes[1] * p.sizes[2];
  shift_from_counter(p.seed, 0, R.a);
  *replica = r;
  return MPCD_OK;
}

int mpcd_batch_add_engine(mpcd_batch* b, mpcd_engine* h, int* replica) {
  if (!b || !h || !replica) return fail(b, MPCD_EINVAL, "add_engine: bad arguments");
  EngineExport ex;
  int rc = engine_export(h, ex);
  if (rc) return fail(b, rc, std::string("add_engine: ") + mpcd_last_error(h));
  mpcd_params p = ex.p;
  p.precision = MPCD_FP32;
  rc = mpcd_batch_add(b, &p, replica);
  if (rc) return rc;
  Replica& R = b->reps[*replica];
  std::memcpy(R.a, ex.a, sizeof R.a);
  R.globalt = ex.globalt;
  R.steps = ex.steps;
  R.nf = ex.nf;
  R.fpos.swap(ex.fpos);
  R.fvel.swap(ex.fvel);
  R.nb = ex.nb;
  R.bpos.swap(ex.bpos);
  R.bvel.swap(ex.bvel);
  R.bmoves.swap(ex.bmoves);
  R.sp_t.swap(ex.sp_t);
  R.sp_o.swap(ex.sp_o);
  R.sp_k.swap(ex.sp_k);
  R.sp_r.swap(ex.sp_r);
  R.sp_rest.swap(ex.sp_rest);
  R.sp_kk.swap(ex.sp_kk);
  R.cil.swap(ex.cil);
  R.newlen.swap(ex.newlen);
  R.oldlen.swap(ex.oldlen);
  return MPCD_OK;
}

int mpcd_batch_set_fluid(mpcd_batch* b, int r, long n, const double* pos, const double* vel) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || n < 0 || (n > 0 && (!pos || !vel)))
    return fail(b, MPCD_EINVAL, "set_fluid: bad arguments or replica already admitted");
  if (n > 0x7fffffffL) return fail(b, MPCD_EINVAL, "set_fluid: too many particles");
  for (long i = 0; i < 3 * n; ++i)
    if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || std::fabs(pos[i]) > 1e12)
      return fail(b, MPCD_EINVAL, "set_fluid: non-finite or out-of-range position or velocity");
  R->nf = n;
  R->fpos.assign(pos, pos + 3 * n);
  R->fvel.assign(vel, vel + 3 * n);
  return MPCD_OK;
}

int mpcd_batch_set_shift(mpcd_batch* b, int r, const double* a3) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || !a3) return fail(b, MPCD_EINVAL, "set_shift: bad arguments");
  for (int q = 0; q < 3; ++q)
    if (!(a3[q] >= 0.0 && a3[q] < 1.0)) return fail(b, MPCD_EINVAL, "set_shift: shift outside [0,1)");
  std::memcpy(R->a, a3, sizeof R->a);
  return MPCD_OK;
}

int mpcd_batch_set_time(mpcd_batch* b, int r, double t) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || !std::isfinite(t)) return fail(b, MPCD_EINVAL, "set_time: bad arguments");
  R->globalt = t;
  return MPCD_OK;
}

int mpcd_batch_set_beads(mpcd_batch* b, int r, long nb, const double* pos, const double* vel, const int* moves) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || nb < 0 || (nb > 0 && (!pos || !vel)))
    return fail(b, MPCD_EINVAL, "set_beads: bad arguments");
  for (long i = 0; i < 3 * nb; ++i)
    if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || std::fabs(pos[i]) > 1e12)
      return fail(b, MPCD_EINVAL, "set_beads: non-finite or out-of-range position or velocity");
  R->nb = nb;
  R->bpos.assign(pos, pos + 3 * nb);
  R->bvel.assign(vel, vel + 3 * nb);
  R->bmoves.assign(nb, 1);
  if (moves)
    for (long i = 0; i < nb; ++i) R->bmoves[i] = moves[i] ? 1 : 0;
  return MPCD_OK;
}

int mpcd_batch_set_springs(mpcd_batch* b, int r, long ns, const int* target, const int* other, const int* kind,
                           const int* ref, const double* rest, const double* k) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || ns < 0 || (ns > 0 && (!target || !other || !kind || !k)))
    return fail(b, MPCD_EINVAL, "set_springs: bad arguments");
  R->sp_t.assign(target, target + ns);
  R->sp_o.assign(other, other + ns);
  R->sp_k.assign(kind, kind + ns);
  R->sp_r.assign(ns, 0);
  R->sp_rest.assign(ns, 0.0);
  for (long i = 0; i < ns; ++i) {
    if (kind[i] < 0 || kind[i] > 3) return fail(b, MPCD_EINVAL, "set_springs: unknown spring kind");
    if (kind[i] >= 2) {
      if (!ref) return fail(b, MPCD_EINVAL, "set_springs: BOND/DIAG springs need ref");
      R->sp_r[i] = ref[i];
    } else {
      if (!rest) return fail(b, MPCD_EINVAL, "set_springs: CONST springs need rest");
      R->sp_rest[i] = rest[i];
    }
  }
  R->sp_kk.assign(k, k + ns);
  return MPCD_OK;
}

int mpcd_batch_set_cilia(mpcd_batch* b, int r, int nc, const mpcd_cilium* cilia, const double* newlength,
                         const double* oldlength) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || nc < 0 || (nc > 0 && !cilia)) return fail(b, MPCD_EINVAL, "set_cilia: bad arguments");
  R->cil.assign(cilia, cilia + nc);
  size_t nbond = 0;
  for (int c = 0; c < nc; ++c) {
    if (cilia[c].rodlength < 2 || cilia[c].bond_base < 0) return fail(b, MPCD_EINVAL, "set_cilia: bad cilium");
    nbond = std::max(nbond, (size_t)(cilia[c].bond_base + cilia[c].rodlength));
  }
  R->newlen.assign(nbond, 0.5);
  R->oldlen.assign(nbond, 0.5);
  if (newlength) R->newlen.assign(newlength, newlength + nbond);
  if (oldlength) R->oldlen.assign(oldlength, oldlength + nbond);
  return MPCD_OK;
}

long long mpcd_batch_estimate(const mpcd_batch* b, long nf, long ncell, long nb, long nsprings, int ncilia,
                              long nbonds) {
  const long T = b ? b->T : 512;
  const long pages = (nf + kPartPage - 1) / kPartPage, cpages = (ncell + kCellPage - 1) / kCellPage;
  long long f = pages * (long long)kPartPage * (2 * (sizeof(float4) * 2 + 4) + 4);  // two buffers + rank
  f += cpages * (long long)kCellPage * (sizeof(float4) * 4 + 3 * 4);               // sum, par, cnt, count, start
  if (nb > 0) {
    const long slots = nb + nb / 8 + 2 * T;                                         // helpers, padding, spare tile
    f += (long long)slots * (6 * 8 + 4 * 4);
    f += (long long)nsprings * 36 + (long long)nb * 4;                              // springs, halo
    f += (long long)ncilia * (sizeof(CiliumDev) + 16) + (long long)nbonds * 24;
  }
  return f;
}

int mpcd_batch_footprint(mpcd_batch* b, int r, long long* bytes) {
  Replica* R = get_rep(b, r);
  if (!R || !bytes) return fail(b, MPCD_EINVAL, "footprint: bad arguments");
  *bytes = mpcd_batch_estimate(b, R->nf, R->ncell, R->nb, (long)R->sp_t.size(), (int)R->cil.size(),
                               (long)R->newlen.size());
  return MPCD_OK;
}

int mpcd_batch_admit(mpcd_batch* b, int r) {
  Replica* Rp = get_rep(b, r);
  if (!Rp || Rp->admitted) return fail(b, MPCD_EINVAL, "admit: bad replica");
  Replica& R = *Rp;
  const int* L = R.p.sizes;
  // MD plan with the batch's fixed cluster layout
  std::string why = plan_replica(b, R);
  if (!why.empty()) return fail(b, MPCD_EINVAL, "admit: " + why);
  const MDPlan& pl = R.plan;
  // device ranges
  R.npages = (R.nf + kPartPage - 1) / kPartPage;
  R.ncpages = (R.ncell + kCellPage - 1) / kCellPage;
  bool ok = true;
  auto take = [&](RangeAlloc& a, long n, long& off) {
    off = n > 0 ? a.alloc(n) : -1;
    if (n > 0 && off < 0) ok = false;
  };
  take(b->a_part, R.npages, R.page0);
  take(b->a_cell, R.ncpages, R.cpage0);
  ok = take_md_ranges(b, R) && ok;
  if (!ok) {
    release_ranges(b, R);
    return fail(b, MPCD_EINVAL, "admit: batch capacity exhausted");
  }
  const long p0 = R.page0 >= 0 ? R.page0 * kPartPage : 0;
  const long cell0 = R.cpage0 * kCellPage;
  const int par = b->cur;
  // fluid: split layout, ordered by cell on the host
  if (R.nf > 0) {
    const long n = R.nf;
    std::vector<float4> P(n), V(n);
    std::vector<uint32_t> cellid(n);
    for (long i = 0; i < n; ++i) {
      int c[3];
      double o[3];
      for (int q = 0; q < 3; ++q) wrap_coord(R.fpos[3 * i + q], L[q], c[q], o[q]);
      float f[3];
      for (int q = 0; q < 3; ++q) {
        f[q] = (float)o[q];
        if (f[q] >= 1.0f) {
          f[q] = 0.0f;
          c[q] = (c[q] + 1) % L[q];
        }
      }
      P[i] = make_float4(f[0], f[1], f[2], bits_to_float(pack_cell(c[0], c[1], c[2])));
      V[i] = make_float4((float)R.fvel[3 * i], (float)R.fvel[3 * i + 1], (float)R.fvel[3 * i + 2], 0.0f);
      cellid[i] = (uint32_t)(c[0] + (long)L[0] * (c[1] + (long)L[1] * c[2]));
    }
    std::vector<uint32_t> cnt(R.ncell + 1, 0);
    for (long i = 0; i < n; ++i) cnt[cellid[i] + 1]++;
    for (long c = 0; c < R.ncell; ++c) cnt[c + 1] += cnt[c];
    std::vector<float4> Ps(n), Vs(n);
    std::vector<uint32_t> ids(n);
    for (long i = 0; i < n; ++i) {
      const long d = cnt[cellid[i]]++;
      Ps[d] = P[i];
      Vs[d] = V[i];
      ids[d] = (uint32_t)i;
    }
    int rc;
    if ((rc = put_range(b, b->fl[par].pos, p0, Ps.data(), n))) return rc;
    if ((rc = put_range(b, b->fl[par].vel, p0, Vs.data(), n))) return rc;
    if ((rc = put_range(b, b->fl[par].id, p0, ids.data(), n))) return rc;
  }
  BK(cudaMemsetAsync(b->cells.sum + cell0, 0, R.ncpages * kCellPage * sizeof(float4), b->s0));
  BK(cudaMemsetAsync(b->cells.cnt + cell0, 0, R.ncpages * kCellPage * sizeof(uint32_t), b->s0));
  // MD, rebased into the shared arrays
  {
    const int rc = upload_md(b, r, R);
    if (rc) return rc;
  }
  MDState& m = b->md;
  // tables
  BatchRep& D = b->rep[r];
  D = BatchRep{};
  D.resident = 1;
  for (int q = 0; q < 3; ++q) D.L[q] = L[q];
  D.walls = 0;
  D.nsub = R.nsub;
  D.cell0 = cell0;
  D.ncell = R.ncell;
  D.p0 = p0;
  D.n = R.nf;
  D.md_tile0 = pl.ntiles > 0 ? (int)R.tile0 : -1;
  D.md_ntiles = pl.ntiles;
  D.seed = R.p.seed;
  D.h = R.p.tstep;
  D.ststep = R.p.ststep;
  D.bead_mass = R.p.bead_mass;
  D.gravity = R.p.gravity;
  D.omega = R.p.omega;
  int rc;
  if ((rc = put_range(b, b->d_rep, r, &D, 1))) return rc;
  BatchState S{};
  S.steps = (uint64_t)R.steps;
  S.steps_left = 0;
  std::memcpy(S.a, R.a, sizeof S.a);
  S.globalt = R.globalt;
  if ((rc = put_range(b, b->d_state, r, &S, 1))) return rc;
  for (long k = 0; k < R.npages; ++k) b->part_page_rep[R.page0 + k] = r;
  for (long k = 0; k < R.ncpages; ++k) b->cell_page_rep[R.cpage0 + k] = r;
  if (R.npages && (rc = put_range(b, b->d_part_page_rep, R.page0, b->part_page_rep.data() + R.page0, R.npages)))
    return rc;
  if ((rc = put_range(b, b->d_cell_page_rep, R.cpage0, b->cell_page_rep.data() + R.cpage0, R.ncpages))) return rc;
  // binning with the current shift (end of Simulation's constructor)
  const BatchTables t = tables(b);
  if (R.npages) b->launches_total += launch_batch_bin_fluid(t, b->fl[par], b->cells, R.page0, R.page0 + R.npages, b->s0);
  if (pl.ntiles)
    b->launches_total += launch_batch_bin_beads(t, m, b->d_tile_rep, b->cells, (int)R.tile0,
                                                (int)(R.tile0 + pl.ntiles), b->s0);
  BK(cudaGetLastError());
  R.admitted = true;
  // the host staging copies are no longer needed
  R.fpos.clear();
  R.fpos.shrink_to_fit();
  R.fvel.clear();
  R.fvel.shrink_to_fit();
  if (pl.ntiles > 0) b->graphs_dirty = true;
  return MPCD_OK;
}

int mpcd_batch_set_steps(mpcd_batch* b, int r, long long nsteps) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted || nsteps < 0) return fail(b, MPCD_EINVAL, "set_steps: bad arguments");
  BK(cudaMemcpyAsync(&b->d_state[r].steps_left, &nsteps, sizeof nsteps, cudaMemcpyHostToDevice, b->s0));
  BK(cudaStreamSynchronize(b->s0));  // nsteps lives on the caller's stack
  return MPCD_OK;
}

int mpcd_batch_run(mpcd_batch* b, int nsteps) {
  if (!b || nsteps < 0) return fail(b, MPCD_EINVAL, "run: bad arguments");
  cudaSetDevice(b->p.device);
  return run_steps(b, nsteps);
}

int mpcd_batch_timed_run(mpcd_batch* b, int nsteps, double* total_ms) {
  if (!b || nsteps < 0) return fail(b, MPCD_EINVAL, "timed_run: bad arguments");
  cudaSetDevice(b->p.device);
  int rc = rebuild_graphs(b);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  BK(cudaEventRecord(e0, b->s0));
  rc = run_steps(b, nsteps);
  BK(cudaEventRecord(e1, b->s0));
  BK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (total_ms) *total_ms = ms;
  return rc;
}

int mpcd_batch_step_inject(mpcd_batch* b, int r, const mpcd_inject* inj) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted || !inj) return fail(b, MPCD_EINVAL, "step_inject: bad arguments");
  if (inj->virt) return fail(b, MPCD_EINVAL, "step_inject: a batch replica has no walls");
  if (inj->shift_next)
    for (int q = 0; q < 3; ++q)
      if (!(inj->shift_next[q] >= 0.0 && inj->shift_next[q] < 1.0))
        return fail(b, MPCD_EINVAL, "step_inject: injected shift outside [0,1)");
  int rc = rebuild_graphs(b);  // plans the MD launches
  if (rc) return rc;
  const long nc = R->ncell;
  double* d = nullptr;  // shift [3] | gamma [nc] | axis [3 nc]
  BK(dalloc(&d, 3 + 4 * (size_t)nc));
  BatchTables t = tables(b);
  t.inj_rep = r;
  cudaError_t e = cudaSuccess;
  if (inj->shift_next && e == cudaSuccess) {
    e = cudaMemcpyAsync(d, inj->shift_next, 3 * sizeof(double), cudaMemcpyHostToDevice, b->s0);
    t.inj_shift = d;
  }
  if (inj->gamma && e == cudaSuccess) {
    e = cudaMemcpyAsync(d + 3, inj->gamma, nc * sizeof(double), cudaMemcpyHostToDevice, b->s0);
    t.inj_gamma = d + 3;
  }
  if (inj->axis && e == cudaSuccess) {
    e = cudaMemcpyAsync(d + 3 + nc, inj->axis, 3 * nc * sizeof(double), cudaMemcpyHostToDevice, b->s0);
    t.inj_axis = d + 3 + nc;
  }
  if (e == cudaSuccess) {
    rc = enqueue_step(b, b->cur, t);  // every replica with steps left advances; r with these draws
    b->launches_total += b->kernels_per_step;
    if (rc == MPCD_OK && ++b->since_sort >= b->tune.sort_interval) {
      enqueue_sort(b, b->cur);
      b->launches_total += b->kernels_per_sort;
      b->cur ^= 1;
      b->since_sort = 0;
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->s0);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(b, e, "step_inject");
  if (rc) return rc;
  BatchState S;
  BK(cudaMemcpy(&S, b->d_state + r, sizeof S, cudaMemcpyDeviceToHost));
  if (S.err & kErrGammaMissing) return fail(b, MPCD_EDEVICE, "step_inject: injected gamma missing for a thermostatted cell");
  return MPCD_OK;
}

int mpcd_batch_sync(mpcd_batch* b) {
  if (!b) return MPCD_EINVAL;
  cudaSetDevice(b->p.device);
  BK(cudaStreamSynchronize(b->s0));
  return MPCD_OK;
}

int mpcd_batch_status(mpcd_batch* b, int r, long long* steps_done, long long* steps_left, double* globalt,
                      unsigned* err_bits) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted) return fail(b, MPCD_EINVAL, "status: bad replica");
  BatchState S;
  BK(cudaMemcpyAsync(&S, b->d_state + r, sizeof S, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaStreamSynchronize(b->s0));
  if (steps_done) *steps_done = (long long)S.steps;
  if (steps_left) *steps_left = S.steps_left;
  if (globalt) *globalt = S.globalt;
  if (err_bits) *err_bits = S.err;
  return MPCD_OK;
}

int mpcd_batch_get_shift(mpcd_batch* b, int r, double* a3) {
  Replica* R = get_rep(b, r);
  if (!R || !a3) return fail(b, MPCD_EINVAL, "get_shift: bad arguments");
  if (!R->admitted) {
    std::memcpy(a3, R->a, sizeof R->a);
    return MPCD_OK;
  }
  BatchState S;
  BK(cudaMemcpyAsync(&S, b->d_state + r, sizeof S, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaStreamSynchronize(b->s0));
  std::memcpy(a3, S.a, sizeof S.a);
  return MPCD_OK;
}

int mpcd_batch_get_fluid(mpcd_batch* b, int r, long n, double* pos, double* vel) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted || n != R->nf) return fail(b, MPCD_EINVAL, "get_fluid: bad replica or size");
  if (n == 0) return MPCD_OK;
  const long p0 = b->rep[r].p0;
  std::vector<float4> P(n), V(n);
  std::vector<uint32_t> ids(n);
  BK(cudaMemcpyAsync(P.data(), b->fl[b->cur].pos + p0, n * sizeof(float4), cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(V.data(), b->fl[b->cur].vel + p0, n * sizeof(float4), cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(ids.data(), b->fl[b->cur].id + p0, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->s0));
  BK(cudaStreamSynchronize(b->s0));
  for (long i = 0; i < n; ++i) {
    const uint32_t k = ids[i];
    if (k >= (uint32_t)n) return fail(b, MPCD_EDEVICE, "get_fluid: corrupt particle ids");
    const uint32_t c = float_to_bits(P[i].w);
    if (pos) {
      pos[3 * k] = cell_x(c) + (double)P[i].x;
      pos[3 * k + 1] = cell_y(c) + (double)P[i].y;
      pos[3 * k + 2] = cell_z(c) + (double)P[i].z;
    }
    if (vel) {
      vel[3 * k] = V[i].x;
      vel[3 * k + 1] = V[i].y;
      vel[3 * k + 2] = V[i].z;
    }
  }
  return MPCD_OK;
}

int mpcd_batch_get_beads(mpcd_batch* b, int r, long nb, double* pos, double* vel) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted || nb != R->nb) return fail(b, MPCD_EINVAL, "get_beads: bad replica or size");
  if (nb == 0) return MPCD_OK;
  int rc = pull_md_state(b, *R);
  if (rc) return rc;
  if (pos) std::memcpy(pos, R->bpos.data(), 3 * nb * sizeof(double));
  if (vel) std::memcpy(vel, R->bvel.data(), 3 * nb * sizeof(double));
  return MPCD_OK;
}

int mpcd_batch_get_cilia(mpcd_batch* b, int r, int nc, double* state2, double* newlength, double* oldlength) {
  Replica* R = get_rep(b, r);
  if (!R || nc != (int)R->cil.size()) return fail(b, MPCD_EINVAL, "get_cilia: bad replica or count");
  if (R->admitted) {
    int rc = pull_md_state(b, *R);
    if (rc) return rc;
  }
  for (int c = 0; c < nc; ++c)
    if (state2) {
      state2[2 * c] = R->cil[c].midpnt;
      state2[2 * c + 1] = R->cil[c].tstroke;
    }
  if (newlength) std::memcpy(newlength, R->newlen.data(), R->newlen.size() * sizeof(double));
  if (oldlength) std::memcpy(oldlength, R->oldlen.data(), R->oldlen.size() * sizeof(double));
  return MPCD_OK;
}

int mpcd_batch_set_step_count(mpcd_batch* b, int r, long long steps_done) {
  Replica* R = get_rep(b, r);
  if (!R || R->admitted || steps_done < 0) return fail(b, MPCD_EINVAL, "set_step_count: bad replica (admitted?)");
  R->steps = steps_done;
  return MPCD_OK;
}

int mpcd_batch_observables(mpcd_batch* b, int r, mpcd_obs* out) {
  Replica* R = get_rep(b, r);
  if (!R || !R->admitted || !out) return fail(b, MPCD_EINVAL, "observables: bad arguments");
  const BatchTables t = tables(b);
  b->launches_total += launch_batch_observables(t, b->fl[b->cur], b->md, b->d_tile_rep, (int)b->tile_cap, b->d_obs,
                                                b->s0);
  double o[8];
  BatchState S;
  BK(cudaMemcpyAsync(o, b->d_obs + 8 * r, sizeof o, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaMemcpyAsync(&S, b->d_state + r, sizeof S, cudaMemcpyDeviceToHost, b->s0));
  BK(cudaStreamSynchronize(b->s0));
  const double M = o[5] > 0 ? o[5] : 1.0, N = o[4] > 0 ? o[4] : 1.0;
  out->momentum[0] = o[0] / M;
  out->momentum[1] = o[1] / M;
  out->momentum[2] = o[2] / M;
  out->n = o[4];
  out->mass = o[5];
  out->kT = o[3] / 3.0 / N;
  out->fluid_T = o[7] > 0 ? o[6] / o[7] / 3.0 : 0.0;
  out->diss_energy = S.diss;
  out->globalt = S.globalt;
  out->energy_fluid = 0.5 * o[6];
  if (S.err) {
    std::string msg = "device check failed for this replica:";
    if (S.err & kErrGammaLoop) msg += " Gamma sampler exceeded its iteration cap;";
    if (S.err & kErrCellRange) msg += " non-finite or out-of-range coordinate (unstable MD step?);";
    if (S.err & kErrLayout) msg += " MD shared-memory layout mismatch;";
    return fail(b, MPCD_EDEVICE, msg);
  }
  return MPCD_OK;
}

int mpcd_batch_remove(mpcd_batch* b, int r) {
  Replica* Rp = get_rep(b, r);
  if (!Rp) return fail(b, MPCD_EINVAL, "remove: bad replica");
  Replica& R = *Rp;
  if (R.admitted) {
    BK(cudaStreamSynchronize(b->s0));
    b->rep[r] = BatchRep{};
    int rc;
    if ((rc = put_range(b, b->d_rep, r, &b->rep[r], 1))) return rc;
    for (long k = 0; k < R.npages; ++k) b->part_page_rep[R.page0 + k] = -1;
    for (long k = 0; k < R.ncpages; ++k) b->cell_page_rep[R.cpage0 + k] = -1;
    if (R.npages && (rc = put_range(b, b->d_part_page_rep, R.page0, b->part_page_rep.data() + R.page0, R.npages)))
      return rc;
    if (R.ncpages &&
        (rc = put_range(b, b->d_cell_page_rep, R.cpage0, b->cell_page_rep.data() + R.cpage0, R.ncpages)))
      return rc;
    if (R.ntiles_alloc > 0) {
      for (long t = 0; t < R.ntiles_alloc; ++t) b->tile_rep[R.tile0 + t] = -1;
      if ((rc = put_range(b, b->d_tile_rep, R.tile0, b->tile_rep.data() + R.tile0, R.ntiles_alloc))) return rc;
      const long ns = R.ntiles_alloc * (long)b->T;
      std::vector<int> neg(ns, -1);
      if ((rc = put_range(b, b->md.moves, R.tile0 * (long)b->T, neg.data(), ns))) return rc;
      b->graphs_dirty = true;
    }
    BK(cudaStreamSynchronize(b->s0));  // the host vectors above must outlive the copies
    release_ranges(b, R);
  }
  R = Replica{};
  return MPCD_OK;
}

int mpcd_batch_resident(const mpcd_batch* b) {
  if (!b) return 0;
  int n = 0;
  for (auto& R : b->reps) n += R.admitted ? 1 : 0;
  return n;
}

int mpcd_batch_set_tuning(mpcd_batch* b, const mpcd_batch_tuning* t) {
  if (!b || !t) return fail(b, MPCD_EINVAL, "set_tuning: bad arguments");
  cudaSetDevice(b->p.device);
  if ((t->fluid_threads != 0 && (t->fluid_threads < 32 || t->fluid_threads > 1024)) || t->fluid_threads % 32 ||
      t->cell_threads < 32 ||
      t->cell_threads > 1024 || t->cell_threads % 32 || t->fluid_blocks < 0 || t->cell_blocks < 0 ||
      t->sort_interval < 1)
    return fail(b, MPCD_EINVAL, "set_tuning: invalid configuration");
  if (b->since_sort != 0) {  // finish the running sort period first
    enqueue_sort(b, b->cur);
    b->launches_total += b->kernels_per_sort;
    b->cur ^= 1;
    b->since_sort = 0;
  }
  b->tune = *t;
  b->graphs_dirty = true;
  return MPCD_OK;
}

int mpcd_batch_get_tuning(const mpcd_batch* b, mpcd_batch_tuning* t) {
  if (!b || !t) return MPCD_EINVAL;
  *t = b->tune;
  return MPCD_OK;
}

int mpcd_batch_autotune(mpcd_batch* b, int trial_steps, mpcd_batch_tuning* chosen) {
  if (!b || trial_steps < 1) return fail(b, MPCD_EINVAL, "autotune: bad arguments");
  cudaSetDevice(b->p.device);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto trial = [&](const mpcd_batch_tuning& t, double* ms_per_step) {
    int rc = mpcd_batch_set_tuning(b, &t);
    if (rc) return rc;
    rc = rebuild_graphs(b);
    if (rc) return rc;
    const int n = std::max(trial_steps, t.sort_interval) / t.sort_interval * t.sort_interval;
    rc = run_steps(b, t.sort_interval);  // warm-up: one sort period
    if (rc) return rc;
    double ms = 0;
    rc = mpcd_batch_timed_run(b, n, &ms);
    *ms_per_step = ms / n;
    return rc;
  };
  mpcd_batch_tuning best = b->tune;
  double best_ms = 1e30;
  // MD layout (threads per slot, slots per CTA): every swimmer is re-planned
  {
    int best_lanes = b->lanes, best_tile = b->T;
    const int layouts[][2] = {{2, 256}, {1, 512}, {2, 128}, {1, 256}, {1, 1024}, {2, 512}};
    for (auto& lt : layouts) {
      if (mpcd_batch_set_md_layout(b, lt[0], lt[1]) != MPCD_OK) continue;  // does not fit: skip
      double ms;
      int rc = trial(best, &ms);
      if (rc) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best_lanes = lt[0];
        best_tile = lt[1];
      }
    }
    int rc = mpcd_batch_set_md_layout(b, best_lanes, best_tile);
    if (rc) return rc;
  }
  // fluid pass: threads per block and grid (persistent multiples of the SM count, or one block per
  // page); threads 0 = the variant staged through shared memory by bulk copies (own block and grid)
  const int threads[] = {0, 256, 512};
  const long grids[] = {0, 4L * sms, 16L * sms, b->npart_pages};
  for (int th : threads)
    for (long g : grids) {
      if (th == 0 && g != 0) continue;
      mpcd_batch_tuning t = best;
      t.fluid_threads = th;
      t.fluid_blocks = (int)std::min<long>(g, 1L << 30);
      double ms;
      int rc = trial(t, &ms);
      if (rc) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  // cell pass
  for (int th : {128, 256, 512}) {
    mpcd_batch_tuning t = best;
    t.cell_threads = th;
    double ms;
    int rc = trial(t, &ms);
    if (rc) return rc;
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
  }
  // sort interval
  for (int si : {10, 25, 50, 100}) {
    mpcd_batch_tuning t = best;
    t.sort_interval = si;
    double ms;
    int rc = trial(t, &ms);
    if (rc) return rc;
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
  }
  int rc = mpcd_batch_set_tuning(b, &best);
  if (rc) return rc;
  if (chosen) *chosen = best;
  return MPCD_OK;
}

int mpcd_batch_stage_times(mpcd_batch* b, int nsteps, double* out4) {
  if (!b || nsteps < 1 || !out4) return fail(b, MPCD_EINVAL, "stage_times: bad arguments");
  cudaSetDevice(b->p.device);
  int rc = rebuild_graphs(b);  // MD launch plan
  if (rc) return rc;
  const BatchTables t = tables(b);
  std::vector<cudaEvent_t> ev(5 * (size_t)nsteps);
  for (auto& e : ev) BK(cudaEventCreate(&e));
  double acc[4] = {0, 0, 0, 0};
  for (int k = 0; k < nsteps; ++k) {
    cudaEvent_t* E = &ev[5 * (size_t)k];
    BK(cudaEventRecord(E[0], b->s0));
    b->launches_total += launch_batch_prologue(t, b->s0);
    b->launches_total += launch_batch_cell_params(t, b->cells, b->tune.cell_threads, b->tune.cell_blocks, b->s0);
    BK(cudaEventRecord(E[1], b->s0));
    b->launches_total +=
        launch_batch_fluid_step(t, b->fl[b->cur], b->cells, b->tune.fluid_threads, b->tune.fluid_blocks, b->s0);
    BK(cudaEventRecord(E[2], b->s0));
    for (const MDLaunch& L : b->launches) {
      cudaError_t st = cudaSuccess;
      b->launches_total += launch_md_cluster_batch(b->md, t, b->cells, b->d_md_reps + L.offset, L.count, L.ctiles,
                                                   L.hmax, L.nsp_max, L.nbond_max, L.nbuf, b->s0, &st);
      if (st != cudaSuccess) return cuda_fail(b, st, "batch MD launch");
    }
    BK(cudaEventRecord(E[3], b->s0));
    if (++b->since_sort >= b->tune.sort_interval) {
      enqueue_sort(b, b->cur);
      b->launches_total += b->kernels_per_sort;
      b->cur ^= 1;
      b->since_sort = 0;
    }
    BK(cudaEventRecord(E[4], b->s0));
  }
  BK(cudaStreamSynchronize(b->s0));
  for (int k = 0; k < nsteps; ++k) {
    cudaEvent_t* E = &ev[5 * (size_t)k];
    for (int j = 0; j < 4; ++j) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, E[j], E[j + 1]);
      acc[j] += ms;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int j = 0; j < 4; ++j) out4[j] = acc[j] / nsteps;
  BK(cudaGetLastError());
  return MPCD_OK;
}

int mpcd_batch_set_md_layout(mpcd_batch* b, int lanes, int tile) {
  if (!b) return MPCD_EINVAL;
  cudaSetDevice(b->p.device);
  if (lanes == 0) lanes = 2;
  if (tile == 0) tile = 512 / lanes;
  if ((lanes != 1 && lanes != 2) || tile < 32 || tile % 32 || tile * lanes > 1024)
    return fail(b, MPCD_EINVAL, "set_md_layout: invalid layout");
  if (lanes == b->lanes && tile == b->T) return MPCD_OK;
  BK(cudaStreamSynchronize(b->s0));
  // current bead and beat state back to the host descriptions
  for (auto& R : b->reps)
    if (R.admitted && R.nb > 0) {
      int rc = pull_md_state(b, R);
      if (rc) return rc;
    }
  // plan every swimmer with the new layout: nothing changes on the device on failure
  const int oldT = b->T, oldL = b->lanes;
  b->T = tile;
  b->lanes = lanes;
  std::vector<MDPlan> plans(b->reps.size());
  long tiles_needed = 0;
  for (size_t r = 0; r < b->reps.size(); ++r) {
    Replica& R = b->reps[r];
    if (!R.admitted || R.nb == 0) continue;
    MDPlan keep;
    keep = std::move(R.plan);
    std::string why = plan_replica(b, R);
    plans[r] = std::move(R.plan);
    R.plan = std::move(keep);
    tiles_needed += plans[r].ntiles + 1;
    if (!why.empty()) {
      b->T = oldT;
      b->lanes = oldL;
      return fail(b, MPCD_EINVAL, "set_md_layout: " + why);
    }
  }
  if (tiles_needed > b->slot_cap / tile) {
    b->T = oldT;
    b->lanes = oldL;
    return fail(b, MPCD_EINVAL, "set_md_layout: the MD slot capacity does not hold the new layout");
  }
  // clear every MD range and table
  b->tile_cap = b->slot_cap / tile;
  b->a_tile.reset(b->tile_cap);
  b->a_sp.reset(b->p.max_springs);
  b->a_halo.reset(b->p.max_halo);
  b->a_cil.reset(b->p.max_cilia);
  b->a_bond.reset(b->p.max_bonds);
  MDState& m = b->md;
  m.tile = tile;
  m.cl_lanes = lanes;
  m.ntiles = (int)b->tile_cap;
  {
    std::vector<int> neg(b->slot_cap, -1);
    BK(cudaMemcpy(m.moves, neg.data(), b->slot_cap * sizeof(int), cudaMemcpyHostToDevice));
    std::fill(b->tile_rep.begin(), b->tile_rep.end(), -1);
    BK(cudaMemcpy(b->d_tile_rep, b->tile_rep.data(), b->tile_arr_cap * sizeof(int), cudaMemcpyHostToDevice));
    BK(cudaMemset(m.tile_help, 0, b->tile_arr_cap * sizeof(int)));
  }
  for (size_t r = 0; r < b->reps.size(); ++r) {
    Replica& R = b->reps[r];
    if (!R.admitted || R.nb == 0) continue;
    R.tile0 = R.sp0 = R.h0 = R.c0 = R.b0 = -1;
    R.plan = std::move(plans[r]);
    if (!take_md_ranges(b, R)) return fail(b, MPCD_EINVAL, "set_md_layout: MD capacity exhausted (batch unusable)");
    int rc = upload_md(b, (int)r, R);
    if (rc) return rc;
    b->rep[r].md_tile0 = (int)R.tile0;
    b->rep[r].md_ntiles = R.plan.ntiles;
    if ((rc = put_range(b, b->d_rep, (long)r, &b->rep[r], 1))) return rc;
  }
  BK(cudaStreamSynchronize(b->s0));
  b->graphs_dirty = true;
  return MPCD_OK;
}

int mpcd_batch_get_md_layout(const mpcd_batch* b, int* lanes, int* tile) {
  if (!b) return MPCD_EINVAL;
  if (lanes) *lanes = b->lanes;
  if (tile) *tile = b->T;
  return MPCD_OK;
}

long long mpcd_batch_launch_count(const mpcd_batch* b) { return b ? b->launches_total : 0; }

}  // extern "C"
