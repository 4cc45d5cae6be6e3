// C ABI of the GB300 MPCD + microswimmer engine (include/mpcd_gpu.h).
//
// Host-side orchestration of one MPC step (Simulation::next_tstep,
// src/simulation.cpp:217-265):
//   1. cell_params   collision maps from the sums binned last step
//   2. fluid_step    collide + stream + bin every fluid particle
//   3. bead_collide  the same collision for MD beads (mass 5 in the sums)
//   4. md            n velocity-Verlet substeps, final half kick, bead binning,
//                    beat state machine (one cooperative launch)
// with the grid shift of the next step known before 2 (it is drawn from a
// counter-based generator, or injected).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mpcd_gpu.h"
#include "df32.cuh"
#include "engine_internal.h"
#include "md_plan.h"
#include "engine_export.h"


using namespace mpcd;

namespace {
constexpr int kObsSlot = 16;  // doubles per observables ring slot (10 used; 128-byte slots)
}

struct mpcd_engine {
  mpcd_params p{};
  Box box{};
  long ncell = 0;
  int nsub = 0;
  cudaStream_t stream = nullptr;
  // the beads' collision and the MD substeps run on their own (higher
  // priority) stream, concurrently with the fluid pass: both only read the
  // step's collision maps and add into the next step's cell sums
  cudaStream_t smd = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool overlap = true;
  // launch shape of the fluid pass beside the MD launch: > 0 persistent with that
  // many CTAs per SM, <= 0 short-lived CTAs of -fluid_per_sm (at least 1)
  // particles per thread
  int fluid_per_sm = -1;
  std::string error;
  long long launches = 0;

  unsigned* d_err = nullptr;
  double* d_diss = nullptr;
  double* d_obs = nullptr;
  // observables read-backs in flight: ticket t lands in slot t % MPCD_OBS_RING
  // of a pinned ring (kObsSlot doubles: the sums, the dissipated energy, the
  // error word), its copy marked by that slot's event
  double* h_ring = nullptr;
  double* d_ring = nullptr;  // the same ring mapped into the device (the cell-sum kernel writes it)
  // staging of the fluid copies (6 doubles per particle), kept between calls
  double* d_stage = nullptr;
  size_t stage_cap = 0;  // doubles
  unsigned* d_stage_flag = nullptr;
  cudaEvent_t ring_ev[MPCD_OBS_RING] = {};
  double ring_t[MPCD_OBS_RING] = {};       // globalt when the ticket was taken
  unsigned char ring_raw[MPCD_OBS_RING] = {};  // 1: error word copied as raw bits, 0: as a double
  long long obs_next = 0;                  // the next ticket
  double* d_obs_part = nullptr;     // per-block partials of the cell-sum observables
  unsigned* d_obs_count = nullptr;  // blocks finished (reset by the last one)
  unsigned* d_bar = nullptr;

  FluidF64 f64, f64tmp;
  FluidF32 f32, f32tmp;
  CellsF64 c64;
  CellsF32 c32;
  uint32_t *d_count = nullptr, *d_start = nullptr, *d_rank = nullptr, *d_blocksums = nullptr;
  double* d_inj_gamma = nullptr;
  double* d_inj_axis = nullptr;
  double* d_inj_virt = nullptr;

  // MD (host copies; device layout built by prepare)
  long nb = 0;
  std::vector<double> bpos, bvel;
  std::vector<int> bmoves;
  std::vector<int> sp_t, sp_o, sp_k, sp_r;
  std::vector<double> sp_rest, sp_kk;
  std::vector<mpcd_cilium> cil;
  std::vector<double> newlen, oldlen;
  std::vector<int> slot_of;  // bead -> slot
  MDState md;
  long md_nsp = 0;  // springs in the device layout
  bool md_dirty = true;

  // profiling: event pairs per launch, resolved on query
  bool profiling = false;
  struct Mark {
    int kernel;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  double prof_ms[8] = {0};
  long long prof_n[8] = {0};
  void* flush_buf = nullptr;

  // bead-first ordering (mpcd_step, MPCD_BEAD_FIRST=1): per-cell claim tags
  // of the bead maps, the deferred bead binning per slot (cell, and m v,
  // m v^2 as double4 or float4).  Off by default: measured slower on
  // swimmer64 (float64 0.353 against 0.330 ms per step, float32 0.249 against
  // 0.246), the MD launch slowing beside the cell-map kernel by more than
  // the cell maps it no longer waits for
  bool bead_first = false;
  uint32_t* d_claim = nullptr;
  uint32_t claim_tag = 0;
  uint32_t* d_bcell = nullptr;
  void* d_bsum = nullptr;
  int bcap = 0;  // slots d_bcell / d_bsum hold
  // contact forces between cilia (mpcd_set_repelling): eps and the candidate pair list
  double repel = 0.0;
  int2* d_cpairs = nullptr;
  int* d_ncpairs = nullptr;
  int cpair_cap = 0;
  // rigid spheres (mpcd_set_rigid_spheres): device state, this step's
  // impulses, running force / torque sums and the steps they cover
  int nsph = 0;
  RigidSphereDev* d_sph = nullptr;
  double* d_sph_acc = nullptr;
  double* d_sph_fsum = nullptr;
  long long sph_steps = 0;

  long steps = 0;
  double globalt = 0.0;
  double a[3] = {0.5, 0.5, 0.5};
  bool have_shift = false;
  bool prepared = false;
  long since_sort = 0;
};

namespace {

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

int fail(mpcd_engine* h, int code, const std::string& msg) {
  if (h) h->error = msg;
  return code;
}

int cuda_fail(mpcd_engine* h, cudaError_t e, const char* what) {
  return fail(h, MPCD_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc((void**)p, (count > 0 ? count : 1) * sizeof(T));
}

void shift_from_counter(uint64_t seed, uint64_t step, double* a) {
  u32x4 r = draw4(seed, step, kStreamShift, 0u, 0u);
  a[0] = u01_dbl(r.x);
  a[1] = u01_dbl(r.y);
  a[2] = u01_dbl(r.z);
}

void free_fluid(FluidF64& f) {
  cudaFree(f.id);
  cudaFree(f.cell);
  cudaFree(f.ox);
  cudaFree(f.oy);
  cudaFree(f.oz);
  cudaFree(f.vx);
  cudaFree(f.vy);
  cudaFree(f.vz);
  f = FluidF64{};
}

void free_md(MDState& m) {
  for (int b = 0; b < 2; ++b) {
    cudaFree(m.x[b]);
    cudaFree(m.y[b]);
    cudaFree(m.z[b]);
  }
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
  for (int b = 0; b < 2; ++b) cudaFree(m.q[b]);
  cudaFree(m.sp_rest2);
  cudaFree(m.sp_m2k2);
  cudaFree(m.sp_code);
  cudaFree(m.sp_split);
  cudaFree(m.tile_b0);
  cudaFree(m.tile_nb);
  cudaFree(m.halo_run);
  cudaFree(m.halo_run_start);
  cudaFree(m.halo_single);
  cudaFree(m.halo_single_start);
  cudaFree(m.pr_start);
  cudaFree(m.pr_local_end);
  cudaFree(m.pr_hub_begin);
  cudaFree(m.pr_code);
  cudaFree(m.pr_rest);
  cudaFree(m.pr_m2k);
  cudaFree(m.pi_start);
  cudaFree(m.pr_pos);
  cudaFree(m.pl_start);
  cudaFree(m.pl_list);
  cudaFree(m.pl_base);
  cudaFree(m.pr_nslot);
  cudaFree(m.hub_slot);
  cudaFree(m.hub_pbase);
  cudaFree(m.hubpart);
  cudaFree(m.th_start);
  cudaFree(m.th);
  cudaFree(m.tr_list);
  GridBarrier bar = m.bar;
  m = MDState{};
  m.bar = bar;
}

int alloc_fluid(mpcd_engine* h, long n) {
  // the same particle count: the arrays are kept (the load rewrites every one)
  const bool f64 = h->p.precision == MPCD_FP64;
  if (h->d_rank && (f64 ? (h->f64.id && h->f64tmp.id && h->f64.n == n && h->f64tmp.n == n)
                        : (h->f32.id && h->f32tmp.id && h->f32.n == n && h->f32tmp.n == n)))
    return MPCD_OK;
  if (f64) {
    free_fluid(h->f64);
    free_fluid(h->f64tmp);
    for (FluidF64* f : {&h->f64, &h->f64tmp}) {
      f->n = n;
      CK(dalloc(&f->id, n));
      CK(dalloc(&f->cell, n));
      CK(dalloc(&f->ox, n));
      CK(dalloc(&f->oy, n));
      CK(dalloc(&f->oz, n));
      CK(dalloc(&f->vx, n));
      CK(dalloc(&f->vy, n));
      CK(dalloc(&f->vz, n));
    }
  } else {
    for (FluidF32* f : {&h->f32, &h->f32tmp}) {
      cudaFree(f->id);
      cudaFree(f->pos);
      cudaFree(f->vel);
    }
    for (FluidF32* f : {&h->f32, &h->f32tmp}) {
      f->n = n;
      CK(dalloc(&f->id, n));
      CK(dalloc(&f->pos, n));
      CK(dalloc(&f->vel, n));
    }
  }
  cudaFree(h->d_rank);
  CK(dalloc(&h->d_rank, n));
  return MPCD_OK;
}

StepArgs step_args(mpcd_engine* h, const double* a_cur, const double* a_next, double t_move) {
  StepArgs s{};
  s.box = h->box;
  for (int q = 0; q < 3; ++q) {
    s.a_cur[q] = a_cur[q];
    s.a_next[q] = a_next[q];
    s.ta_cur[q] = 1.0 - a_cur[q];
    s.ta_next[q] = 1.0 - a_next[q];
  }
  s.h = h->p.tstep;
  s.gkick = h->p.gravity != 0.0 ? h->p.gravity * std::cos(t_move * h->p.omega) * h->p.tstep : 0.0;
  s.walls = h->p.walls;
  s.bead_mass = h->p.bead_mass;
  s.seed = h->p.seed;
  s.step = (uint64_t)h->steps + 1;
  s.err = h->d_err;
  s.diss = h->d_diss;
  for (int q = 0; q < 3; ++q) {
    s.fta_cur[q] = (float)s.ta_cur[q];
    s.fta_next[q] = (float)s.ta_next[q];
  }
  s.fh = (float)s.h;
  s.fgkick = (float)s.gkick;
  s.fbead_mass = (float)s.bead_mass;
  if (h->nsph > 0) {
    s.sph.n = h->nsph;
    s.sph.s = h->d_sph;
    s.sph.acc = h->d_sph_acc;
  }
  return s;
}

int check_launch(mpcd_engine* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return MPCD_OK;
}

// Build the MD device layout (md_plan.cu plans it on the host; this uploads
// it into freshly allocated device arrays).
int build_md(mpcd_engine* h) {
  free_md(h->md);
  MDState& m = h->md;
  if (h->nb == 0) {
    h->md_dirty = false;
    return MPCD_OK;
  }
  MDInput in;
  in.nb = h->nb;
  in.bpos = h->bpos.data();
  in.bvel = h->bvel.data();
  in.bmoves = h->bmoves.data();
  in.nsp = (long)h->sp_t.size();
  in.sp_t = h->sp_t.data();
  in.sp_o = h->sp_o.data();
  in.sp_k = h->sp_k.data();
  in.sp_r = h->sp_r.data();
  in.sp_rest = h->sp_rest.data();
  in.sp_kk = h->sp_kk.data();
  in.ncil = (int)h->cil.size();
  in.cil = h->cil.data();
  in.nbond = (long)h->newlen.size();
  in.newlen = h->newlen.data();
  in.oldlen = h->oldlen.data();
  // -1: the grid kernel of md_df.cu (faster on GB300 than the float64 kernel
  // and than the split-arithmetic cluster kernel for one box), with
  // double-float springs for the float64 path and float springs on the same
  // double-float positions for the float32 split path (swimmer64 MD 0.204
  // against 0.215 ms, swimmer128 0.423 against 0.526)
  // contact forces between cilia run on the float64 grid kernel only
  const int arith = h->repel != 0.0 ? 0 : h->p.md_split < 0 ? (h->p.precision == MPCD_FP32 ? 3 : 2) : h->p.md_split;
  if (arith > 5) return fail(h, MPCD_EINVAL, "md_split must be -1 or 0 to 5");
  in.split = arith == 1;
  in.df = arith >= 2;
  in.pair = arith == 4 ? 1 : (arith == 5 ? 2 : 0);
  MDPlan pl;
  // MPCD_MD_NO_CLUSTER=1 keeps split arithmetic on the cooperative grid layout
  const char* no_cl = std::getenv("MPCD_MD_NO_CLUSTER");
  const bool allow_cluster = !(no_cl && std::atoi(no_cl) != 0) && h->repel == 0.0;
  // MPCD_MD_MIN_TILE: narrowest grid-layout tile (tests of the wide layouts on small bead sets)
  const char* mt = std::getenv("MPCD_MD_MIN_TILE");
  const int min_tile = mt ? std::max(0, std::min(256, std::atoi(mt))) : 0;
  const std::string why =
      plan_md(in, MDForce{}, allow_cluster, false, h->p.precision == MPCD_FP32 ? 1 : 0, pl, min_tile);
  if (!why.empty()) return fail(h, MPCD_EINVAL, why);
  if (const char* ps = std::getenv("MPCD_MD_PLAN_STATS"); ps && std::atoi(ps) && pl.pair) {
    // the pair layout's per-tile sizes: force entries (of them reaching only
    // the tile), halo, incidences, hubs reached
    for (int t = 0; t < pl.ntiles; ++t)
      std::fprintf(stderr, "md tile %d entries %d local %d halo %d incidences %d hubs %d\n", t,
                   pl.pr_start[t + 1] - pl.pr_start[t], pl.pr_local_end[t] - pl.pr_start[t],
                   pl.hstart[t + 1] - pl.hstart[t], pl.pi_start[(t + 1) * pl.tile] - pl.pi_start[t * pl.tile],
                   pl.th_start[t + 1] - pl.th_start[t]);
  }
  if (pl.hstart.size() != (size_t)pl.ntiles + 1 || pl.halo.size() != (size_t)pl.hstart.back())
    return fail(h, MPCD_EINVAL, "MD plan: halo lists inconsistent with their offsets");
  m.split = pl.split;
  m.pair = pl.pair;
  m.df = pl.df && !pl.pair ? (arith == 3 ? 2 : 1) : 0;
  m.cluster = pl.cluster;
  m.cl_lanes = pl.cl_lanes;
  m.cl_nsp_max = pl.cl_nsp_max;
  m.cl_nbond_max = pl.cl_nbond_max;
  m.cl_nbuf = pl.cl_nbuf;
  m.tile = pl.tile;
  m.ntiles = pl.ntiles;
  m.nslots = pl.nslots;
  m.hmax = pl.hmax;
  const int ns = m.nslots;
  const long nspk = pl.nsp_kept();
  h->md_nsp = nspk;
  const size_t nbond = pl.newlen.size();
  const size_t ncil = pl.cd.size();
  for (int b = 0; b < 2; ++b) {
    CK(dalloc(&m.x[b], ns));
    CK(dalloc(&m.y[b], ns));
    CK(dalloc(&m.z[b], ns));
  }
  CK(dalloc(&m.vx, ns));
  CK(dalloc(&m.vy, ns));
  CK(dalloc(&m.vz, ns));
  CK(dalloc(&m.moves, ns));
  CK(dalloc(&m.prim, ns));
  CK(dalloc(&m.nhelp, ns));
  CK(dalloc(&m.tile_help, m.ntiles));
  CK(dalloc(&m.sp_start, ns + 1));
  CK(dalloc(&m.sp_other, nspk));
  CK(dalloc(&m.sp_local, nspk));
  CK(dalloc(&m.halo, pl.halo.size()));
  CK(dalloc(&m.halo_start, m.ntiles + 1));
  CK(dalloc(&m.diag, nbond));
  CK(dalloc(&m.sp_kind, nspk));
  CK(dalloc(&m.sp_ref, nspk));
  CK(dalloc(&m.sp_rest, nspk));
  CK(dalloc(&m.sp_m2k, nspk));
  CK(dalloc(&m.tile_react, m.ntiles));
  m.ncil = (int)ncil;
  CK(dalloc(&m.cil, ncil));
  CK(dalloc(&m.midpnt, ncil));
  CK(dalloc(&m.tstroke, ncil));
  CK(dalloc(&m.newlen, nbond));
  CK(dalloc(&m.oldlen, nbond));
  CK(dalloc(&m.tile_cil, m.ntiles + 1));
  auto up = [&](void* d, const void* src, size_t bytes) { return cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice); };
  for (int b = 0; b < 2; ++b) {
    CK(up(m.x[b], pl.X.data(), ns * 8));
    CK(up(m.y[b], pl.Y.data(), ns * 8));
    CK(up(m.z[b], pl.Z.data(), ns * 8));
  }
  CK(up(m.vx, pl.VX.data(), ns * 8));
  CK(up(m.vy, pl.VY.data(), ns * 8));
  CK(up(m.vz, pl.VZ.data(), ns * 8));
  CK(up(m.moves, pl.mv.data(), ns * 4));
  CK(up(m.prim, pl.prim.data(), ns * 4));
  CK(up(m.nhelp, pl.nhelp.data(), ns * 4));
  CK(up(m.tile_help, pl.thelp.data(), m.ntiles * 4));
  CK(up(m.sp_start, pl.start.data(), (ns + 1) * 4));
  if (nspk) {
    CK(up(m.sp_other, pl.so.data(), nspk * 4));
    CK(up(m.sp_local, pl.sl.data(), nspk * 4));
    CK(up(m.sp_kind, pl.sk.data(), nspk * 4));
    CK(up(m.sp_ref, pl.sr.data(), nspk * 4));
    CK(up(m.sp_rest, pl.srest.data(), nspk * 8));
    CK(up(m.sp_m2k, pl.sm2k.data(), nspk * 8));
  }
  CK(up(m.tile_react, pl.tile_react.data(), m.ntiles * 4));
  if (ncil) {
    CK(up(m.cil, pl.cd.data(), ncil * sizeof(CiliumDev)));
    CK(up(m.midpnt, pl.mid.data(), ncil * 8));
    CK(up(m.tstroke, pl.ts.data(), ncil * 8));
  }
  if (nbond) {
    CK(up(m.newlen, pl.newlen.data(), nbond * 8));
    CK(up(m.oldlen, pl.oldlen.data(), nbond * 8));
    CK(up(m.diag, pl.diag.data(), nbond * 8));
  }
  if (m.pair) {
    // force entries, incidences and long beads of the pair kernel
    m.pr_nent_max = pl.pr_nent_max;
    m.pr_ninc_max = pl.pr_ninc_max;
    m.pr_nlong_max = pl.pr_nlong_max;
    const size_t ne = pl.pr_code.size(), nlg = pl.pl_list.size();
    CK(dalloc(&m.pr_start, m.ntiles + 1));
    CK(dalloc(&m.pr_local_end, m.ntiles));
    CK(dalloc(&m.pr_hub_begin, m.ntiles));
    CK(dalloc(&m.pr_code, std::max<size_t>(1, ne)));
    CK(dalloc(&m.pr_rest, std::max<size_t>(1, ne)));
    CK(dalloc(&m.pr_m2k, std::max<size_t>(1, ne)));
    CK(dalloc(&m.pi_start, ns + 1));
    CK(dalloc(&m.pr_pos, std::max<size_t>(1, ne)));
    CK(dalloc(&m.pl_start, m.ntiles + 1));
    CK(dalloc(&m.pl_list, std::max<size_t>(1, nlg)));
    CK(dalloc(&m.pl_base, std::max<size_t>(1, nlg)));
    CK(dalloc(&m.pr_nslot, m.ntiles));
    CK(up(m.pr_start, pl.pr_start.data(), (m.ntiles + 1) * sizeof(int)));
    CK(up(m.pr_local_end, pl.pr_local_end.data(), m.ntiles * sizeof(int)));
    CK(up(m.pr_hub_begin, pl.pr_hub_begin.data(), m.ntiles * sizeof(int)));
    if (ne) {
      CK(up(m.pr_code, pl.pr_code.data(), ne * sizeof(uint2)));
      CK(up(m.pr_rest, pl.pr_rest.data(), ne * sizeof(double)));
      CK(up(m.pr_m2k, pl.pr_m2k.data(), ne * sizeof(double)));
    }
    CK(up(m.pi_start, pl.pi_start.data(), (ns + 1) * sizeof(int)));
    if (ne) CK(up(m.pr_pos, pl.pr_pos.data(), ne * sizeof(uint32_t)));
    CK(up(m.pl_start, pl.pl_start.data(), (m.ntiles + 1) * sizeof(int)));
    if (nlg) CK(up(m.pl_list, pl.pl_list.data(), nlg * sizeof(int)));
    if (nlg) CK(up(m.pl_base, pl.pl_base.data(), nlg * sizeof(int)));
    CK(up(m.pr_nslot, pl.pr_nslot.data(), m.ntiles * sizeof(int)));
    // hubs: their slots, the partial sums' offsets and two buffers of them,
    // the tiles' references
    m.nhub = (int)pl.hub_slot.size();
    m.hub_ncon = pl.hub_pbase.empty() ? 0 : pl.hub_pbase.back();
    m.ntr = (int)pl.tr_list.size();
    CK(dalloc(&m.hub_slot, std::max<size_t>(1, pl.hub_slot.size())));
    CK(dalloc(&m.hub_pbase, (size_t)m.nhub + 1));
    CK(dalloc(&m.hubpart, std::max<size_t>(1, 8 * (size_t)m.hub_ncon)));
    CK(dalloc(&m.th_start, m.ntiles + 1));
    CK(dalloc(&m.th, std::max<size_t>(1, pl.th.size())));
    CK(dalloc(&m.tr_list, std::max<size_t>(1, pl.tr_list.size())));
    if (m.nhub) CK(up(m.hub_slot, pl.hub_slot.data(), m.nhub * sizeof(int)));
    CK(up(m.hub_pbase, pl.hub_pbase.data(), (m.nhub + 1) * sizeof(int)));
    CK(up(m.th_start, pl.th_start.data(), (m.ntiles + 1) * sizeof(int)));
    if (!pl.th.empty()) CK(up(m.th, pl.th.data(), pl.th.size() * sizeof(HubRef)));
    if (m.ntr) CK(up(m.tr_list, pl.tr_list.data(), m.ntr * sizeof(int)));
  }
  if (m.df || m.pair) {
    // float pairs of the spring data and the packed layout; the position pair
    // buffers are filled by the kernel (the pair kernel's four float64 per
    // slot take the same 32 bytes)
    std::vector<float2> r2(nspk), k2(nspk);
    for (long i = 0; i < nspk; ++i) {
      const dfloat a = df_from_double(pl.srest[i]), b = df_from_double(pl.sm2k[i]);
      r2[i] = make_float2(a.h, a.l);
      k2[i] = make_float2(b.h, b.l);
    }
    m.df_nsp_max = pl.df_nsp_max;
    m.df_nb_max = pl.df_nb_max;
    m.df_nrun_max = pl.df_nrun_max;
    m.df_nsingle_max = pl.df_nsingle_max;
    for (int b = 0; b < 2; ++b) CK(dalloc(&m.q[b], 2 * (size_t)ns));
    CK(dalloc(&m.sp_rest2, nspk));
    CK(dalloc(&m.sp_m2k2, nspk));
    CK(dalloc(&m.sp_code, nspk));
    CK(dalloc(&m.sp_split, ns));
    CK(dalloc(&m.tile_b0, m.ntiles));
    CK(dalloc(&m.tile_nb, m.ntiles));
    if (nspk) {
      CK(up(m.sp_rest2, r2.data(), nspk * sizeof(float2)));
      CK(up(m.sp_m2k2, k2.data(), nspk * sizeof(float2)));
      CK(up(m.sp_code, pl.df_code.data(), nspk * sizeof(uint32_t)));
    }
    CK(up(m.sp_split, pl.df_split.data(), ns * sizeof(int)));
    CK(up(m.tile_b0, pl.df_b0.data(), m.ntiles * sizeof(int)));
    CK(up(m.tile_nb, pl.df_nb.data(), m.ntiles * sizeof(int)));
    CK(dalloc(&m.halo_run, std::max<size_t>(1, pl.df_runs.size())));
    CK(dalloc(&m.halo_run_start, m.ntiles + 1));
    if (!pl.df_runs.empty()) CK(up(m.halo_run, pl.df_runs.data(), pl.df_runs.size() * sizeof(int4)));
    CK(up(m.halo_run_start, pl.df_run_start.data(), (m.ntiles + 1) * sizeof(int)));
    CK(dalloc(&m.halo_single, std::max<size_t>(1, pl.df_single.size())));
    CK(dalloc(&m.halo_single_start, m.ntiles + 1));
    if (!pl.df_single.empty()) CK(up(m.halo_single, pl.df_single.data(), pl.df_single.size() * sizeof(int2)));
    CK(up(m.halo_single_start, pl.df_single_start.data(), (m.ntiles + 1) * sizeof(int)));
  }
  if (!pl.halo.empty()) CK(up(m.halo, pl.halo.data(), pl.halo.size() * 4));
  CK(up(m.halo_start, pl.hstart.data(), (m.ntiles + 1) * 4));
  CK(up(m.tile_cil, pl.tcil.data(), (m.ntiles + 1) * 4));
  m.bar.count = h->d_bar;
  m.bar.gen = h->d_bar + 1;
  if (h->repel != 0.0) {
    for (size_t c = 0; c < ncil; ++c)
      if (pl.cd[c].len > 64) return fail(h, MPCD_EINVAL, "repelling: cilia of at most 64 beads per filament");
    const long need = std::max<long>(1, std::min<long>((long)ncil * ((long)ncil - 1) / 2, 1L << 20));
    if (h->cpair_cap < need) {
      cudaFree(h->d_cpairs);
      h->d_cpairs = nullptr;
      h->cpair_cap = 0;
      CK(dalloc(&h->d_cpairs, need));
      h->cpair_cap = (int)need;
    }
    if (!h->d_ncpairs) CK(dalloc(&h->d_ncpairs, 1));
    m.repel = h->repel;
    m.cpairs = h->d_cpairs;
    m.ncpairs = h->d_ncpairs;
    m.cpair_cap = h->cpair_cap;
  }
  if (h->bcap < ns) {  // the deferred bead binning of the bead-first step
    cudaFree(h->d_bcell);
    cudaFree(h->d_bsum);
    h->d_bcell = nullptr;
    h->d_bsum = nullptr;
    h->bcap = 0;
    CK(dalloc(&h->d_bcell, ns));
    CK(dalloc(reinterpret_cast<double4**>(&h->d_bsum), ns));
    h->bcap = ns;
  }
  h->slot_of = pl.slot_of;
  h->md_dirty = false;
  return MPCD_OK;
}
// copy device bead state back into the host arrays
int pull_md(mpcd_engine* h) {
  MDState& m = h->md;
  if (h->nb == 0 || m.nslots == 0 || h->md_dirty) return MPCD_OK;
  const int ns = m.nslots;
  std::vector<double> X(ns), Y(ns), Z(ns), VX(ns), VY(ns), VZ(ns);
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(X.data(), m.x[0], ns * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(Y.data(), m.y[0], ns * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(Z.data(), m.z[0], ns * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(VX.data(), m.vx, ns * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(VY.data(), m.vy, ns * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(VZ.data(), m.vz, ns * 8, cudaMemcpyDeviceToHost));
  for (long b = 0; b < h->nb; ++b) {
    int s = h->slot_of[b];
    h->bpos[3 * b] = X[s];
    h->bpos[3 * b + 1] = Y[s];
    h->bpos[3 * b + 2] = Z[s];
    h->bvel[3 * b] = VX[s];
    h->bvel[3 * b + 1] = VY[s];
    h->bvel[3 * b + 2] = VZ[s];
  }
  if (m.ncil) {
    std::vector<double> mid(m.ncil), ts(m.ncil);
    CK(cudaMemcpy(mid.data(), m.midpnt, m.ncil * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ts.data(), m.tstroke, m.ncil * 8, cudaMemcpyDeviceToHost));
    for (int c = 0; c < m.ncil; ++c) {
      h->cil[c].midpnt = mid[c];
      h->cil[c].tstroke = ts[c];
    }
    CK(cudaMemcpy(h->newlen.data(), m.newlen, h->newlen.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->oldlen.data(), m.oldlen, h->oldlen.size() * 8, cudaMemcpyDeviceToHost));
  }
  return MPCD_OK;
}

static std::string error_text(unsigned e) {
  std::string msg = "device check failed:";
  if (e & kErrGammaMissing) msg += " injected gamma missing for a thermostatted cell;";
  if (e & kErrGammaLoop) msg += " Gamma sampler exceeded its iteration cap;";
  if (e & kErrBarrier) msg += " MD grid barrier timed out;";
  if (e & kErrCellRange) msg += " non-finite or out-of-range coordinate (unstable MD step?);";
  if (e & kErrCellOverflow) msg += " cell occupancy overflow;";
  if (e & kErrLayout) msg += " MD shared-memory layout mismatch;";
  return msg;
}

int device_error(mpcd_engine* h) {
  unsigned e = 0;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&e, h->d_err, sizeof e, cudaMemcpyDeviceToHost));
  if (e == 0) return MPCD_OK;
  cudaMemset(h->d_err, 0, sizeof(unsigned));
  return fail(h, MPCD_EDEVICE, error_text(e));
}

// brackets one launch with events when profiling is on
struct ProfScope {
  mpcd_engine* h;
  int kernel;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(mpcd_engine* hh, int k, cudaStream_t st = nullptr) : h(hh), kernel(k), s(st ? st : hh->stream) {
    if (h->profiling) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (h->profiling) {
      cudaEventRecord(b, s);
      h->marks.push_back({kernel, a, b});
    }
  }
};

void resolve_marks(mpcd_engine* h) {
  if (h->marks.empty()) return;
  cudaStreamSynchronize(h->stream);
  for (auto& m : h->marks) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) {
      h->prof_ms[m.kernel] += ms;
      h->prof_n[m.kernel] += 1;
    }
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  h->marks.clear();
}

int sort_fluid(mpcd_engine* h) {
  ProfScope ps(h, MPCD_K_SORT);
  if (h->p.precision == MPCD_FP64) {
    if (h->f64.n == 0) return MPCD_OK;
    h->launches += launch_sort_f64(h->f64, h->f64tmp, h->box, h->d_count, h->d_start, h->d_rank, h->d_blocksums,
                                   h->stream);
  } else {
    if (h->f32.n == 0) return MPCD_OK;
    h->launches += launch_sort_f32(h->f32, h->f32tmp, h->box, h->d_count, h->d_start, h->d_rank, h->d_blocksums,
                                   h->stream);
  }
  h->since_sort = 0;
  return check_launch(h, "sort");
}

}  // namespace

namespace mpcd {

int engine_export(mpcd_engine* h, EngineExport& out) {
  if (!h) return MPCD_EINVAL;
  int rc = pull_md(h);
  if (rc) return rc;
  out = EngineExport{};
  out.p = h->p;
  std::memcpy(out.a, h->a, sizeof out.a);
  out.globalt = h->globalt;
  out.steps = h->steps;
  out.nf = mpcd_fluid_count(h);
  if (out.nf > 0) {
    out.fpos.resize(3 * out.nf);
    out.fvel.resize(3 * out.nf);
    rc = mpcd_get_fluid(h, out.nf, out.fpos.data(), out.fvel.data());
    if (rc) return rc;
  }
  out.nb = h->nb;
  out.bpos = h->bpos;
  out.bvel = h->bvel;
  out.bmoves = h->bmoves;
  out.sp_t = h->sp_t;
  out.sp_o = h->sp_o;
  out.sp_k = h->sp_k;
  out.sp_r = h->sp_r;
  out.sp_rest = h->sp_rest;
  out.sp_kk = h->sp_kk;
  out.cil = h->cil;
  out.newlen = h->newlen;
  out.oldlen = h->oldlen;
  return MPCD_OK;
}

}  // namespace mpcd

extern "C" {

int mpcd_create(const mpcd_params* params, mpcd_engine** out) {
  if (params == nullptr || out == nullptr) return MPCD_EINVAL;
  *out = nullptr;
  const mpcd_params& p = *params;
  for (int q = 0; q < 3; ++q)
    if (p.sizes[q] < 2 || p.sizes[q] > 1024) return MPCD_EINVAL;
  if (!(p.tstep > 0) || !(p.ststep > 0) || (p.precision != MPCD_FP64 && p.precision != MPCD_FP32) ||
      p.walls < 0 || p.walls > 2 || !(p.bead_mass > 0))
    return MPCD_EINVAL;
  mpcd_engine* h = new (std::nothrow) mpcd_engine();
  if (!h) return MPCD_ENOMEM;
  h->p = p;
  // auto: every 50 steps (swimmer64 ms per step, float64 / float32: every 10
  // steps 0.343 / 0.251, 25 0.334 / 0.246, 50 0.331 / 0.244, 100 0.331 / 0.244)
  if (h->p.sort_interval <= 0) h->p.sort_interval = 50;
  for (int q = 0; q < 3; ++q) h->box.L[q] = p.sizes[q];
  h->ncell = (long)p.sizes[0] * p.sizes[1] * p.sizes[2];
  h->nsub = (int)((p.tstep + 0.00000001) / p.ststep);
  if (h->nsub < 1 || h->nsub > 511) {
    delete h;
    return MPCD_EINVAL;  // 1 .. 511 MD substeps per MPC step
  }
  auto bail = [&](cudaError_t e, const char* what) {
    fprintf(stderr, "mpcd_create: %s: %s\n", what, cudaGetErrorString(e));
    mpcd_destroy(h);
    return e == cudaErrorMemoryAllocation ? MPCD_ENOMEM : MPCD_ECUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(p.device)) != cudaSuccess) return bail(e, "cudaSetDevice");
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
  {
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if ((e = cudaStreamCreateWithPriority(&h->smd, cudaStreamNonBlocking, prio_greatest)) != cudaSuccess)
      return bail(e, "stream");
    if ((e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
    const char* env = std::getenv("MPCD_MD_OVERLAP");  // 0: MD after the fluid pass on one stream
    h->overlap = !(env && std::atoi(env) == 0);
    if (const char* f = std::getenv("MPCD_FLUID_PER_SM")) h->fluid_per_sm = std::max(-64, std::min(8, std::atoi(f)));
  }
  if ((e = dalloc(&h->d_err, 1)) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_diss, 1)) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_obs, 16)) != cudaSuccess) return bail(e, "alloc");
  if ((e = cudaHostAlloc((void**)&h->h_ring, kObsSlot * sizeof(double) * MPCD_OBS_RING,
                         cudaHostAllocMapped | cudaHostAllocPortable)) != cudaSuccess)
    return bail(e, "alloc");
  if ((e = cudaHostGetDevicePointer((void**)&h->d_ring, h->h_ring, 0)) != cudaSuccess) return bail(e, "map");
  if ((e = dalloc(&h->d_obs_part, 7 * (size_t)kObsBlocks)) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_obs_count, 1)) != cudaSuccess) return bail(e, "alloc");
  if ((e = cudaMemset(h->d_obs_count, 0, sizeof(unsigned))) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_bar, 2)) != cudaSuccess) return bail(e, "alloc");
  cudaMemset(h->d_err, 0, sizeof(unsigned));
  cudaMemset(h->d_diss, 0, sizeof(double));
  cudaMemset(h->d_bar, 0, 2 * sizeof(unsigned));
  const long nc = h->ncell;
  if (p.precision == MPCD_FP64) {
    h->c64.ncell = nc;
    if ((e = dalloc(&h->c64.sum, nc)) != cudaSuccess) return bail(e, "alloc cells");
    if ((e = dalloc(&h->c64.cnt, nc)) != cudaSuccess) return bail(e, "alloc cells");
    if ((e = dalloc(&h->c64.par, 12 * nc)) != cudaSuccess) return bail(e, "alloc cells");
    cudaMemset(h->c64.sum, 0, nc * sizeof(double4));
    cudaMemset(h->c64.cnt, 0, nc * sizeof(uint32_t));
  } else {
    h->c32.ncell = nc;
    if ((e = dalloc(&h->c32.sum, nc)) != cudaSuccess) return bail(e, "alloc cells");
    if ((e = dalloc(&h->c32.cnt, nc)) != cudaSuccess) return bail(e, "alloc cells");
    if ((e = dalloc(&h->c32.par, 2 * nc)) != cudaSuccess) return bail(e, "alloc cells");
    cudaMemset(h->c32.sum, 0, nc * sizeof(float4));
    cudaMemset(h->c32.cnt, 0, nc * sizeof(uint32_t));
  }
  if ((e = dalloc(&h->d_count, nc)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&h->d_start, nc)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&h->d_blocksums, nc / 1024 + 2)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&h->d_claim, nc)) != cudaSuccess) return bail(e, "alloc cells");
  cudaMemset(h->d_claim, 0, nc * sizeof(uint32_t));
  if (const char* bf = std::getenv("MPCD_BEAD_FIRST")) h->bead_first = std::atoi(bf) != 0;
  shift_from_counter(p.seed, 0, h->a);
  *out = h;
  return MPCD_OK;
}

int mpcd_destroy(mpcd_engine* h) {
  if (!h) return MPCD_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_fluid(h->f64);
  free_fluid(h->f64tmp);
  for (FluidF32* f : {&h->f32, &h->f32tmp}) {
    cudaFree(f->id);
    cudaFree(f->pos);
    cudaFree(f->vel);
  }
  cudaFree(h->c64.sum);
  cudaFree(h->c64.cnt);
  cudaFree(h->c64.par);
  cudaFree(h->c32.sum);
  cudaFree(h->c32.cnt);
  cudaFree(h->c32.par);
  cudaFree(h->d_count);
  cudaFree(h->d_start);
  cudaFree(h->d_rank);
  cudaFree(h->d_blocksums);
  cudaFree(h->d_inj_gamma);
  cudaFree(h->d_inj_axis);
  cudaFree(h->d_inj_virt);
  free_md(h->md);
  cudaFree(h->d_err);
  cudaFree(h->d_diss);
  cudaFree(h->d_obs);
  cudaFreeHost(h->h_ring);
  cudaFree(h->d_stage);
  cudaFree(h->d_stage_flag);
  for (cudaEvent_t ev : h->ring_ev)
    if (ev) cudaEventDestroy(ev);
  cudaFree(h->d_obs_part);
  cudaFree(h->d_obs_count);
  cudaFree(h->d_bar);
  cudaFree(h->d_cpairs);
  cudaFree(h->d_ncpairs);
  cudaFree(h->d_claim);
  cudaFree(h->d_bcell);
  cudaFree(h->d_bsum);
  cudaFree(h->d_sph);
  cudaFree(h->d_sph_acc);
  cudaFree(h->d_sph_fsum);
  cudaFree(h->flush_buf);
  for (auto& m : h->marks) {
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->smd) cudaStreamDestroy(h->smd);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  delete h;
  return MPCD_OK;
}

const char* mpcd_last_error(const mpcd_engine* h) { return h ? h->error.c_str() : "null handle"; }
long mpcd_cell_count(const mpcd_engine* h) { return h ? h->ncell : 0; }
long long mpcd_launch_count(const mpcd_engine* h) { return h ? h->launches : 0; }
long mpcd_fluid_count(const mpcd_engine* h) {
  if (!h) return 0;
  return h->p.precision == MPCD_FP64 ? h->f64.n : h->f32.n;
}

// Device staging of the caller's N x 3 float64 arrays (pos, vel): 48 bytes per
// particle and a flag word (cleared), kept by the handle and grown to the
// largest fluid copied, so that repeated uploads and downloads allocate nothing.
struct Staging {
  double* d = nullptr;
  unsigned* flag = nullptr;
};
int staging(mpcd_engine* h, long n, Staging& st) {
  const size_t need = 6 * (size_t)(n > 0 ? n : 1);
  if (need > h->stage_cap) {
    cudaFree(h->d_stage);
    h->d_stage = nullptr;
    h->stage_cap = 0;
    CK(dalloc(&h->d_stage, need));
    h->stage_cap = need;
  }
  if (!h->d_stage_flag) CK(dalloc(&h->d_stage_flag, 1));
  CK(cudaMemsetAsync(h->d_stage_flag, 0, sizeof(unsigned), h->stream));
  st.d = h->d_stage;
  st.flag = h->d_stage_flag;
  return MPCD_OK;
}

int mpcd_set_fluid(mpcd_engine* h, long n, const double* pos, const double* vel) {
  if (!h || n < 0 || (n > 0 && (!pos || !vel))) return fail(h, MPCD_EINVAL, "set_fluid: bad arguments");
  if (n > 0x7fffffffL) return fail(h, MPCD_EINVAL, "set_fluid: more than 2^31 - 1 particles");
  Staging st;
  if (int rc_st = staging(h, n, st)) return rc_st;
  double* dpos = st.d;
  double* dvel = st.d + 3 * (size_t)n;
  if (n > 0) {
    // the caller's arrays as they are; validation, wrapping into cell +
    // offset and the split into the kernels' layout run on the device
    CK(cudaMemcpyAsync(dpos, pos, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dvel, vel, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->launches += launch_check_fluid(n, dpos, dvel, st.flag, h->stream);
    unsigned bad = 0;
    CK(cudaMemcpyAsync(&bad, st.flag, sizeof bad, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (bad) return fail(h, MPCD_EINVAL, "set_fluid: non-finite or out-of-range position or velocity");
  }
  int rc = alloc_fluid(h, n);
  if (rc) return rc;
  if (h->p.precision == MPCD_FP64)
    h->launches += launch_load_fluid_f64(n, dpos, dvel, h->box, h->f64, h->stream);
  else
    h->launches += launch_load_fluid_f32(n, dpos, dvel, h->box, h->f32, h->stream);
  CK(cudaStreamSynchronize(h->stream));  // the staging buffer is free again on return
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_get_fluid(mpcd_engine* h, long n, double* pos, double* vel) {
  if (!h) return MPCD_EINVAL;
  const long have = mpcd_fluid_count(h);
  if (n != have) return fail(h, MPCD_EINVAL, "get_fluid: n does not match the fluid size");
  if (n == 0) return device_error(h);
  Staging st;
  if (int rc_st = staging(h, n, st)) return rc_st;
  double* dpos = st.d;
  double* dvel = st.d + 3 * (size_t)n;
  // back into the caller's order (by particle id) and layout on the device
  if (h->p.precision == MPCD_FP64)
    h->launches += launch_store_fluid_f64(h->f64, dpos, dvel, st.flag, h->stream);
  else
    h->launches += launch_store_fluid_f32(h->f32, dpos, dvel, st.flag, h->stream);
  unsigned bad = 0;
  CK(cudaMemcpyAsync(&bad, st.flag, sizeof bad, cudaMemcpyDeviceToHost, h->stream));
  if (pos) CK(cudaMemcpyAsync(pos, dpos, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (vel) CK(cudaMemcpyAsync(vel, dvel, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (bad) return fail(h, MPCD_EDEVICE, "particle id out of range");
  return device_error(h);
}

// Page-locks a caller's buffer so that the fluid and bead copies of this
// library run as direct DMA instead of through the CUDA driver's staging of
// pageable memory (no counterpart in the reference, which has no device).
int mpcd_pin_host(mpcd_engine* h, void* p, size_t bytes) {
  if (!h || !p || bytes == 0) return MPCD_EINVAL;
  CK(cudaHostRegister(p, bytes, cudaHostRegisterPortable));
  return MPCD_OK;
}
int mpcd_unpin_host(mpcd_engine* h, void* p) {
  if (!h || !p) return MPCD_EINVAL;
  CK(cudaHostUnregister(p));
  return MPCD_OK;
}

int mpcd_set_shift(mpcd_engine* h, const double* a3) {
  if (!h || !a3) return MPCD_EINVAL;
  for (int q = 0; q < 3; ++q)
    if (!(a3[q] >= 0.0 && a3[q] < 1.0)) return fail(h, MPCD_EINVAL, "shift components must lie in [0,1)");
  std::memcpy(h->a, a3, sizeof h->a);
  h->prepared = false;
  return MPCD_OK;
}
int mpcd_get_shift(mpcd_engine* h, double* a3) {
  if (!h || !a3) return MPCD_EINVAL;
  std::memcpy(a3, h->a, sizeof h->a);
  return MPCD_OK;
}
int mpcd_set_time(mpcd_engine* h, double t) {
  if (!h) return MPCD_EINVAL;
  h->globalt = t;
  return MPCD_OK;
}
int mpcd_get_time(mpcd_engine* h, double* t) {
  if (!h || !t) return MPCD_EINVAL;
  *t = h->globalt;
  return MPCD_OK;
}

int mpcd_set_beads(mpcd_engine* h, long nb, const double* pos, const double* vel, const int* moves) {
  if (!h || nb < 0 || (nb > 0 && (!pos || !vel))) return fail(h, MPCD_EINVAL, "set_beads: bad arguments");
  for (long i = 0; i < 3 * nb; ++i)
    if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || std::fabs(pos[i]) > 1e12)
      return fail(h, MPCD_EINVAL, "set_beads: non-finite or out-of-range position or velocity");
  if (h->nb != nb) {
    h->md_dirty = true;
    h->nb = nb;
  }
  h->bpos.assign(pos, pos + 3 * nb);
  h->bvel.assign(vel, vel + 3 * nb);
  h->bmoves.assign(nb, 1);
  if (moves)
    for (long i = 0; i < nb; ++i) h->bmoves[i] = moves[i] ? 1 : 0;
  h->md_dirty = true;
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_get_beads(mpcd_engine* h, long nb, double* pos, double* vel) {
  if (!h || nb != h->nb) return fail(h, MPCD_EINVAL, "get_beads: n does not match the bead count");
  int rc = pull_md(h);
  if (rc) return rc;
  if (pos) std::memcpy(pos, h->bpos.data(), 3 * nb * sizeof(double));
  if (vel) std::memcpy(vel, h->bvel.data(), 3 * nb * sizeof(double));
  return device_error(h);
}

int mpcd_set_springs(mpcd_engine* h, long ns, const int* target, const int* other, const int* kind, const int* ref,
                     const double* rest, const double* k) {
  if (!h || ns < 0 || (ns > 0 && (!target || !other || !kind || !k))) return fail(h, MPCD_EINVAL, "set_springs: bad arguments");
  int rc = pull_md(h);
  if (rc) return rc;
  h->sp_t.assign(target, target + ns);
  h->sp_o.assign(other, other + ns);
  h->sp_k.assign(kind, kind + ns);
  h->sp_r.assign(ns, 0);
  h->sp_rest.assign(ns, 0.0);
  for (long i = 0; i < ns; ++i) {
    if (kind[i] < 0 || kind[i] > 3) return fail(h, MPCD_EINVAL, "set_springs: unknown spring kind");
    if (kind[i] >= 2) {
      if (!ref) return fail(h, MPCD_EINVAL, "set_springs: BOND/DIAG springs need ref");
      h->sp_r[i] = ref[i];
    } else {
      if (!rest) return fail(h, MPCD_EINVAL, "set_springs: CONST springs need rest");
      h->sp_rest[i] = rest[i];
    }
  }
  h->sp_kk.assign(k, k + ns);
  h->md_dirty = true;
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_set_cilia(mpcd_engine* h, int nc, const mpcd_cilium* cilia, const double* newlength,
                   const double* oldlength) {
  if (!h || nc < 0 || (nc > 0 && !cilia)) return fail(h, MPCD_EINVAL, "set_cilia: bad arguments");
  int rc = pull_md(h);
  if (rc) return rc;
  h->cil.assign(cilia, cilia + nc);
  size_t nbond = 0;
  for (int c = 0; c < nc; ++c) {
    if (cilia[c].rodlength < 2 || cilia[c].bond_base < 0) return fail(h, MPCD_EINVAL, "set_cilia: bad cilium");
    nbond = std::max(nbond, (size_t)(cilia[c].bond_base + cilia[c].rodlength));
  }
  h->newlen.assign(nbond, 0.5);
  h->oldlen.assign(nbond, 0.5);
  if (newlength) h->newlen.assign(newlength, newlength + nbond);
  if (oldlength) h->oldlen.assign(oldlength, oldlength + nbond);
  h->md_dirty = true;
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_get_cilia(mpcd_engine* h, int nc, double* state2, double* newlength, double* oldlength) {
  if (!h || nc != (int)h->cil.size()) return fail(h, MPCD_EINVAL, "get_cilia: count mismatch");
  int rc = pull_md(h);
  if (rc) return rc;
  for (int c = 0; c < nc; ++c) {
    if (state2) {
      state2[2 * c] = h->cil[c].midpnt;
      state2[2 * c + 1] = h->cil[c].tstroke;
    }
  }
  if (newlength) std::memcpy(newlength, h->newlen.data(), h->newlen.size() * 8);
  if (oldlength) std::memcpy(oldlength, h->oldlen.data(), h->oldlen.size() * 8);
  return MPCD_OK;
}

int mpcd_prepare(mpcd_engine* h) {
  if (!h) return MPCD_EINVAL;
  if (h->md_dirty) {
    int rc = build_md(h);
    if (rc) return rc;
  }
  const long nc = h->ncell;
  if (h->p.precision == MPCD_FP64) {
    CK(cudaMemsetAsync(h->c64.sum, 0, nc * sizeof(double4), h->stream));
    CK(cudaMemsetAsync(h->c64.cnt, 0, nc * sizeof(uint32_t), h->stream));
  } else {
    CK(cudaMemsetAsync(h->c32.sum, 0, nc * sizeof(float4), h->stream));
    CK(cudaMemsetAsync(h->c32.cnt, 0, nc * sizeof(uint32_t), h->stream));
  }
  int rc = sort_fluid(h);
  if (rc) return rc;
  StepArgs s = step_args(h, h->a, h->a, h->globalt);
  if (h->p.precision == MPCD_FP64) {
    h->launches += launch_bin_fluid_f64(h->f64, h->c64, s, h->stream);
    h->launches += launch_bin_beads_f64(h->md, h->c64, s, h->stream);
  } else {
    h->launches += launch_bin_fluid_f32(h->f32, h->c32, s, h->stream);
    h->launches += launch_bin_beads_f32(h->md, h->c32, s, h->stream);
  }
  rc = check_launch(h, "prepare");
  if (rc) return rc;
  h->prepared = true;
  return MPCD_OK;
}

int mpcd_step(mpcd_engine* h, const mpcd_inject* inj) {
  if (!h) return MPCD_EINVAL;
  if (!h->prepared) {
    int rc = mpcd_prepare(h);
    if (rc) return rc;
  }
  double a_next[3];
  if (inj && inj->shift_next) {
    for (int q = 0; q < 3; ++q) {
      a_next[q] = inj->shift_next[q];
      if (!(a_next[q] >= 0.0 && a_next[q] < 1.0)) return fail(h, MPCD_EINVAL, "injected shift outside [0,1)");
    }
  } else {
    shift_from_counter(h->p.seed, (uint64_t)h->steps + 1, a_next);
  }
  // simulation time as the reference accumulates it (n additions of ststep)
  const double t0 = h->globalt;
  double t_move = t0;
  for (int k = 1; k < h->nsub; ++k) t_move += h->p.ststep;
  t_move += h->p.ststep;
  StepArgs s = step_args(h, h->a, a_next, t_move);
  if (inj && inj->virt) {
    if (!h->d_inj_virt) CK(dalloc(&h->d_inj_virt, 3 * h->ncell));
    CK(cudaMemcpyAsync(h->d_inj_virt, inj->virt, 3 * h->ncell * 8, cudaMemcpyHostToDevice, h->stream));
    s.inj_virt = h->d_inj_virt;
  }
  if (inj && (inj->gamma || inj->axis)) {
    if (!h->d_inj_gamma) {
      CK(dalloc(&h->d_inj_gamma, h->ncell));
      CK(dalloc(&h->d_inj_axis, 3 * h->ncell));
    }
    if (inj->gamma) {
      CK(cudaMemcpyAsync(h->d_inj_gamma, inj->gamma, h->ncell * 8, cudaMemcpyHostToDevice, h->stream));
      s.inj_gamma = h->d_inj_gamma;
    }
    if (inj->axis) {
      CK(cudaMemcpyAsync(h->d_inj_axis, inj->axis, 3 * h->ncell * 8, cudaMemcpyHostToDevice, h->stream));
      s.inj_axis = h->d_inj_axis;
    }
  }
  MDStepArgs ma{};
  ma.t0 = t0;
  ma.dt = h->p.ststep;
  ma.tstep = h->p.tstep;
  ma.n = h->nsub;
  ma.t_end = t_move;
  // rest-length refresh schedule of the force evaluations (src/cilia.cpp:206-215):
  // evaluation 0 and 1 at t0, evaluation k+1 after k additions of ststep
  {
    double te = t0;
    for (int e = 0; e <= h->nsub && e < 512; ++e) {
      if (e >= 2) te += h->p.ststep;
      if (std::fmod(te + h->p.ststep / 10., 0.01) < h->p.ststep) ma.refresh[e >> 6] |= 1ull << (e & 63);
    }
  }
  ma.box = h->box;
  for (int q = 0; q < 3; ++q) {
    ma.a_cur[q] = h->a[q];
    ma.a_next[q] = a_next[q];
  }
  ma.bead_mass = h->p.bead_mass;
  ma.err = h->d_err;
  cudaError_t coop = cudaSuccess;
  const bool f64 = h->p.precision == MPCD_FP64;
  const bool md = h->md.nslots > 0;
  // the double-float grid kernel applies the beads' collision itself (one
  // launch less on the MD chain); the other MD kernels after the bead kernel
  const bool folded = md && !h->md.cluster && (h->md.df || h->md.pair);
  // bead first (MPCD_BEAD_FIRST=1, folded MD launch only): only the maps of
  // the cells that hold beads are made before the MD launch; it is forked
  // right after them, and the maps of the other cells and the fluid pass run
  // beside it (the beads' binning is deferred to a kernel after the join).
  // Otherwise every map is made before the fork.
  const bool first = folded && h->bead_first;
  if (first) {
    s.premapped = 1;
    ma.deferred = 1;
    ma.bcell = h->d_bcell;
    ma.bsum = h->d_bsum;
    ProfScope ps(h, MPCD_K_CELL);
    h->launches += f64 ? launch_bead_maps_f64(h->md, h->c64, s, h->d_claim, ++h->claim_tag, h->stream)
                       : launch_bead_maps_f32(h->md, h->c32, s, h->d_claim, ++h->claim_tag, h->stream);
  } else {
    ProfScope ps(h, MPCD_K_CELL);
    h->launches += f64 ? launch_cell_params_f64(h->c64, s, h->stream) : launch_cell_params_f32(h->c32, s, h->stream);
  }
  // fluid pass on the engine's stream; beads' collision and MD on smd, forked
  // after the collision maps they read and joined before anything reads the
  // new state (kernel timing runs them one after the other, so that each is
  // timed alone)
  const bool fork = md && h->overlap && !h->profiling;
  cudaStream_t sm = fork ? h->smd : h->stream;
  if (fork) {
    CK(cudaEventRecord(h->ev_fork, h->stream));
    CK(cudaStreamWaitEvent(h->smd, h->ev_fork, 0));
  }
  if (md) {
    if (folded) {
      ma.collide = 1;
      ma.diss = h->d_diss;
    } else {
      ProfScope ps(h, MPCD_K_BEAD, sm);
      h->launches += f64 ? launch_bead_collide_f64(h->md, h->c64, s, sm) : launch_bead_collide_f32(h->md, h->c32, s, sm);
    }
    if (h->md.repel != 0.0) h->launches += launch_contact_pairs(h->md, sm);
    ProfScope ps(h, MPCD_K_MD, sm);
    if (h->md.cluster)
      h->launches += f64 ? launch_md_cluster_f64cells(h->md, h->c64, ma, sm, &coop)
                         : launch_md_cluster_f32cells(h->md, h->c32, ma, sm, &coop);
    else if (h->md.pair)
      h->launches += f64 ? launch_md_pair_f64cells(h->md, h->c64, ma, sm, &coop)
                         : launch_md_pair_f32cells(h->md, h->c32, ma, sm, &coop);
    else if (h->md.df)
      h->launches += f64 ? launch_md_df_f64cells(h->md, h->c64, ma, sm, &coop)
                         : launch_md_df_f32cells(h->md, h->c32, ma, sm, &coop);
    else
      h->launches += f64 ? launch_md_f64(h->md, h->c64, ma, sm, &coop)
                         : launch_md_f32cells(h->md, h->c32, ma, sm, &coop);
  }
  if (first) {  // the other cells' maps, beside the MD launch
    ProfScope ps(h, MPCD_K_CELL);
    h->launches += f64 ? launch_cell_params_f64(h->c64, s, h->stream) : launch_cell_params_f32(h->c32, s, h->stream);
  }
  {
    // beside the MD launch the fluid pass runs as many short-lived CTAs (one
    // round of particles per thread): as they retire, the higher-priority MD
    // CTAs take their place, and the fluid CTAs fill what the MD leaves of
    // every SM (swimmer64 float64: 0.336 ms per step against 0.405 with a
    // persistent grid of 3 CTAs per SM)
    ProfScope ps(h, MPCD_K_FLUID);
    const int per_sm = fork ? h->fluid_per_sm : 4;
    h->launches += f64 ? launch_fluid_step_f64(h->f64, h->c64, s, h->stream, per_sm)
                       : launch_fluid_step_f32(h->f32, h->c32, s, h->stream, per_sm);
  }
  if (h->nsph > 0) {
    h->launches += launch_spheres_update(h->d_sph, h->nsph, h->d_sph_acc, h->d_sph_fsum, h->p.tstep, h->box, h->stream);
    h->sph_steps++;
  }
  if (fork) {
    CK(cudaEventRecord(h->ev_join, h->smd));
    CK(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
  }
  if (first) {  // the beads' binning the MD launch deferred
    ProfScope ps(h, MPCD_K_BEAD);
    h->launches += f64 ? launch_bead_add_f64(h->md, h->c64, h->d_bcell, h->d_bsum, h->stream)
                       : launch_bead_add_f32(h->md, h->c32, h->d_bcell, h->d_bsum, h->stream);
  }
  if (coop != cudaSuccess) return cuda_fail(h, coop, "cooperative MD launch");
  int rc = check_launch(h, "step");
  if (rc) return rc;
  h->globalt = t_move;
  std::memcpy(h->a, a_next, sizeof h->a);
  h->steps++;
  if (++h->since_sort >= h->p.sort_interval) {
    rc = sort_fluid(h);
    if (rc) return rc;
  }
  if (inj && (inj->gamma || inj->axis)) return device_error(h);  // injected runs check every step
  return MPCD_OK;
}

int mpcd_run(mpcd_engine* h, int nsteps) {
  if (!h || nsteps < 0) return MPCD_EINVAL;
  for (int i = 0; i < nsteps; ++i) {
    int rc = mpcd_step(h, nullptr);
    if (rc) return rc;
  }
  return MPCD_OK;
}

int mpcd_sync(mpcd_engine* h) {
  if (!h) return MPCD_EINVAL;
  return device_error(h);
}

int mpcd_reset_diss(mpcd_engine* h) {
  if (!h) return MPCD_EINVAL;
  CK(cudaMemsetAsync(h->d_diss, 0, sizeof(double), h->stream));
  return MPCD_OK;
}

// Enqueues the observables of the current state behind the work issued so far
// and returns at once; no counterpart in the reference (MPCD::debug,
// src/libcilia/mpcd.cpp:404-467, sums and prints in one go).  The sums land in
// ring slot ticket % MPCD_OBS_RING; every later call on the handle is ordered
// after the kernel (and copies) that write them on the stream, so the next step
// runs while the host has not yet read them.
int mpcd_observables_async(mpcd_engine* h, long long* ticket) {
  if (!h || !ticket) return MPCD_EINVAL;
  if (h->md_dirty && h->nb) {
    int rc = build_md(h);
    if (rc) return rc;
  }
  const long long t = h->obs_next;
  const int slot = (int)(t % MPCD_OBS_RING);
  double* o = h->h_ring + (size_t)slot * kObsSlot;
  if (!h->ring_ev[slot]) CK(cudaEventCreateWithFlags(&h->ring_ev[slot], cudaEventDisableTiming));
  if (h->p.precision == MPCD_FP64 && h->prepared) {
    // the cell sums of the last binning (the state has not changed since: every
    // setter clears `prepared`) hold the totals; one kernel, which writes the
    // ten results straight into the mapped ring slot
    h->launches += launch_observables_cells_f64(h->c64, h->md, h->p.bead_mass, h->d_diss, h->d_err, h->d_obs_part,
                                                h->d_obs_count, h->d_ring + (size_t)slot * kObsSlot, h->stream);
    h->ring_raw[slot] = 0;
  } else {
    CK(cudaMemsetAsync(h->d_obs, 0, 8 * sizeof(double), h->stream));
    if (h->p.precision == MPCD_FP64)
      h->launches += launch_observables_f64(h->f64, h->md, h->p.bead_mass, h->d_obs, h->stream);
    else
      h->launches += launch_observables_f32(h->f32, h->md, h->p.bead_mass, h->d_obs, h->stream);
    CK(cudaMemcpyAsync(o, h->d_obs, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(o + 8, h->d_diss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(o + 9, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    h->ring_raw[slot] = 1;
  }
  if (int rc = check_launch(h, "observables")) return rc;  // no ticket for a launch that failed
  CK(cudaEventRecord(h->ring_ev[slot], h->stream));
  h->ring_t[slot] = h->globalt;
  h->obs_next = t + 1;
  *ticket = t;
  return MPCD_OK;
}

// Waits for the read-back of one ticket (not for later work on the stream) and
// converts it as mpcd_observables does.
int mpcd_observables_result(mpcd_engine* h, long long ticket, mpcd_obs* out) {
  if (!h || !out) return MPCD_EINVAL;
  if (ticket < 0 || ticket >= h->obs_next)
    return fail(h, MPCD_EINVAL, "observables ticket " + std::to_string(ticket) + " was not issued");
  if (ticket < h->obs_next - MPCD_OBS_RING)
    return fail(h, MPCD_EINVAL, "observables ticket " + std::to_string(ticket) + " was overwritten (more than " +
                                    std::to_string(MPCD_OBS_RING) + " newer tickets)");
  const int slot = (int)(ticket % MPCD_OBS_RING);
  CK(cudaEventSynchronize(h->ring_ev[slot]));
  const double* o = h->h_ring + (size_t)slot * kObsSlot;
  unsigned err_bits = 0;
  if (h->ring_raw[slot])
    std::memcpy(&err_bits, o + 9, sizeof err_bits);
  else
    err_bits = (unsigned)o[9];
  const double diss = o[8];
  const double M = o[5] > 0 ? o[5] : 1.0, N = o[4] > 0 ? o[4] : 1.0;
  out->momentum[0] = o[0] / M;
  out->momentum[1] = o[1] / M;
  out->momentum[2] = o[2] / M;
  out->n = o[4];
  out->mass = o[5];
  out->kT = o[3] / 3.0 / N;
  out->fluid_T = o[7] > 0 ? o[6] / o[7] / 3.0 : 0.0;
  out->diss_energy = diss;
  out->globalt = h->ring_t[slot];
  out->energy_fluid = 0.5 * o[6];
  if (!err_bits) return MPCD_OK;
  // the error word as it was at the ticket (a later call may have cleared it)
  const int rc = device_error(h);
  return rc ? rc : fail(h, MPCD_EDEVICE, error_text(err_bits));
}

int mpcd_observables(mpcd_engine* h, mpcd_obs* out) {
  if (!h || !out) return MPCD_EINVAL;
  long long t = 0;
  const int rc = mpcd_observables_async(h, &t);
  return rc ? rc : mpcd_observables_result(h, t, out);
}

int mpcd_timed_run(mpcd_engine* h, int nsteps, int flush_l2, double* step_ms) {
  if (!h || nsteps < 0) return MPCD_EINVAL;
  if (!h->prepared) {
    int rc = mpcd_prepare(h);
    if (rc) return rc;
  }
  const size_t kFlush = 256u << 20;
  if (flush_l2 && !h->flush_buf) CK(cudaMalloc(&h->flush_buf, kFlush));
  std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  int rc = MPCD_OK;
  for (int i = 0; i < nsteps && rc == MPCD_OK; ++i) {
    if (flush_l2) CK(cudaMemsetAsync(h->flush_buf, i & 0xff, kFlush, h->stream));
    CK(cudaEventRecord(ev[2 * i], h->stream));
    rc = mpcd_step(h, nullptr);
    CK(cudaEventRecord(ev[2 * i + 1], h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < nsteps; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    if (step_ms) step_ms[i] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  return device_error(h);
}

int mpcd_set_profiling(mpcd_engine* h, int on) {
  if (!h) return MPCD_EINVAL;
  resolve_marks(h);
  h->profiling = on != 0;
  for (int k = 0; k < 8; ++k) {
    h->prof_ms[k] = 0.0;
    h->prof_n[k] = 0;
  }
  return MPCD_OK;
}

int mpcd_kernel_time(mpcd_engine* h, int kernel, double* total_ms, long long* launches) {
  if (!h || kernel < 0 || kernel > 7) return MPCD_EINVAL;
  resolve_marks(h);
  if (total_ms) *total_ms = h->prof_ms[kernel];
  if (launches) *launches = h->prof_n[kernel];
  return MPCD_OK;
}

int mpcd_set_rigid_spheres(mpcd_engine* h, int n, const mpcd_rigid_sphere* spheres) {
  if (!h || n < 0 || n > MPCD_MAX_RIGID_SPHERES || (n > 0 && !spheres))
    return fail(h, MPCD_EINVAL, "set_rigid_spheres: bad arguments");
  std::vector<RigidSphereDev> dev(kMaxSpheres);
  for (int k = 0; k < n; ++k) {
    const mpcd_rigid_sphere& q = spheres[k];
    RigidSphereDev& d = dev[k];
    if (!(q.radius > 0.0) || !std::isfinite(q.radius) || !std::isfinite(q.mass))
      return fail(h, MPCD_EINVAL, "set_rigid_spheres: radius must be positive and finite");
    for (int j = 0; j < 3; ++j) {
      if (!std::isfinite(q.center[j]) || !std::isfinite(q.velocity[j]) || !std::isfinite(q.omega[j]))
        return fail(h, MPCD_EINVAL, "set_rigid_spheres: non-finite centre, velocity or angular velocity");
      double c = q.center[j];
      const double L = h->box.L[j];
      if (q.radius < 0.5 * L) c -= std::floor(c / L) * L;  // spheres with periodic images: into [0, L)
      if (c >= L && q.radius < 0.5 * L) c = 0.0;
      d.c[j] = c;
      d.v[j] = q.velocity[j];
      d.w[j] = q.omega[j];
    }
    d.r = q.radius;
    d.mass = q.mass;
    d.inertia = q.mass > 0.0 ? 0.4 * q.mass * q.radius * q.radius : 0.0;
  }
  if (!h->d_sph) {
    CK(dalloc(&h->d_sph, kMaxSpheres));
    CK(dalloc(&h->d_sph_acc, 6 * kMaxSpheres));
    CK(dalloc(&h->d_sph_fsum, 6 * kMaxSpheres));
  }
  CK(cudaMemcpyAsync(h->d_sph, dev.data(), kMaxSpheres * sizeof(RigidSphereDev), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemsetAsync(h->d_sph_acc, 0, 6 * kMaxSpheres * sizeof(double), h->stream));
  CK(cudaMemsetAsync(h->d_sph_fsum, 0, 6 * kMaxSpheres * sizeof(double), h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->nsph = n;
  h->sph_steps = 0;
  return MPCD_OK;
}

int mpcd_get_rigid_spheres(mpcd_engine* h, int n, mpcd_rigid_sphere* spheres, double* force_torque) {
  if (!h || n != h->nsph || (n > 0 && !spheres && !force_torque))
    return fail(h, MPCD_EINVAL, "get_rigid_spheres: n does not match the sphere count");
  if (n == 0) return MPCD_OK;
  std::vector<RigidSphereDev> dev(n);
  std::vector<double> fs(6 * (size_t)n);
  CK(cudaMemcpyAsync(dev.data(), h->d_sph, n * sizeof(RigidSphereDev), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(fs.data(), h->d_sph_fsum, 6 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < n; ++k) {
    if (spheres) {
      for (int j = 0; j < 3; ++j) {
        spheres[k].center[j] = dev[k].c[j];
        spheres[k].velocity[j] = dev[k].v[j];
        spheres[k].omega[j] = dev[k].w[j];
      }
      spheres[k].radius = dev[k].r;
      spheres[k].mass = dev[k].mass;
    }
    if (force_torque)
      for (int j = 0; j < 6; ++j) force_torque[6 * k + j] = h->sph_steps > 0 ? fs[6 * k + j] / h->sph_steps : 0.0;
  }
  return device_error(h);
}

int mpcd_rigid_sphere_count(const mpcd_engine* h) { return h ? h->nsph : 0; }

int mpcd_set_repelling(mpcd_engine* h, double eps) {
  if (!h || !std::isfinite(eps)) return fail(h, MPCD_EINVAL, "set_repelling: eps must be finite");
  int rc = pull_md(h);
  if (rc) return rc;
  h->repel = eps;
  h->md_dirty = true;
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_reset_rigid_sphere_forces(mpcd_engine* h) {
  if (!h) return MPCD_EINVAL;
  if (h->d_sph_fsum) CK(cudaMemsetAsync(h->d_sph_fsum, 0, 6 * kMaxSpheres * sizeof(double), h->stream));
  h->sph_steps = 0;
  return MPCD_OK;
}

int mpcd_collision_draws(int nc, unsigned long long seed, unsigned long long step, long n, double* gamma,
                         double* axis, int device) {
  if (nc < 2 || nc > 0xffff || n < 0 || n > 0xffffffffL || (!gamma && !axis)) return MPCD_EINVAL;
  if (n == 0) return MPCD_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MPCD_ECUDA;
  double *dg = nullptr, *da = nullptr;
  unsigned* derr = nullptr;
  int rc = MPCD_OK;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == MPCD_OK) rc = e == cudaErrorMemoryAllocation ? MPCD_ENOMEM : MPCD_ECUDA;
    return rc == MPCD_OK;
  };
  unsigned err = 0;
  if (ok(dalloc(&derr, 1)) && ok(cudaMemset(derr, 0, sizeof(unsigned))) && (!gamma || ok(dalloc(&dg, n))) &&
      (!axis || ok(dalloc(&da, 3 * n)))) {
    launch_collision_draws(nc, seed, step, n, dg, da, derr, nullptr);
    if (ok(cudaGetLastError()) && ok(cudaDeviceSynchronize()) &&
        (!gamma || ok(cudaMemcpy(gamma, dg, n * sizeof(double), cudaMemcpyDeviceToHost))) &&
        (!axis || ok(cudaMemcpy(axis, da, 3 * n * sizeof(double), cudaMemcpyDeviceToHost))))
      ok(cudaMemcpy(&err, derr, sizeof err, cudaMemcpyDeviceToHost));
  }
  cudaFree(dg);
  cudaFree(da);
  cudaFree(derr);
  if (rc == MPCD_OK && err) rc = MPCD_EDEVICE;
  return rc;
}

// ------------------------------------------------------------ snapshots ---
// A snapshot is the whole state of a handle as host bytes: a header, then the
// fluid in the engine's own layout (no conversion, so nothing is rounded),
// the beads, springs and cilia (the host copies, brought up to date first),
// the rigid spheres and the accumulators.  The cell sums are not stored: the
// first step after a restore bins the restored particles again, which gives
// the same sums up to the order of the atomic additions.
namespace {

struct SnapHeader {
  char magic[8];
  int32_t version, precision, sizes[3], nsph;
  int64_t nf, nb, nsp, ncil, nbond, steps, since_sort, sph_steps;
  double globalt, a[3], diss, tstep, ststep;
  uint64_t seed;
};
constexpr char kSnapMagic[8] = {'M', 'P', 'C', 'D', 'S', 'N', 'P', '1'};

// serialises (store = true) into, or reads (store = false) from, a byte cursor
struct SnapCursor {
  unsigned char* p;
  size_t left;
  bool ok = true;
  void io(void* data, size_t bytes, bool store) {
    if (!ok || bytes > left) {
      ok = false;
      return;
    }
    if (store)
      std::memcpy(p, data, bytes);
    else
      std::memcpy(data, p, bytes);
    p += bytes;
    left -= bytes;
  }
};

size_t fluid_bytes(const mpcd_engine* h, long n) {
  return h->p.precision == MPCD_FP64 ? (size_t)n * (4 + 4 + 6 * 8) : (size_t)n * (4 + 2 * 16);
}

size_t snapshot_bytes(const mpcd_engine* h) {
  const long nf = mpcd_fluid_count(h);
  return sizeof(SnapHeader) + fluid_bytes(h, nf) + (size_t)h->nb * (6 * 8 + 4) + h->sp_t.size() * (4 * 4 + 2 * 8) +
         h->cil.size() * sizeof(mpcd_cilium) + h->newlen.size() * 2 * 8 +
         (size_t)h->nsph * (sizeof(RigidSphereDev) + 6 * 8);
}

}  // namespace

int mpcd_snapshot_size(mpcd_engine* h, long long* bytes) {
  if (!h || !bytes) return MPCD_EINVAL;
  *bytes = (long long)snapshot_bytes(h);
  return MPCD_OK;
}

int mpcd_snapshot(mpcd_engine* h, void* buf, long long bytes) {
  if (!h || !buf) return MPCD_EINVAL;
  int rc = pull_md(h);
  if (rc) return rc;
  if (bytes < (long long)snapshot_bytes(h)) return fail(h, MPCD_EINVAL, "snapshot: buffer smaller than mpcd_snapshot_size");
  SnapHeader hd{};
  std::memcpy(hd.magic, kSnapMagic, 8);
  hd.version = 1;
  hd.precision = h->p.precision;
  for (int q = 0; q < 3; ++q) hd.sizes[q] = h->p.sizes[q];
  hd.nsph = h->nsph;
  hd.nf = mpcd_fluid_count(h);
  hd.nb = h->nb;
  hd.nsp = (int64_t)h->sp_t.size();
  hd.ncil = (int64_t)h->cil.size();
  hd.nbond = (int64_t)h->newlen.size();
  hd.steps = h->steps;
  hd.since_sort = h->since_sort;
  hd.sph_steps = h->sph_steps;
  hd.globalt = h->globalt;
  std::memcpy(hd.a, h->a, sizeof hd.a);
  hd.tstep = h->p.tstep;
  hd.ststep = h->p.ststep;
  hd.seed = h->p.seed;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&hd.diss, h->d_diss, sizeof(double), cudaMemcpyDeviceToHost));
  SnapCursor c{static_cast<unsigned char*>(buf), (size_t)bytes};
  c.io(&hd, sizeof hd, true);
  const size_t n = (size_t)hd.nf;
  auto dev = [&](const void* d, size_t nbytes) {  // device array -> cursor
    if (!c.ok || nbytes > c.left) {
      c.ok = false;
      return cudaSuccess;
    }
    cudaError_t e = nbytes ? cudaMemcpy(c.p, d, nbytes, cudaMemcpyDeviceToHost) : cudaSuccess;
    c.p += nbytes;
    c.left -= nbytes;
    return e;
  };
  if (h->p.precision == MPCD_FP64) {
    const FluidF64& f = h->f64;
    CK(dev(f.id, 4 * n));
    CK(dev(f.cell, 4 * n));
    for (double* a : {f.ox, f.oy, f.oz, f.vx, f.vy, f.vz}) CK(dev(a, 8 * n));
  } else {
    CK(dev(h->f32.id, 4 * n));
    CK(dev(h->f32.pos, 16 * n));
    CK(dev(h->f32.vel, 16 * n));
  }
  c.io(h->bpos.data(), 8 * h->bpos.size(), true);
  c.io(h->bvel.data(), 8 * h->bvel.size(), true);
  c.io(h->bmoves.data(), 4 * h->bmoves.size(), true);
  for (std::vector<int>* v : {&h->sp_t, &h->sp_o, &h->sp_k, &h->sp_r}) c.io(v->data(), 4 * v->size(), true);
  c.io(h->sp_rest.data(), 8 * h->sp_rest.size(), true);
  c.io(h->sp_kk.data(), 8 * h->sp_kk.size(), true);
  c.io(h->cil.data(), sizeof(mpcd_cilium) * h->cil.size(), true);
  c.io(h->newlen.data(), 8 * h->newlen.size(), true);
  c.io(h->oldlen.data(), 8 * h->oldlen.size(), true);
  if (h->nsph) {
    CK(dev(h->d_sph, sizeof(RigidSphereDev) * h->nsph));
    CK(dev(h->d_sph_fsum, 6 * 8 * (size_t)h->nsph));
  }
  if (!c.ok) return fail(h, MPCD_EINVAL, "snapshot: buffer too small");
  return device_error(h);
}

int mpcd_restore(mpcd_engine* h, const void* buf, long long bytes) {
  if (!h || !buf || bytes < (long long)sizeof(SnapHeader)) return fail(h, MPCD_EINVAL, "restore: bad arguments");
  SnapCursor c{const_cast<unsigned char*>(static_cast<const unsigned char*>(buf)), (size_t)bytes};
  SnapHeader hd;
  c.io(&hd, sizeof hd, false);
  if (std::memcmp(hd.magic, kSnapMagic, 8) != 0 || hd.version != 1)
    return fail(h, MPCD_EINVAL, "restore: not a snapshot of this library");
  if (hd.precision != h->p.precision || hd.sizes[0] != h->p.sizes[0] || hd.sizes[1] != h->p.sizes[1] ||
      hd.sizes[2] != h->p.sizes[2] || hd.tstep != h->p.tstep || hd.ststep != h->p.ststep)
    return fail(h, MPCD_EINVAL, "restore: the snapshot's box, precision or time steps differ from the handle's");
  if (hd.nf < 0 || hd.nb < 0 || hd.nsp < 0 || hd.ncil < 0 || hd.nbond < 0 || hd.nsph < 0 ||
      hd.nsph > kMaxSpheres || hd.nf > 0x7fffffffL)
    return fail(h, MPCD_EINVAL, "restore: corrupt header");
  const size_t n = (size_t)hd.nf;
  const size_t need = sizeof(SnapHeader) + (h->p.precision == MPCD_FP64 ? n * 56 : n * 36) + (size_t)hd.nb * 52 +
                      (size_t)hd.nsp * 32 + (size_t)hd.ncil * sizeof(mpcd_cilium) + (size_t)hd.nbond * 16 +
                      (size_t)hd.nsph * (sizeof(RigidSphereDev) + 48);
  if ((size_t)bytes < need) return fail(h, MPCD_EINVAL, "restore: snapshot truncated");
  int rc = alloc_fluid(h, (long)n);
  if (rc) return rc;
  auto dev = [&](void* d, size_t nbytes) {  // cursor -> device array
    cudaError_t e = nbytes ? cudaMemcpy(d, c.p, nbytes, cudaMemcpyHostToDevice) : cudaSuccess;
    c.p += nbytes;
    c.left -= nbytes;
    return e;
  };
  if (h->p.precision == MPCD_FP64) {
    FluidF64& f = h->f64;
    CK(dev(f.id, 4 * n));
    CK(dev(f.cell, 4 * n));
    for (double* a : {f.ox, f.oy, f.oz, f.vx, f.vy, f.vz}) CK(dev(a, 8 * n));
  } else {
    CK(dev(h->f32.id, 4 * n));
    CK(dev(h->f32.pos, 16 * n));
    CK(dev(h->f32.vel, 16 * n));
  }
  h->nb = (long)hd.nb;
  h->bpos.resize(3 * hd.nb);
  h->bvel.resize(3 * hd.nb);
  h->bmoves.resize(hd.nb);
  c.io(h->bpos.data(), 8 * h->bpos.size(), false);
  c.io(h->bvel.data(), 8 * h->bvel.size(), false);
  c.io(h->bmoves.data(), 4 * h->bmoves.size(), false);
  for (std::vector<int>* v : {&h->sp_t, &h->sp_o, &h->sp_k, &h->sp_r}) {
    v->resize(hd.nsp);
    c.io(v->data(), 4 * v->size(), false);
  }
  h->sp_rest.resize(hd.nsp);
  h->sp_kk.resize(hd.nsp);
  c.io(h->sp_rest.data(), 8 * h->sp_rest.size(), false);
  c.io(h->sp_kk.data(), 8 * h->sp_kk.size(), false);
  h->cil.resize(hd.ncil);
  c.io(h->cil.data(), sizeof(mpcd_cilium) * h->cil.size(), false);
  h->newlen.resize(hd.nbond);
  h->oldlen.resize(hd.nbond);
  c.io(h->newlen.data(), 8 * h->newlen.size(), false);
  c.io(h->oldlen.data(), 8 * h->oldlen.size(), false);
  if (hd.nsph) {
    if (!h->d_sph) {
      CK(dalloc(&h->d_sph, kMaxSpheres));
      CK(dalloc(&h->d_sph_acc, 6 * kMaxSpheres));
      CK(dalloc(&h->d_sph_fsum, 6 * kMaxSpheres));
    }
    CK(dev(h->d_sph, sizeof(RigidSphereDev) * hd.nsph));
    CK(dev(h->d_sph_fsum, 48 * (size_t)hd.nsph));
    CK(cudaMemset(h->d_sph_acc, 0, 6 * kMaxSpheres * sizeof(double)));
  }
  h->nsph = hd.nsph;
  h->sph_steps = hd.sph_steps;
  if (!c.ok) return fail(h, MPCD_EINVAL, "restore: snapshot truncated");
  CK(cudaMemcpy(h->d_diss, &hd.diss, sizeof(double), cudaMemcpyHostToDevice));
  h->steps = (long)hd.steps;
  h->since_sort = (long)hd.since_sort;
  h->globalt = hd.globalt;
  std::memcpy(h->a, hd.a, sizeof h->a);
  h->p.seed = hd.seed;
  h->md_dirty = true;
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_md_layout(mpcd_engine* h, int* info) {
  if (!h || !info) return MPCD_EINVAL;
  if (h->md_dirty) {
    const int rc = build_md(h);
    if (rc) return rc;
  }
  const MDState& m = h->md;
  info[0] = m.cluster;
  info[1] = m.cluster ? m.cl_lanes : (m.pair ? md_pair_threads(m.tile) / m.tile : (m.df ? md_df_lanes(m.tile) : 4));
  info[2] = m.tile;
  info[3] = m.ntiles;
  info[4] = m.nslots;
  info[5] = (int)h->md_nsp;
  info[6] = m.hmax;
  info[7] = m.pair ? 3 + m.pair : (m.df ? m.df + 1 : m.split);
  return MPCD_OK;
}

}  // extern "C"
