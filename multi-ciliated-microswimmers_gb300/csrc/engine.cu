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
#include "engine_internal.h"


using namespace mpcd;

struct mpcd_engine {
  mpcd_params p{};
  Box box{};
  long ncell = 0;
  int nsub = 0;
  cudaStream_t stream = nullptr;
  std::string error;
  long long launches = 0;

  unsigned* d_err = nullptr;
  double* d_diss = nullptr;
  double* d_obs = nullptr;
  unsigned* d_bar = nullptr;

  FluidF64 f64, f64tmp;
  FluidF32 f32, f32tmp;
  CellsF64 c64;
  CellsF32 c32;
  uint32_t *d_count = nullptr, *d_start = nullptr, *d_rank = nullptr, *d_blocksums = nullptr;
  double* d_inj_gamma = nullptr;
  double* d_inj_axis = nullptr;

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
  GridBarrier bar = m.bar;
  m = MDState{};
  m.bar = bar;
}

int alloc_fluid(mpcd_engine* h, long n) {
  if (h->p.precision == MPCD_FP64) {
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

// wrap an unwrapped coordinate into cell index + offset in [0,1)
inline void wrap_coord(double x, int L, int& i, double& o) {
  double xw = x - std::floor(x / L) * L;
  if (xw >= L) xw -= L;
  if (xw < 0) xw += L;
  double fi = std::floor(xw);
  i = (int)fi;
  o = xw - fi;
  if (i >= L) {
    i -= L;
  }
  if (o >= 1.0) {
    o = 0.0;
    i = (i + 1) % L;
  }
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
  return s;
}

int check_launch(mpcd_engine* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return MPCD_OK;
}

// Build the MD device layout: tiles of `tile` slots, one CTA each.  A bead
// owns 1 + h consecutive slots (h helper slots when its spring list is longer
// than kChunk, each helper summing one chunk).  Every cilium occupies
// contiguous slots of one tile; the other beads fill the remaining space.
int build_md(mpcd_engine* h, bool allow_cluster = true, bool no_react = false) {
  // springs per helper slot: the longest serial spring chain of any thread.
  // Odd, so that the helper slots' spring lists start in different
  // shared-memory banks.
  int kChunk = 31;
  if (const char* env = std::getenv("MPCD_MD_CHUNK")) kChunk = std::max(2, std::min(256, std::atoi(env)));
  free_md(h->md);
  MDState& m = h->md;
  if (h->nb == 0) {
    h->md_dirty = false;
    return MPCD_OK;
  }
  const long nb = h->nb;
  const long nsp = (long)h->sp_t.size();
  std::vector<int> nspr(nb, 0);
  for (long i = 0; i < nsp; ++i) {
    if (h->sp_t[i] < 0 || h->sp_t[i] >= nb || h->sp_o[i] < 0 || h->sp_o[i] >= nb)
      return fail(h, MPCD_EINVAL, "spring bead index out of range");
    nspr[h->sp_t[i]]++;
  }
  std::vector<int> width(nb);
  for (long b = 0; b < nb; ++b) width[b] = 1 + (nspr[b] > kChunk ? (nspr[b] + kChunk - 1) / kChunk - 1 : 0);
  std::vector<int> owner(nb, -1);  // cilium owning the bead
  for (size_t c = 0; c < h->cil.size(); ++c)
    for (int k = 0; k < 3 * h->cil[c].rodlength; ++k) {
      const long b = (long)h->cil[c].bead0 + k;
      if (b < 0 || b >= nb) return fail(h, MPCD_EINVAL, "cilium bead range outside the bead array");
      if (owner[b] >= 0) return fail(h, MPCD_EINVAL, "beads shared by two cilia");
      owner[b] = (int)c;
    }
  // Hubs (a sphere's centre: one spring to every surface bead).  When every
  // spring of a hub has an exact reverse partner inside the same run of
  // non-cilium beads, the cluster layout drops the hub's own list and sums the
  // partners' forces, negated, over the tile (react[j] marks the partners).
  std::vector<int> run_id(nb, -1);
  for (long b = 0, r = 0; b < nb; ++b)
    if (owner[b] < 0) run_id[b] = (b > 0 && owner[b - 1] < 0) ? run_id[b - 1] : (int)r++;
  std::vector<int> bstart(nb + 1, 0), blist(nsp);
  for (long i = 0; i < nsp; ++i) bstart[h->sp_t[i] + 1]++;
  for (long b = 0; b < nb; ++b) bstart[b + 1] += bstart[b];
  {
    std::vector<int> fillp(bstart.begin(), bstart.end() - 1);
    for (long i = 0; i < nsp; ++i) blist[fillp[h->sp_t[i]]++] = (int)i;
  }
  std::vector<char> hub(nb, 0), react(nsp, 0), dropped(nsp, 0);
  if (!no_react) {
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0 || nspr[b] <= kChunk) continue;
      std::vector<int> partners;
      bool ok = true;
      for (int q = bstart[b]; q < bstart[b + 1] && ok; ++q) {
        const int i = blist[q];
        const int o = h->sp_o[i];
        if (h->sp_k[i] != MPCD_SPRING_CONST || run_id[o] != run_id[b] || o == b) {
          ok = false;
          break;
        }
        int found = -1;
        for (int r = bstart[o]; r < bstart[o + 1]; ++r) {
          const int j = blist[r];
          if (h->sp_o[j] == b && h->sp_k[j] == MPCD_SPRING_CONST && h->sp_rest[j] == h->sp_rest[i] &&
              h->sp_kk[j] == h->sp_kk[i] && !react[j]) {
            found = j;
            break;
          }
        }
        if (found < 0) ok = false;
        else partners.push_back(found);
      }
      if (!ok) continue;
      hub[b] = 1;
      for (int j : partners) react[j] = 1;
      for (int q = bstart[b]; q < bstart[b + 1]; ++q) dropped[blist[q]] = 1;
    }
  }
  // every bead of a cilium owns the same number of slots (the kernels address
  // a cilium's beads as slot0 + stride * (filament * rodlength + bead))
  auto pad_cilia = [&]() {
    for (size_t c = 0; c < h->cil.size(); ++c) {
      int wmax = 1;
      for (int k = 0; k < 3 * h->cil[c].rodlength; ++k) wmax = std::max(wmax, width[h->cil[c].bead0 + k]);
      for (int k = 0; k < 3 * h->cil[c].rodlength; ++k) width[h->cil[c].bead0 + k] = wmax;
    }
  };
  pad_cilia();
  std::vector<int> width_grid = width;
  int cl_chunk = kChunk;  // springs per slot of the chosen layout
  int maxw = 0;
  for (size_t c = 0; c < h->cil.size(); ++c) {
    const mpcd_cilium& cl = h->cil[c];
    int w = 0;
    for (int k = 0; k < 3 * cl.rodlength; ++k) w += width[(long)cl.bead0 + k];
    maxw = std::max(maxw, w);
  }
  for (long b = 0; b < nb; ++b)
    if (owner[b] < 0) maxw = std::max(maxw, width[b]);
  // Pack: cilia first (each contiguous in one tile), then the other beads in
  // the remaining space.  Returns the number of tiles.
  std::vector<int> fill, slot_of(nb, -1), cil_tile(h->cil.size());
  auto pack = [&](int tile) {
    fill.clear();
    std::fill(slot_of.begin(), slot_of.end(), -1);
    for (size_t c = 0; c < h->cil.size(); ++c) {
      const mpcd_cilium& cl = h->cil[c];
      int w = 0;
      for (int k = 0; k < 3 * cl.rodlength; ++k) w += width[cl.bead0 + k];
      if (fill.empty() || fill.back() + w > tile) fill.push_back(0);
      const int t = (int)fill.size() - 1;
      cil_tile[c] = t;
      for (int k = 0; k < 3 * cl.rodlength; ++k) {
        slot_of[cl.bead0 + k] = t * tile + fill[t];
        fill[t] += width[cl.bead0 + k];
      }
    }
    size_t tcur = 0;
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0) continue;
      while (tcur < fill.size() && fill[tcur] + width[b] > tile) ++tcur;
      if (tcur == fill.size()) fill.push_back(0);
      slot_of[b] = (int)tcur * tile + fill[tcur];
      fill[tcur] += width[b];
    }
    return (int)fill.size();
  };
  m.split = h->p.md_split < 0 ? (h->p.precision == MPCD_FP32 ? 1 : 0) : (h->p.md_split ? 1 : 0);
  // Cluster packing (split arithmetic): runs of consecutive non-cilium beads
  // wider than 64 slots (a sphere, whose centre bead reaches every surface
  // bead) each stay whole in one tile; cilia follow in order (next fit, so a
  // tile's cilia have contiguous bond tables); the remaining beads fill gaps.
  bool keep_hubs_whole = false;  // one-lane layout: hub runs stay in one tile (reactions)
  auto pack_cluster = [&](int tile) {
    fill.clear();
    std::fill(slot_of.begin(), slot_of.end(), -1);
    std::vector<std::pair<long, long>> runs;  // [begin, end) of non-cilium beads
    for (long b = 0; b < nb;) {
      if (owner[b] >= 0) {
        ++b;
        continue;
      }
      long e = b;
      while (e < nb && owner[e] < 0) ++e;
      runs.push_back({b, e});
      b = e;
    }
    std::vector<char> placed(nb, 0);
    for (auto& r : runs) {
      long w = 0;
      bool has_hub = false;
      for (long b = r.first; b < r.second; ++b) {
        w += width[b];
        has_hub = has_hub || hub[b];
      }
      if (has_hub && keep_hubs_whole && w > tile) return 1 << 20;  // a hub's run must stay whole
      if (w <= 64 || w > tile) continue;
      fill.push_back(0);
      const int t = (int)fill.size() - 1;
      for (long b = r.first; b < r.second; ++b) {
        slot_of[b] = t * tile + fill[t];
        fill[t] += width[b];
        placed[b] = 1;
      }
    }
    const int first_cil_tile = (int)fill.size();
    for (size_t c = 0; c < h->cil.size(); ++c) {
      const mpcd_cilium& cl = h->cil[c];
      int w = 0;
      for (int k = 0; k < 3 * cl.rodlength; ++k) w += width[cl.bead0 + k];
      if ((int)fill.size() == first_cil_tile || fill.back() + w > tile) fill.push_back(0);
      const int t = (int)fill.size() - 1;
      cil_tile[c] = t;
      for (int k = 0; k < 3 * cl.rodlength; ++k) {
        slot_of[cl.bead0 + k] = t * tile + fill[t];
        fill[t] += width[cl.bead0 + k];
      }
    }
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0 || placed[b]) continue;
      size_t t = 0;
      while (t < fill.size() && fill[t] + width[b] > tile) ++t;
      if (t == fill.size()) fill.push_back(0);
      slot_of[b] = (int)t * tile + fill[t];
      fill[t] += width[b];
    }
    return (int)fill.size();
  };
  int tile = 0;
  m.cluster = 0;
  if (m.split && allow_cluster) {
    int lanes_hi = 2, lanes_lo = 1;
    if (const char* env = std::getenv("MPCD_MD_LANES")) lanes_hi = lanes_lo = std::max(1, std::min(2, std::atoi(env)));
    for (int lanes = lanes_hi; lanes >= lanes_lo && !m.cluster; --lanes) {
      // one lane per slot: short chunks (two slots per cilium bead) keep the
      // serial spring chains short; hubs take their force from reactions
      const int chunk = lanes == 2 ? kChunk : std::min(kChunk, 11);
      keep_hubs_whole = lanes == 1;
      for (long b = 0; b < nb; ++b)
        width[b] = (hub[b] && keep_hubs_whole) ? 1
                                               : 1 + (nspr[b] > chunk ? (nspr[b] + chunk - 1) / chunk - 1 : 0);
      cl_chunk = chunk;
      pad_cilia();
      int maxw_cl = 0;
      for (size_t c = 0; c < h->cil.size(); ++c) {
        int w = 0;
        for (int k = 0; k < 3 * h->cil[c].rodlength; ++k) w += width[h->cil[c].bead0 + k];
        maxw_cl = std::max(maxw_cl, w);
      }
      for (long b = 0; b < nb; ++b)
        if (owner[b] < 0) maxw_cl = std::max(maxw_cl, width[b]);
      maxw = maxw_cl;
      const int tmax = 1024 / lanes;
      for (int t = std::max(32, ((maxw + 31) / 32) * 32); t <= tmax; t += 32)
        if (pack_cluster(t) <= 16) {
          tile = t;
          m.cluster = 1;
          m.cl_lanes = lanes;
          break;
        }
    }
  }
  if (m.cluster && !keep_hubs_whole) {  // two-lane layout: hubs keep their own lists and helpers
    std::fill(hub.begin(), hub.end(), 0);
    std::fill(react.begin(), react.end(), 0);
    std::fill(dropped.begin(), dropped.end(), 0);
  }
  if (!m.cluster) {
    width = width_grid;
    cl_chunk = kChunk;
    std::fill(hub.begin(), hub.end(), 0);
    std::fill(react.begin(), react.end(), 0);
    std::fill(dropped.begin(), dropped.end(), 0);
    maxw = 0;
    for (size_t c = 0; c < h->cil.size(); ++c) {
      int w = 0;
      for (int k = 0; k < 3 * h->cil[c].rodlength; ++k) w += width[h->cil[c].bead0 + k];
      maxw = std::max(maxw, w);
    }
    for (long b = 0; b < nb; ++b)
      if (owner[b] < 0) maxw = std::max(maxw, width[b]);
    tile = std::max(32, ((maxw + 15) / 16) * 16);
    if (tile > 1024) return fail(h, MPCD_EINVAL, "an MD group needs more than 1024 slots");
    pack(tile);
  }
  // a hub and all its partners must share one tile, one hub per tile
  std::vector<int> tile_react;
  {
    const int nt = (int)fill.size();
    tile_react.assign(nt, -1);
    bool bad = false;
    for (long b = 0; b < nb && !bad; ++b) {
      if (!hub[b]) continue;
      const int t = slot_of[b] / tile;
      if (tile_react[t] >= 0) bad = true;
      tile_react[t] = slot_of[b] - t * tile;
    }
    for (long i = 0; i < nsp && !bad; ++i)
      if (react[i] && slot_of[h->sp_t[i]] / tile != slot_of[h->sp_o[i]] / tile) bad = true;
    if (bad) return build_md(h, allow_cluster, true);
  }
  m.tile = tile;
  m.ntiles = (int)fill.size();
  m.nslots = m.ntiles * tile;
  const int ns = m.nslots;
  std::vector<double> X(ns, 0.0), Y(ns, 0.0), Z(ns, 0.0), VX(ns, 0.0), VY(ns, 0.0), VZ(ns, 0.0);
  std::vector<int> mv(ns, -1), prim(ns, 0), nhelp(ns, 0), thelp(m.ntiles, 0);
  for (long b = 0; b < nb; ++b) {
    const int s = slot_of[b];
    X[s] = h->bpos[3 * b];
    Y[s] = h->bpos[3 * b + 1];
    Z[s] = h->bpos[3 * b + 2];
    VX[s] = h->bvel[3 * b];
    VY[s] = h->bvel[3 * b + 1];
    VZ[s] = h->bvel[3 * b + 2];
    mv[s] = h->bmoves[b] ? 1 : 0;
    prim[s] = s;
    nhelp[s] = width[b] - 1;
    for (int k = 1; k < width[b]; ++k) {
      mv[s + k] = 2;
      prim[s + k] = s;
      X[s + k] = X[s];
      Y[s + k] = Y[s];
      Z[s + k] = Z[s];
    }
    if (width[b] > 1) thelp[s / tile] = 1;
  }
  // springs: CSR by slot; a bead's list (in input order) is cut into chunks of
  // kChunk over its primary and helper slots
  std::vector<int> start(ns + 1, 0);
  std::vector<int> seen(nb, 0);
  std::vector<int> sslot(nsp);
  for (long i = 0; i < nsp; ++i) {
    if (dropped[i]) {
      sslot[i] = -1;
      continue;
    }
    const int b = h->sp_t[i];
    const int chunk = width[b] > 1 ? seen[b] / cl_chunk : 0;
    seen[b]++;
    sslot[i] = slot_of[b] + chunk;
    start[sslot[i] + 1]++;
  }
  for (int s = 0; s < ns; ++s) start[s + 1] += start[s];
  std::vector<int> pos(start.begin(), start.end() - 1);
  const long nspk = start[ns];  // springs kept
  std::vector<int> so(nspk), sk(nspk), sr(nspk);
  std::vector<double> srest(nspk), sm2k(nspk);
  for (long i = 0; i < nsp; ++i) {
    if (sslot[i] < 0) continue;
    const int d = pos[sslot[i]]++;
    so[d] = slot_of[h->sp_o[i]];
    sk[d] = h->sp_k[i] | (react[i] ? kSpringReact : 0);
    sr[d] = h->sp_r[i];
    srest[d] = h->sp_rest[i];
    sm2k[d] = -2.0 * h->sp_kk[i];
  }
  // halos: per tile the distinct slots of other tiles its springs reach, and
  // every spring's other bead as an index into the tile's staged positions
  std::vector<int> sl(nspk), halo, hstart(m.ntiles + 1, 0);
  int hmax = 0;
  for (int t = 0; t < m.ntiles; ++t) {
    const int b0 = t * tile, b1 = b0 + tile;
    std::vector<int> ext;
    for (int s2 = start[b0]; s2 < start[b1]; ++s2)
      if (so[s2] < b0 || so[s2] >= b1) ext.push_back(so[s2]);
    std::sort(ext.begin(), ext.end());
    ext.erase(std::unique(ext.begin(), ext.end()), ext.end());
    for (int s2 = start[b0]; s2 < start[b1]; ++s2) {
      if (so[s2] >= b0 && so[s2] < b1)
        sl[s2] = so[s2] - b0;
      else
        sl[s2] = tile + (int)(std::lower_bound(ext.begin(), ext.end(), so[s2]) - ext.begin());
    }
    hstart[t + 1] = hstart[t] + (int)ext.size();
    halo.insert(halo.end(), ext.begin(), ext.end());
    hmax = std::max(hmax, (int)ext.size());
  }
  m.hmax = hmax;
  if (m.cluster) {
    // per-tile maxima for the cluster kernel's shared-memory layout
    m.cl_nsp_max = 0;
    m.cl_nbond_max = 0;
    std::vector<int> tb(m.ntiles, 0);
    for (size_t c = 0; c < h->cil.size(); ++c) tb[cil_tile[c]] += h->cil[c].rodlength;
    for (int t = 0; t < m.ntiles; ++t) {
      m.cl_nsp_max = std::max(m.cl_nsp_max, start[(t + 1) * tile] - start[t * tile]);
      m.cl_nbond_max = std::max(m.cl_nbond_max, tb[t]);
    }
    if (!md_cluster_feasible(m)) return build_md(h, false);  // grid layout instead
  } else {
    const int cap = md_max_coresident_blocks(m, h->p.precision == MPCD_FP32 ? 1 : 0);
    if (m.ntiles > cap) return fail(h, MPCD_EINVAL, "MD tiles exceed the co-resident CTA limit of the device");
  }
  // cilia
  std::vector<CiliumDev> cd(h->cil.size());
  std::vector<double> mid(h->cil.size()), ts(h->cil.size());
  std::vector<int> tcil(m.ntiles + 1, 0);
  for (size_t c = 0; c < h->cil.size(); ++c) {
    const mpcd_cilium& cl = h->cil[c];
    CiliumDev& d = cd[c];
    d.stride = width[cl.bead0];
    d.kind = cl.kind;
    d.len = cl.rodlength;
    d.num_anker = cl.num_anker;
    d.slot0 = slot_of[cl.bead0];
    d.bond_base = cl.bond_base;
    d.beatstrength = cl.beatstrength;
    d.bending = cl.bending;
    d.max_bend = cl.max_bend;
    d.m_speed = cl.m_speed;
    d.power_dur = cl.power_stroke_duration;
    d.recovery_dur = cl.recovery_stroke_duration;
    d.start = cl.start;
    mid[c] = cl.midpnt;
    ts[c] = cl.tstroke;
    tcil[cil_tile[c] + 1]++;
  }
  for (int t = 0; t < m.ntiles; ++t) tcil[t + 1] += tcil[t];
  const size_t nbond = h->newlen.size();
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
  CK(dalloc(&m.halo, halo.size()));
  CK(dalloc(&m.halo_start, m.ntiles + 1));
  CK(dalloc(&m.diag, nbond));
  CK(dalloc(&m.sp_kind, nspk));
  CK(dalloc(&m.sp_ref, nspk));
  CK(dalloc(&m.sp_rest, nspk));
  CK(dalloc(&m.sp_m2k, nspk));
  CK(dalloc(&m.tile_react, m.ntiles));
  m.ncil = (int)h->cil.size();
  CK(dalloc(&m.cil, cd.size()));
  CK(dalloc(&m.midpnt, cd.size()));
  CK(dalloc(&m.tstroke, cd.size()));
  CK(dalloc(&m.newlen, nbond));
  CK(dalloc(&m.oldlen, nbond));
  CK(dalloc(&m.tile_cil, m.ntiles + 1));
  auto up = [&](void* d, const void* src, size_t bytes) { return cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice); };
  for (int b = 0; b < 2; ++b) {
    CK(up(m.x[b], X.data(), ns * 8));
    CK(up(m.y[b], Y.data(), ns * 8));
    CK(up(m.z[b], Z.data(), ns * 8));
  }
  CK(up(m.vx, VX.data(), ns * 8));
  CK(up(m.vy, VY.data(), ns * 8));
  CK(up(m.vz, VZ.data(), ns * 8));
  CK(up(m.moves, mv.data(), ns * 4));
  CK(up(m.prim, prim.data(), ns * 4));
  CK(up(m.nhelp, nhelp.data(), ns * 4));
  CK(up(m.tile_help, thelp.data(), m.ntiles * 4));
  CK(up(m.sp_start, start.data(), (ns + 1) * 4));
  if (nspk) {
    CK(up(m.sp_other, so.data(), nspk * 4));
    CK(up(m.sp_local, sl.data(), nspk * 4));
    CK(up(m.sp_kind, sk.data(), nspk * 4));
    CK(up(m.sp_ref, sr.data(), nspk * 4));
    CK(up(m.sp_rest, srest.data(), nspk * 8));
    CK(up(m.sp_m2k, sm2k.data(), nspk * 8));
  }
  CK(up(m.tile_react, tile_react.data(), m.ntiles * 4));
  if (!cd.empty()) {
    CK(up(m.cil, cd.data(), cd.size() * sizeof(CiliumDev)));
    CK(up(m.midpnt, mid.data(), cd.size() * 8));
    CK(up(m.tstroke, ts.data(), cd.size() * 8));
  }
  if (nbond) {
    std::vector<double> dg(nbond);
    for (size_t k = 0; k < nbond; ++k) dg[k] = std::sqrt(0.5 * 0.5 + 0.5 * h->newlen[k]);
    CK(up(m.newlen, h->newlen.data(), nbond * 8));
    CK(up(m.oldlen, h->oldlen.data(), nbond * 8));
    CK(up(m.diag, dg.data(), nbond * 8));
  }
  if (!halo.empty()) CK(up(m.halo, halo.data(), halo.size() * 4));
  CK(up(m.halo_start, hstart.data(), (m.ntiles + 1) * 4));
  CK(up(m.tile_cil, tcil.data(), (m.ntiles + 1) * 4));
  m.bar.count = h->d_bar;
  m.bar.gen = h->d_bar + 1;
  h->slot_of = slot_of;
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

int device_error(mpcd_engine* h) {
  unsigned e = 0;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&e, h->d_err, sizeof e, cudaMemcpyDeviceToHost));
  if (e == 0) return MPCD_OK;
  std::string msg = "device check failed:";
  if (e & kErrGammaMissing) msg += " injected gamma missing for a thermostatted cell;";
  if (e & kErrGammaLoop) msg += " Gamma sampler exceeded its iteration cap;";
  if (e & kErrBarrier) msg += " MD grid barrier timed out;";
  if (e & kErrCellRange) msg += " non-finite or out-of-range coordinate (unstable MD step?);";
  if (e & kErrCellOverflow) msg += " cell occupancy overflow;";
  cudaMemset(h->d_err, 0, sizeof(unsigned));
  return fail(h, MPCD_EDEVICE, msg);
}

// brackets one launch with events when profiling is on
struct ProfScope {
  mpcd_engine* h;
  int kernel;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(mpcd_engine* hh, int k) : h(hh), kernel(k) {
    if (h->profiling) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, h->stream);
    }
  }
  ~ProfScope() {
    if (h->profiling) {
      cudaEventRecord(b, h->stream);
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
  if (h->p.sort_interval <= 0) h->p.sort_interval = 25;
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
  if ((e = dalloc(&h->d_err, 1)) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_diss, 1)) != cudaSuccess) return bail(e, "alloc");
  if ((e = dalloc(&h->d_obs, 16)) != cudaSuccess) return bail(e, "alloc");
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
    if ((e = dalloc(&h->c32.par, 3 * nc)) != cudaSuccess) return bail(e, "alloc cells");
    cudaMemset(h->c32.sum, 0, nc * sizeof(float4));
    cudaMemset(h->c32.cnt, 0, nc * sizeof(uint32_t));
  }
  if ((e = dalloc(&h->d_count, nc)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&h->d_start, nc)) != cudaSuccess) return bail(e, "alloc sort");
  if ((e = dalloc(&h->d_blocksums, nc / 1024 + 2)) != cudaSuccess) return bail(e, "alloc sort");
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
  free_md(h->md);
  cudaFree(h->d_err);
  cudaFree(h->d_diss);
  cudaFree(h->d_obs);
  cudaFree(h->d_bar);
  cudaFree(h->flush_buf);
  for (auto& m : h->marks) {
    cudaEventDestroy(m.a);
    cudaEventDestroy(m.b);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
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

int mpcd_set_fluid(mpcd_engine* h, long n, const double* pos, const double* vel) {
  if (!h || n < 0 || (n > 0 && (!pos || !vel))) return fail(h, MPCD_EINVAL, "set_fluid: bad arguments");
  if (n > 0x7fffffffL) return fail(h, MPCD_EINVAL, "set_fluid: more than 2^31 - 1 particles");
  for (long i = 0; i < 3 * n; ++i)
    if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || std::fabs(pos[i]) > 1e12)
      return fail(h, MPCD_EINVAL, "set_fluid: non-finite or out-of-range position or velocity");
  int rc = alloc_fluid(h, n);
  if (rc) return rc;
  const int* L = h->box.L;
  if (h->p.precision == MPCD_FP64) {
    std::vector<uint32_t> cell(n);
    std::vector<double> o[3], v[3];
    for (int q = 0; q < 3; ++q) {
      o[q].resize(n);
      v[q].resize(n);
    }
    for (long i = 0; i < n; ++i) {
      int c[3];
      for (int q = 0; q < 3; ++q) {
        wrap_coord(pos[3 * i + q], L[q], c[q], o[q][i]);
        v[q][i] = vel[3 * i + q];
      }
      cell[i] = pack_cell(c[0], c[1], c[2]);
    }
    std::vector<uint32_t> ids(n);
    for (long i = 0; i < n; ++i) ids[i] = (uint32_t)i;
    CK(cudaMemcpy(h->f64.id, ids.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.cell, cell.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.ox, o[0].data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.oy, o[1].data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.oz, o[2].data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.vx, v[0].data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.vy, v[1].data(), n * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f64.vz, v[2].data(), n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float4> P(n), V(n);
    for (long i = 0; i < n; ++i) {
      int c[3];
      double o[3];
      for (int q = 0; q < 3; ++q) wrap_coord(pos[3 * i + q], L[q], c[q], o[q]);
      float f[3];
      for (int q = 0; q < 3; ++q) {
        f[q] = (float)o[q];
        if (f[q] >= 1.0f) {  // rounding up to 1: move to the next cell
          f[q] = 0.0f;
          c[q] = (c[q] + 1) % L[q];
        }
      }
      P[i] = make_float4(f[0], f[1], f[2], bits_to_float(pack_cell(c[0], c[1], c[2])));
      V[i] = make_float4((float)vel[3 * i], (float)vel[3 * i + 1], (float)vel[3 * i + 2], 0.0f);
    }
    std::vector<uint32_t> ids(n);
    for (long i = 0; i < n; ++i) ids[i] = (uint32_t)i;
    CK(cudaMemcpy(h->f32.id, ids.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f32.pos, P.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->f32.vel, V.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  }
  h->prepared = false;
  return MPCD_OK;
}

int mpcd_get_fluid(mpcd_engine* h, long n, double* pos, double* vel) {
  if (!h) return MPCD_EINVAL;
  const long have = mpcd_fluid_count(h);
  if (n != have) return fail(h, MPCD_EINVAL, "get_fluid: n does not match the fluid size");
  CK(cudaStreamSynchronize(h->stream));
  if (h->p.precision == MPCD_FP64) {
    std::vector<uint32_t> cell(n);
    std::vector<double> o[3], v[3];
    for (int q = 0; q < 3; ++q) {
      o[q].resize(n);
      v[q].resize(n);
    }
    CK(cudaMemcpy(cell.data(), h->f64.cell, n * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(o[0].data(), h->f64.ox, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(o[1].data(), h->f64.oy, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(o[2].data(), h->f64.oz, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v[0].data(), h->f64.vx, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v[1].data(), h->f64.vy, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(v[2].data(), h->f64.vz, n * 8, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> ids(n);
    CK(cudaMemcpy(ids.data(), h->f64.id, n * 4, cudaMemcpyDeviceToHost));
    for (long i = 0; i < n; ++i) {
      const long d = ids[i];
      if (d < 0 || d >= n) return fail(h, MPCD_EDEVICE, "particle id out of range");
      const int c[3] = {cell_x(cell[i]), cell_y(cell[i]), cell_z(cell[i])};
      for (int q = 0; q < 3; ++q) {
        if (pos) pos[3 * d + q] = c[q] + o[q][i];
        if (vel) vel[3 * d + q] = v[q][i];
      }
    }
  } else {
    std::vector<float4> P(n), V(n);
    CK(cudaMemcpy(P.data(), h->f32.pos, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(V.data(), h->f32.vel, n * sizeof(float4), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> ids(n);
    CK(cudaMemcpy(ids.data(), h->f32.id, n * 4, cudaMemcpyDeviceToHost));
    for (long i = 0; i < n; ++i) {
      const long d = ids[i];
      if (d < 0 || d >= n) return fail(h, MPCD_EDEVICE, "particle id out of range");
      uint32_t cp = float_to_bits(P[i].w);
      if (pos) {
        pos[3 * d] = cell_x(cp) + (double)P[i].x;
        pos[3 * d + 1] = cell_y(cp) + (double)P[i].y;
        pos[3 * d + 2] = cell_z(cp) + (double)P[i].z;
      }
      if (vel) {
        vel[3 * d] = V[i].x;
        vel[3 * d + 1] = V[i].y;
        vel[3 * d + 2] = V[i].z;
      }
    }
  }
  return device_error(h);
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
  {
    ProfScope ps(h, MPCD_K_CELL);
    h->launches += f64 ? launch_cell_params_f64(h->c64, s, h->stream) : launch_cell_params_f32(h->c32, s, h->stream);
  }
  {
    ProfScope ps(h, MPCD_K_FLUID);
    h->launches += f64 ? launch_fluid_step_f64(h->f64, h->c64, s, h->stream)
                       : launch_fluid_step_f32(h->f32, h->c32, s, h->stream);
  }
  if (h->md.nslots) {
    {
      ProfScope ps(h, MPCD_K_BEAD);
      h->launches += f64 ? launch_bead_collide_f64(h->md, h->c64, s, h->stream)
                         : launch_bead_collide_f32(h->md, h->c32, s, h->stream);
    }
    ProfScope ps(h, MPCD_K_MD);
    if (h->md.cluster)
      h->launches += f64 ? launch_md_cluster_f64cells(h->md, h->c64, ma, h->stream, &coop)
                         : launch_md_cluster_f32cells(h->md, h->c32, ma, h->stream, &coop);
    else
      h->launches += f64 ? launch_md_f64(h->md, h->c64, ma, h->stream, &coop)
                         : launch_md_f32cells(h->md, h->c32, ma, h->stream, &coop);
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

int mpcd_observables(mpcd_engine* h, mpcd_obs* out) {
  if (!h || !out) return MPCD_EINVAL;
  if (h->md_dirty && h->nb) {
    int rc = build_md(h);
    if (rc) return rc;
  }
  CK(cudaMemsetAsync(h->d_obs, 0, 8 * sizeof(double), h->stream));
  if (h->p.precision == MPCD_FP64)
    h->launches += launch_observables_f64(h->f64, h->md, h->p.bead_mass, h->d_obs, h->stream);
  else
    h->launches += launch_observables_f32(h->f32, h->md, h->p.bead_mass, h->d_obs, h->stream);
  double o[8], diss = 0.0;
  CK(cudaMemcpyAsync(o, h->d_obs, sizeof o, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(&diss, h->d_diss, sizeof diss, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const double M = o[5] > 0 ? o[5] : 1.0, N = o[4] > 0 ? o[4] : 1.0;
  out->momentum[0] = o[0] / M;
  out->momentum[1] = o[1] / M;
  out->momentum[2] = o[2] / M;
  out->n = o[4];
  out->mass = o[5];
  out->kT = o[3] / 3.0 / N;
  out->fluid_T = o[7] > 0 ? o[6] / o[7] / 3.0 : 0.0;
  out->diss_energy = diss;
  out->globalt = h->globalt;
  out->energy_fluid = 0.5 * o[6];
  return device_error(h);
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

}  // extern "C"
