// Fluid-side kernels of the replica batch (batch_internal.h).
//
// One MPC step of every active replica (Simulation::next_tstep,
// src/simulation.cpp:217-265) is
//   prologue      per replica: the next grid shift, the step's times and the
//                 beat refresh schedule; commits the replica's counters
//   cell_params   per cell of every replica: collision map from the sums
//   fluid_step    per particle of every replica: collide, stream, wrap, bin
//                 into the next shift's sums            } concurrently
//   md            per swimmer: bead collision, substeps, } (md_cluster.cu)
//                 binning, beat state machine
// The kernels walk fixed-size pages; a page belongs to one replica, whose
// parameters are loaded once per page.  A replica's random numbers are keyed
// by its own seed, step counter and box-local cell index, exactly as for the
// same box run alone (engine.cu), so its trajectory does not depend on the
// company it keeps.
#include <cstdlib>

#include "batch_internal.h"
#include "fluid_device.cuh"
#include "tma.cuh"

namespace mpcd {

namespace {

__global__ void k_batch_prologue(BatchTables t) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= t.nrep) return;
  const BatchRep& R = t.rep[r];
  BatchStep& S = t.step[r];
  BatchState& st = t.state[r];
  if (!R.resident || st.steps_left <= 0) {
    S.active = 0;
    return;
  }
  S.active = 1;
  const uint64_t step = st.steps + 1;
  S.step = step;
  double an[3];
  if (r == t.inj_rep && t.inj_shift) {
    an[0] = t.inj_shift[0];
    an[1] = t.inj_shift[1];
    an[2] = t.inj_shift[2];
  } else {
    const u32x4 q = draw4(R.seed, step, kStreamShift, 0u, 0u);  // shift_from_counter (engine.cu)
    an[0] = u01_dbl(q.x);
    an[1] = u01_dbl(q.y);
    an[2] = u01_dbl(q.z);
  }
  // simulation time as the reference accumulates it (n additions of ststep)
  const double t0 = st.globalt;
  double t_move = t0;
  for (int k = 0; k < R.nsub; ++k) t_move += R.ststep;
  MDStepArgs& m = S.md;
  m.t0 = t0;
  m.dt = R.ststep;
  m.tstep = R.h;
  m.n = R.nsub;
  m.t_end = t_move;
  // rest-length refresh of force evaluation e (src/cilia.cpp:206-215):
  // evaluations 0 and 1 at t0, evaluation k+1 after k additions of ststep
  for (int w = 0; w < 8; ++w) m.refresh[w] = 0ull;
  double te = t0;
  for (int e = 0; e <= R.nsub && e < 512; ++e) {
    if (e >= 2) te += R.ststep;
    if (fmod(te + R.ststep / 10., 0.01) < R.ststep) m.refresh[e >> 6] |= 1ull << (e & 63);
  }
  m.box.L[0] = R.L[0];
  m.box.L[1] = R.L[1];
  m.box.L[2] = R.L[2];
  for (int q = 0; q < 3; ++q) {
    m.a_cur[q] = st.a[q];
    m.a_next[q] = an[q];
    S.fta_cur[q] = (float)(1.0 - st.a[q]);
    S.fta_next[q] = (float)(1.0 - an[q]);
  }
  m.bead_mass = R.bead_mass;
  m.err = &st.err;
  S.fh = (float)R.h;
  S.fbead_mass = (float)R.bead_mass;
  S.fgkick = R.gravity != 0.0 ? (float)(R.gravity * cos(t_move * R.omega) * R.h) : 0.0f;
  // commit: the other kernels of this step read S only
  st.steps = step;
  st.globalt = t_move;
  st.a[0] = an[0];
  st.a[1] = an[1];
  st.a[2] = an[2];
  st.steps_left -= 1;
}

__global__ void k_batch_cell_params(BatchTables t, BatchCells c) {
  for (long pg = blockIdx.x; pg < t.ncell_pages; pg += gridDim.x) {
    const int r = t.cell_page_rep[pg];
    if (r < 0) continue;
    const BatchStep& S = t.step[r];
    if (!S.active) continue;
    const BatchRep& R = t.rep[r];
    const long c0 = pg * kCellPage;
    const long c1 = min(c0 + kCellPage, R.cell0 + R.ncell);
    const uint64_t seed = R.seed, step = S.step;
    const float mb = S.fbead_mass;
    const long cell0 = R.cell0;
    const bool inj = r == t.inj_rep;
    const double* inj_gamma = inj ? t.inj_gamma : nullptr;
    const double* inj_axis = inj ? t.inj_axis : nullptr;
    float ldiss = 0.0f;
    unsigned errbits = 0;
    bool gfail = false;
    // four cells per thread at a time: their count words and sums are loaded
    // together, so the latency of the loads is paid once per four cells
    constexpr int kU = 4;
    const long stride = blockDim.x;
    for (long cb = c0 + threadIdx.x; cb < c1; cb += kU * stride) {
      uint32_t w[kU];
      float4 sm[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const long cid = cb + u * stride;
        w[u] = cid < c1 ? __ldcg(c.cnt + cid) : 0u;
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const long cid = cb + u * stride;
        sm[u] = w[u] ? __ldcg(c.sum + cid) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (!w[u]) continue;
        const long cid = cb + u * stride;
        c.sum[cid] = make_float4(0.f, 0.f, 0.f, 0.f);
        c.cnt[cid] = 0u;
        cell_map_f32(sm[u], w[u], (uint32_t)(cid - cell0), seed, step, mb, inj_gamma, inj_axis, c.par + 2 * cid,
                     ldiss, errbits, gfail);
      }
    }
    if (gfail) errbits |= kErrGammaLoop;
    if (errbits) atomicOr(&t.state[r].err, errbits);
    const double tot = block_sum_f32(ldiss);
    if (threadIdx.x == 0 && tot != 0.0) atomicAdd(&t.state[r].diss, tot);
  }
}

// The replica parameters one fluid page needs.
struct FluidPage {
  int L[3];
  float tc[3], tn[3];
  float h, gk;
  float4* sum;
  uint32_t* cnt;
  const float4* par;
};

__device__ __forceinline__ FluidPage fluid_page(const BatchTables& t, const BatchCells& c, int r) {
  const BatchStep& S = t.step[r];
  const BatchRep& R = t.rep[r];
  FluidPage P;
  for (int q = 0; q < 3; ++q) {
    P.L[q] = R.L[q];
    P.tc[q] = S.fta_cur[q];
    P.tn[q] = S.fta_next[q];
  }
  P.h = S.fh;
  P.gk = S.fgkick;
  P.sum = c.sum + R.cell0;
  P.cnt = c.cnt + R.cell0;
  P.par = c.par + 2 * R.cell0;
  return P;
}

// The shifted cell of a fluid particle under the current grid shift: the
// cell whose collision map it takes.
// (box cells < 2^30: 32-bit index)
__device__ __forceinline__ uint32_t fluid_cell_cur(const FluidPage& P, const float4 p) {
  const uint32_t cp = __float_as_uint(p.w);
  return (uint32_t)shifted_f(cell_x(cp), p.x, P.tc[0], P.L[0]) +
         (uint32_t)P.L[0] * ((uint32_t)shifted_f(cell_y(cp), p.y, P.tc[1], P.L[1]) +
                             (uint32_t)P.L[1] * (uint32_t)shifted_f(cell_z(cp), p.z, P.tc[2], P.L[2]));
}

// One fluid particle (MPCD::next_tstep's rotation, MPCD::move, Fluid::move,
// add_impuls: src/libcilia/mpcd.cpp:140-267, src/libcilia/fluid.cpp:152-167):
// collide with its cell's map (mk, mu), stream, wrap, body force, bin into the
// sums of the next shift.  Returns the new state.
__device__ __forceinline__ void fluid_particle(const FluidPage& P, const float4 p, const float4 v, const float4 mk,
                                               const float4 mu, float4& po, float4& vo, float& ke_after, unsigned& bad) {
  const int Lx = P.L[0], Ly = P.L[1], Lz = P.L[2];
  const uint32_t cp = __float_as_uint(p.w);
  int ix = cell_x(cp), iy = cell_y(cp), iz = cell_z(cp);
  float ox = p.x, oy = p.y, oz = p.z, vx = v.x, vy = v.y, vz = v.z;
  apply_map_f32(mk, mu, vx, vy, vz);
  ke_after += vx * vx + vy * vy + vz * vz;
  ox = fmaf(vx, P.h, ox);
  oy = fmaf(vy, P.h, oy);
  oz = fmaf(vz, P.h, oz);
  rewrap_f(ox, ix, Lx, bad);
  rewrap_f(oy, iy, Ly, bad);
  rewrap_f(oz, iz, Lz, bad);
  if (P.gk != 0.0f) vx += P.gk;
  const uint32_t cn = (uint32_t)shifted_f(ix, ox, P.tn[0], Lx) +
                      (uint32_t)Lx * ((uint32_t)shifted_f(iy, oy, P.tn[1], Ly) + (uint32_t)Ly * (uint32_t)shifted_f(iz, oz, P.tn[2], Lz));
  red_add_v4(P.sum + cn, make_float4(vx, vy, vz, vx * vx + vy * vy + vz * vz));
  atomicAdd(P.cnt + cn, 1u);
  po = make_float4(ox, oy, oz, __uint_as_float(pack_cell(ix, iy, iz)));
  vo = make_float4(vx, vy, vz, 0.f);
}

__device__ __forceinline__ void fluid_particle(const FluidPage& P, const float4 p, const float4 v, float4& po,
                                               float4& vo, float& ke_after, unsigned& bad) {
  const float4* m = P.par + 2 * (size_t)fluid_cell_cur(P, p);
  fluid_particle(P, p, v, __ldg(m), __ldg(m + 1), po, vo, ke_after, bad);
}

// Particles per thread whose loads (state, then collision map) are issued
// together before their reductions and stores (one or two measured alike on
// the 64-replica ensemble: 0.549-0.555 ms; four spill registers).
constexpr int kFluidBatchB = 2;

template <int U>
__global__ void __launch_bounds__(512, 2) k_batch_fluid_step(BatchTables t, BatchFluid f, BatchCells c) {
  for (long pg = blockIdx.x; pg < t.npart_pages; pg += gridDim.x) {
    const int r = t.part_page_rep[pg];
    if (r < 0) continue;
    if (!t.step[r].active) continue;
    const BatchRep& R = t.rep[r];
    const long i0 = pg * kPartPage;
    const long i1 = min(i0 + kPartPage, R.p0 + R.n);
    const FluidPage P = fluid_page(t, c, r);
    float ke_after = 0.0f;
    unsigned bad = 0;
    const int np = (int)(i1 - i0);  // page-local indices: 32-bit
    float4* const pos = f.pos + i0;
    float4* const vel = f.vel + i0;
    for (int base = threadIdx.x; base < np; base += U * blockDim.x) {
      float4 p[U], v[U], mk[U], mu[U];
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int j = base + q * blockDim.x;
        if (j < np) {
          p[q] = __ldcs(pos + j);
          v[q] = __ldcs(vel + j);
        }
      }
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int j = base + q * blockDim.x;
        if (j < np) {
          const float4* m = P.par + 2 * (size_t)fluid_cell_cur(P, p[q]);
          mk[q] = __ldg(m);
          mu[q] = __ldg(m + 1);
        }
      }
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int j = base + q * blockDim.x;
        if (j < np) {
          float4 po, vo;
          fluid_particle(P, p[q], v[q], mk[q], mu[q], po, vo, ke_after, bad);
          __stcs(pos + j, po);
          __stcs(vel + j, vo);
        }
      }
    }
    if (bad) atomicOr(&t.state[r].err, bad);
    const double tot = block_sum_f32(ke_after);
    if (threadIdx.x == 0 && tot != 0.0) atomicAdd(&t.state[r].diss, -tot);
  }
}

// The same pass with the particle state staged through shared memory by bulk
// asynchronous copies (TMA): chunks of kTmaChunk particles, two buffers, the
// copy of the next chunk in flight while the current one is processed.  The
// chunks are the pages' quarters, taken in a grid-stride order that every
// thread of the block derives alike; waits are bounded (a timeout sets
// kErrBarrier for the chunk's replica and ends the block after its copies
// are drained).
constexpr int kTmaChunk = 1024;
constexpr int kTmaThreads = 256;
constexpr uint32_t kTmaWaitLimit = 1u << 22;

__global__ void __launch_bounds__(kTmaThreads) k_batch_fluid_step_tma(BatchTables t, BatchFluid f, BatchCells c) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  float4* const buf = reinterpret_cast<float4*>(tma_smem);  // [b][pos | vel][kTmaChunk]
  __shared__ __align__(8) uint64_t bar[2];
  constexpr int kParts = kPartPage / kTmaChunk;
  const long nchunks = t.npart_pages * kParts;
  auto chunk = [&](long q, long& i0, int& n, int& r) -> bool {
    const long pg = q / kParts;
    r = t.part_page_rep[pg];
    if (r < 0 || !t.step[r].active) return false;
    const BatchRep& R = t.rep[r];
    i0 = pg * kPartPage + (q % kParts) * kTmaChunk;
    const long e = min(i0 + kTmaChunk, R.p0 + R.n);
    n = (int)(e - i0);
    return n > 0;
  };
  auto issue = [&](long i0, int n, int b) {
    const uint32_t bytes = (uint32_t)n * sizeof(float4);
    mbar_arrive_expect_tx(&bar[b], 2 * bytes);
    bulk_load(buf + (2 * b) * kTmaChunk, f.pos + i0, bytes, &bar[b]);
    bulk_load(buf + (2 * b + 1) * kTmaChunk, f.vel + i0, bytes, &bar[b]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  long q = blockIdx.x, i0 = 0;
  int n = 0, r = -1;
  while (q < nchunks && !chunk(q, i0, n, r)) q += gridDim.x;
  if (q >= nchunks) return;
  if (threadIdx.x == 0) issue(i0, n, 0);
  int b = 0;
  uint32_t phase = 0u;  // bit k: parity of the next phase of bar[k]
  for (;;) {
    long qn = q + gridDim.x, i0n = 0;
    int nn = 0, rn = -1;
    while (qn < nchunks && !chunk(qn, i0n, nn, rn)) qn += gridDim.x;
    const bool has_next = qn < nchunks;
    if (threadIdx.x == 0 && has_next) {  // buffer b ^ 1 was released by the last barrier
      fence_proxy_async_smem();
      issue(i0n, nn, b ^ 1);
    }
    const bool ok = mbar_wait(&bar[b], (phase >> b) & 1u, kTmaWaitLimit);
    phase ^= 1u << b;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(&t.state[r].err, kErrBarrier);
      if (has_next) mbar_wait(&bar[b ^ 1], (phase >> (b ^ 1)) & 1u, kTmaWaitLimit);  // drain the copy in flight
      return;
    }
    const FluidPage P = fluid_page(t, c, r);
    const float4* sp = buf + (2 * b) * kTmaChunk;
    const float4* sv = buf + (2 * b + 1) * kTmaChunk;
    float ke_after = 0.0f;
    unsigned bad = 0;
    for (int j = threadIdx.x; j < n; j += kTmaThreads) {
      float4 po, vo;
      fluid_particle(P, sp[j], sv[j], po, vo, ke_after, bad);
      f.pos[i0 + j] = po;
      f.vel[i0 + j] = vo;
    }
    if (bad) atomicOr(&t.state[r].err, bad);
    const double tot = block_sum_f32(ke_after);  // its barriers also release buffer b
    if (threadIdx.x == 0 && tot != 0.0) atomicAdd(&t.state[r].diss, -tot);
    __syncthreads();
    if (!has_next) break;
    q = qn;
    i0 = i0n;
    n = nn;
    r = rn;
    b ^= 1;
  }
}

__global__ void k_batch_bin_fluid(BatchTables t, BatchFluid f, BatchCells c, long page0, long page1) {
  for (long pg = page0 + blockIdx.x; pg < page1; pg += gridDim.x) {
    const int r = t.part_page_rep[pg];
    if (r < 0) continue;
    const BatchRep& R = t.rep[r];
    const BatchState& st = t.state[r];
    const long i0 = pg * kPartPage;
    const long i1 = min(i0 + kPartPage, R.p0 + R.n);
    const int Lx = R.L[0], Ly = R.L[1], Lz = R.L[2];
    const float tcx = (float)(1.0 - st.a[0]), tcy = (float)(1.0 - st.a[1]), tcz = (float)(1.0 - st.a[2]);
    for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const float4 p = f.pos[i];
      const float4 v = f.vel[i];
      const uint32_t cp = __float_as_uint(p.w);
      const long cid = shifted_f(cell_x(cp), p.x, tcx, Lx) +
                       (long)Lx * (shifted_f(cell_y(cp), p.y, tcy, Ly) + (long)Ly * shifted_f(cell_z(cp), p.z, tcz, Lz));
      red_add_v4(c.sum + R.cell0 + cid, make_float4(v.x, v.y, v.z, v.x * v.x + v.y * v.y + v.z * v.z));
      atomicAdd(c.cnt + R.cell0 + cid, 1u);
    }
  }
}

__global__ void k_batch_bin_beads(BatchTables t, MDState m, const int* tile_rep, BatchCells c, int tile0, int tile1) {
  const long s0 = (long)tile0 * m.tile, s1 = (long)tile1 * m.tile;
  for (long s = s0 + (long)blockIdx.x * blockDim.x + threadIdx.x; s < s1; s += (long)gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const int r = tile_rep[s / m.tile];
    if (r < 0) continue;
    const BatchRep& R = t.rep[r];
    BatchState& st = t.state[r];
    Box box;
    box.L[0] = R.L[0];
    box.L[1] = R.L[1];
    box.L[2] = R.L[2];
    const long cid = unwrapped_cell(box, st.a, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      atomicOr(&st.err, kErrCellRange);
      continue;
    }
    const float mb = (float)R.bead_mass;
    const float vx = (float)m.vx[s], vy = (float)m.vy[s], vz = (float)m.vz[s];
    red_add_v4(c.sum + R.cell0 + cid, make_float4(vx * mb, vy * mb, vz * mb, mb * (vx * vx + vy * vy + vz * vz)));
    atomicAdd(c.cnt + R.cell0 + cid, 1u << 16);
  }
}

// ------------------------------------------------------------------ sort ---
// Counting sort by cell within every replica's own particle range: the global
// exclusive scan of the per-cell counts gives start[], and a particle of
// replica r goes to p0 + start[cell] - start[cell0] + rank.

__global__ void k_batch_sort_count(BatchTables t, BatchFluid f, uint32_t* count, uint32_t* rank) {
  for (long pg = blockIdx.x; pg < t.npart_pages; pg += gridDim.x) {
    const int r = t.part_page_rep[pg];
    if (r < 0) continue;
    const BatchRep& R = t.rep[r];
    const long i0 = pg * kPartPage;
    const long i1 = min(i0 + kPartPage, R.p0 + R.n);
    for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const uint32_t cp = __float_as_uint(f.pos[i].w);
      const long cell = R.cell0 + cell_x(cp) + (long)R.L[0] * (cell_y(cp) + (long)R.L[1] * cell_z(cp));
      rank[i] = atomicAdd(count + cell, 1u);
    }
  }
}

__global__ void k_batch_sort_scatter(BatchTables t, BatchFluid src, BatchFluid dst, const uint32_t* start,
                                     const uint32_t* rank) {
  for (long pg = blockIdx.x; pg < t.npart_pages; pg += gridDim.x) {
    const int r = t.part_page_rep[pg];
    if (r < 0) continue;
    const BatchRep& R = t.rep[r];
    const long i0 = pg * kPartPage;
    const long i1 = min(i0 + kPartPage, R.p0 + R.n);
    const long base = R.p0 - (long)start[R.cell0];
    for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const float4 p = src.pos[i];
      const uint32_t cp = __float_as_uint(p.w);
      const long cell = R.cell0 + cell_x(cp) + (long)R.L[0] * (cell_y(cp) + (long)R.L[1] * cell_z(cp));
      const long d = base + (long)start[cell] + rank[i];
      dst.id[d] = src.id[i];
      dst.pos[d] = p;
      dst.vel[d] = src.vel[i];
    }
  }
}

// ----------------------------------------------------------- observables ---

__global__ void k_batch_obs_fluid(BatchTables t, BatchFluid f, double* out) {
  for (long pg = blockIdx.x; pg < t.npart_pages; pg += gridDim.x) {
    const int r = t.part_page_rep[pg];
    if (r < 0) continue;
    const BatchRep& R = t.rep[r];
    const long i0 = pg * kPartPage;
    const long i1 = min(i0 + kPartPage, R.p0 + R.n);
    double px = 0, py = 0, pz = 0, e = 0, n = 0;
    for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const float4 v = f.vel[i];
      const double vx = v.x, vy = v.y, vz = v.z;
      px += vx;
      py += vy;
      pz += vz;
      e += vx * vx + vy * vy + vz * vz;
      n += 1.0;
    }
    // fluid: mass 1, so sum m v^2 = sum v^2, N = M
    const double vals[8] = {px, py, pz, e, n, n, e, n};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const double s = block_sum_f64(vals[k]);
      if (threadIdx.x == 0 && s != 0.0) atomicAdd(out + 8 * r + k, s);
    }
  }
}

__global__ void k_batch_obs_beads(BatchTables t, MDState m, const int* tile_rep, int ntiles, double* out) {
  const long ns = (long)ntiles * m.tile;
  for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (long)gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const int r = tile_rep[s / m.tile];
    if (r < 0) continue;
    const double mb = t.rep[r].bead_mass;
    const double vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    double* o = out + 8 * r;
    atomicAdd(o + 0, mb * vx);
    atomicAdd(o + 1, mb * vy);
    atomicAdd(o + 2, mb * vz);
    atomicAdd(o + 3, mb * (vx * vx + vy * vy + vz * vz));
    atomicAdd(o + 4, 1.0);
    atomicAdd(o + 5, mb);
  }
}

inline int sm_count_b() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

inline int page_grid(long pages, int per_sm = 8) {
  long g = pages;
  const long cap = (long)sm_count_b() * per_sm;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int launch_batch_prologue(const BatchTables& t, cudaStream_t s) {
  k_batch_prologue<<<(t.nrep + 127) / 128, 128, 0, s>>>(t);
  return 1;
}

int launch_batch_cell_params(const BatchTables& t, BatchCells c, int threads, int blocks, cudaStream_t s) {
  if (blocks <= 0) blocks = page_grid(t.ncell_pages);
  k_batch_cell_params<<<blocks, threads, 0, s>>>(t, c);
  return 1;
}

int launch_batch_fluid_step(const BatchTables& t, BatchFluid f, BatchCells c, int threads, int blocks,
                            cudaStream_t s) {
  if (threads == 0) {  // shared-memory staged variant: fixed block, two 32 KB buffers, three blocks per SM
    const size_t smem = 4 * sizeof(float4) * kTmaChunk;
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute((const void*)k_batch_fluid_step_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
      attr = true;
    }
    const long nchunks = t.npart_pages * (kPartPage / kTmaChunk);
    if (blocks <= 0) blocks = (int)std::min<long>(nchunks, 3L * sm_count_b());
    k_batch_fluid_step_tma<<<blocks, kTmaThreads, smem, s>>>(t, f, c);
    return 1;
  }
  if (blocks <= 0) blocks = page_grid(t.npart_pages);
  // particles per thread and round: kFluidBatchB unless MPCD_FLUID_BATCH is 1
  static const int batch = [] {
    const char* e = std::getenv("MPCD_FLUID_BATCH");
    return e && std::atoi(e) == 1 ? 1 : kFluidBatchB;
  }();
  if (batch == 1)
    k_batch_fluid_step<1><<<blocks, threads, 0, s>>>(t, f, c);
  else
    k_batch_fluid_step<kFluidBatchB><<<blocks, threads, 0, s>>>(t, f, c);
  return 1;
}

int launch_batch_bin_fluid(const BatchTables& t, BatchFluid f, BatchCells c, long page0, long page1,
                           cudaStream_t s) {
  if (page1 <= page0) return 0;
  k_batch_bin_fluid<<<page_grid(page1 - page0), 256, 0, s>>>(t, f, c, page0, page1);
  return 1;
}

int launch_batch_bin_beads(const BatchTables& t, const MDState& m, const int* tile_rep, BatchCells c, int tile0,
                           int tile1, cudaStream_t s) {
  if (tile1 <= tile0 || m.tile == 0) return 0;
  const long ns = (long)(tile1 - tile0) * m.tile;
  const int blocks = (int)std::min<long>((ns + 255) / 256, 4L * sm_count_b());
  k_batch_bin_beads<<<blocks, 256, 0, s>>>(t, m, tile_rep, c, tile0, tile1);
  return 1;
}

int launch_batch_sort(const BatchTables& t, BatchFluid src, BatchFluid dst, uint32_t* count, uint32_t* start,
                      uint32_t* rank, uint32_t* blocksums, long ncell_total, cudaStream_t s) {
  cudaMemsetAsync(count, 0, sizeof(uint32_t) * ncell_total, s);
  const int g = page_grid(t.npart_pages);
  k_batch_sort_count<<<g, 256, 0, s>>>(t, src, count, rank);
  int n = 2 + scan_counts_ext(count, ncell_total, start, blocksums, s);
  k_batch_sort_scatter<<<g, 256, 0, s>>>(t, src, dst, start, rank);
  return n;
}

int launch_batch_observables(const BatchTables& t, BatchFluid f, const MDState& m, const int* tile_rep, int ntiles,
                             double* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(double) * 8 * t.nrep, s);
  k_batch_obs_fluid<<<page_grid(t.npart_pages), 256, 0, s>>>(t, f, out);
  int n = 1;
  if (ntiles > 0 && m.tile > 0) {
    const long ns = (long)ntiles * m.tile;
    const int blocks = (int)std::min<long>((ns + 255) / 256, 4L * sm_count_b());
    k_batch_obs_beads<<<blocks, 256, 0, s>>>(t, m, tile_rep, ntiles, out);
    ++n;
  }
  return n;
}

}  // namespace mpcd
