// MD substeps of one MPC step for all beads (src/simulation.cpp:217-265 inner
// loop; src/libcilia/mdobject.cpp:36-72 integrator; spring forces of
// src/cilia.cpp:127-239, src/sphere.cpp:87-119, src/clami.cpp:188-198).
//
// One cooperative launch runs all substeps.  A CTA owns one tile of bead
// slots; every cilium lies inside one tile, so its rest-length refresh
// (Cilia::length, src/cilia.cpp:79-121) and beat state machine
// (src/cilia.cpp:241-258, src/ConstantBeatCilia.cpp:8-23) need only
// __syncthreads.  Four lanes share one slot and split its spring list (a
// fixed-order shuffle reduction combines them); beads with long lists (the
// sphere centre has 642 radial springs) also own helper slots whose partial
// sums the primary adds in order.  Each substep the tile stages positions in
// shared memory: its own beads from registers, the beads of other tiles its
// springs reach ("halo") from the global position buffer written before the
// last grid barrier.  Positions go through two global buffers (read one,
// write the other), so one bounded grid barrier per substep suffices.
//
// Spring arithmetic: float64 (plain path) or split (kSplit): positions as
// float hi + float lo pairs, the difference x_i - x_j formed in float from the
// pairs, the rest of the spring in float; state and integration stay float64.
#include <algorithm>

#include "md_common.cuh"

namespace mpcd {

namespace {

constexpr int kLanes = 4;


// partial spring force on bead `me` (local index) from the springs
// [s0 + lane, s1) step kLanes
__device__ __forceinline__ void springs_f64(const MDState& m, const Stage<false>& st, int me, int s0, int s1,
                                            int lane, double& fx, double& fy, double& fz) {
  fx = fy = fz = 0.0;
  const double x = st.x[me], y = st.y[me], z = st.z[me];
  for (int s = s0 + lane; s < s1; s += kLanes) {
    const int o = __ldg(m.sp_local + s);
    const int kind = __ldg(m.sp_kind + s);
    const double b = kind <= 1 ? __ldg(m.sp_rest + s) : (kind == 2 ? m.newlen[__ldg(m.sp_ref + s)] : m.diag[__ldg(m.sp_ref + s)]);
    const double dx = x - st.x[o], dy = y - st.y[o], dz = z - st.z[o];
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (kind == 1 && d2 == 0.0) continue;  // vector-form spring: no force at zero distance
    const double fac = __ldg(m.sp_m2k + s) * (1.0 - b * rsqrt(d2));
    fx = fma(dx, fac, fx);
    fy = fma(dy, fac, fy);
    fz = fma(dz, fac, fz);
  }
}

__device__ __forceinline__ void springs_split(const MDState& m, const Stage<true>& st, int me, int s0, int s1,
                                              int lane, double& fx, double& fy, double& fz) {
  float ax = 0.f, ay = 0.f, az = 0.f;
  const float hx = st.hx[me], hy = st.hy[me], hz = st.hz[me];
  const float lx = st.lx[me], ly = st.ly[me], lz = st.lz[me];
  for (int s = s0 + lane; s < s1; s += kLanes) {
    const int o = __ldg(m.sp_local + s);
    const int kind = __ldg(m.sp_kind + s);
    const float b = (float)(kind <= 1 ? __ldg(m.sp_rest + s)
                                      : (kind == 2 ? m.newlen[__ldg(m.sp_ref + s)] : m.diag[__ldg(m.sp_ref + s)]));
    const float dx = (hx - st.hx[o]) + (lx - st.lx[o]);
    const float dy = (hy - st.hy[o]) + (ly - st.ly[o]);
    const float dz = (hz - st.hz[o]) + (lz - st.lz[o]);
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (kind == 1 && d2 == 0.0f) continue;
    const float fac = (float)__ldg(m.sp_m2k + s) * (1.0f - b * rsqrtf(d2));
    ax = fmaf(dx, fac, ax);
    ay = fmaf(dy, fac, ay);
    az = fmaf(dz, fac, az);
  }
  fx = ax;
  fy = ay;
  fz = az;
}


// ------------------------------------------------------------ contacts ---
// Contact forces between cilia: GlobalForces::recalc_forces / vdw_force with
// -DREPELLING=eps (src/libcilia/globalforces.cpp:22-95, constants
// src/libcilia/globalforces.h:22-28: cutoff 1.5, N = 4), over the cilia in
// their input order (the reference's own code names a `cilias` list its class
// does not declare, so its -DREPELLING build does not compile).  For a pair
// i < j, every filament-0 bead pair (k, l) on the lattices k = 3, 7, ... and
// l = len_j - 3, len_j - 7, ... (l >= k) closer than N * cutoff adds, for
// sections kk = k - 2 .. k + 1 and ll = l + 2 down to max(l - 2, kk), the
// repulsion F = -2 eps (1 - cutoff / |d|) d of the section centroids d
// (|d| < cutoff) to the three beads of section kk and -F to those of ll.  The
// reference gates these loops by a bounding-box overlap within the cutoff;
// that gate never removes a pair closer than the cutoff, so only candidate
// pairs (boxes within cutoff + 1 at the start of the MPC step: beads move far
// less than 0.5 in one step) are looked at.  Sections past a cilium's end are
// skipped.
constexpr double kRepelCutoff = 1.5;
constexpr int kRepelN = 4;
constexpr double kRepelReach = kRepelCutoff + 1.0;

__device__ __forceinline__ int cil_slot(const CiliumDev& c, int f, int j) { return c.slot0 + c.stride * (f * c.len + j); }

__device__ __forceinline__ void section_sum(const double* X, const double* Y, const double* Z, const CiliumDev& c, int j,
                                            double* s) {
  s[0] = s[1] = s[2] = 0.0;
  for (int f = 0; f < 3; ++f) {
    const int sl = cil_slot(c, f, j);
    s[0] += X[sl];
    s[1] += Y[sl];
    s[2] += Z[sl];
  }
}

__global__ void k_contact_pairs(MDState m) {
  const long n = m.ncil;
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < n * n; p += (long)gridDim.x * blockDim.x) {
    const int i = (int)(p / n), j = (int)(p % n);
    if (j <= i) continue;
    const CiliumDev ci = m.cil[i], cj = m.cil[j];
    double lo[2][3], hi[2][3];
    for (int w = 0; w < 2; ++w) {
      const CiliumDev& c = w ? cj : ci;
      for (int q = 0; q < 3; ++q) {
        lo[w][q] = 1e300;
        hi[w][q] = -1e300;
      }
      for (int s = 0; s < c.len; ++s) {
        double x[3];
        section_sum(m.x[0], m.y[0], m.z[0], c, s, x);
        for (int q = 0; q < 3; ++q) {
          lo[w][q] = fmin(lo[w][q], x[q] / 3.0);
          hi[w][q] = fmax(hi[w][q], x[q] / 3.0);
        }
      }
    }
    bool near = true;
    for (int q = 0; q < 3; ++q) near = near && lo[1][q] - hi[0][q] < kRepelReach && lo[0][q] - hi[1][q] < kRepelReach;
    if (!near) continue;
    const int k = atomicAdd(m.ncpairs, 1);
    if (k < m.cpair_cap) m.cpairs[k] = make_int2(i, j);
  }
}

// contact forces on this tile's beads into cf[3 * local slot] (shared, zeroed by the caller)
__device__ void contact_forces(const MDState& m, int b, int tile, int base, double* cf) {
  const int np = min(*m.ncpairs, m.cpair_cap);
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  const double* X = m.x[b];
  const double* Y = m.y[b];
  const double* Z = m.z[b];
  const int N = kRepelN;
  // work items: (pair, coarse k index, coarse l index), 16 x 16 per pair
  for (int w = threadIdx.x; w < np * 256; w += blockDim.x) {
    const int2 pr = m.cpairs[w >> 8];
    const bool mi = pr.x >= c0 && pr.x < c1, mj = pr.y >= c0 && pr.y < c1;
    if (!mi && !mj) continue;
    const CiliumDev ci = m.cil[pr.x], cj = m.cil[pr.y];
    const int k = 1 + N / 2 + N * ((w >> 4) & 15);
    const int l = cj.len - 1 - N / 2 - N * (w & 15);
    if (k >= ci.len || l < k) continue;
    const int sk = cil_slot(ci, 0, k), sl = cil_slot(cj, 0, l);
    const double ex = X[sk] - X[sl], ey = Y[sk] - Y[sl], ez = Z[sk] - Z[sl];
    if (!(sqrt(ex * ex + ey * ey + ez * ez) < N * kRepelCutoff)) continue;
    for (int kk = k - N / 2; kk < k + N / 2 && kk < ci.len; ++kk) {
      double x0[3];
      section_sum(X, Y, Z, ci, kk, x0);
      for (int ll = l + N / 2; ll >= l - N / 2 && ll >= kk; --ll) {
        double x1[3];
        section_sum(X, Y, Z, cj, ll, x1);
        const double dx = (x0[0] - x1[0]) / 3.0, dy = (x0[1] - x1[1]) / 3.0, dz = (x0[2] - x1[2]) / 3.0;
        const double dis = sqrt(dx * dx + dy * dy + dz * dz);
        if (!(dis < kRepelCutoff)) continue;
        const double f = -2.0 * m.repel * (1.0 - kRepelCutoff / dis);
        for (int r = 0; r < 3; ++r) {
          if (mi) {
            double* c = cf + 3 * (cil_slot(ci, r, kk) - base);
            atomicAdd(c, dx * f);
            atomicAdd(c + 1, dy * f);
            atomicAdd(c + 2, dz * f);
          }
          if (mj) {
            double* c = cf + 3 * (cil_slot(cj, r, ll) - base);
            atomicAdd(c, -(dx * f));
            atomicAdd(c + 1, -(dy * f));
            atomicAdd(c + 2, -(dz * f));
          }
        }
      }
    }
  }
}

template <bool kSplit, typename Bin>
__device__ void md_body(const MDState& m, const MDStepArgs& a, Bin bin) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int T = m.tile;
  const int NP = T + m.hmax;
  Stage<kSplit> st;
  st.init(smem, NP);
  double* part = reinterpret_cast<double*>(smem + Stage<kSplit>::bytes(NP));
  const int tile = blockIdx.x;
  const int base = tile * T;
  const int q = threadIdx.x / kLanes, lane = threadIdx.x % kLanes;
  const int slot = base + q;
  const bool valid = q < T && slot < m.nslots;
  const int mv = valid ? m.moves[slot] : -1;
  const bool moves = mv == 1;
  const bool primary = mv == 0 || mv == 1;
  const int me = valid && mv >= 0 ? m.prim[slot] - base : 0;
  const int nh = primary ? m.nhelp[slot] : 0;
  const int s0 = valid ? m.sp_start[slot] : 0, s1 = valid ? m.sp_start[slot + 1] : 0;
  const bool helpers = m.tile_help[tile] != 0;
  const int h0 = m.halo_start[tile], hn = m.halo_start[tile + 1] - h0;
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  const double dt = a.dt;
  double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0, fx = 0, fy = 0, fz = 0;
  if (primary) {
    x = m.x[0][slot];
    y = m.y[0][slot];
    z = m.z[0][slot];
    vx = m.vx[slot];
    vy = m.vy[slot];
    vz = m.vz[slot];
  }
  const unsigned nblocks = gridDim.x;
  unsigned barriers = 0;  // barriers passed in this launch
  double t = a.t0;
  int cur = 0;
  int eval = 0;  // index of the force evaluation within this MPC step

  auto stage = [&](int b) {
    if (primary && lane == 0) st.put(q, x, y, z);
    for (int i = threadIdx.x; i < hn; i += blockDim.x) {
      const int g = m.halo[h0 + i];
      st.put(T + i, m.x[b][g], m.y[b][g], m.z[b][g]);
    }
    __syncthreads();
  };
  auto evaluate = [&]() {
    const bool due = refresh_due(a, eval++);
    if (c1 > c0 && due) {
      // flatten (cilium, bond) pairs of this tile over the CTA's threads
      int off = 0;
      for (int c = c0; c < c1; ++c) {
        const CiliumDev cl = m.cil[c];
        const int nbnd = cl.len - cl.num_anker;
        const int w = (int)threadIdx.x - off;
        if (w >= 0 && w < nbnd) {
          const int i = cl.num_anker - 1 + w;
          const int k = cl.bond_base + i;
          const int l0 = cl.slot0 - base;
          const double l =
              cilium_length(cl, i, m.midpnt[c], m.oldlen[k], st.dist(l0 + cl.stride * i, l0 + cl.stride * (i + 1)));
          m.newlen[k] = l;
          m.oldlen[k] = l;
          m.diag[k] = sqrt(0.5 * 0.5 + 0.5 * l);
        }
        off += nbnd;
      }
      __syncthreads();
    }
    if (mv >= 0) {
      if constexpr (kSplit)
        springs_split(m, st, me, s0, s1, lane, fx, fy, fz);
      else
        springs_f64(m, st, me, s0, s1, lane, fx, fy, fz);
    } else {
      fx = fy = fz = 0.0;
    }
    // fixed-order reduction over the four lanes of the slot
    fx += __shfl_xor_sync(0xffffffffu, fx, 1);
    fy += __shfl_xor_sync(0xffffffffu, fy, 1);
    fz += __shfl_xor_sync(0xffffffffu, fz, 1);
    fx += __shfl_xor_sync(0xffffffffu, fx, 2);
    fy += __shfl_xor_sync(0xffffffffu, fy, 2);
    fz += __shfl_xor_sync(0xffffffffu, fz, 2);
    if (helpers) {
      if (lane == 0 && q < T) {
        part[3 * q] = fx;
        part[3 * q + 1] = fy;
        part[3 * q + 2] = fz;
      }
      __syncthreads();
      if (primary && lane == 0)
        for (int k = 1; k <= nh; ++k) {
          fx += part[3 * (q + k)];
          fy += part[3 * (q + k) + 1];
          fz += part[3 * (q + k) + 2];
        }
    }
    if (m.repel != 0.0) {  // contact forces between cilia, summed per bead in shared memory
      double* cf = part + 3 * T;
      for (int i = threadIdx.x; i < 3 * T; i += blockDim.x) cf[i] = 0.0;
      __syncthreads();
      contact_forces(m, cur, tile, base, cf);
      __syncthreads();
      if (primary && lane == 0) {
        fx += cf[3 * q];
        fy += cf[3 * q + 1];
        fz += cf[3 * q + 2];
      }
      __syncthreads();
    }
  };
  auto publish = [&](int b) {
    if (primary && lane == 0) {
      m.x[b][slot] = x;
      m.y[b][slot] = y;
      m.z[b][slot] = z;
    }
  };

  // md_loop_start: forces at t0, v += F dt/2, x += v dt
  stage(cur);
  evaluate();
  if (moves && lane == 0) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
    x = fma(vx, dt, x);
    y = fma(vy, dt, y);
    z = fma(vz, dt, z);
  }
  publish(cur ^ 1);
  if (!grid_sync(m.bar, ++barriers * nblocks, a.err)) return;
  cur ^= 1;
  stage(cur);
  evaluate();
  // md_loop: t += dt, v += F dt, x += v dt, forces
  for (int k = 1; k < a.n; ++k) {
    t += dt;
    if (moves && lane == 0) {
      vx = fma(fx, dt, vx);
      vy = fma(fy, dt, vy);
      vz = fma(fz, dt, vz);
      x = fma(vx, dt, x);
      y = fma(vy, dt, y);
      z = fma(vz, dt, z);
    }
    publish(cur ^ 1);
    if (!grid_sync(m.bar, ++barriers * nblocks, a.err)) return;
    cur ^= 1;
    stage(cur);
    evaluate();
  }
  t += dt;
  // md_loop_stop: v += F dt/2, then bin with the next shift
  if (moves && lane == 0) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
  }
  if (primary && lane == 0) {
    m.x[0][slot] = x;
    m.y[0][slot] = y;
    m.z[0][slot] = z;
    m.vx[slot] = vx;
    m.vy[slot] = vy;
    m.vz[slot] = vz;
    if (moves) bin(x, y, z, vx, vy, vz);
  }
  // switch_logic for the cilia of this tile (positions are unchanged since the last stage)
  for (int c = c0 + (int)threadIdx.x; c < c1; c += (int)blockDim.x) cilium_switch(m, a, c, t, base, st);
}


template <bool kSplit>
__global__ void k_md_f64cells(MDState m, CellsF64 c, MDStepArgs a) {
  md_body<kSplit>(m, a, BinF64{c, &a});
}

template <bool kSplit>
__global__ void k_md_f32cells(MDState m, CellsF32 c, MDStepArgs a) {
  md_body<kSplit>(m, a, BinF32{c, &a});
}

size_t md_smem(const MDState& m) {
  const int np = m.tile + m.hmax;
  return (m.split ? Stage<true>::bytes(np) : Stage<false>::bytes(np)) +
         (m.repel != 0.0 ? 6 : 3) * sizeof(double) * (size_t)m.tile;
}

template <typename K, typename C>
int launch_coop(K kernel, const MDState& m, const C& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  if (m.nslots == 0 || m.ntiles == 0) return 0;
  cudaMemsetAsync(m.bar.count, 0, 2 * sizeof(unsigned), s);  // count and gen are adjacent
  MDState mm = m;
  C cc = c;
  MDStepArgs aa = a;
  void* args[] = {&mm, &cc, &aa};
  const size_t smem = md_smem(m);
  if (smem > 48 * 1024) cudaFuncSetAttribute((const void*)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  *st = cudaLaunchCooperativeKernel((const void*)kernel, dim3(m.ntiles), dim3(kLanes * m.tile), args, smem, s);
  return 1;
}

}  // namespace

int launch_md_f64(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return m.split ? launch_coop(k_md_f64cells<true>, m, c, a, s, st) : launch_coop(k_md_f64cells<false>, m, c, a, s, st);
}

int launch_md_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return m.split ? launch_coop(k_md_f32cells<true>, m, c, a, s, st) : launch_coop(k_md_f32cells<false>, m, c, a, s, st);
}

int launch_contact_pairs(const MDState& m, cudaStream_t s) {
  if (m.repel == 0.0 || m.ncil < 2) return 0;
  cudaMemsetAsync(m.ncpairs, 0, sizeof(int), s);
  const long n2 = (long)m.ncil * m.ncil;
  const int g = (int)std::min<long>((n2 + 255) / 256, 4096);
  k_contact_pairs<<<g, 256, 0, s>>>(m);
  return 1;
}

// co-resident CTA limit for the cooperative launch of this layout
int md_max_coresident_blocks(const MDState& m, int f32cells) {
  if (m.pair) return md_pair_max_coresident_blocks(m, f32cells);
  if (m.df) return md_df_max_coresident_blocks(m, f32cells);
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = md_smem(m);
  const void* k = f32cells ? (m.split ? (const void*)k_md_f32cells<true> : (const void*)k_md_f32cells<false>)
                           : (m.split ? (const void*)k_md_f64cells<true> : (const void*)k_md_f64cells<false>);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kLanes * m.tile, smem);
  return per_sm * sms;
}

}  // namespace mpcd
