// MD substeps of one MPC step for all beads (src/simulation.cpp:217-265 inner
// loop; src/libcilia/mdobject.cpp:36-72 integrator; spring forces of
// src/cilia.cpp:127-239, src/sphere.cpp:87-119, src/clami.cpp:188-198).
//
// One cooperative launch runs every substep.  One thread owns one bead slot
// and keeps its velocity and force in registers; positions are shared through
// two global buffers (read one, write the other), so a single bounded grid
// barrier per substep orders the writes of substep k before the reads of
// substep k+1.  Every cilium lies inside one CTA: its rest-length refresh
// (Cilia::length, src/cilia.cpp:79-121) and beat state machine
// (src/cilia.cpp:241-258, src/ConstantBeatCilia.cpp:8-23) only need __syncthreads.
#include "engine_internal.h"

namespace mpcd {

namespace {

// Cilia::length(i) (src/cilia.cpp:79-121) for bond i of cilium `cl`, reading
// filament-0 positions from the current buffer.
__device__ double cilium_length(const CiliumDev& cl, int i, double midpnt, double oldlen, const double* X,
                                const double* Y, const double* Z) {
  const double bondlength = 0.5;
  const int s0 = cl.slot0 + i, s1 = s0 + 1;
  const double dx = X[s0] - X[s1], dy = Y[s0] - Y[s1], dz = Z[s0] - Z[s1];
  double tl = sqrt(dx * dx + dy * dy + dz * dz);
  double l;
  if (i < midpnt - 2.0) {
    l = bondlength + cl.beatstrength *
                         pow(1.0 - (i - cl.num_anker - 1.0) / (cl.len - cl.num_anker - 1.0), 2.5) * 0.5 *
                         (1.0 - 1.0 / (midpnt - i - 1.0));
  } else {
    const double di = i - midpnt;
    l = bondlength - 2.0 * cl.beatstrength / (di * di + 1.0);
  }
  if (fabs(l - tl) > cl.bending) {
    tl = tl + cl.bending - 2.0 * cl.bending * (l < tl ? 1.0 : 0.0);
    if ((l - oldlen) * (tl - oldlen) > 0) {
      l = tl;
    } else {
      l = oldlen;
    }
  }
  return l;
}

// refresh of the active rest lengths every 0.01 time units (src/cilia.cpp:206-215)
__device__ __forceinline__ bool refresh_due(double t, double dt) { return fmod(t + dt / 10., 0.01) < dt; }

__device__ void refresh_tile(const MDState& m, int tile, const double* X, const double* Y, const double* Z) {
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  // flatten (cilium, bond) pairs of this tile over the CTA's threads
  int base = 0;
  for (int c = c0; c < c1; ++c) {
    const CiliumDev cl = m.cil[c];
    const int nb = cl.len - 1 - (cl.num_anker - 1);
    for (int w = (int)threadIdx.x - base; w >= 0 && w < nb; w += (int)blockDim.x) {
      const int i = cl.num_anker - 1 + w;
      const int k = cl.bond_base + i;
      const double l = cilium_length(cl, i, m.midpnt[c], m.oldlen[k], X, Y, Z);
      m.newlen[k] = l;
      m.oldlen[k] = l;
    }
    base += nb;
  }
}

__device__ __forceinline__ void spring_force(const MDState& m, int slot, double x, double y, double z,
                                             const double* X, const double* Y, const double* Z, double& fx,
                                             double& fy, double& fz) {
  fx = fy = fz = 0.0;
  const int s1 = m.sp_start[slot + 1];
  for (int s = m.sp_start[slot]; s < s1; ++s) {
    const int o = m.sp_other[s];
    const int kind = m.sp_kind[s];
    double b;
    if (kind <= 1) {
      b = m.sp_rest[s];
    } else {
      const double nl = m.newlen[m.sp_ref[s]];
      b = kind == 2 ? nl : sqrt(0.5 * 0.5 + 0.5 * nl);
    }
    const double dx = x - X[o], dy = y - Y[o], dz = z - Z[o];
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (kind == 1 && d2 == 0.0) continue;  // vector-form spring: no force at zero distance
    const double fac = m.sp_m2k[s] * (1.0 - b * rsqrt(d2));
    fx = fma(dx, fac, fx);
    fy = fma(dy, fac, fy);
    fz = fma(dz, fac, fz);
  }
}

// Cilia::localbend(0, rodlength) (src/cilia.cpp:68-77)
__device__ double cilium_localbend(const CiliumDev& cl, const double* X, const double* Y, const double* Z) {
  double l = 0.0;
  for (int i = 0; i < cl.len - 1; ++i) {
    for (int f = 0; f < 3; ++f) {
      const int a = cl.slot0 + f * cl.len + i, b = a + 1;
      const double dx = X[a] - X[b], dy = Y[a] - Y[b], dz = Z[a] - Z[b];
      const double d = sqrt(dx * dx + dy * dy + dz * dz);
      l += f == 0 ? 2.0 * d : -d;
    }
  }
  return l;
}

template <typename Bin>
__device__ void md_body(MDState m, MDStepArgs a, Bin bin) {
  // partial forces of helper slots (beads with long spring lists own several
  // consecutive slots; the primary adds its helpers' partial sums in order)
  extern __shared__ double part[];
  const int tile = blockIdx.x;
  const int slot = tile * m.tile + threadIdx.x;
  const bool valid = threadIdx.x < m.tile && slot < m.nslots;
  const int mv = valid ? m.moves[slot] : -1;
  const bool moves = mv == 1;
  const bool primary = mv == 0 || mv == 1;
  const int me = valid ? m.prim[slot] : 0;  // slot holding this bead's position
  const int nh = primary ? m.nhelp[slot] : 0;
  const bool helpers = m.tile_help[tile] != 0;
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
  double t = a.t0;
  int cur = 0;
  // force evaluation at buffer b (refresh of the active rest lengths first when due)
  auto evaluate = [&](int b) {
    if (refresh_due(t, dt) && m.tile_cil[tile + 1] > m.tile_cil[tile]) {
      refresh_tile(m, tile, m.x[b], m.y[b], m.z[b]);
      __syncthreads();
    }
    if (primary) {
      spring_force(m, slot, x, y, z, m.x[b], m.y[b], m.z[b], fx, fy, fz);
    } else if (mv == 2) {
      spring_force(m, slot, m.x[b][me], m.y[b][me], m.z[b][me], m.x[b], m.y[b], m.z[b], fx, fy, fz);
    }
    if (helpers) {
      const int j = threadIdx.x;
      part[3 * j] = fx;
      part[3 * j + 1] = fy;
      part[3 * j + 2] = fz;
      __syncthreads();
      if (primary) {
        for (int k = 1; k <= nh; ++k) {
          fx += part[3 * (j + k)];
          fy += part[3 * (j + k) + 1];
          fz += part[3 * (j + k) + 2];
        }
      }
    }
  };
  // md_loop_start: v += F dt/2, x += v dt
  evaluate(cur);
  if (moves) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
    x = fma(vx, dt, x);
    y = fma(vy, dt, y);
    z = fma(vz, dt, z);
  }
  if (primary) {
    m.x[cur ^ 1][slot] = x;
    m.y[cur ^ 1][slot] = y;
    m.z[cur ^ 1][slot] = z;
  }
  if (!grid_sync(m.bar, nblocks, a.err)) return;
  cur ^= 1;
  evaluate(cur);
  for (int k = 1; k < a.n; ++k) {
    t += dt;
    if (moves) {
      vx = fma(fx, dt, vx);
      vy = fma(fy, dt, vy);
      vz = fma(fz, dt, vz);
      x = fma(vx, dt, x);
      y = fma(vy, dt, y);
      z = fma(vz, dt, z);
    }
    if (primary) {
      m.x[cur ^ 1][slot] = x;
      m.y[cur ^ 1][slot] = y;
      m.z[cur ^ 1][slot] = z;
    }
    if (!grid_sync(m.bar, nblocks, a.err)) return;
    cur ^= 1;
    evaluate(cur);
  }
  t += dt;
  // md_loop_stop: v += F dt/2, then bin with the next shift
  if (moves) {
    vx = fma(fx, dt / 2.0, vx);
    vy = fma(fy, dt / 2.0, vy);
    vz = fma(fz, dt / 2.0, vz);
  }
  if (primary) {
    if (cur == 1) {
      m.x[0][slot] = x;
      m.y[0][slot] = y;
      m.z[0][slot] = z;
    }
    m.vx[slot] = vx;
    m.vy[slot] = vy;
    m.vz[slot] = vz;
  }
  if (moves) bin(x, y, z, vx, vy, vz);
  __syncthreads();
  // switch_logic for the cilia of this tile
  const int c0 = m.tile_cil[tile], c1 = m.tile_cil[tile + 1];
  for (int c = c0 + (int)threadIdx.x; c < c1; c += (int)blockDim.x) {
    const CiliumDev cl = m.cil[c];
    double mp = m.midpnt[c], ts = m.tstroke[c];
    if (cl.kind == 1) {
      if (t - ts >= cl.power_dur && mp == cl.start) mp += 1;
      if (t - ts - cl.power_dur >= cl.recovery_dur && mp > cl.start) {
        ts = t;
        mp = cl.start;
      }
    } else {
      if (mp == cl.start && t - ts > 100.0) mp += 1;
      if (cilium_localbend(cl, m.x[0], m.y[0], m.z[0]) > cl.max_bend && mp > cl.start) {
        ts = t;
        mp = cl.start;
      }
    }
    if (mp > cl.start) mp += a.tstep / cl.m_speed;
    m.midpnt[c] = mp;
    m.tstroke[c] = ts;
  }
}

__device__ __forceinline__ int cell_axis(double x, double a, int L) {
  double xa = x + a;
  int c = (int)(floor(xa) - floor(xa / L) * L);
  if (c < 0) c += L;
  if (c >= L) c -= L;
  return c;
}

__global__ void k_md_f64(MDState m, CellsF64 c, MDStepArgs a) {
  md_body(m, a, [&](double x, double y, double z, double vx, double vy, double vz) {
    const long cid = cell_axis(x, a.a_next[0], a.box.L[0]) +
                     (long)a.box.L[0] * (cell_axis(y, a.a_next[1], a.box.L[1]) +
                                         (long)a.box.L[1] * cell_axis(z, a.a_next[2], a.box.L[2]));
    const double mb = a.bead_mass;
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, vx * mb);
    atomicAdd(sp + 1, vy * mb);
    atomicAdd(sp + 2, vz * mb);
    atomicAdd(sp + 3, mb * (vx * vx + vy * vy + vz * vz));
    atomicAdd(c.cnt + cid, 1u << 16);
  });
}

__global__ void k_md_f32cells(MDState m, CellsF32 c, MDStepArgs a) {
  md_body(m, a, [&](double x, double y, double z, double vx, double vy, double vz) {
    const long cid = cell_axis(x, a.a_next[0], a.box.L[0]) +
                     (long)a.box.L[0] * (cell_axis(y, a.a_next[1], a.box.L[1]) +
                                         (long)a.box.L[1] * cell_axis(z, a.a_next[2], a.box.L[2]));
    const float mb = (float)a.bead_mass;
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    float* sp = reinterpret_cast<float*>(c.sum + cid);
    atomicAdd(sp + 0, fvx * mb);
    atomicAdd(sp + 1, fvy * mb);
    atomicAdd(sp + 2, fvz * mb);
    atomicAdd(sp + 3, mb * (fvx * fvx + fvy * fvy + fvz * fvz));
    atomicAdd(c.cnt + cid, 1u << 16);
  });
}

template <typename K, typename C>
int launch_coop(K kernel, const MDState& m, const C& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  if (m.nslots == 0 || m.ntiles == 0) return 0;
  cudaMemsetAsync(m.bar.count, 0, 2 * sizeof(unsigned), s);  // count and gen are adjacent
  MDState mm = m;
  C cc = c;
  MDStepArgs aa = a;
  void* args[] = {&mm, &cc, &aa};
  *st = cudaLaunchCooperativeKernel((const void*)kernel, dim3(m.ntiles), dim3(m.tile), args,
                                    3 * sizeof(double) * m.tile, s);
  return 1;
}

}  // namespace

int launch_md_f64(const MDState& m, const CellsF64& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return launch_coop(k_md_f64, m, c, a, s, st);
}

int launch_md_f32cells(const MDState& m, const CellsF32& c, const MDStepArgs& a, cudaStream_t s, cudaError_t* st) {
  return launch_coop(k_md_f32cells, m, c, a, s, st);
}

// occupancy check used by the host before the first cooperative launch
int md_max_coresident_blocks(int tile, int f32cells) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 3 * sizeof(double) * tile;
  if (f32cells)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_md_f32cells, tile, smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_md_f64, tile, smem);
  return per_sm * sms;
}

}  // namespace mpcd
