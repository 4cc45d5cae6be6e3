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
#include "engine_internal.h"

namespace mpcd {

namespace {

constexpr int kLanes = 4;

// Cilia::length(i) (src/cilia.cpp:79-121): active rest length of bond i
__device__ double cilium_length(const CiliumDev& cl, int i, double midpnt, double oldlen, double tl) {
  const double bondlength = 0.5;
  double l;
  if (i < midpnt - 2.0) {
    // base^2.5 as base^2 sqrt(base) (base > 0 for every refreshed bond)
    const double base = 1.0 - (i - cl.num_anker - 1.0) / (cl.len - cl.num_anker - 1.0);
    l = bondlength + cl.beatstrength * (base * base * sqrt(base)) * 0.5 * (1.0 - 1.0 / (midpnt - i - 1.0));
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

// refresh every 0.01 time units (src/cilia.cpp:206-215); the schedule of the
// step's force evaluations is computed on the host
__device__ __forceinline__ bool refresh_due(const MDStepArgs& a, int e) { return (a.refresh[e >> 6] >> (e & 63)) & 1ull; }

// Positions of one tile (own slots, then halo) in shared memory.
template <bool kSplit>
struct Stage;

template <>
struct Stage<false> {
  double *x, *y, *z;
  __device__ void init(unsigned char* base, int np) {
    x = reinterpret_cast<double*>(base);
    y = x + np;
    z = y + np;
  }
  __host__ __device__ static size_t bytes(int np) { return 3 * sizeof(double) * (size_t)np; }
  __device__ void put(int i, double px, double py, double pz) {
    x[i] = px;
    y[i] = py;
    z[i] = pz;
  }
  __device__ void get(int i, double& px, double& py, double& pz) const {
    px = x[i];
    py = y[i];
    pz = z[i];
  }
  __device__ double dist(int i, int j) const {
    const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

template <>
struct Stage<true> {
  float *hx, *hy, *hz, *lx, *ly, *lz;
  __device__ void init(unsigned char* base, int np) {
    hx = reinterpret_cast<float*>(base);
    hy = hx + np;
    hz = hy + np;
    lx = hz + np;
    ly = lx + np;
    lz = ly + np;
  }
  __host__ __device__ static size_t bytes(int np) { return 6 * sizeof(float) * (size_t)np; }
  __device__ void put(int i, double px, double py, double pz) {
    const float a = (float)px, b = (float)py, c = (float)pz;
    hx[i] = a;
    hy[i] = b;
    hz[i] = c;
    lx[i] = (float)(px - (double)a);
    ly[i] = (float)(py - (double)b);
    lz[i] = (float)(pz - (double)c);
  }
  __device__ void get(int i, double& px, double& py, double& pz) const {
    px = (double)hx[i] + (double)lx[i];
    py = (double)hy[i] + (double)ly[i];
    pz = (double)hz[i] + (double)lz[i];
  }
  __device__ double dist(int i, int j) const {
    double xi, yi, zi, xj, yj, zj;
    get(i, xi, yi, zi);
    get(j, xj, yj, zj);
    const double dx = xi - xj, dy = yi - yj, dz = zi - zj;
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

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

// Cilia::localbend(0, rodlength) (src/cilia.cpp:68-77) from staged positions
template <bool kSplit>
__device__ double cilium_localbend(const CiliumDev& cl, int l0, const Stage<kSplit>& st) {
  double l = 0.0;
  const int sd = cl.stride;
  for (int i = 0; i < cl.len - 1; ++i) {
    l += 2.0 * st.dist(l0 + sd * i, l0 + sd * (i + 1));
    l -= st.dist(l0 + sd * (cl.len + i), l0 + sd * (cl.len + i + 1));
    l -= st.dist(l0 + sd * (2 * cl.len + i), l0 + sd * (2 * cl.len + i + 1));
  }
  return l;
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
      if (cilium_localbend<kSplit>(cl, cl.slot0 - base, st) > cl.max_bend && mp > cl.start) {
        ts = t;
        mp = cl.start;
      }
    }
    if (mp > cl.start) mp += a.tstep / cl.m_speed;
    m.midpnt[c] = mp;
    m.tstroke[c] = ts;
  }
}

struct BinF64 {
  CellsF64 c;
  const MDStepArgs* a;
  __device__ void operator()(double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(a->box, a->a_next, x, y, z);
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      return;
    }
    const double mb = a->bead_mass;
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, vx * mb);
    atomicAdd(sp + 1, vy * mb);
    atomicAdd(sp + 2, vz * mb);
    atomicAdd(sp + 3, mb * (vx * vx + vy * vy + vz * vz));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
};

struct BinF32 {
  CellsF32 c;
  const MDStepArgs* a;
  __device__ void operator()(double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(a->box, a->a_next, x, y, z);
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      return;
    }
    const float mb = (float)a->bead_mass;
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    float* sp = reinterpret_cast<float*>(c.sum + cid);
    atomicAdd(sp + 0, fvx * mb);
    atomicAdd(sp + 1, fvy * mb);
    atomicAdd(sp + 2, fvz * mb);
    atomicAdd(sp + 3, mb * (fvx * fvx + fvy * fvy + fvz * fvz));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
};

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
  return (m.split ? Stage<true>::bytes(np) : Stage<false>::bytes(np)) + 3 * sizeof(double) * (size_t)m.tile;
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

// co-resident CTA limit for the cooperative launch of this layout
int md_max_coresident_blocks(const MDState& m, int f32cells) {
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
