// Pieces shared by the cooperative-grid MD kernels (md_kernels.cu: float64 and
// split spring arithmetic; md_df.cu: double-float arithmetic): the cilia's
// active rest lengths and beat state machine, the staged-position layouts in
// shared memory, and the binning of beads into the next collision's cells.
#pragma once
#include "engine_internal.h"
#include "fluid_device.cuh"

namespace mpcd {

namespace {

// Cilia::length(i) (src/cilia.cpp:79-121), first part: the beat's rest
// length of bond i for the current midpoint (constant during one MPC step's
// substeps; the midpoint moves in switch_logic after them)
__device__ inline double cilium_target(const CiliumDev& cl, int i, double midpnt) {
  const double bondlength = 0.5;
  if (i < midpnt - 2.0) {
    // base^2.5 as base^2 sqrt(base) (base > 0 for every refreshed bond)
    const double base = 1.0 - (i - cl.num_anker - 1.0) / (cl.len - cl.num_anker - 1.0);
    return bondlength + cl.beatstrength * (base * base * sqrt(base)) * 0.5 * (1.0 - 1.0 / (midpnt - i - 1.0));
  }
  const double di = i - midpnt;
  return bondlength - 2.0 * cl.beatstrength / (di * di + 1.0);
}

// Cilia::length(i), second part: the change from the previous rest length is
// limited by the bending rate; l is the target, tl the bond's current length
__device__ inline double cilium_limit(double l, double bending, double oldlen, double tl) {
  if (fabs(l - tl) > bending) {
    tl = tl + bending - 2.0 * bending * (l < tl ? 1.0 : 0.0);
    if ((l - oldlen) * (tl - oldlen) > 0) {
      l = tl;
    } else {
      l = oldlen;
    }
  }
  return l;
}
__device__ inline double cilium_length(const CiliumDev& cl, int i, double midpnt, double oldlen, double tl) {
  return cilium_limit(cilium_target(cl, i, midpnt), cl.bending, oldlen, tl);
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

// Cilia::localbend(0, rodlength) (src/cilia.cpp:68-77) from staged positions
template <typename St>
__device__ double cilium_localbend(const CiliumDev& cl, int l0, const St& st) {
  double l = 0.0;
  const int sd = cl.stride;
  for (int i = 0; i < cl.len - 1; ++i) {
    l += 2.0 * st.dist(l0 + sd * i, l0 + sd * (i + 1));
    l -= st.dist(l0 + sd * (cl.len + i), l0 + sd * (cl.len + i + 1));
    l -= st.dist(l0 + sd * (2 * cl.len + i), l0 + sd * (2 * cl.len + i + 1));
  }
  return l;
}

// switch_logic of cilium c at time t (src/cilia.cpp:241-258,
// src/ConstantBeatCilia.cpp:8-23); `st` holds the tile's staged positions
template <typename St>
__device__ void cilium_switch(const MDState& m, const MDStepArgs& a, int c, double t, int base, const St& st) {
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
    if (cilium_localbend(cl, cl.slot0 - base, st) > cl.max_bend && mp > cl.start) {
      ts = t;
      mp = cl.start;
    }
  }
  if (mp > cl.start) mp += a.tstep / cl.m_speed;
  m.midpnt[c] = mp;
  m.tstroke[c] = ts;
}

struct BinF64 {
  using Cells = CellsF64;
  CellsF64 c;
  const MDStepArgs* a;
  // a moving bead in the collision (its cell's map, MPCD::next_tstep,
  // src/libcilia/mpcd.cpp:140-247): the new velocity and its m v'^2, as k_bead_collide_f64
  __device__ double collide(double x, double y, double z, double& vx, double& vy, double& vz) const {
    const long cid = unwrapped_cell(a->box, a->a_cur, x, y, z);
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      return 0.0;
    }
    apply_map_f64(c.par + 12 * cid, vx, vy, vz);
    return a->bead_mass * (vx * vx + vy * vy + vz * vz);
  }
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
  // the same contribution kept per slot (MDStepArgs::deferred)
  __device__ void defer(int slot, double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(a->box, a->a_next, x, y, z);
    uint32_t* bc = a->bcell;
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      bc[slot] = 0xffffffffu;
      return;
    }
    const double mb = a->bead_mass;
    bc[slot] = (uint32_t)cid;
    static_cast<double4*>(a->bsum)[slot] = make_double4(vx * mb, vy * mb, vz * mb, mb * (vx * vx + vy * vy + vz * vz));
  }
};

struct BinF32 {
  using Cells = CellsF32;
  CellsF32 c;
  const MDStepArgs* a;
  // as k_bead_collide_f32: the map applied in float to the rounded velocity
  __device__ double collide(double x, double y, double z, double& vx, double& vy, double& vz) const {
    const long cid = unwrapped_cell(a->box, a->a_cur, x, y, z);
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      return 0.0;
    }
    float fx = (float)vx, fy = (float)vy, fz = (float)vz;
    apply_map_f32(c.par + 2 * cid, fx, fy, fz);
    vx = fx;
    vy = fy;
    vz = fz;
    return a->bead_mass * ((double)fx * fx + (double)fy * fy + (double)fz * fz);
  }
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
  // the same contribution kept per slot (MDStepArgs::deferred)
  __device__ void defer(int slot, double x, double y, double z, double vx, double vy, double vz) const {
    const long cid = unwrapped_cell(a->box, a->a_next, x, y, z);
    uint32_t* bc = a->bcell;
    if (cid < 0) {
      atomicOr(a->err, kErrCellRange);
      bc[slot] = 0xffffffffu;
      return;
    }
    const float mb = (float)a->bead_mass;
    const float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    bc[slot] = (uint32_t)cid;
    static_cast<float4*>(a->bsum)[slot] = make_float4(fvx * mb, fvy * mb, fvz * mb, mb * (fvx * fvx + fvy * fvy + fvz * fvz));
  }
};

}  // namespace

}  // namespace mpcd
