// MPCD fluid kernels: per-cell collision maps, fused collide + stream + bin,
// bead coupling, observables and the periodic counting-sort reorder.
//
// One MPC step of the fluid (src/libcilia/mpcd.cpp:140-247 collision,
// src/libcilia/fluid.cpp:152-167 + mpcd.cpp:340-394 streaming, mpcd.cpp:257-267
// binning) is two kernels:
//   cell_params : per cell, from the sums binned at the end of the previous step:
//                 u = P/M, E_rel = K - M u^2, thermostat factor sc, rotation R,
//                 and the affine collision map v' = A v + b (A = sc R, b = u - A u);
//                 clears the sums for the next step.
//   fluid_step  : per particle: v' = A v + b with the map of its shifted cell,
//                 x' = x + v' h with periodic wrap, bin into the next shifted cell
//                 (atomic sums).  One read and one write of the particle state.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "engine_internal.h"
#include "fluid_device.cuh"

namespace mpcd {

namespace {

constexpr int kThreads = 256;

// Persistent grid-stride sizing: a few resident CTAs per SM, every thread
// handling many particles, so per-thread set-up and reductions amortise.
inline int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

inline int grid_for(long n, int threads = kThreads, int per_sm = 4) {
  long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (per_sm <= 0) {
    // not persistent: -per_sm items per thread, short-lived CTAs, at most
    // kMaxShortCTAs of them (more rounds per thread beyond that: every CTA
    // ends with one float64 atomic into the same dissipated-energy word;
    // 128^3 boxes measured best at about 10 k CTAs, like 64^3 ones)
    constexpr long kMaxShortCTAs = 10240;
    const long per = (long)threads * (per_sm < 0 ? -per_sm : 1);
    g = (n + per - 1) / per;
    return (int)(g < 1 ? 1 : (g > kMaxShortCTAs ? kMaxShortCTAs : g));
  }
  const long cap = (long)sm_count() * per_sm;
  return (int)(g < cap ? g : cap);
}

// Threshold 1 - a of one axis as the two 32-bit halves of its IEEE pattern.
struct Thresh {
  int hi;
  uint32_t lo;
};
__device__ __forceinline__ Thresh thresh(double t) { return {__double2hiint(t), (uint32_t)__double2loint(t)}; }

// shifted cell along one axis from the cell index and the in-cell offset:
// floor(i + o + a) = i + (o >= 1 - a), compared on the IEEE bit patterns
// (for a non-negative threshold, integer order of the patterns = numeric
// order), high word signed then low word unsigned: 32-bit integer
// instructions only (64-bit compares take GB300's small FP64 pipe)
__device__ __forceinline__ int shifted(int i, double o, Thresh t, int L) {
  const int hi = __double2hiint(o);
  const bool ge = hi > t.hi || (hi == t.hi && (uint32_t)__double2loint(o) >= t.lo);
  const int s = i + (ge ? 1 : 0);
  return s == L ? 0 : s;
}

// true unless 0 <= o < 1 (negative, -0, >= 1, NaN): one 32-bit compare of the
// high word (0x3FF00000 = high word of 1.0; the sign bit makes a negative
// pattern larger)
__device__ __forceinline__ bool off_unit(double o) { return (uint32_t)__double2hiint(o) >= 0x3FF00000u; }

// reduce an offset that left [0,1) back into the cell.  A streaming step
// moves a particle by less than one cell almost always: 1 <= o < 2 and
// -1 < o < 0 are told apart on the high word and corrected by one exact
// float64 add (the same result as o - floor(o), without the FP64 floor and
// compares); the general path takes the rest.
__device__ __forceinline__ void rewrap(double& o, int& i, int L, unsigned& bad) {
  const uint32_t hw = (uint32_t)__double2hiint(o);
  if (hw < 0x3FF00000u) return;  // 0 <= o < 1
  const bool up = hw < 0x40000000u;                       // 1 <= o < 2: o - 1 is exact
  const bool down = hw >= 0x80000000u && hw < 0xBFF00000u;  // -1 < o < 0 (or -0)
  if (up || down) {
    o += up ? -1.0 : 1.0;  // one add for either case
    if (up) {
      i = i + 1 == L ? 0 : i + 1;
    } else if (__double2hiint(o) == 0x3FF00000 && __double2loint(o) == 0) {
      o = 0.0;  // rounded up to 1: the particle stays in its cell at offset 0
    } else {
      i = i == 0 ? L - 1 : i - 1;
    }
    return;
  }
  if (off_unit(o)) {
    if (!(o > -1.0e9 && o < 1.0e9)) {  // non-finite: keep the particle in its cell and report
      o = 0.5;
      bad |= kErrCellRange;
      return;
    }
    double fl = floor(o);
    o -= fl;
    i += (int)fl;
    if (o >= 1.0) {  // o was a tiny negative number: o - floor(o) rounded to 1
      o = 0.0;
      i += 1;
    }
    i %= L;
    if (i < 0) i += L;
  }
}

// 1/n for the particle counts of bead-free cells, rounded once as the IEEE
// division rounds it (the same bits as 1.0 / n at run time), so that the
// common cell needs no float64 division on GB300's small FP64 pipe
struct InvTable {
  double v[256];
};
constexpr InvTable make_inv_table() {
  InvTable t{};
  for (int i = 1; i < 256; ++i) t.v[i] = 1.0 / i;
  return t;
}
__device__ const InvTable g_inv_n = make_inv_table();

// Free-running rotation axis of the float64 path: the direction drawn in
// float (cos theta = 2u - 1, phi = 2 pi u', as generate_collision_matrix,
// src/libcilia/mpcd.cpp:269-284), normalised in float64 so that the rotation
// is orthogonal to float64 precision.  |r|^2 = 1 + e with |e| of a few float
// roundings: two Newton steps for 1/sqrt from 1 (y1 = 1.5 - n2/2 is within
// 3e^2/8, y2 within float64 rounding) on the FMA chain instead of the general
// reciprocal square root.
__device__ __forceinline__ void draw_axis_f64(uint64_t seed, uint64_t step, uint32_t cid, double& rx, double& ry,
                                              double& rz) {
  const u32x4 r = draw4(seed, step, kStreamCell, cid, 0u);
  const float ct = 2.0f * u01_flt(r.y) - 1.0f;
  const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  float sp, cp;
  sincospif(2.0f * u01_flt(r.x), &sp, &cp);
  rx = (double)(st * cp);
  ry = (double)(st * sp);
  rz = (double)ct;
  const double n2 = fma(rx, rx, fma(ry, ry, rz * rz));
  const double y1 = fma(-0.5, n2, 1.5);
  const double y2 = y1 * fma(-0.5, (n2 * y1) * y1, 1.5);
  rx *= y2;
  ry *= y2;
  rz *= y2;
}

__device__ __forceinline__ void collision_map(double4 s, uint32_t w, long cid, const StepArgs& a, double* A,
                                              double* b, double& ldiss, unsigned& errbits, bool& gfail) {
  const int nf = cnt_fluid(w), nb = cnt_beads(w);
  int num = nf + nb;
  double M = (double)nf + (double)nb * a.bead_mass;
  const double preal[3] = {s.x, s.y, s.z}, mreal = M;  // the real particles' momentum and mass
  int sk = -1;  // rigid sphere whose surface cuts the cell
  double rel[3];
  if (a.sph.n && num < 10 && !(a.walls && wall_layer_cell(a.box, cid))) {
    const int L0 = a.box.L[0], L1 = a.box.L[1];
    sk = sphere_cut_cell(a.sph, a.box, a.a_cur, (int)(cid % L0), (int)((cid / L0) % L1), (int)(cid / ((long)L0 * L1)),
                         rel);
    if (sk >= 0) {  // virtual particles up to rho = 10, moving with the surface
      const int dm = 10 - num;
      double pv[3];
      sphere_virtual(a.sph.s[sk], rel, dm, a.seed, a.step, (uint32_t)cid, a.inj_virt, pv);
      s.x += pv[0];
      s.y += pv[1];
      s.z += pv[2];
      s.w += (pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]) / dm;
      M += dm;
      num += dm;
    }
  }
  if (a.walls && num < 10 && wall_layer_cell(a.box, cid)) {  // virtual particles up to rho = 10
    const int dm = 10 - num;
    double pv[3];
    if (a.inj_virt) {
      pv[0] = a.inj_virt[3 * cid];
      pv[1] = a.inj_virt[3 * cid + 1];
      pv[2] = a.inj_virt[3 * cid + 2];
    } else {
      virtual_momentum(a.seed, a.step, (uint32_t)cid, dm, pv);
    }
    s.x += pv[0];
    s.y += pv[1];
    s.z += pv[2];
    s.w += (pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]) / dm;
    M += dm;
    num += dm;
  }
  const double inv = (nb == 0 && num < 256) ? __ldg(g_inv_n.v + num) : 1.0 / M;  // M = num without beads
  const double ux = s.x * inv, uy = s.y * inv, uz = s.z * inv;
  const double erel = s.w - (ux * s.x + uy * s.y + uz * s.z);  // K - M u^2
  double sc = 1.0;
  if (erel > 0 && num > 1) {
    double g;
    if (a.inj_gamma) {
      g = a.inj_gamma[cid];
      if (g < 0) {
        errbits |= kErrGammaMissing;
        g = 0.0;
      }
    } else {
      g = (double)gamma_mt(num, a.seed, a.step, (uint32_t)cid, &gfail);
    }
    // sqrt(g / (erel / 2)) = 2g / sqrt(2g erel): one reciprocal square root in
    // place of a float64 division and square root (the cell pass is bound
    // by the float64 pipe); outside the float range the direct form
    const double q = 2.0 * g, x = q * erel;
    sc = (x > 1e-30 && x < 1e30) ? q * rsqrt_f64(x) : sqrt(g / (erel * 0.5));
  }
  double rx, ry, rz;
  if (a.inj_axis) {
    rx = a.inj_axis[3 * cid + 0];
    ry = a.inj_axis[3 * cid + 1];
    rz = a.inj_axis[3 * cid + 2];
  } else {
    draw_axis_f64(a.seed, a.step, (uint32_t)cid, rx, ry, rz);
  }
  const double ca = kCosAlpha, sa = kSinAlpha, oc = 1.0 - kCosAlpha;
  // A = sc R, R the rotation about (rx, ry, rz) by alpha with the entries of
  // src/libcilia/mpcd.cpp:285-293 (R_ii = r_i^2 + (1 - r_i^2) ca,
  // R_ij = r_i r_j (1 - ca) -+ r_k sa), the factor sc folded in:
  // A_ii = (sc oc r_i) r_i + sc ca, A_ij = (sc oc r_i) r_j -+ sc sa r_k
  const double sco = sc * oc, scc = sc * ca, scs = sc * sa;
  const double tx = sco * rx, ty = sco * ry, tz = sco * rz;
  const double qx = scs * rx, qy = scs * ry, qz = scs * rz;
  A[0] = fma(tx, rx, scc);
  A[1] = fma(tx, ry, -qz);
  A[2] = fma(tx, rz, qy);
  A[3] = fma(tx, ry, qz);
  A[4] = fma(ty, ry, scc);
  A[5] = fma(ty, rz, -qx);
  A[6] = fma(tx, rz, -qy);
  A[7] = fma(ty, rz, qx);
  A[8] = fma(tz, rz, scc);
  b[0] = ux - (A[0] * ux + A[1] * uy + A[2] * uz);
  b[1] = uy - (A[3] * ux + A[4] * uy + A[5] * uz);
  b[2] = uz - (A[6] * ux + A[7] * uy + A[8] * uz);
  if (sk >= 0) {
    // the real particles' momentum after the collision is A P + M b; what
    // they gained came from the virtual particles, i.e. from the sphere
    double J[3];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      J[q] = preal[q] - (A[3 * q] * preal[0] + A[3 * q + 1] * preal[1] + A[3 * q + 2] * preal[2] + mreal * b[q]);
    add_impulse(a.sph.acc + 6 * sk, rel, J);
  }
  // dissipated energy (src/libcilia/mpcd.cpp:166-168, 232-234, 243-246): every
  // cell adds sum m v^2 before the collision here, and every particle
  // subtracts its m v'^2 after it (fluid_step, bead_collide), so the total
  // matches the reference's bookkeeping including the rounding of its
  // rotation constants
  ldiss += s.w;
}

// ============================================================== float64 ===

__global__ void k_cell_params_f64(CellsF64 c, StepArgs a) {
  double ldiss = 0.0;
  unsigned errbits = 0;
  bool gfail = false;
  for (long cid = (long)blockIdx.x * blockDim.x + threadIdx.x; cid < c.ncell; cid += (long)gridDim.x * blockDim.x) {
    const uint32_t w = c.cnt[cid];
    if (w == 0) continue;
    const double4 s = c.sum[cid];
    c.sum[cid] = make_double4(0.0, 0.0, 0.0, 0.0);
    c.cnt[cid] = 0u;
    if (a.premapped && cnt_beads(w) > 0) continue;  // mapped by k_bead_maps_f64
    double A[9], b[3];
    collision_map(s, w, cid, a, A, b, ldiss, errbits, gfail);
    double2* p = reinterpret_cast<double2*>(c.par + 12 * cid);
    p[0] = make_double2(A[0], A[1]);
    p[1] = make_double2(A[2], A[3]);
    p[2] = make_double2(A[4], A[5]);
    p[3] = make_double2(A[6], A[7]);
    p[4] = make_double2(A[8], b[0]);
    p[5] = make_double2(b[1], b[2]);
  }
  if (gfail) errbits |= kErrGammaLoop;
  if (errbits) atomicOr(a.err, errbits);
  double tot = block_sum_f64(ldiss);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, tot);
}

// Walls along z (NOSLIP / SLIP, src/libcilia/mpcd.cpp:346-376): the channel is
// 0 <= z <= Lz - 1; a particle that crossed a wall during the streaming step
// is reflected.  Returns the (possibly changed) unwrapped z.
__device__ __forceinline__ void wall_bounce(int walls, double ztop, double& x, double& y, double& z, double& vx,
                                            double& vy, double& vz) {
  if (z > ztop) {
    if (walls == 1) {
      double t2 = (z - ztop) / vz;
      vx = -vx;
      vy = -vy;
      vz = -vz;
      x += 2.0 * t2 * vx;
      y += 2.0 * t2 * vy;
      z += 2.0 * t2 * vz;
    } else {
      vz = -vz;
      z = -z + ztop * 2.0;
    }
  }
  if (z < 0) {
    double t2 = z / vz;
    vx = -vx;
    vy = -vy;
    vz = -vz;
    x += vx * 2.0 * t2;
    y += vy * 2.0 * t2;
    z += vz * 2.0 * t2;
  }
}

// I: particle index type (32-bit whenever the particle count allows, so that
// no 64-bit integer work competes with the float64 arithmetic).
// kBoundary: walls or rigid spheres, streaming in unwrapped coordinates with
// bounce-back; a separate instantiation, so that the common periodic pass
// keeps the registers (about 60) that let its CTAs share the SMs with the MD
// launch (the sphere bounce-back alone takes the kernel to over 100).
template <typename I, bool kBoundary>
__global__ void __launch_bounds__(kThreads) k_fluid_step_f64(FluidF64 f, CellsF64 c, StepArgs a) {
  const int Lx = a.box.L[0], Ly = a.box.L[1], Lz = a.box.L[2];
  const Thresh tcx = thresh(a.ta_cur[0]), tcy = thresh(a.ta_cur[1]), tcz = thresh(a.ta_cur[2]);
  const Thresh tnx = thresh(a.ta_next[0]), tny = thresh(a.ta_next[1]), tnz = thresh(a.ta_next[2]);
  const double h = a.h, gk = a.gkick;
  const bool kick = gk != 0.0, walls = kBoundary;
  const I n = (I)f.n;
  double ke_after = 0.0;
  unsigned bad = 0;
  for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
    const uint32_t cp = f.cell[i];
    int ix = cell_x(cp), iy = cell_y(cp), iz = cell_z(cp);
    double ox = f.ox[i], oy = f.oy[i], oz = f.oz[i];
    double vx = f.vx[i], vy = f.vy[i], vz = f.vz[i];
    // collision with the map of the shifted cell (box cells < 2^30: 32-bit index)
    const uint32_t cid = (uint32_t)shifted(ix, ox, tcx, Lx) +
                         (uint32_t)Lx * ((uint32_t)shifted(iy, oy, tcy, Ly) + (uint32_t)Ly * (uint32_t)shifted(iz, oz, tcz, Lz));
    apply_map_f64(c.par + 12 * (size_t)cid, vx, vy, vz);
    const double k_post = vx * vx + vy * vy + vz * vz;
    ke_after += k_post;
    // streaming
    if (!walls) {
      ox = fma(vx, h, ox);
      oy = fma(vy, h, oy);
      oz = fma(vz, h, oz);
    } else {
      double x = ix + ox, y = iy + oy, z = iz + oz;
      double X[3] = {x, y, z}, V[3] = {vx, vy, vz};
      if (a.sph.n && sphere_bounce(a.sph, a.box, h, X, V)) {
        x = X[0];
        y = X[1];
        z = X[2];
        vx = V[0];
        vy = V[1];
        vz = V[2];
      } else {
        x += vx * h;
        y += vy * h;
        z += vz * h;
      }
      if (a.walls) wall_bounce(a.walls, (double)(Lz - 1), x, y, z, vx, vy, vz);
      double fx = floor(x), fy = floor(y), fz = floor(z);
      ox = x - fx;
      oy = y - fy;
      oz = z - fz;
      ix = (((int)fx % Lx) + Lx) % Lx;
      iy = (((int)fy % Ly) + Ly) % Ly;
      iz = (((int)fz % Lz) + Lz) % Lz;
    }
    rewrap(ox, ix, Lx, bad);
    rewrap(oy, iy, Ly, bad);
    rewrap(oz, iz, Lz, bad);
    if (kick) vx += gk;
    // bin with the next shift
    const uint32_t cn = (uint32_t)shifted(ix, ox, tnx, Lx) +
                        (uint32_t)Lx * ((uint32_t)shifted(iy, oy, tny, Ly) + (uint32_t)Ly * (uint32_t)shifted(iz, oz, tnz, Lz));
    const double K = (kick || walls) ? vx * vx + vy * vy + vz * vz : k_post;
    double* sp = reinterpret_cast<double*>(c.sum + cn);
    atomicAdd(sp + 0, vx);
    atomicAdd(sp + 1, vy);
    atomicAdd(sp + 2, vz);
    atomicAdd(sp + 3, K);
    atomicAdd(c.cnt + cn, 1u);
    f.cell[i] = pack_cell(ix, iy, iz);
    f.ox[i] = ox;
    f.oy[i] = oy;
    f.oz[i] = oz;
    f.vx[i] = vx;
    f.vy[i] = vy;
    f.vz[i] = vz;
  }
  if (bad) atomicOr(a.err, bad);
  const double tot = block_sum_f64(ke_after);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
}

__global__ void k_bin_fluid_f64(FluidF64 f, CellsF64 c, StepArgs a) {
  const int Lx = a.box.L[0], Ly = a.box.L[1], Lz = a.box.L[2];
  const Thresh tcx = thresh(a.ta_cur[0]), tcy = thresh(a.ta_cur[1]), tcz = thresh(a.ta_cur[2]);
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t cp = f.cell[i];
    const long cid = shifted(cell_x(cp), f.ox[i], tcx, Lx) +
                     (long)Lx * (shifted(cell_y(cp), f.oy[i], tcy, Ly) + (long)Ly * shifted(cell_z(cp), f.oz[i], tcz, Lz));
    const double vx = f.vx[i], vy = f.vy[i], vz = f.vz[i];
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, vx);
    atomicAdd(sp + 1, vy);
    atomicAdd(sp + 2, vz);
    atomicAdd(sp + 3, vx * vx + vy * vy + vz * vz);
    atomicAdd(c.cnt + cid, 1u);
  }
}

__global__ void k_bead_collide_f64(MDState m, CellsF64 c, StepArgs a) {
  double ke_after = 0.0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      atomicOr(a.err, kErrCellRange);
      continue;
    }
    double vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    apply_map_f64(c.par + 12 * cid, vx, vy, vz);
    ke_after += a.bead_mass * (vx * vx + vy * vy + vz * vz);
    m.vx[s] = vx;
    m.vy[s] = vy;
    m.vz[s] = vz;
  }
  const double tot = block_sum_f64(ke_after);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
}

__global__ void k_bin_beads_f64(MDState m, CellsF64 c, StepArgs a) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      atomicOr(a.err, kErrCellRange);
      continue;
    }
    const double mb = a.bead_mass, vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, vx * mb);
    atomicAdd(sp + 1, vy * mb);
    atomicAdd(sp + 2, vz * mb);
    atomicAdd(sp + 3, mb * (vx * vx + vy * vy + vz * vz));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
}

__global__ void k_observables_f64(FluidF64 f, MDState m, double bead_mass, double* out) {
  double px = 0, py = 0, pz = 0, e = 0, n = 0, ms = 0, ef = 0, nf = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const double vx = f.vx[i], vy = f.vy[i], vz = f.vz[i];
    const double v2 = vx * vx + vy * vy + vz * vz;
    px += vx;
    py += vy;
    pz += vz;
    e += v2;
    ef += v2;
    n += 1.0;
    ms += 1.0;
    nf += 1.0;
  }
  for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += (long)gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const double vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    px += bead_mass * vx;
    py += bead_mass * vy;
    pz += bead_mass * vz;
    e += bead_mass * (vx * vx + vy * vy + vz * vz);
    n += 1.0;
    ms += bead_mass;
  }
  double vals[8] = {px, py, pz, e, n, ms, ef, nf};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    double t = block_sum_f64(vals[k]);
    if (threadIdx.x == 0) atomicAdd(out + k, t);
  }
}

// Observables from the cell sums binned at the end of the last step (float64
// path): the sums hold every moving particle's m v and m v^2 once, so their
// totals are the fluid + bead momentum and energy, read from 36 B per cell
// instead of 24 B per particle.  The beads' own energy (moving beads, a few
// thousand) is summed beside it to split off the fluid's.  Per-block
// partials, added in block order by the last block to finish (no memset, no
// float atomics into the result); out = {P x, y, z, sum m v^2, n, mass,
// fluid sum v^2, fluid n, dissipated energy, error bits}, device memory or a
// mapped page-locked host slot (then no copy follows the kernel).
// GB300 runs float64 adds at a small fraction of its float32 rate, so the
// counts are summed as integers and the grid is one block per SM (fewer
// block reductions); four cells' loads are in flight per thread.
__global__ void __launch_bounds__(kThreads) k_observables_cells_f64(CellsF64 c, MDState m, double bead_mass,
                                                                    const double* diss, const unsigned* err,
                                                                    double* part, unsigned* counter, double* out) {
  double px = 0, py = 0, pz = 0, e = 0, eb = 0;
  uint32_t nf = 0, nb = 0;
  const long stride = (long)gridDim.x * blockDim.x;
  long cid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; cid + 3 * stride < c.ncell; cid += 4 * stride) {
    uint32_t w[4];
    double4 s[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) w[u] = c.cnt[cid + u * stride];
#pragma unroll
    for (int u = 0; u < 4; ++u) s[u] = c.sum[cid + u * stride];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (w[u] != 0) {
        px += s[u].x;
        py += s[u].y;
        pz += s[u].z;
        e += s[u].w;
        nf += (uint32_t)cnt_fluid(w[u]);
        nb += (uint32_t)cnt_beads(w[u]);
      }
  }
  for (; cid < c.ncell; cid += stride) {
    const uint32_t w = c.cnt[cid];
    if (w == 0) continue;
    const double4 s = c.sum[cid];
    px += s.x;
    py += s.y;
    pz += s.z;
    e += s.w;
    nf += (uint32_t)cnt_fluid(w);
    nb += (uint32_t)cnt_beads(w);
  }
  for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += stride) {
    if (m.moves[s] != 1) continue;
    const double vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    eb += bead_mass * (vx * vx + vy * vy + vz * vz);
  }
  // the counts as integers up to the block total, then exact in float64
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nf += __shfl_xor_sync(0xffffffffu, nf, o);
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
  }
  __shared__ uint32_t s_cnt[2][32];
  if ((threadIdx.x & 31) == 0) {
    s_cnt[0][threadIdx.x >> 5] = nf;
    s_cnt[1][threadIdx.x >> 5] = nb;
  }
  const double v5[5] = {px, py, pz, e, eb};
  __shared__ bool last;
  __shared__ double t5[5];
  __shared__ double tot[7];
  block_sums_f64<5>(v5, t5);  // t5 for every thread after it (its barriers order s_cnt too)
  if (threadIdx.x < 7) {  // partial k: P x, y, z, sum m v^2, fluid n, bead n, bead sum m v^2
    double r;
    if (threadIdx.x < 4) {
      r = t5[threadIdx.x];
    } else if (threadIdx.x == 6) {
      r = t5[4];
    } else {
      uint32_t t = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s_cnt[threadIdx.x - 4][i];
      r = (double)t;
    }
    part[7 * blockIdx.x + threadIdx.x] = r;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  double vals[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    double v = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += __ldcg(part + 7 * b + k);
    vals[k] = v;
  }
  block_sums_f64<7>(vals, tot);
  if (threadIdx.x == 0) {
    out[0] = tot[0];
    out[1] = tot[1];
    out[2] = tot[2];
    out[3] = tot[3];
    out[4] = tot[4] + tot[5];
    out[5] = tot[4] + tot[5] * bead_mass;
    out[6] = tot[3] - tot[6];
    out[7] = tot[4];
    out[8] = *diss;
    out[9] = (double)*err;  // bit flags (below 2^16): exact
    *counter = 0u;  // ready for the next call
  }
}

// ================================================================== sort ===

__global__ void k_sort_count(const uint32_t* cell, long n, Box box, uint32_t* count, uint32_t* rank) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t cp = cell[i];
    const long c = box.lin(cell_x(cp), cell_y(cp), cell_z(cp));
    rank[i] = atomicAdd(count + c, 1u);
  }
}

__global__ void k_sort_count_f32(const float4* pos, long n, Box box, uint32_t* count, uint32_t* rank) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t cp = __float_as_uint(pos[i].w);
    const long c = box.lin(cell_x(cp), cell_y(cp), cell_z(cp));
    rank[i] = atomicAdd(count + c, 1u);
  }
}

// exclusive scan of `count` (n entries) into `start`, three passes
constexpr int kScanBlock = 1024;

__global__ void k_scan_blocks(const uint32_t* in, long n, uint32_t* blocksums) {
  __shared__ uint32_t red[32];
  long i = (long)blockIdx.x * kScanBlock + threadIdx.x;
  uint32_t v = i < n ? in[i] : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t r = red[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) blocksums[blockIdx.x] = r;
  }
}

__global__ void k_scan_blocksums(uint32_t* blocksums, int nb) {
  // single block: sequential over chunks of 1024 with an in-block scan
  __shared__ uint32_t wsum[32];
  uint32_t carry = 0;
  for (int base = 0; base < nb; base += kScanBlock) {
    int i = base + threadIdx.x;
    uint32_t v = i < nb ? blocksums[i] : 0u;
    uint32_t x = v;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t w = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    uint32_t incl = x + (wid > 0 ? wsum[wid - 1] : 0u);
    if (i < nb) blocksums[i] = carry + incl - v;  // exclusive
    uint32_t total = wsum[31];
    __syncthreads();
    carry += total;
  }
}

__global__ void k_scan_apply(const uint32_t* in, long n, const uint32_t* blockoff, uint32_t* out) {
  __shared__ uint32_t wsum[32];
  long i = (long)blockIdx.x * kScanBlock + threadIdx.x;
  uint32_t v = i < n ? in[i] : 0u;
  uint32_t x = v;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  uint32_t incl = x + (wid > 0 ? wsum[wid - 1] : 0u);
  if (i < n) out[i] = blockoff[blockIdx.x] + incl - v;
}

__global__ void k_sort_scatter_f64(FluidF64 src, FluidF64 dst, Box box, const uint32_t* start, const uint32_t* rank) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < src.n; i += (long)gridDim.x * blockDim.x) {
    const uint32_t cp = src.cell[i];
    const long c = box.lin(cell_x(cp), cell_y(cp), cell_z(cp));
    const long d = (long)start[c] + rank[i];
    dst.id[d] = src.id[i];
    dst.cell[d] = cp;
    dst.ox[d] = src.ox[i];
    dst.oy[d] = src.oy[i];
    dst.oz[d] = src.oz[i];
    dst.vx[d] = src.vx[i];
    dst.vy[d] = src.vy[i];
    dst.vz[d] = src.vz[i];
  }
}

__global__ void k_sort_scatter_f32(FluidF32 src, FluidF32 dst, Box box, const uint32_t* start, const uint32_t* rank) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < src.n; i += (long)gridDim.x * blockDim.x) {
    const float4 p = src.pos[i];
    const uint32_t cp = __float_as_uint(p.w);
    const long c = box.lin(cell_x(cp), cell_y(cp), cell_z(cp));
    const long d = (long)start[c] + rank[i];
    dst.id[d] = src.id[i];
    dst.pos[d] = p;
    dst.vel[d] = src.vel[i];
  }
}

int scan_counts(const uint32_t* count, long ncell, uint32_t* start, uint32_t* blocksums, cudaStream_t s) {
  const int nb = (int)((ncell + kScanBlock - 1) / kScanBlock);
  k_scan_blocks<<<nb, kScanBlock, 0, s>>>(count, ncell, blocksums);
  k_scan_blocksums<<<1, kScanBlock, 0, s>>>(blocksums, nb);
  k_scan_apply<<<nb, kScanBlock, 0, s>>>(count, ncell, blocksums, start);
  return 3;
}

// ============================================================== float32 ===
// Split precision: position = packed cell + float32 offset, velocity float32,
// per-cell sums and collision maps float32.  The thermostat factor and the
// rotation are computed per cell in float64 and rounded once.

// Split-precision collision map: everything per cell in float (the sums
// are float); the dissipated-energy bookkeeping accumulates in float64.
__global__ void k_cell_params_f32(CellsF32 c, StepArgs a) {
  float ldiss = 0.0f;
  unsigned errbits = 0;
  bool gfail = false;
  // four cells per thread at a time, their loads issued together
  constexpr int kU = 4;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long cb = (long)blockIdx.x * blockDim.x + threadIdx.x; cb < c.ncell; cb += kU * stride) {
    uint32_t w[kU];
    float4 sm[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const long cid = cb + u * stride;
      w[u] = cid < c.ncell ? __ldcg(c.cnt + cid) : 0u;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) sm[u] = w[u] ? __ldcg(c.sum + cb + u * stride) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (!w[u]) continue;
      const long cid = cb + u * stride;
      c.sum[cid] = make_float4(0.f, 0.f, 0.f, 0.f);
      c.cnt[cid] = 0u;
      if (a.premapped && cnt_beads(w[u]) > 0) continue;  // mapped by k_bead_maps_f32
      cell_map_f32(sm[u], w[u], (uint32_t)cid, a.seed, a.step, a.fbead_mass, a.inj_gamma, a.inj_axis, c.par + 2 * cid,
                   ldiss, errbits, gfail, a.walls != 0 && wall_layer_cell(a.box, cid), a.inj_virt, &a);
    }
  }
  if (gfail) errbits |= kErrGammaLoop;
  if (errbits) atomicOr(a.err, errbits);
  const double tot = block_sum_f32(ldiss);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, tot);
}

// Particles per thread whose loads (state, then collision map) are issued
// together before any of their reductions and stores.  The pass is bound by
// the latency of the dependent chain particle -> cell -> map; the chains in
// flight per SM are bounded by the register file, so one, two and four per
// thread measured alike (two: 48.6 us on 2.6 M particles, one 47.5, four 58.8
// at half the resident CTAs).  MPCD_FLUID_BATCH selects 1, 2 or 4.
constexpr int kFluidBatch = 2;
// resident CTAs per SM the register budget of a batch size allows
template <int U>
struct FluidMinBlocks {
  static constexpr int value = U >= 4 ? 2 : 4;
};
// default options of the split-precision fluid pass (kOptPrefetch | kOptAggregate
// bits): both (2.62 M particles, persistent grid: 45.8 us against 49.2 us
// without either, 50.4 with the prefetch alone, 49.1 with the aggregation
// alone; the same order with one particle per thread)
constexpr int kFluidOpt = 3;

// Options of the split-precision fluid pass (bits of kOpt):
//   kOptPrefetch  one thread per CTA and round sends the particle state of the
//                 chunk `pf_dist` particles ahead (the chunk a later round or
//                 a later CTA takes) from HBM into L2 by a bulk prefetch, so
//                 that the dependent chain particle -> cell -> map starts
//                 from L2
//   kOptAggregate the warp's particles binned into the same next cell are
//                 summed in registers (peer_sum) and added by one vector
//                 reduction and one count add per cell and warp
constexpr int kOptPrefetch = 1;
constexpr int kOptAggregate = 2;

// kWalls: the bounce-back path (its float64 temporaries would otherwise
// crowd the registers of the batched loads).
template <int U, bool kWalls, typename I, int kOpt>
__global__ void __launch_bounds__(kThreads, FluidMinBlocks<U>::value)
    k_fluid_step_f32(FluidF32 f, CellsF32 c, StepArgs a, long pf_dist) {
  const int Lx = a.box.L[0], Ly = a.box.L[1], Lz = a.box.L[2];
  const float tcx = a.fta_cur[0], tcy = a.fta_cur[1], tcz = a.fta_cur[2];
  const float tnx = a.fta_next[0], tny = a.fta_next[1], tnz = a.fta_next[2];
  const float h = a.fh, gk = a.fgkick;
  float ke_after = 0.0f;
  unsigned bad = 0;
  const I n = (I)f.n;
  const I lane = (I)(threadIdx.x & 31);
  // each block takes U x blockDim consecutive particles per round; the loop
  // runs while the warp's first particle exists, so that every lane of a
  // warp takes part in the warp-wide operations of each round
  for (I base = (I)blockIdx.x * U * blockDim.x + threadIdx.x; base - lane < n; base += (I)gridDim.x * U * blockDim.x) {
    if ((kOpt & kOptPrefetch) && threadIdx.x == 0) {
      const long s = (long)base + pf_dist;
      if (s < (long)n) {
        const long cnt = min((long)U * blockDim.x, (long)n - s);
        prefetch_l2(f.pos + s, (uint32_t)(cnt * sizeof(float4)));
        prefetch_l2(f.vel + s, (uint32_t)(cnt * sizeof(float4)));
      }
    }
    float4 p[U], v[U], mk[U], mu[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const I i = base + (I)q * blockDim.x;
      if (i < n) {
        p[q] = __ldcs(f.pos + i);
        v[q] = __ldcs(f.vel + i);
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const I i = base + (I)q * blockDim.x;
      if (i < n) {
        const uint32_t cp = __float_as_uint(p[q].w);
        const uint32_t cid = (uint32_t)shifted_f(cell_x(cp), p[q].x, tcx, Lx) +
                             (uint32_t)Lx * ((uint32_t)shifted_f(cell_y(cp), p[q].y, tcy, Ly) +
                                             (uint32_t)Ly * (uint32_t)shifted_f(cell_z(cp), p[q].z, tcz, Lz));
        const float4* m = c.par + 2 * (size_t)cid;
        mk[q] = __ldg(m);
        mu[q] = __ldg(m + 1);
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const I i = base + (I)q * blockDim.x;
      if (kOpt & kOptAggregate) {
        if (base + (I)q * blockDim.x - lane >= n) continue;  // warp-uniform: no particle of this warp
      } else if (i >= n) {
        continue;
      }
      const bool valid = i < n;
      if (!valid) p[q] = v[q] = mk[q] = mu[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      const uint32_t cp = __float_as_uint(p[q].w);
      int ix = cell_x(cp), iy = cell_y(cp), iz = cell_z(cp);
      float ox = p[q].x, oy = p[q].y, oz = p[q].z, vx = v[q].x, vy = v[q].y, vz = v[q].z;
      apply_map_f32(mk[q], mu[q], vx, vy, vz);
      ke_after += vx * vx + vy * vy + vz * vz;
      if (!kWalls) {
        ox = fmaf(vx, h, ox);
        oy = fmaf(vy, h, oy);
        oz = fmaf(vz, h, oz);
      } else {
        double x = ix + (double)ox, y = iy + (double)oy, z = iz + (double)oz;
        double dvx = vx, dvy = vy, dvz = vz;
        double X[3] = {x, y, z}, V[3] = {dvx, dvy, dvz};
        if (a.sph.n && sphere_bounce(a.sph, a.box, a.h, X, V)) {
          x = X[0];
          y = X[1];
          z = X[2];
          dvx = V[0];
          dvy = V[1];
          dvz = V[2];
        } else {
          x += dvx * a.h;
          y += dvy * a.h;
          z += dvz * a.h;
        }
        if (a.walls) wall_bounce(a.walls, (double)(Lz - 1), x, y, z, dvx, dvy, dvz);
        double fx = floor(x), fy = floor(y), fz = floor(z);
        ox = (float)(x - fx);
        oy = (float)(y - fy);
        oz = (float)(z - fz);
        ix = (((int)fx % Lx) + Lx) % Lx;
        iy = (((int)fy % Ly) + Ly) % Ly;
        iz = (((int)fz % Lz) + Lz) % Lz;
        vx = (float)dvx;
        vy = (float)dvy;
        vz = (float)dvz;
      }
      rewrap_f(ox, ix, Lx, bad);
      rewrap_f(oy, iy, Ly, bad);
      rewrap_f(oz, iz, Lz, bad);
      if (gk != 0.0f) vx += gk;
      const uint32_t cn = (uint32_t)shifted_f(ix, ox, tnx, Lx) +
                          (uint32_t)Lx * ((uint32_t)shifted_f(iy, oy, tny, Ly) + (uint32_t)Ly * (uint32_t)shifted_f(iz, oz, tnz, Lz));
      const float4 contrib = make_float4(vx, vy, vz, vx * vx + vy * vy + vz * vz);
      if (kOpt & kOptAggregate) {
        const uint32_t key = valid ? cn : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const float4 tot = peer_sum(peers, valid ? contrib : make_float4(0.f, 0.f, 0.f, 0.f));
        if (valid && (unsigned)(__ffs(peers) - 1) == (unsigned)lane) {
          red_add_v4(c.sum + cn, tot);
          atomicAdd(c.cnt + cn, (uint32_t)__popc(peers));
        }
      } else {
        red_add_v4(c.sum + cn, contrib);
        atomicAdd(c.cnt + cn, 1u);
      }
      if (valid) {  // (a lane past the end carried a zero particle: nothing to store, nothing added to ke_after)
        __stcs(f.pos + i, make_float4(ox, oy, oz, __uint_as_float(pack_cell(ix, iy, iz))));
        __stcs(f.vel + i, make_float4(vx, vy, vz, 0.f));
      }
    }
  }
  if (bad) atomicOr(a.err, bad);
  const double tot = block_sum_f32(ke_after);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
}

__global__ void k_bin_fluid_f32(FluidF32 f, CellsF32 c, StepArgs a) {
  const int Lx = a.box.L[0], Ly = a.box.L[1], Lz = a.box.L[2];
  const float tcx = a.fta_cur[0], tcy = a.fta_cur[1], tcz = a.fta_cur[2];
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const float4 p = f.pos[i];
    const float4 v = f.vel[i];
    const uint32_t cp = __float_as_uint(p.w);
    const long cid = shifted_f(cell_x(cp), p.x, tcx, Lx) +
                     (long)Lx * (shifted_f(cell_y(cp), p.y, tcy, Ly) + (long)Ly * shifted_f(cell_z(cp), p.z, tcz, Lz));
    red_add_v4(c.sum + cid, make_float4(v.x, v.y, v.z, v.x * v.x + v.y * v.y + v.z * v.z));
    atomicAdd(c.cnt + cid, 1u);
  }
}

__global__ void k_bead_collide_f32(MDState m, CellsF32 c, StepArgs a) {
  double ke_after = 0.0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      atomicOr(a.err, kErrCellRange);
      continue;
    }
    float vx = (float)m.vx[s], vy = (float)m.vy[s], vz = (float)m.vz[s];
    apply_map_f32(c.par + 2 * cid, vx, vy, vz);
    ke_after += a.bead_mass * ((double)vx * vx + (double)vy * vy + (double)vz * vz);
    m.vx[s] = vx;
    m.vy[s] = vy;
    m.vz[s] = vz;
  }
  const double tot = block_sum_f64(ke_after);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, -tot);
}

__global__ void k_bin_beads_f32(MDState m, CellsF32 c, StepArgs a) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      atomicOr(a.err, kErrCellRange);
      continue;
    }
    const float mb = (float)a.bead_mass;
    const float vx = (float)m.vx[s], vy = (float)m.vy[s], vz = (float)m.vz[s];
    red_add_v4(c.sum + cid, make_float4(vx * mb, vy * mb, vz * mb, mb * (vx * vx + vy * vy + vz * vz)));
    atomicAdd(c.cnt + cid, 1u << 16);
  }
}

__global__ void k_observables_f32(FluidF32 f, MDState m, double bead_mass, double* out) {
  double px = 0, py = 0, pz = 0, e = 0, n = 0, ms = 0, ef = 0, nf = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const float4 v = f.vel[i];
    const double vx = v.x, vy = v.y, vz = v.z;
    const double v2 = vx * vx + vy * vy + vz * vz;
    px += vx;
    py += vy;
    pz += vz;
    e += v2;
    ef += v2;
    n += 1.0;
    ms += 1.0;
    nf += 1.0;
  }
  for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += (long)gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const double vx = m.vx[s], vy = m.vy[s], vz = m.vz[s];
    px += bead_mass * vx;
    py += bead_mass * vy;
    pz += bead_mass * vz;
    e += bead_mass * (vx * vx + vy * vy + vz * vz);
    n += 1.0;
    ms += bead_mass;
  }
  double vals[8] = {px, py, pz, e, n, ms, ef, nf};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    double t = block_sum_f64(vals[k]);
    if (threadIdx.x == 0) atomicAdd(out + k, t);
  }
}

// ====================================================== host interchange ===
// Fluid state to and from the caller's float64 arrays (positions N x 3,
// unwrapped allowed; velocities N x 3), staged in device memory as they
// are: the conversion to cell + offset, the split into the kernels' layout
// and the return to input order by particle id run here, one thread per
// particle, instead of in host loops.

// 1 for a non-finite or out-of-range (|x| > 1e12) position or velocity
__global__ void k_check_fluid(long n, const double* pos, const double* vel, unsigned* bad) {
  unsigned b = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += (long)gridDim.x * blockDim.x) {
    const double x = pos[i], v = vel[i];
    if (!(fabs(x) <= 1e12) || !isfinite(v)) b = 1u;
  }
  if (__syncthreads_or(b) && threadIdx.x == 0) atomicOr(bad, 1u);
}

// an unwrapped coordinate as cell index + offset in [0,1); explicit
// roundings (no contraction into a fused multiply-add) so that the result is
// the same as the host's plain float64 arithmetic
__device__ __forceinline__ void wrap_coord_dev(double x, int L, int& i, double& o) {
  const double dl = (double)L;
  double xw = __dsub_rn(x, __dmul_rn(floor(__ddiv_rn(x, dl)), dl));
  if (xw >= dl) xw = __dsub_rn(xw, dl);
  if (xw < 0) xw = __dadd_rn(xw, dl);
  const double fi = floor(xw);
  i = (int)fi;
  o = __dsub_rn(xw, fi);
  if (i >= L) i -= L;
  if (o >= 1.0) {
    o = 0.0;
    i = (i + 1) % L;
  }
}

__global__ void k_load_fluid_f64(long n, const double* pos, const double* vel, Box box, FluidF64 f) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    int c[3];
    double o[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) wrap_coord_dev(pos[3 * i + q], box.L[q], c[q], o[q]);
    f.id[i] = (uint32_t)i;
    f.cell[i] = pack_cell(c[0], c[1], c[2]);
    f.ox[i] = o[0];
    f.oy[i] = o[1];
    f.oz[i] = o[2];
    f.vx[i] = vel[3 * i];
    f.vy[i] = vel[3 * i + 1];
    f.vz[i] = vel[3 * i + 2];
  }
}

__global__ void k_load_fluid_f32(long n, const double* pos, const double* vel, Box box, FluidF32 f) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    int c[3];
    float o[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double od;
      wrap_coord_dev(pos[3 * i + q], box.L[q], c[q], od);
      o[q] = __double2float_rn(od);
      if (o[q] >= 1.0f) {  // rounding up to 1: move to the next cell
        o[q] = 0.0f;
        c[q] = (c[q] + 1) % box.L[q];
      }
    }
    f.id[i] = (uint32_t)i;
    f.pos[i] = make_float4(o[0], o[1], o[2], __uint_as_float(pack_cell(c[0], c[1], c[2])));
    f.vel[i] = make_float4(__double2float_rn(vel[3 * i]), __double2float_rn(vel[3 * i + 1]),
                           __double2float_rn(vel[3 * i + 2]), 0.0f);
  }
}

// back to input order: particle k of the caller is the one with id k
__global__ void k_store_fluid_f64(FluidF64 f, double* pos, double* vel, unsigned* bad) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const long d = f.id[i];
    if (d >= f.n) {
      atomicOr(bad, 1u);
      continue;
    }
    const uint32_t cp = f.cell[i];
    pos[3 * d] = __dadd_rn((double)cell_x(cp), f.ox[i]);
    pos[3 * d + 1] = __dadd_rn((double)cell_y(cp), f.oy[i]);
    pos[3 * d + 2] = __dadd_rn((double)cell_z(cp), f.oz[i]);
    vel[3 * d] = f.vx[i];
    vel[3 * d + 1] = f.vy[i];
    vel[3 * d + 2] = f.vz[i];
  }
}

__global__ void k_store_fluid_f32(FluidF32 f, double* pos, double* vel, unsigned* bad) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += (long)gridDim.x * blockDim.x) {
    const long d = f.id[i];
    if (d >= f.n) {
      atomicOr(bad, 1u);
      continue;
    }
    const float4 p = f.pos[i], v = f.vel[i];
    const uint32_t cp = __float_as_uint(p.w);
    pos[3 * d] = __dadd_rn((double)cell_x(cp), (double)p.x);
    pos[3 * d + 1] = __dadd_rn((double)cell_y(cp), (double)p.y);
    pos[3 * d + 2] = __dadd_rn((double)cell_z(cp), (double)p.z);
    vel[3 * d] = v.x;
    vel[3 * d + 1] = v.y;
    vel[3 * d + 2] = v.z;
  }
}

// The collision maps of the cells holding moving beads (the same map
// k_cell_params_* would make from the same sums and generator keys), one
// thread per bead slot; the first bead of a cell to take the cell's claim
// word with this step's tag makes it.  The sums are left for the cell-map
// kernel to clear.
__global__ void k_bead_maps_f64(MDState m, CellsF64 c, StepArgs a, uint32_t* claim, uint32_t tag) {
  double ldiss = 0.0;
  unsigned errbits = 0;
  bool gfail = false;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      errbits |= kErrCellRange;
      continue;
    }
    if (atomicExch(claim + cid, tag) == tag) continue;  // another bead of the cell makes it
    const uint32_t w = c.cnt[cid];
    if (w == 0) continue;
    double A[9], b[3];
    collision_map(c.sum[cid], w, cid, a, A, b, ldiss, errbits, gfail);
    double2* p = reinterpret_cast<double2*>(c.par + 12 * cid);
    p[0] = make_double2(A[0], A[1]);
    p[1] = make_double2(A[2], A[3]);
    p[2] = make_double2(A[4], A[5]);
    p[3] = make_double2(A[6], A[7]);
    p[4] = make_double2(A[8], b[0]);
    p[5] = make_double2(b[1], b[2]);
  }
  if (gfail) errbits |= kErrGammaLoop;
  if (errbits) atomicOr(a.err, errbits);
  const double tot = block_sum_f64(ldiss);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, tot);
}

__global__ void k_bead_maps_f32(MDState m, CellsF32 c, StepArgs a, uint32_t* claim, uint32_t tag) {
  float ldiss = 0.0f;
  unsigned errbits = 0;
  bool gfail = false;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const long cid = unwrapped_cell(a.box, a.a_cur, m.x[0][s], m.y[0][s], m.z[0][s]);
    if (cid < 0) {
      errbits |= kErrCellRange;
      continue;
    }
    if (atomicExch(claim + cid, tag) == tag) continue;
    const uint32_t w = c.cnt[cid];
    if (w == 0) continue;
    cell_map_f32(c.sum[cid], w, (uint32_t)cid, a.seed, a.step, a.fbead_mass, a.inj_gamma, a.inj_axis, c.par + 2 * cid,
                 ldiss, errbits, gfail, a.walls != 0 && wall_layer_cell(a.box, cid), a.inj_virt, &a);
  }
  if (gfail) errbits |= kErrGammaLoop;
  if (errbits) atomicOr(a.err, errbits);
  const double tot = block_sum_f32(ldiss);
  if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.diss, tot);
}

// the MD launch's deferred bead binning into the cell sums
__global__ void k_bead_add_f64(MDState m, CellsF64 c, const uint32_t* bcell, const double4* bsum) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const uint32_t cid = bcell[s];
    if (cid == 0xffffffffu) continue;
    const double4 v = bsum[s];
    double* sp = reinterpret_cast<double*>(c.sum + cid);
    atomicAdd(sp + 0, v.x);
    atomicAdd(sp + 1, v.y);
    atomicAdd(sp + 2, v.z);
    atomicAdd(sp + 3, v.w);
    atomicAdd(c.cnt + cid, 1u << 16);
  }
}

__global__ void k_bead_add_f32(MDState m, CellsF32 c, const uint32_t* bcell, const float4* bsum) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < m.nslots; s += gridDim.x * blockDim.x) {
    if (m.moves[s] != 1) continue;
    const uint32_t cid = bcell[s];
    if (cid == 0xffffffffu) continue;
    red_add_v4(c.sum + cid, bsum[s]);
    atomicAdd(c.cnt + cid, 1u << 16);
  }
}

// Rigid spheres after a step: the impulse and angular impulse the fluid gave
// them this step are added to the running force and torque sums (divided by
// h) and cleared; every sphere moves with the velocity it had during the
// step; a free sphere (mass > 0) then takes the impulses into its velocity
// and angular velocity (solid sphere, I = 2/5 m r^2).  Float64 throughout.
__global__ void k_spheres_update(RigidSphereDev* s, int n, double* acc, double* fsum, double h, Box box) {
  const int k = threadIdx.x;
  if (k >= n) return;
  RigidSphereDev S = s[k];
  double* A = acc + 6 * k;
  for (int j = 0; j < 6; ++j) fsum[6 * k + j] += A[j] / h;
  for (int q = 0; q < 3; ++q) {
    S.c[q] += S.v[q] * h;
    if (S.r < 0.5 * box.L[q]) {  // spheres with periodic images stay in [0, L)
      if (S.c[q] >= box.L[q]) S.c[q] -= box.L[q];
      if (S.c[q] < 0.0) S.c[q] += box.L[q];
    }
  }
  if (S.mass > 0.0) {
    for (int q = 0; q < 3; ++q) {
      S.v[q] += A[q] / S.mass;
      S.w[q] += A[3 + q] / S.inertia;
    }
  }
  for (int j = 0; j < 6; ++j) A[j] = 0.0;
  s[k] = S;
}

// The generator's per-cell draws, as the collision kernels take them: cell k
// of step `step` gets the Gamma(3(nc-1)/2) variate of gamma_mt and the
// float64 path's rotation axis.  Used to check the samplers' distributions.
__global__ void k_collision_draws(int nc, uint64_t seed, uint64_t step, long n, double* gamma, double* axis,
                                  unsigned* err) {
  bool gfail = false;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    if (gamma) gamma[k] = (double)gamma_mt(nc, seed, step, (uint32_t)k, &gfail);
    if (axis) draw_axis_f64(seed, step, (uint32_t)k, axis[3 * k], axis[3 * k + 1], axis[3 * k + 2]);
  }
  if (gfail) atomicOr(err, kErrGammaLoop);
}

}  // namespace

// ============================================================ launchers ===

int launch_bead_maps_f64(const MDState& m, const CellsF64& c, const StepArgs& a, uint32_t* claim, uint32_t tag,
                         cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_maps_f64<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a, claim, tag);
  return 1;
}
int launch_bead_maps_f32(const MDState& m, const CellsF32& c, const StepArgs& a, uint32_t* claim, uint32_t tag,
                         cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_maps_f32<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a, claim, tag);
  return 1;
}
int launch_bead_add_f64(const MDState& m, const CellsF64& c, const uint32_t* bcell, const void* bsum, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_add_f64<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, bcell, static_cast<const double4*>(bsum));
  return 1;
}
int launch_bead_add_f32(const MDState& m, const CellsF32& c, const uint32_t* bcell, const void* bsum, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_add_f32<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, bcell, static_cast<const float4*>(bsum));
  return 1;
}

int launch_spheres_update(RigidSphereDev* sph, int n, double* acc, double* fsum, double h, const Box& box,
                          cudaStream_t s) {
  if (n <= 0) return 0;
  k_spheres_update<<<1, 32, 0, s>>>(sph, n, acc, fsum, h, box);
  return 1;
}

int launch_collision_draws(int nc, uint64_t seed, uint64_t step, long n, double* gamma, double* axis, unsigned* err,
                           cudaStream_t s) {
  if (n == 0) return 0;
  k_collision_draws<<<grid_for(n), kThreads, 0, s>>>(nc, seed, step, n, gamma, axis, err);
  return 1;
}

int launch_cell_params_f64(const CellsF64& c, const StepArgs& a, cudaStream_t s) {
  k_cell_params_f64<<<grid_for(c.ncell), kThreads, 0, s>>>(c, a);
  return 1;
}
int launch_fluid_step_f64(const FluidF64& f, const CellsF64& c, const StepArgs& a, cudaStream_t s, int per_sm) {
  if (f.n == 0) return 0;
  const int grid = grid_for(f.n, kThreads, per_sm);
  const bool i32 = f.n + (long)grid * kThreads < (1L << 32);
  if (a.walls != 0 || a.sph.n > 0)
    i32 ? k_fluid_step_f64<uint32_t, true><<<grid, kThreads, 0, s>>>(f, c, a)
        : k_fluid_step_f64<long, true><<<grid, kThreads, 0, s>>>(f, c, a);
  else
    i32 ? k_fluid_step_f64<uint32_t, false><<<grid, kThreads, 0, s>>>(f, c, a)
        : k_fluid_step_f64<long, false><<<grid, kThreads, 0, s>>>(f, c, a);
  return 1;
}
int launch_bin_fluid_f64(const FluidF64& f, const CellsF64& c, const StepArgs& a, cudaStream_t s) {
  if (f.n == 0) return 0;
  k_bin_fluid_f64<<<grid_for(f.n), kThreads, 0, s>>>(f, c, a);
  return 1;
}
int launch_bead_collide_f64(const MDState& m, const CellsF64& c, const StepArgs& a, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_collide_f64<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a);
  return 1;
}
int launch_bin_beads_f64(const MDState& m, const CellsF64& c, const StepArgs& a, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bin_beads_f64<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a);
  return 1;
}
int launch_observables_cells_f64(const CellsF64& c, const MDState& m, double bead_mass, const double* diss,
                                 const unsigned* err, double* part, unsigned* counter, double* out, cudaStream_t s) {
  const long n = c.ncell > m.nslots ? c.ncell : m.nslots;
  const int g1 = grid_for(n, kThreads, 1);  // at most one block per SM
  const int g = g1 < kObsBlocks ? g1 : kObsBlocks;
  k_observables_cells_f64<<<g, kThreads, 0, s>>>(c, m, bead_mass, diss, err, part, counter, out);
  return 1;
}
int launch_observables_f64(const FluidF64& f, const MDState& m, double bead_mass, double* out, cudaStream_t s) {
  long n = f.n > m.nslots ? f.n : m.nslots;
  k_observables_f64<<<grid_for(n) < 1024 ? grid_for(n) : 1024, kThreads, 0, s>>>(f, m, bead_mass, out);
  return 1;
}
int launch_sort_f64(FluidF64& f, FluidF64& tmp, const Box& box, uint32_t* count, uint32_t* start, uint32_t* rank,
                    uint32_t* blocksums, cudaStream_t s) {
  const long ncell = (long)box.L[0] * box.L[1] * box.L[2];
  cudaMemsetAsync(count, 0, ncell * sizeof(uint32_t), s);
  k_sort_count<<<grid_for(f.n), kThreads, 0, s>>>(f.cell, f.n, box, count, rank);
  int k = 1 + scan_counts(count, ncell, start, blocksums, s);
  tmp.n = f.n;
  k_sort_scatter_f64<<<grid_for(f.n), kThreads, 0, s>>>(f, tmp, box, start, rank);
  FluidF64 t = f;
  f = tmp;
  tmp = t;
  return k + 1;
}

int scan_counts_ext(const uint32_t* count, long ncell, uint32_t* start, uint32_t* blocksums, cudaStream_t s) {
  return scan_counts(count, ncell, start, blocksums, s);
}

int launch_cell_params_f32(const CellsF32& c, const StepArgs& a, cudaStream_t s) {
  k_cell_params_f32<<<grid_for(c.ncell), kThreads, 0, s>>>(c, a);
  return 1;
}
template <int U, int kOpt>
void launch_fluid_f32_opt(const FluidF32& f, const CellsF32& c, const StepArgs& a, cudaStream_t s, int per_sm) {
  const int ps = per_sm <= 0 ? per_sm : std::min(per_sm, FluidMinBlocks<U>::value);
  const int gb = grid_for((f.n + U - 1) / U, kThreads, ps);
  const bool i32 = f.n + 4L * gb * kThreads < (1L << 32);
  long pf = 0;
  if (kOpt & kOptPrefetch) {
    // the chunk the CTA starting after the current wave (or this CTA's next
    // round, for a grid of at most one wave) will take
    static int resident = 0;
    if (resident == 0) {
      int per = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fluid_step_f32<U, false, uint32_t, kOpt>, kThreads, 0);
      resident = std::max(1, per) * sm_count();
    }
    pf = (long)std::min(gb, resident) * U * kThreads;
  }
  if (i32)
    k_fluid_step_f32<U, false, uint32_t, kOpt><<<gb, kThreads, 0, s>>>(f, c, a, pf);
  else
    k_fluid_step_f32<U, false, long, kOpt><<<gb, kThreads, 0, s>>>(f, c, a, pf);
}

int launch_fluid_step_f32(const FluidF32& f, const CellsF32& c, const StepArgs& a, cudaStream_t s, int per_sm) {
  if (f.n == 0) return 0;
  if (a.walls != 0 || a.sph.n > 0) {
    const int g1 = grid_for(f.n, kThreads, per_sm);
    const bool i32 = f.n + 4L * g1 * kThreads < (1L << 32);
    i32 ? k_fluid_step_f32<1, true, uint32_t, 0><<<g1, kThreads, 0, s>>>(f, c, a, 0)
        : k_fluid_step_f32<1, true, long, 0><<<g1, kThreads, 0, s>>>(f, c, a, 0);
    return 1;
  }
  // particles per thread and round: kFluidBatch unless MPCD_FLUID_BATCH (1, 2) says otherwise;
  // options: kFluidOpt unless MPCD_FLUID_OPT (0..3: bit 0 prefetch, bit 1 aggregation) says otherwise
  static const int batch = [] {
    const char* e = std::getenv("MPCD_FLUID_BATCH");
    const int b = e ? std::atoi(e) : kFluidBatch;
    return b == 1 ? 1 : 2;
  }();
  static const int opt = [] {
    const char* e = std::getenv("MPCD_FLUID_OPT");
    const int o = e ? std::atoi(e) : kFluidOpt;
    return o & 3;
  }();
  switch (batch * 4 + opt) {
    case 4: launch_fluid_f32_opt<1, 0>(f, c, a, s, per_sm); break;
    case 5: launch_fluid_f32_opt<1, 1>(f, c, a, s, per_sm); break;
    case 6: launch_fluid_f32_opt<1, 2>(f, c, a, s, per_sm); break;
    case 7: launch_fluid_f32_opt<1, 3>(f, c, a, s, per_sm); break;
    case 8: launch_fluid_f32_opt<2, 0>(f, c, a, s, per_sm); break;
    case 9: launch_fluid_f32_opt<2, 1>(f, c, a, s, per_sm); break;
    case 10: launch_fluid_f32_opt<2, 2>(f, c, a, s, per_sm); break;
    default: launch_fluid_f32_opt<2, 3>(f, c, a, s, per_sm); break;
  }
  return 1;
}
int launch_bin_fluid_f32(const FluidF32& f, const CellsF32& c, const StepArgs& a, cudaStream_t s) {
  if (f.n == 0) return 0;
  k_bin_fluid_f32<<<grid_for(f.n), kThreads, 0, s>>>(f, c, a);
  return 1;
}
int launch_bead_collide_f32(const MDState& m, const CellsF32& c, const StepArgs& a, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bead_collide_f32<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a);
  return 1;
}
int launch_bin_beads_f32(const MDState& m, const CellsF32& c, const StepArgs& a, cudaStream_t s) {
  if (m.nslots == 0) return 0;
  k_bin_beads_f32<<<grid_for(m.nslots), kThreads, 0, s>>>(m, c, a);
  return 1;
}
int launch_observables_f32(const FluidF32& f, const MDState& m, double bead_mass, double* out, cudaStream_t s) {
  long n = f.n > m.nslots ? f.n : m.nslots;
  k_observables_f32<<<grid_for(n) < 1024 ? grid_for(n) : 1024, kThreads, 0, s>>>(f, m, bead_mass, out);
  return 1;
}
int launch_sort_f32(FluidF32& f, FluidF32& tmp, const Box& box, uint32_t* count, uint32_t* start, uint32_t* rank,
                    uint32_t* blocksums, cudaStream_t s) {
  const long ncell = (long)box.L[0] * box.L[1] * box.L[2];
  cudaMemsetAsync(count, 0, ncell * sizeof(uint32_t), s);
  k_sort_count_f32<<<grid_for(f.n), kThreads, 0, s>>>(f.pos, f.n, box, count, rank);
  int k = 1 + scan_counts(count, ncell, start, blocksums, s);
  tmp.n = f.n;
  k_sort_scatter_f32<<<grid_for(f.n), kThreads, 0, s>>>(f, tmp, box, start, rank);
  FluidF32 t = f;
  f = tmp;
  tmp = t;
  return k + 1;
}

int launch_check_fluid(long n, const double* pos, const double* vel, unsigned* bad, cudaStream_t s) {
  if (n == 0) return 0;
  k_check_fluid<<<grid_for(3 * n), kThreads, 0, s>>>(n, pos, vel, bad);
  return 1;
}
int launch_load_fluid_f64(long n, const double* pos, const double* vel, const Box& box, const FluidF64& f,
                          cudaStream_t s) {
  if (n == 0) return 0;
  k_load_fluid_f64<<<grid_for(n), kThreads, 0, s>>>(n, pos, vel, box, f);
  return 1;
}
int launch_load_fluid_f32(long n, const double* pos, const double* vel, const Box& box, const FluidF32& f,
                          cudaStream_t s) {
  if (n == 0) return 0;
  k_load_fluid_f32<<<grid_for(n), kThreads, 0, s>>>(n, pos, vel, box, f);
  return 1;
}
int launch_store_fluid_f64(const FluidF64& f, double* pos, double* vel, unsigned* bad, cudaStream_t s) {
  if (f.n == 0) return 0;
  k_store_fluid_f64<<<grid_for(f.n), kThreads, 0, s>>>(f, pos, vel, bad);
  return 1;
}
int launch_store_fluid_f32(const FluidF32& f, double* pos, double* vel, unsigned* bad, cudaStream_t s) {
  if (f.n == 0) return 0;
  k_store_fluid_f32<<<grid_for(f.n), kThreads, 0, s>>>(f, pos, vel, bad);
  return 1;
}

}  // namespace mpcd
