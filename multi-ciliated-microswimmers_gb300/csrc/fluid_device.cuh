// Device helpers shared by the single-box fluid kernels (fluid_kernels.cu)
// and the replica batch (batch_kernels.cu).
#pragma once
#include "engine_internal.h"

namespace mpcd {

// sum over the block, float lanes, one float64 result (thread 0)
__device__ __forceinline__ double block_sum_f32(float v) {
  __shared__ double red32[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red32[wid] = (double)v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += red32[w];
  return r;
}

__device__ __forceinline__ double block_sum_f64(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// N sums over the block at once (blockDim.x a multiple of 32, N <= 32):
// shuffles within each warp, then one shared-memory round adds the warps in
// warp order; out (shared) holds the totals for every thread on return.
template <int N>
__device__ __forceinline__ void block_sums_f64(const double (&v)[N], double* out) {
  __shared__ double red[N][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double w[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    w[k] = x;
  }
  __syncthreads();  // earlier readers of red and out are done
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) red[k][wid] = w[k];
  }
  __syncthreads();
  if (threadIdx.x < N) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[threadIdx.x][i];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ int shifted_f(int i, float o, float ta, int L) {
  int s = i + (o >= ta ? 1 : 0);
  return s == L ? 0 : s;
}

__device__ __forceinline__ void rewrap_f(float& o, int& i, int L, unsigned& bad) {
  if (o < 0.0f || o >= 1.0f) {
    if (!(o > -1.0e9f && o < 1.0e9f)) {
      o = 0.5f;
      bad |= kErrCellRange;
      return;
    }
    float fl = floorf(o);
    o -= fl;
    i += (int)fl;
    if (o >= 1.0f) {
      o = 0.0f;
      i += 1;
    }
    i %= L;
    if (i < 0) i += L;
  }
}

// Vector reduction into a cell sum.  No "memory" clobber: the sums are only
// reduced into during a kernel (never read back in it), so the compiler may
// move the other loads and stores of the thread across it.
__device__ __forceinline__ void red_add_v4(float4* addr, float4 v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w));
}

// Bulk prefetch of `bytes` (a multiple of 16, 16-byte aligned) from global
// memory into L2, no destination in the SM: the state of particles a later
// round (or a later CTA) will read is on its way from HBM before any warp
// waits on it.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Sum of x over the lanes holding the same key (peers = __match_any_sync of
// the key): a tree over the peers' ranks, one round per doubling of the
// largest group (log2 of it), every lane taking part in every shuffle.  The
// lowest lane of each group ends with the group's total; the other lanes'
// results are partial.  (Peer reduction by rank halving, E. Westphal's
// warp-aggregated atomics with __match_any_sync.)
__device__ __forceinline__ float4 peer_sum(unsigned peers, float4 x) {
  const int lane = threadIdx.x & 31;
  int rank = __popc(peers & ((1u << lane) - 1u));
  unsigned up = peers & (0xfffffffeu << lane);  // my peers above me still holding a value
  while (__any_sync(0xffffffffu, up != 0u)) {
    const int next = __ffs(up);  // 1-based lane of the next peer above, 0: none
    const int src = next ? next - 1 : lane;
    const float tx = __shfl_sync(0xffffffffu, x.x, src), ty = __shfl_sync(0xffffffffu, x.y, src);
    const float tz = __shfl_sync(0xffffffffu, x.z, src), tw = __shfl_sync(0xffffffffu, x.w, src);
    if (next) {
      x.x += tx;
      x.y += ty;
      x.z += tz;
      x.w += tw;
    }
    // odd ranks were added into their lower neighbour this round: drop them
    up &= ~__ballot_sync(0xffffffffu, rank & 1);
    rank >>= 1;
  }
  return x;
}

// ------------------------------------------------------- rigid spheres ---
// No-slip bounce-back off rigid spheres and virtual particles in the cells
// their surface cuts: the reference's planar-wall rules (bounce-back
// src/libcilia/mpcd.cpp:346-376, virtual particles mpcd.cpp:175-198)
// generalised to a sphere that may move and rotate.  Exchanges with the fluid
// are accumulated in float64 (impulse and angular impulse per sphere).

// displacement x - c along one axis: the nearest periodic image for spheres
// smaller than half the box, the plain difference for larger ones (a sphere
// far larger than the box stands for a curved wall and has no images)
__device__ __forceinline__ double sph_disp(double x, double c, int L, double r) {
  double d = x - c;
  if (r < 0.5 * L) {
    if (d > 0.5 * L)
      d -= L;
    else if (d < -0.5 * L)
      d += L;
  }
  return d;
}

__device__ __forceinline__ void add_impulse(double* acc, const double* rc, const double* J) {
  atomicAdd(acc + 0, J[0]);
  atomicAdd(acc + 1, J[1]);
  atomicAdd(acc + 2, J[2]);
  atomicAdd(acc + 3, rc[1] * J[2] - rc[2] * J[1]);
  atomicAdd(acc + 4, rc[2] * J[0] - rc[0] * J[2]);
  atomicAdd(acc + 5, rc[0] * J[1] - rc[1] * J[0]);
}

// One streaming step of a particle (mass 1) that starts at x (any periodic
// image) with the post-collision velocity v, against the rigid spheres.
// Returns false when it touches none (the caller streams it freely);
// otherwise x and v are replaced by its end position and velocity: it moves
// to the first contact with the surface (the sphere moving with its
// velocity during the step), leaves with v' = 2 u_s - v, u_s the surface
// velocity V + W x r_c at the contact, for the rest of the step, and the
// sphere receives the impulse v - v' and its moment.  A particle found
// inside at the start (after the sphere moved onto it) is put on the surface
// along the radius and reflected there if it approaches the centre; one that
// is leaving (a particle a previous reflection left on the surface) streams
// freely, as it would a hair outside: otherwise a rounding-level difference
// in the sphere's state decides whether it is turned back.
__device__ __forceinline__ bool sphere_bounce(const SphereSet& ss, const Box& box, double h, double* x, double* v) {
  for (int k = 0; k < ss.n; ++k) {
    const RigidSphereDev& S = ss.s[k];
    const double R = S.r;
    double r0[3], w[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      r0[q] = sph_disp(x[q], S.c[q], box.L[q], R);
      w[q] = v[q] - S.v[q];
    }
    const double A = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double B = r0[0] * w[0] + r0[1] * w[1] + r0[2] * w[2];
    const double C = r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2] - R * R;
    double tc, rc[3];
    if (C < 0.0) {  // inside at the start: onto the surface along the radius
      if (B >= 0.0) continue;  // leaving
      const double s = R / sqrt(C + R * R);
      tc = 0.0;
#pragma unroll
      for (int q = 0; q < 3; ++q) rc[q] = r0[q] * s;
    } else {
      // first root of |r0 + w t| = R within the step, moving inwards
      if (B >= 0.0 || A == 0.0) continue;
      const double disc = B * B - A * C;
      if (disc < 0.0) continue;
      tc = C / (-B + sqrt(disc));  // = (-B - sqrt(disc)) / A, without cancellation
      if (tc > h) continue;
#pragma unroll
      for (int q = 0; q < 3; ++q) rc[q] = r0[q] + w[q] * tc;
    }
    double vn[3], J[3], re[3];
    const double us[3] = {S.v[0] + S.w[1] * rc[2] - S.w[2] * rc[1], S.v[1] + S.w[2] * rc[0] - S.w[0] * rc[2],
                          S.v[2] + S.w[0] * rc[1] - S.w[1] * rc[0]};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      vn[q] = 2.0 * us[q] - v[q];
      J[q] = v[q] - vn[q];
      re[q] = rc[q] + (vn[q] - S.v[q]) * (h - tc);  // relative position at the end of the step
    }
    const double e2 = re[0] * re[0] + re[1] * re[1] + re[2] * re[2];
    if (e2 < R * R) {  // a rotating surface can leave it inside: onto the surface
      const double s = R / sqrt(e2 > 0.0 ? e2 : 1e-300);
#pragma unroll
      for (int q = 0; q < 3; ++q) re[q] *= s;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      x[q] += (re[q] - r0[q]) + S.v[q] * h;
      v[q] = vn[q];
    }
    add_impulse(ss.acc + 6 * k, rc, J);
    return true;
  }
  return false;
}

// The rigid sphere whose surface cuts shifted cell (sx, sy, sz) of a grid
// shifted by a, or -1; rel receives the cell centre relative to the sphere
// centre.  A cell is cut when its nearest point lies inside the sphere and
// its farthest point outside.
__device__ __forceinline__ int sphere_cut_cell(const SphereSet& ss, const Box& box, const double* a, int sx, int sy,
                                               int sz, double* rel) {
  const int sc[3] = {sx, sy, sz};
  for (int k = 0; k < ss.n; ++k) {
    const RigidSphereDev& S = ss.s[k];
    double dn = 0.0, df = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      rel[q] = sph_disp((double)sc[q] + 0.5 - a[q], S.c[q], box.L[q], S.r);
      const double e = fabs(rel[q]);
      const double n = e > 0.5 ? e - 0.5 : 0.0;
      dn += n * n;
      df += (e + 0.5) * (e + 0.5);
    }
    if (dn < S.r * S.r && df > S.r * S.r) return k;
  }
  return -1;
}

// Virtual particles of a cut cell holding num < 10 particles: dm = 10 - num
// particles of unit mass moving with the surface velocity at the cell centre
// plus thermal noise at kT = 1 (the wall rule of src/libcilia/mpcd.cpp:
// 175-198, whose wall is at rest): momentum p = dm u_s + sqrt(dm) N(0,1)^3
// (or the injected thermal part).
__device__ __forceinline__ void sphere_virtual(const RigidSphereDev& S, const double* rel, int dm, uint64_t seed,
                                               uint64_t step, uint32_t cid, const double* inj_virt, double* p) {
  if (inj_virt) {
    p[0] = inj_virt[3 * cid];
    p[1] = inj_virt[3 * cid + 1];
    p[2] = inj_virt[3 * cid + 2];
  } else {
    virtual_momentum(seed, step, cid, dm, p);
  }
  const double us[3] = {S.v[0] + S.w[1] * rel[2] - S.w[2] * rel[1], S.v[1] + S.w[2] * rel[0] - S.w[0] * rel[2],
                        S.v[2] + S.w[0] * rel[1] - S.w[1] * rel[0]};
  p[0] += dm * us[0];
  p[1] += dm * us[1];
  p[2] += dm * us[2];
}

// Split-precision collision map of one cell (MPCD::next_tstep,
// src/libcilia/mpcd.cpp:140-247): mean velocity, relative kinetic energy, the
// MBS thermostat factor from a Gamma(3(N-1)/2) draw and the rotation about a
// random axis, written as three float4 rows (A row, b) of v' = A v + b.  The
// cell's sum m v^2 before the collision goes into ldiss.  `cid` keys the
// generator (the cell's index within its own box).
__device__ __forceinline__ void cell_map_f32(const float4 s0, const uint32_t w, const uint32_t cid, const uint64_t seed,
                                             const uint64_t step, const float mb, const double* inj_gamma,
                                             const double* inj_axis, float4* par_out, float& ldiss, unsigned& errbits,
                                             bool& gfail, const bool wall_cell = false,
                                             const double* inj_virt = nullptr, const StepArgs* sa = nullptr) {
  const int nf = cnt_fluid(w), nb = cnt_beads(w);
  int num = nf + nb;
  float M = (float)nf + (float)nb * mb;
  float4 s = s0;
  int sk = -1;  // rigid sphere whose surface cuts the cell
  double rel[3];
  if (sa && sa->sph.n && num < 10 && !wall_cell) {
    const int L0 = sa->box.L[0], L1 = sa->box.L[1];
    sk = sphere_cut_cell(sa->sph, sa->box, sa->a_cur, (int)(cid % L0), (int)((cid / L0) % L1),
                         (int)(cid / ((uint32_t)L0 * L1)), rel);
    if (sk >= 0) {  // virtual particles up to rho = 10, moving with the surface
      const int dm = 10 - num;
      double pv[3];
      sphere_virtual(sa->sph.s[sk], rel, dm, seed, step, cid, inj_virt, pv);
      s.x += (float)pv[0];
      s.y += (float)pv[1];
      s.z += (float)pv[2];
      s.w += (float)((pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]) / dm);
      M += (float)dm;
      num += dm;
    }
  }
  if (wall_cell && num < 10) {  // virtual particles up to rho = 10 (src/libcilia/mpcd.cpp:175-198)
    const int dm = 10 - num;
    double pv[3];
    if (inj_virt) {
      pv[0] = inj_virt[3 * cid];
      pv[1] = inj_virt[3 * cid + 1];
      pv[2] = inj_virt[3 * cid + 2];
    } else {
      virtual_momentum(seed, step, cid, dm, pv);
    }
    s.x += (float)pv[0];
    s.y += (float)pv[1];
    s.z += (float)pv[2];
    s.w += (float)((pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]) / dm);
    M += (float)dm;
    num += dm;
  }
  const float inv = 1.0f / M;
  const float ux = s.x * inv, uy = s.y * inv, uz = s.z * inv;
  const float erel = s.w - (ux * s.x + uy * s.y + uz * s.z);
  float sc = 1.0f;
  if (erel > 0.f && num > 1) {
    float g;
    if (inj_gamma) {
      g = (float)inj_gamma[cid];
      if (g < 0.f) {
        errbits |= kErrGammaMissing;
        g = 0.f;
      }
    } else {
      g = gamma_mt(num, seed, step, cid, &gfail);
    }
    sc = sqrtf(2.0f * g / erel);
  }
  float rx, ry, rz;
  if (inj_axis) {
    rx = (float)inj_axis[3 * cid + 0];
    ry = (float)inj_axis[3 * cid + 1];
    rz = (float)inj_axis[3 * cid + 2];
  } else {
    const u32x4 r = draw4(seed, step, kStreamCell, cid, 0u);
    const float ct = 2.0f * u01_flt(r.y) - 1.0f;
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float sp, cp;
    sincospif(2.0f * u01_flt(r.x), &sp, &cp);
    rx = st * cp;
    ry = st * sp;
    rz = ct;
  }
  // v' = u + sc R (v - u), R the rotation about (rx, ry, rz) with the
  // reference's matrix entries (src/libcilia/mpcd.cpp:285-293), applied as
  // R w = ca w + sa (r x w) + (1 - ca) (r . w) r: one 32-byte map per cell
  float4* p = par_out;
  p[0] = make_float4(rx, ry, rz, sc);
  p[1] = make_float4(ux, uy, uz, 0.0f);
  ldiss += s.w;
  if (sk >= 0) {
    // the real particles' momentum after the collision, in float64:
    // M u + sc R (P - M u) (R applied in Rodrigues form, as apply_map_f32);
    // what they gained came from the virtual particles, i.e. from the sphere
    const double Mr = (double)nf + (double)nb * mb;
    const double u[3] = {ux, uy, uz}, r[3] = {rx, ry, rz};
    const double q[3] = {(double)s0.x - Mr * u[0], (double)s0.y - Mr * u[1], (double)s0.z - Mr * u[2]};
    const double ca = kCosAlpha, sa_ = kSinAlpha, oc = 1.0 - kCosAlpha;
    const double rq = oc * (r[0] * q[0] + r[1] * q[1] + r[2] * q[2]);
    const double cr[3] = {r[1] * q[2] - r[2] * q[1], r[2] * q[0] - r[0] * q[2], r[0] * q[1] - r[1] * q[0]};
    const double p0[3] = {s0.x, s0.y, s0.z};
    double J[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) J[k] = p0[k] - (Mr * u[k] + (double)sc * (ca * q[k] + sa_ * cr[k] + rq * r[k]));
    add_impulse(sa->sph.acc + 6 * sk, rel, J);
  }
}

// v' = A v + b with the float64 map of one cell (A row-major, then b)
__device__ __forceinline__ void apply_map_f64(const double* par, double& vx, double& vy, double& vz) {
  const double2* p = reinterpret_cast<const double2*>(par);
  const double2 p0 = __ldg(p + 0), p1 = __ldg(p + 1), p2 = __ldg(p + 2);
  const double2 p3 = __ldg(p + 3), p4 = __ldg(p + 4), p5 = __ldg(p + 5);
  const double nx = fma(p0.x, vx, fma(p0.y, vy, fma(p1.x, vz, p4.y)));
  const double ny = fma(p1.y, vx, fma(p2.x, vy, fma(p2.y, vz, p5.x)));
  const double nz = fma(p3.x, vx, fma(p3.y, vy, fma(p4.x, vz, p5.y)));
  vx = nx;
  vy = ny;
  vz = nz;
}

// v' = u + sc R (v - u) with the map k = {rx, ry, rz, sc}, u = {ux, uy, uz, 0}
__device__ __forceinline__ void apply_map_f32(const float4 k, const float4 u, float& vx, float& vy, float& vz) {
  const float ca = (float)kCosAlpha, sa = (float)kSinAlpha, oc = 1.0f - (float)kCosAlpha;
  const float wx = vx - u.x, wy = vy - u.y, wz = vz - u.z;
  const float kw = oc * (k.x * wx + k.y * wy + k.z * wz);
  const float cx = k.y * wz - k.z * wy, cy = k.z * wx - k.x * wz, cz = k.x * wy - k.y * wx;
  vx = fmaf(k.w, fmaf(ca, wx, fmaf(sa, cx, kw * k.x)), u.x);
  vy = fmaf(k.w, fmaf(ca, wy, fmaf(sa, cy, kw * k.y)), u.y);
  vz = fmaf(k.w, fmaf(ca, wz, fmaf(sa, cz, kw * k.z)), u.z);
}

__device__ __forceinline__ void apply_map_f32(const float4* par, float& vx, float& vy, float& vz) {
  apply_map_f32(__ldg(par + 0), __ldg(par + 1), vx, vy, vz);
}

}  // namespace mpcd
