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
                                             const double* inj_virt = nullptr) {
  const int nf = cnt_fluid(w), nb = cnt_beads(w);
  int num = nf + nb;
  float M = (float)nf + (float)nb * mb;
  float4 s = s0;
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
