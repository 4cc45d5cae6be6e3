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
  const float ca = (float)kCosAlpha, sa = (float)kSinAlpha, oc = 1.0f - (float)kCosAlpha;
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
  const float A00 = sc * (rx * rx + (1.0f - rx * rx) * ca), A01 = sc * (rx * ry * oc - rz * sa),
              A02 = sc * (rx * rz * oc + ry * sa);
  const float A10 = sc * (rx * ry * oc + rz * sa), A11 = sc * (ry * ry + (1.0f - ry * ry) * ca),
              A12 = sc * (ry * rz * oc - rx * sa);
  const float A20 = sc * (rx * rz * oc - ry * sa), A21 = sc * (ry * rz * oc + rx * sa),
              A22 = sc * (rz * rz + (1.0f - rz * rz) * ca);
  float4* p = par_out;
  p[0] = make_float4(A00, A01, A02, ux - (A00 * ux + A01 * uy + A02 * uz));
  p[1] = make_float4(A10, A11, A12, uy - (A10 * ux + A11 * uy + A12 * uz));
  p[2] = make_float4(A20, A21, A22, uz - (A20 * ux + A21 * uy + A22 * uz));
  ldiss += s.w;
}

__device__ __forceinline__ void apply_map_f32(const float4* par, float& vx, float& vy, float& vz) {
  const float4 r0 = __ldg(par + 0), r1 = __ldg(par + 1), r2 = __ldg(par + 2);
  const float nx = fmaf(r0.x, vx, fmaf(r0.y, vy, fmaf(r0.z, vz, r0.w)));
  const float ny = fmaf(r1.x, vx, fmaf(r1.y, vy, fmaf(r1.z, vz, r1.w)));
  const float nz = fmaf(r2.x, vx, fmaf(r2.y, vy, fmaf(r2.z, vz, r2.w)));
  vx = nx;
  vy = ny;
  vz = nz;
}

}  // namespace mpcd
