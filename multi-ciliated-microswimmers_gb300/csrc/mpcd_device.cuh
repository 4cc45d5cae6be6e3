// Device-side building blocks shared by the MPCD kernels.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#ifndef MPCD_HD
#define MPCD_HD __host__ __device__ __forceinline__
#endif

namespace mpcd {

// -------------------------------------------------------------- errors ---
// Bits of the device error word (read back by mpcd_sync / the getters).
enum : unsigned {
  kErrGammaMissing = 1u,   // injected Gamma < 0 for a cell that needs one
  kErrGammaLoop = 2u,      // Marsaglia-Tsang loop exceeded its iteration cap
  kErrBarrier = 4u,        // grid barrier wait exceeded its iteration cap
  kErrCellRange = 8u,      // a non-finite or out-of-range coordinate (e.g. an unstable MD step)
  kErrCellOverflow = 16u,  // more than 65535 particles of one kind in a cell
  kErrLayout = 32u,        // MD shared-memory layout smaller than the tile needs (planner mismatch)
};

// ----------------------------------------------------------- constants ---
// SRD rotation by 130 degrees: the reference's cos/sin constants
// (src/libcilia/mpcd.h:72-76), used as given.
constexpr double kCosAlpha = -0.6427876;
constexpr double kSinAlpha = 0.76604444;
constexpr double kPi = 3.14159265358979323846;

// ------------------------------------------------------------- Philox ---
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies on a 128-bit
// counter with a 64-bit key bumped by the Weyl constants each round.
struct u32x4 {
  uint32_t x, y, z, w;
};

MPCD_HD void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

MPCD_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(M0, c.x, hi0, lo0);
    mulhilo(M1, c.z, hi1, lo1);
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Stream identifiers: which quantity a counter block feeds.
enum : uint32_t { kStreamShift = 1, kStreamCell = 2, kStreamWall = 3, kStreamInit = 4 };

// counter = (index, step_lo, step_hi ^ (stream << 24), round)
MPCD_HD u32x4 draw4(uint64_t seed, uint64_t step, uint32_t stream, uint32_t index, uint32_t round) {
  u32x4 c{index, (uint32_t)step, (uint32_t)(step >> 32) ^ (stream << 24), round};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uniform in (0,1), 32-bit resolution, like MTRand::randDblExc
MPCD_HD double u01_dbl(uint32_t u) { return ((double)u + 0.5) * (1.0 / 4294967296.0); }
// uniform in (0,1), float (24-bit)
MPCD_HD float u01_flt(uint32_t u) { return ((float)(u >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// Gamma(k = 3(N-1)/2, 1) by Marsaglia & Tsang (2000), the method of
// src/libcilia/mpcd.cpp:13-43, driven by Philox draws in float.  The loop is
// capped; on exhaustion it returns the mean and sets *failed.
__device__ __forceinline__ float gamma_mt(int nc, uint64_t seed, uint64_t step, uint32_t cell, bool* failed) {
  const float d = 1.5f * (float)nc - 1.8333333333f;
  const float c = (1.0f / 3.0f) * rsqrtf(d);
  for (uint32_t round = 0; round < 64; ++round) {
    u32x4 r = draw4(seed, step, kStreamCell, cell, 16u + round);
    float u1 = u01_flt(r.x), u2 = u01_flt(r.y);
    float x = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    float v = 1.0f + c * x;
    if (v <= 0.0f) continue;
    v = v * v * v;
    float u = u01_flt(r.z);
    float x2 = x * x;
    if (u < 1.0f - 0.0331f * x2 * x2) return d * v;
    if (logf(u) < 0.5f * x2 + d * (1.0f - v + logf(v))) return d * v;
  }
  *failed = true;
  return d;
}

// Virtual particles of a wall-layer cell (src/libcilia/mpcd.cpp:175-198): dm
// particles of mass 1 at kT = 1 enter the cell's sums as one momentum vector
// with components sqrt(dm) N(0,1); the normals come from one counter block of
// the wall stream by Box-Muller (both branches of the first pair).
__device__ __forceinline__ void virtual_momentum(uint64_t seed, uint64_t step, uint32_t cell, int dm, double* p) {
  const u32x4 r = draw4(seed, step, kStreamWall, cell, 0u);
  const double r1 = sqrt(-2.0 * log(u01_dbl(r.x))), r3 = sqrt(-2.0 * log(u01_dbl(r.z)));
  double s2, c2;
  sincospi(2.0 * u01_dbl(r.y), &s2, &c2);
  const double c4 = cospi(2.0 * u01_dbl(r.w));
  const double sd = sqrt((double)dm);
  p[0] = sd * r1 * c2;
  p[1] = sd * r1 * s2;
  p[2] = sd * r3 * c4;
}

// ---------------------------------------------------------------- cells ---
// A particle's cell is packed as ix | iy << 10 | iz << 20 (edges up to 1024).
MPCD_HD uint32_t pack_cell(int ix, int iy, int iz) { return (uint32_t)ix | ((uint32_t)iy << 10) | ((uint32_t)iz << 20); }
MPCD_HD int cell_x(uint32_t c) { return (int)(c & 1023u); }
MPCD_HD int cell_y(uint32_t c) { return (int)((c >> 10) & 1023u); }
MPCD_HD int cell_z(uint32_t c) { return (int)((c >> 20) & 1023u); }

struct Box {
  int L[3];
  MPCD_HD int lin(int ix, int iy, int iz) const { return ix + L[0] * (iy + L[1] * iz); }
};

// Cell along one axis of an unwrapped coordinate, floor(x + a) - floor((x + a)/L) L
// (src/libcilia/mpcd.cpp:130-138).  Returns -1 for a non-finite or absurdly
// large coordinate, so that callers report an error instead of indexing with it.
MPCD_HD int unwrapped_cell_axis(double x, double a, int L) {
  const double xa = x + a;
  if (!(xa > -1.0e15 && xa < 1.0e15)) return -1;
  double c = floor(xa) - floor(xa / L) * L;
  if (c < 0) c += L;  // rounding edge where (x + a)/L rounds to an integer
  if (c >= L) c -= L;
  if (!(c >= 0.0 && c < (double)L)) return -1;
  return (int)c;
}

// linear cell of an unwrapped position, -1 if invalid
MPCD_HD long unwrapped_cell(const Box& b, const double* a, double x, double y, double z) {
  const int cx = unwrapped_cell_axis(x, a[0], b.L[0]);
  const int cy = unwrapped_cell_axis(y, a[1], b.L[1]);
  const int cz = unwrapped_cell_axis(z, a[2], b.L[2]);
  if (cx < 0 || cy < 0 || cz < 0) return -1;
  return cx + (long)b.L[0] * (cy + (long)b.L[1] * cz);
}

// A cell of the bottom or top layer in the reference's wall test
// (src/libcilia/mpcd.cpp:177-178; strict `>` at the top, so the first cell of
// the top layer is not one).
MPCD_HD bool wall_layer_cell(const Box& b, long cid) {
  const long layer = (long)b.L[0] * b.L[1];
  return cid < layer || cid > layer * (b.L[2] - 1);
}

// Count word of a cell: fluid particles in the low 16 bits, beads in the high.
MPCD_HD int cnt_fluid(uint32_t w) { return (int)(w & 0xffffu); }
MPCD_HD int cnt_beads(uint32_t w) { return (int)(w >> 16); }

// ----------------------------------------------------------- barriers ---
// Grid-wide barrier for cooperative launches: a monotonic arrival counter,
// reset to zero by the host before every launch.  The k-th barrier of a
// launch (k = 1, 2, ...) waits until the counter reaches k * nblocks.  Each
// CTA publishes its writes with one gpu-scope release add (cumulative over
// the CTA's writes, which __syncthreads made visible to the adding thread),
// then polls with acquire loads, back to back (the wait is the critical path
// of every MD substep).  Every wait is bounded: on timeout the CTA
// sets kErrBarrier in *err and returns false, and the caller leaves the kernel
// (the other CTAs then time out as well, so the launch always ends).
struct GridBarrier {
  unsigned* count;
  unsigned* gen;  // unused word next to the counter (both cleared per launch)
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_sync(const GridBarrier& b, unsigned target, unsigned* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(b.count) : "memory");
    unsigned long long spins = 0;
    while (ld_acquire(b.count) < target) {
      if (++spins > (1ull << 23)) {  // bounded wait (each poll is an L2 round trip: a few seconds)
        atomicOr(err, kErrBarrier);
        ok = 0;
        break;
      }
    }
  }
  __syncthreads();
  return ok != 0;
}

// 1 / sqrt(x) for x in the float range (about 1e-30 to 1e30): the float
// reciprocal square root (relative error about 2^-23) refined by one cubic
// step of the Householder iteration for f(y) = y^-2 - x: with r = 1 - x y^2,
// y' = y + y r (1/2 + 3/8 r), whose error is of order r^3 (about 2^-69), below
// float64 rounding (within about one ulp, like the library's rsqrt); five
// float64 operations, where GB300's float64 division and square root cost
// several times more
__device__ __forceinline__ double rsqrt_f64(double x) {
  const double y = (double)rsqrtf((float)x);
  const double r = fma(-x * y, y, 1.0);
  return fma(y * r, fma(0.375, r, 0.5), y);
}

}  // namespace mpcd
