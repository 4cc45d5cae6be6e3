// Bead coordinates of the double-float MD kernels (md_df.cu, md_pair.cu):
// an integer cell plus an offset held as a pair of floats, exact differences
// of two coordinates, and the Verlet updates in pairs.
#pragma once
#include <cstdint>

#include "df32.cuh"

namespace mpcd {

namespace {

// A bead coordinate is an integer c plus an offset o in [0, 1) held as a
// pair: o.h on the grid of multiples of 2^-24 (so that the difference of two
// offsets is exact in float) and o.l the rest, |o.l| <= 2^-25.  Its resolution
// (about 2^-48) does not depend on the distance from the origin.  Staged and
// published entry: two float4,
//   {ohx, ohy, ohz, olx} and {oly, olz, bits(cx | cy << 16), cz}
// (cx, cy as 16-bit integers, cz as a float).
struct BeadCoord {
  int c;
  dfloat o;
};
constexpr float kGrid = 16777216.0f;  // 2^24
__device__ __forceinline__ BeadCoord coord_from_double(double x) {
  const double c = floor(x);
  const double o = x - c;                     // exact
  const double h = floor(o * 16777216.0) / 16777216.0;  // exact, on the grid
  return {(int)c, {(float)h, (float)(o - h)}};
}
__device__ __forceinline__ double coord_to_double(const BeadCoord& q) {
  return (double)q.c + ((double)q.o.h + (double)q.o.l);
}
// q += v c; the offset's high part back on the grid and in [0, 1)
__device__ __forceinline__ void coord_kick(BeadCoord& q, dfloat v, dfloat c) {
  const dfloat o = df_add(q.o, df_mul(v, c));
  float g = __fmul_rn(rintf(__fmul_rn(o.h, kGrid)), 1.0f / kGrid);  // exact
  const float lo = __fadd_rn(__fsub_rn(o.h, g), o.l);                  // o.h - g exact
  const float k = floorf(g);
  g = __fsub_rn(g, k);  // exact: a grid value minus an integer
  q.c += (int)k;
  q.o = {g, lo};
}
__device__ __forceinline__ void pack_coords(const BeadCoord& x, const BeadCoord& y, const BeadCoord& z, float4& p0,
                                            float4& p1) {
  p0 = make_float4(x.o.h, y.o.h, z.o.h, x.o.l);
  p1 = make_float4(y.o.l, z.o.l, __uint_as_float(((uint32_t)x.c & 0xffffu) | ((uint32_t)y.c << 16)), (float)z.c);
}
__device__ __forceinline__ int cell_x(const float4 p1) { return (int)(short)(__float_as_uint(p1.z) & 0xffffu); }
__device__ __forceinline__ int cell_y(const float4 p1) { return (int)__float_as_uint(p1.z) >> 16; }

struct StageDF {
  const float4* p;
  // float64 distance (switch_logic's bend measure)
  __device__ double dist(int i, int j) const {
    const float4 a0 = p[2 * i], a1 = p[2 * i + 1], b0 = p[2 * j], b1 = p[2 * j + 1];
    const double dx = (double)(cell_x(a1) - cell_x(b1)) + (df_to_double({a0.x, a0.w}) - df_to_double({b0.x, b0.w}));
    const double dy = (double)(cell_y(a1) - cell_y(b1)) + (df_to_double({a0.y, a1.x}) - df_to_double({b0.y, b1.x}));
    const double dz = ((double)a1.w - (double)b1.w) + (df_to_double({a0.z, a1.y}) - df_to_double({b0.z, b1.y}));
    return sqrt(dx * dx + dy * dy + dz * dz);
  }
};

// one component of a difference: the cells' difference dc (an exact small
// integer) plus the high parts' (exact: both on the 2^-24 grid, |difference|
// < 1), summed exactly (FastTwoSum: |dc| >= 1 > |s| or dc == 0), then the
// low parts
__device__ __forceinline__ dfloat coord_diff(float dc, float ha, float hb, float la, float lb) {
  const dfloat t = df_fast_two_sum(dc, __fsub_rn(ha, hb));
  return {t.h, __fadd_rn(t.l, __fsub_rn(la, lb))};
}

// Difference of two staged positions as pairs and its squared length as a
// normalised pair.
struct DfDiff {
  dfloat dx, dy, dz, d2;
};
__device__ __forceinline__ DfDiff df_diff(const float4 a0, const float4 a1, const float4 b0, const float4 b1) {
  DfDiff r;
  r.dx = coord_diff((float)(cell_x(a1) - cell_x(b1)), a0.x, b0.x, a0.w, b0.w);
  r.dy = coord_diff((float)(cell_y(a1) - cell_y(b1)), a0.y, b0.y, a1.x, b1.x);
  r.dz = coord_diff(__fsub_rn(a1.w, b1.w), a0.z, b0.z, a1.y, b1.y);
  const dfloat px = df_two_prod(r.dx.h, r.dx.h), py = df_two_prod(r.dy.h, r.dy.h), pz = df_two_prod(r.dz.h, r.dz.h);
  const dfloat q1 = df_two_sum(px.h, py.h);
  const dfloat q2 = df_two_sum(q1.h, pz.h);
  float low = (q1.l + q2.l) + (px.l + py.l + pz.l);
  low += 2.0f * (r.dx.h * r.dx.l + r.dy.h * r.dy.l + r.dz.h * r.dz.l);
  low += r.dx.l * r.dx.l + r.dy.l * r.dy.l + r.dz.l * r.dz.l;
  r.d2 = df_fast_two_sum(q2.h, low);
  return r;
}

// v += F c (pairs)
__device__ __forceinline__ void kick(dfloat& v, dfloat f, dfloat c) { v = df_add(v, df_mul(f, c)); }

}  // namespace

}  // namespace mpcd
