// Double-float arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum h + l of two floats; normalised pairs have
// |l| <= ulp(h) / 2, about 48 significand bits.  The building blocks are the
// error-free transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the
// product error of a fused multiply-add (TwoProd); the sums and products
// follow the double-double algorithms of Dekker (1971) and of Hida, Li and
// Bailey's QD library, with floats in place of doubles.  The __f*_rn
// intrinsics keep the compiler from contracting the steps whose rounding
// error is being captured.
#pragma once
#include <cuda_runtime.h>

namespace mpcd {

struct dfloat {
  float h, l;
};

// s + e == a + b exactly, s = fl(a + b)
__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// as df_two_sum when |a| >= |b| (or a == 0)
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// p + e == a * b exactly, p = fl(a * b)
__device__ __forceinline__ dfloat df_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, fmaf(a, b, -p)};
}

// normalised a + b
__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.h, b.h);
  const dfloat t = df_two_sum(a.l, b.l);
  dfloat r = df_fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return df_fast_two_sum(r.h, __fadd_rn(r.l, t.l));
}

// normalised a * b
__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
  const dfloat p = df_two_prod(a.h, b.h);
  return df_fast_two_sum(p.h, fmaf(a.h, b.l, fmaf(a.l, b.h, p.l)));
}

// compensated accumulation: h carries the rounded running sum, l the sum of
// the rounding errors (and of the addends' low parts); normalise at the end
__device__ __forceinline__ void df_acc(float& h, float& l, float gh, float gl) {
  const dfloat s = df_two_sum(h, gh);
  h = s.h;
  l = __fadd_rn(l, __fadd_rn(s.l, gl));
}

__device__ __forceinline__ dfloat df_norm(float h, float l) { return df_two_sum(h, l); }

__device__ __forceinline__ dfloat df_neg(dfloat a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dfloat df_sub(dfloat a, dfloat b) { return df_add(a, df_neg(b)); }

// comparisons and sign of normalised pairs
__device__ __forceinline__ bool df_lt(dfloat a, dfloat b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ int df_sign(dfloat a) {
  return a.h > 0.0f ? 1 : (a.h < 0.0f ? -1 : (a.l > 0.0f ? 1 : (a.l < 0.0f ? -1 : 0)));
}
__device__ __forceinline__ dfloat df_abs(dfloat a) { return df_sign(a) < 0 ? df_neg(a) : a; }

// 1/sqrt(a) for a normalised positive pair: the rsqrtf seed y refined by one
// third-order step r = y (1 + e/2 + 3e^2/8), e = 1 - a y^2 formed from exact
// products (Karp and Markstein, "High-precision division and square root",
// ACM TOMS 23, 1997); relative error about 2^-46
__device__ __forceinline__ dfloat df_rsqrt(dfloat a) {
  const float y = rsqrtf(a.h);
  const dfloat yy = df_two_prod(y, y);
  const dfloat t = df_two_prod(a.h, yy.h);
  const float e = ((__fsub_rn(1.0f, t.h) - t.l) - a.h * yy.l) - a.l * yy.h;
  return df_fast_two_sum(y, y * e * fmaf(0.375f, e, 0.5f));
}

__device__ __forceinline__ dfloat df_sqrt(dfloat a) { return df_mul(a, df_rsqrt(a)); }

__host__ __device__ inline dfloat df_from_double(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

__host__ __device__ inline double df_to_double(dfloat a) { return (double)a.h + (double)a.l; }

}  // namespace mpcd
