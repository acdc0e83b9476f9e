// fe_df.cuh -- double-float ("float-float") arithmetic for the few places of
// the mixed-precision path whose sums must match the FP64 oracle far below
// FP32's rounding: the intramolecular Ewald correction energy, a large sum of
// same-sign terms (one per excluded pair) that cancels most of the Ewald self
// energy.  A value is an unevaluated sum hi + lo of two floats (about 48
// significant bits); the building blocks are the error-free transformations
// of Knuth (TwoSum) and Dekker / FMA (TwoProduct).  On this GPU FP32 runs 70x
// faster than FP64, so a double-float operation of 5-20 FP32 instructions is
// much cheaper than the FP64 one.
//
// The exponential uses exp(x) = exp(k/64) * exp(r), |r| <= 1/128, with the
// table exp(k/64) in double-float computed on the host in FP64 and a degree-4
// Taylor polynomial for exp(r) (truncation below 3e-13 relative).
#pragma once

#include <cmath>

namespace fe {

struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dfl df_quick_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ dfl df_from_double(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__host__ inline void df_split(double x, float &hi, float &lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}
// an integer of up to 2^53 exactly as hi + lo
__device__ __forceinline__ dfl df_from_ll(long long x) {
  float h = __ll2float_rn(x);
  return {h, __ll2float_rn(x - __float2ll_rn(h))};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, b.hi);
  dfl t = df_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = df_quick_sum(s.hi, s.lo);
  s.lo += t.lo;
  return df_quick_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  dfl p = df_two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return df_quick_sum(p.hi, p.lo);
}
__device__ __forceinline__ dfl df_mul_f(dfl a, float b) {
  dfl p = df_two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return df_quick_sum(p.hi, p.lo);
}
// 1 / a: IEEE float reciprocal refined by one Newton step in double-float
__device__ __forceinline__ dfl df_recip(dfl a) {
  float y = 1.0f / a.hi;
  dfl e = df_add({1.0f, 0.0f}, df_neg(df_mul_f(a, y)));  // 1 - a y, about 2^-24
  return df_quick_sum(y, y * e.hi);
}
// sqrt(a), a > 0: IEEE float root refined by one Newton step
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  float s = sqrtf(a.hi);
  dfl p = df_two_prod(s, s);
  float d = ((a.hi - p.hi) - p.lo) + a.lo;  // a - s^2, small and exact enough
  return df_quick_sum(s, d * 0.5f / s);
}

constexpr int kDfExpLo = -1024;  // table of exp(k/64), k in [kDfExpLo, kDfExpHi]
constexpr int kDfExpHi = 64;
constexpr int kDfExpN = kDfExpHi - kDfExpLo + 1;

// exp(x) for x in [-16, 1]; tab = {hi, lo} pairs of exp(k/64)
__device__ __forceinline__ dfl df_exp(dfl x, const float2 *__restrict__ tab) {
  float kf = rintf(x.hi * 64.0f);
  kf = fminf(fmaxf(kf, (float)kDfExpLo), (float)kDfExpHi);
  dfl r = df_two_sum(x.hi - kf * 0.015625f, x.lo);  // the first difference is exact
  float rh = r.hi;
  float p = rh * rh * (0.5f + rh * (1.0f / 6.0f + rh * (1.0f / 24.0f)));  // r^2/2 + ..
  dfl e = df_add(df_two_sum(1.0f, rh), {r.lo + p, 0.0f});
  float2 t = tab[(int)kf - kDfExpLo];
  return df_mul(e, {t.x, t.y});
}

// erfc(z) with the reference's erfc fit (ewald.c:817-836, Numerical
// Recipes "erfcc") evaluated in double-float: same function as the oracle's
// FP64 evaluation to about 1e-13 relative.  z >= 0.
struct DfErfcCoef {
  float2 c[10];  // the fit's coefficients, constant term first, as hi / lo
};

// Constants of the double-float intramolecular correction energy.
struct DfIntra {
  DfErfcCoef C;
  float2 kappa, qf;  // kappa, QFACTOR (qa qb qf: kJ/mol A)
  float2 sl[3];      // L / 2^32 per axis
};

__device__ __forceinline__ dfl df_erfc_nr(dfl z, const DfErfcCoef &C,
                                          const float2 *__restrict__ tab) {
  dfl t = df_recip(df_add({1.0f, 0.0f}, df_mul_f(z, 0.5f)));
  dfl p = {C.c[9].x, C.c[9].y};
#pragma unroll
  for (int k = 8; k >= 0; k--) p = df_add(df_mul(p, t), {C.c[k].x, C.c[k].y});
  dfl arg = df_add(df_neg(df_mul(z, z)), p);
  return df_mul(t, df_exp(arg, tab));
}

}  // namespace fe
