// tempo_dfloat.cuh -- double-float ("float-float") arithmetic for the precision islands
// of the mixed-precision step.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the quantities that
// the reference needs in FP64 -- temperature and vapour state, saturation mixing
// ratios and their differences (supersaturation, saturation adjustment), the
// sedimentation flux divergence and the precipitation sums -- are carried as an
// unevaluated sum hi + lo of two floats (about 48 significant bits) and computed on
// the FP32 pipes.  The algorithms are the classical error-free transformations:
// Knuth's TwoSum, Dekker's Fast2Sum, and the FMA form of Dekker's TwoProduct, combined
// as in the double-double arithmetic of Hida, Li and Bailey (QD library, 2001) with
// accurate (cancellation-safe) addition.  Relative error of + - * / is a few units
// of 2^-48.
#pragma once

#include <cuda_runtime.h>

namespace tg {

struct df {
  float hi, lo;
  df() = default;
  __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
  // exact for floats; for doubles the rounding error of hi goes to lo
  __host__ __device__ constexpr df(float x) : hi(x), lo(0.0f) {}
  __host__ __device__ constexpr df(double x)
      : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ constexpr df(int x) : hi((float)x), lo(0.0f) {}  // |x| < 2^24
  __host__ __device__ explicit constexpr operator float() const { return hi + lo; }
  __host__ __device__ explicit constexpr operator double() const { return (double)hi + (double)lo; }
};

namespace dfo {
// Knuth TwoSum: s + e == a + b exactly
__host__ __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// Dekker Fast2Sum, |a| >= |b|
__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// TwoProduct with one FMA: p + e == a * b exactly
__host__ __device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
}  // namespace dfo

__host__ __device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }

// accurate addition (QD's IEEE-style add): both halves summed with TwoSum, so a sum
// that cancels -- a saturation difference qv - qvs -- keeps its relative accuracy
__host__ __device__ __forceinline__ df operator+(df a, df b) {
  float s1, s2, t1, t2;
  dfo::two_sum(a.hi, b.hi, s1, s2);
  dfo::two_sum(a.lo, b.lo, t1, t2);
  s2 += t1;
  dfo::fast_two_sum(s1, s2, s1, s2);
  s2 += t2;
  dfo::fast_two_sum(s1, s2, s1, s2);
  return df(s1, s2);
}
__host__ __device__ __forceinline__ df operator+(df a, float b) {
  float s1, s2, t1, t2;
  dfo::two_sum(a.hi, b, s1, s2);
  dfo::two_sum(s2, a.lo, t1, t2);
  dfo::two_sum(s1, t1, s1, s2);
  s2 += t2;
  dfo::fast_two_sum(s1, s2, s1, s2);
  return df(s1, s2);
}
__host__ __device__ __forceinline__ df operator+(float a, df b) { return b + a; }
__host__ __device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__host__ __device__ __forceinline__ df operator-(df a, float b) { return a + (-b); }
__host__ __device__ __forceinline__ df operator-(float a, df b) { return (-b) + a; }

__host__ __device__ __forceinline__ df operator*(df a, df b) {
  float p, e;
  dfo::two_prod(a.hi, b.hi, p, e);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float h, l;
  dfo::fast_two_sum(p, e, h, l);
  return df(h, l);
}
__host__ __device__ __forceinline__ df operator*(df a, float b) {
  float p, e;
  dfo::two_prod(a.hi, b, p, e);
  e = fmaf(a.lo, b, e);
  float h, l;
  dfo::fast_two_sum(p, e, h, l);
  return df(h, l);
}
__host__ __device__ __forceinline__ df operator*(float a, df b) { return b * a; }

// long division with two correction steps (QD's accurate division)
__host__ __device__ __forceinline__ df operator/(df a, df b) {
  float q1 = a.hi / b.hi;
  df r = a - b * q1;
  float q2 = r.hi / b.hi;
  r = r - b * q2;
  float q3 = r.hi / b.hi;
  float h, l;
  dfo::fast_two_sum(q1, q2, h, l);
  return df(h, l) + q3;
}
__host__ __device__ __forceinline__ df operator/(df a, float b) { return a / df(b); }
__host__ __device__ __forceinline__ df operator/(float a, df b) { return df(a) / b; }

// double operands (constants): converted to df, never narrowed to float
__host__ __device__ __forceinline__ df operator+(df a, double b) { return a + df(b); }
__host__ __device__ __forceinline__ df operator+(double a, df b) { return df(a) + b; }
__host__ __device__ __forceinline__ df operator-(df a, double b) { return a - df(b); }
__host__ __device__ __forceinline__ df operator-(double a, df b) { return df(a) - b; }
__host__ __device__ __forceinline__ df operator*(df a, double b) { return a * df(b); }
__host__ __device__ __forceinline__ df operator*(double a, df b) { return df(a) * b; }
__host__ __device__ __forceinline__ df operator/(df a, double b) { return a / df(b); }
__host__ __device__ __forceinline__ df operator/(double a, df b) { return df(a) / b; }

__host__ __device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__host__ __device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }

// comparisons on the represented value (hi and lo are normalised: |lo| <= ulp(hi)/2)
__host__ __device__ __forceinline__ bool operator<(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__host__ __device__ __forceinline__ bool operator>(df a, df b) { return b < a; }
__host__ __device__ __forceinline__ bool operator<=(df a, df b) { return !(b < a); }
__host__ __device__ __forceinline__ bool operator>=(df a, df b) { return !(a < b); }
__host__ __device__ __forceinline__ bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
__host__ __device__ __forceinline__ bool operator!=(df a, df b) { return !(a == b); }

__host__ __device__ __forceinline__ bool operator<(df a, double b) { return a < df(b); }
__host__ __device__ __forceinline__ bool operator>(df a, double b) { return a > df(b); }
__host__ __device__ __forceinline__ bool operator<=(df a, double b) { return a <= df(b); }
__host__ __device__ __forceinline__ bool operator>=(df a, double b) { return a >= df(b); }
__host__ __device__ __forceinline__ bool operator<(double a, df b) { return df(a) < b; }
__host__ __device__ __forceinline__ bool operator>(double a, df b) { return df(a) > b; }

__host__ __device__ __forceinline__ df Fabs(df a) { return a.hi < 0.0f ? -a : a; }
__host__ __device__ __forceinline__ df Max(df a, df b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ df Min(df a, df b) { return a < b ? a : b; }

// square root: one Newton correction of the float root (QD's sqrt)
__host__ __device__ __forceinline__ df Sqrt(df a) {
  if (a.hi <= 0.0f) return df(0.0f);
  const float q = sqrtf(a.hi);
  df r = a - df(q) * df(q);
  float h, l;
  dfo::fast_two_sum(q, r.hi / (2.0f * q), h, l);
  return df(h, l);
}

// exp for |x| < 80: x = n ln2 + r with |r| <= ln2/2 (ln2 split in two floats so that
// n * ln2 is exact to ~2^-48), then r / 16, Taylor series to the 9th power, and four
// squarings; relative error below 1e-14 over the range used by the step.
__host__ __device__ __forceinline__ df Exp(df x) {
  const df ln2(0.6931471805599453);
  const float n = rintf(x.hi * 1.4426950408889634f);
  df r = x - ln2 * n;
  r = r * 0.0625f;
  // Horner: 1 + r (1 + r/2 (1 + r/3 (... (1 + r/9))))
  df s = df(1.0f) + r * (1.0f / 9.0f);
  s = df(1.0f) + r * s * df(1.0 / 8.0);
  s = df(1.0f) + r * s * df(1.0 / 7.0);
  s = df(1.0f) + r * s * df(1.0 / 6.0);
  s = df(1.0f) + r * s * df(1.0 / 5.0);
  s = df(1.0f) + r * s * df(1.0 / 4.0);
  s = df(1.0f) + r * s * df(1.0 / 3.0);
  s = df(1.0f) + r * s * 0.5f;
  s = df(1.0f) + r * s;
  s = s * s;
  s = s * s;
  s = s * s;
  s = s * s;
  const float sc = ldexpf(1.0f, (int)n);
  return df(s.hi * sc, s.lo * sc);
}

}  // namespace tg
