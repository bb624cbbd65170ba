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
// as in the double-double arithmetic of Hida, Li and Bailey (QD library, 2001), and the
// addition and division algorithms of Joldes, Muller and Popescu ("Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2),
// 2017).  Relative error of * is a few units of 2^-48 (u^2, u = 2^-24), of / at most
// 15 u^2; the error of + and - is a few u^2 of the operands' magnitude.
#pragma once

#include <cuda_runtime.h>

namespace tg {

// 8-byte aligned, so that a value in a scratch plane moves with one 64-bit load or store
struct __align__(8) df {
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

// addition of two double-words: QD's sloppy_add (SloppyDWPlusDW of Joldes, Muller and
// Popescu), 11 FP32 operations against 20 for the cancellation-safe form.  Its absolute
// error is a few u^2 (|a| + |b|): relative to its operands, not to a result that
// cancels.  That is the accuracy the step needs -- a saturation difference qv - qvs,
// for example, is then exact to ~1e-17 kg/kg, far below any threshold the step
// compares it with, and the decision census and the precision study of the mixed
// form came out the same with either addition.
__host__ __device__ __forceinline__ df operator+(df a, df b) {
  float s, e;
  dfo::two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  dfo::fast_two_sum(s, e, s, e);
  return df(s, e);
}
// double-word plus float, DWPlusFP of the same paper: relative error at most 2 u^2
__host__ __device__ __forceinline__ df operator+(df a, float b) {
  float s, e;
  dfo::two_sum(a.hi, b, s, e);
  const float v = a.lo + e;
  dfo::fast_two_sum(s, v, s, e);
  return df(s, e);
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

// Division, DWDivDW2 of Joldes, Muller and Popescu (2017): one float quotient th, the
// remainder x - y th (y th as a double-word by DWTimesFP3; xh - rh is exact), one
// correction tl = remainder / yh.  Relative error at most 15 u^2 + 56 u^3.
__host__ __device__ __forceinline__ df operator/(df x, df y) {
  const float th = x.hi / y.hi;
  float rh, rl;
  dfo::two_prod(y.hi, th, rh, rl);
  rl = fmaf(y.lo, th, rl);
  dfo::fast_two_sum(rh, rl, rh, rl);
  const float ph = x.hi - rh;
  const float dl = x.lo - rl;
  const float tl = (ph + dl) / y.hi;
  float h, l;
  dfo::fast_two_sum(th, tl, h, l);
  return df(h, l);
}
// double-word by float, DWDivFP3 of the same paper: relative error at most 3 u^2
__host__ __device__ __forceinline__ df operator/(df x, float y) {
  const float th = x.hi / y;
  float ph, pl;
  dfo::two_prod(th, y, ph, pl);
  const float d = ((x.hi - ph) - pl) + x.lo;
  const float tl = d / y;
  float h, l;
  dfo::fast_two_sum(th, tl, h, l);
  return df(h, l);
}
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

// c + x s for one Horner step of a polynomial: the sum by the sloppy double-word
// addition (QD's sloppy_add; SloppyDWPlusDW of Joldes, Muller and Popescu), whose
// absolute error is a few u^2 (|c| + |x s|).  Horner's own error is of that form
// (u^2 times the sum of the terms' magnitudes) whatever the addition, so the accurate
// addition buys nothing here.
__host__ __device__ __forceinline__ df horner_step(df x, df s, double c) {
  const df p = x * s, a(c);
  float sh, sl;
  dfo::two_sum(a.hi, p.hi, sh, sl);
  const float w = sl + (a.lo + p.lo);
  float h, l;
  dfo::fast_two_sum(sh, w, h, l);
  return df(h, l);
}

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
