// tempo_powers.h -- powers with the compile-time exponents of the rain and graupel
// size distributions, for the mixed form's FP32 bulk (host and device: the host check
// tests/power_check.cpp runs the same arithmetic).
#pragma once

#include <cmath>

#include "tempo_consts.h"

namespace tg {

// Exponents of the rain and graupel size distributions that the host puts in cre and
// cge (params:511-523, 558-571), as constants: with the scheme's mu_r = mu_g = 0,
// bm = 3 and bv_r = 1 all of cre and the entries of cge that do not involve the graupel
// fall-speed exponent are integers or half-integers (negative entries: depends on
// bv_g).
constexpr double kCre[13] = {bm_r + 1.0, mu_r + 1.0, bm_r + mu_r + 1.0, bm_r * 2.0 + mu_r + 1.0,
                             mu_r + bv_r + 1.0, bm_r + mu_r + bv_r + 1.0,
                             bm_r * 0.5 + mu_r + bv_r + 1.0, bm_r + mu_r + bv_r + 3.0,
                             mu_r + bv_r + 3.0, mu_r + 2.0, 0.5 * (bv_r + 5.0 + 2.0 * mu_r),
                             bm_r * 0.5 + mu_r + 1.0, bm_r * 2.0 + mu_r + bv_r + 1.0};
constexpr double kCge[12] = {bm_g + 1.0, mu_g + 1.0, bm_g + mu_g + 1.0, bm_g * 2.0 + mu_g + 1.0,
                             -1.0, -1.0, -1.0, -1.0, -1.0, mu_g + 2.0, -1.0,
                             bm_g * 0.5 + mu_g + 1.0};
// x**N and x**(TW/2) for compile-time N and TW: binary powering, one square root for a
// half-integer, one division for a negative exponent; at most 5.5 units of 2^-24 over the
// slopes the size checks allow (tests/power_check.cpp)
template <int N> TG_HD inline float ipow_ct(float x) {
  if constexpr (N == 0) {
    return 1.0f;
  } else if constexpr (N == 1) {
    return x;
  } else {
    const float h = ipow_ct<N / 2>(x);
    if constexpr (N % 2) return h * h * x;
    else return h * h;
  }
}
template <int TW> TG_HD inline float pow_twice(float x) {
  constexpr int A = TW < 0 ? -TW : TW;
  float r = ipow_ct<A / 2>(x);
  if constexpr (A % 2 != 0) r = r * sqrtf(x);
  if constexpr (TW < 0) r = 1.0f / r;
  return r;
}
// the exponent S E[K] (S = +1 or -1) as twice an integer, checked at compile time
template <double const* E, int K, int S> struct FixedExp {
  static constexpr double e = S * E[K];
  static constexpr int tw = (int)(2.0 * e);
  static_assert(e * 2.0 == (double)tw && E[K] >= 0.0, "an integer or half-integer exponent");
};

}  // namespace tg
