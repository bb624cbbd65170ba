// Host check of the mixed form's powers with compile-time exponents
// (tempo_gb300/csrc/tempo_powers.h): each x**e the rain and graupel size distributions
// use with an integer or half-integer e, formed by products, a square root and a
// division in FP32 (IEEE-rounded on the host as on the device), against long double
// pow on seeded random arguments over the range the step feeds it (the slopes that the
// size checks allow; there no power leaves the normal FP32 range).  Prints one line per
// exponent: the exponent, samples, and the maximum relative error in units of 2^-24.
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "tempo_powers.h"

using LD = long double;

static uint64_t g_state = 0x2545f4914f6cdd1dull;
static double uniform() {  // splitmix64 -> [0, 1)
  uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53;
}

template <double const* E, int K, int S>
static void check(const char* name, double lo, double hi) {
  constexpr int tw = tg::FixedExp<E, K, S>::tw;
  const LD e = (LD)tw / 2;
  LD worst = 0;
  const int n = 200000;
  for (int i = 0; i < n; i++) {
    // log-uniform in [lo, hi]: slopes and diameters span decades
    const float x = (float)(lo * std::pow(hi / lo, uniform()));
    const LD want = std::pow((LD)x, e);
    const LD got = (LD)tg::pow_twice<tw>(x);
    const LD rel = std::fabs((got - want) / want);
    if (rel > worst) worst = rel;
  }
  std::printf("%s %.1Lf %d %.3Lf\n", name, e, n, worst / std::ldexp((LD)1.0, -24));
}

int main() {
  using tg::kCge;
  using tg::kCre;
  // rain: the size checks keep the median volume diameter within [0.75 d0r, d0r_max]
  // = [37.5 um, 2.5 mm], so the slope lamr = 3.672 / D lies in [1.5e3, 9.8e4] m^-1
  // (ilamr its inverse; lamr + fv_r and lamr + fv_r / 2 slightly above)
  check<kCre, 0, 1>("cre0", 1.4e3, 1.0e5);
  check<kCre, 1, 1>("cre1", 1.4e3, 1.0e5);
  check<kCre, 2, 1>("cre2", 1.4e3, 1.0e5);
  check<kCre, 3, 1>("cre3", 1.0e-5, 7.0e-4);
  check<kCre, 5, -1>("cre5n", 1.6e3, 1.0e5);
  check<kCre, 6, -1>("cre6n", 1.6e3, 1.0e5);
  check<kCre, 7, -1>("cre7n", 1.6e3, 1.0e5);
  check<kCre, 8, -1>("cre8n", 1.6e3, 1.0e5);
  check<kCre, 9, 1>("cre9", 1.0e-5, 7.0e-4);
  check<kCre, 10, -1>("cre10n", 1.5e3, 1.0e5);
  check<kCre, 11, 1>("cre11", 1.4e3, 1.0e5);
  // graupel: median volume diameter within [d0r, 25.4 mm], slope lamg in [1.4e2, 7.4e4]
  check<kCge, 0, 1>("cge0", 1.4e2, 7.5e4);
  check<kCge, 1, 1>("cge1", 1.4e2, 7.5e4);
  check<kCge, 3, 1>("cge3", 1.3e-5, 7.0e-3);
  check<kCge, 9, 1>("cge9", 1.3e-5, 7.0e-3);
  return 0;
}
