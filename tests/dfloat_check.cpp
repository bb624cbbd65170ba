// Host check of the double-float building blocks of the mixed-precision island
// (tempo_gb300/csrc/tempo_dfloat.cuh): division, division by a float, addition,
// addition of a float, multiplication and the Horner step of the saturation
// polynomials, each against long double arithmetic on seeded random operands.  Prints
// one line per operation: name, samples, maximum relative error in units of u^2
// (u = 2^-24); for the double-word addition the error in units of u^2 (|a| + |b|) (its
// bound, also where the sum cancels) and the relative error of same-sign sums; for the
// polynomials the error in units of u^2 times the sum of the terms' magnitudes
// (Horner's error scale).
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "tempo_dfloat.cuh"

using tg::df;
using LD = long double;

static uint64_t g_state = 0x9e3779b97f4a7c15ull;
static double uniform() {  // splitmix64 -> [0, 1)
  uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53;
}
// a value with a random sign, mantissa and decimal exponent in [lo, hi]
static double random_value(double lo, double hi) {
  const double m = 1.0 + 9.0 * uniform();
  const double e = std::floor(lo + (hi - lo + 1.0) * uniform());
  return (uniform() < 0.5 ? -1.0 : 1.0) * m * std::pow(10.0, e);
}
static LD exact(df a) { return (LD)a.hi + (LD)a.lo; }
static const LD kU2 = std::ldexp((LD)1.0, -48);

static LD rel(LD got, LD want) { return want == 0 ? std::fabs(got) : std::fabs((got - want) / want); }

int main() {
  const int n = 200000;
  LD e_div = 0, e_divf = 0, e_add = 0, e_add_same = 0, e_addf = 0, e_mul = 0;
  for (int i = 0; i < n; i++) {
    const df a(random_value(-12, 6)), b(random_value(-12, 6));
    const float f = (float)random_value(-12, 6);
    LD q = rel(exact(a / b), exact(a) / exact(b));
    if (q > e_div) e_div = q;
    q = rel(exact(a / f), exact(a) / (LD)f);
    if (q > e_divf) e_divf = q;
    q = rel(exact(a * b), exact(a) * exact(b));
    if (q > e_mul) e_mul = q;
    // sums of nearly equal values (the saturation differences) and of unrelated ones
    const df c = (i % 2) ? df(-(double)exact(a) * (1.0 + 1e-6 * uniform())) : b;
    q = std::fabs(exact(a + c) - (exact(a) + exact(c))) / (std::fabs(exact(a)) + std::fabs(exact(c)));
    if (q > e_add) e_add = q;
    const df bs = (exact(a) < 0) == (exact(b) < 0) ? b : -b;
    q = rel(exact(a + bs), exact(a) + exact(bs));
    if (q > e_add_same) e_add_same = q;
    const float g = (i % 2) ? -(float)exact(a) * (float)(1.0 + 1e-3 * uniform()) : f;
    q = rel(exact(a + g), exact(a) + (LD)g);
    if (q > e_addf) e_addf = q;
  }
  std::printf("div %d %.3Lf\n", n, e_div / kU2);
  std::printf("div_float %d %.3Lf\n", n, e_divf / kU2);
  std::printf("mul %d %.3Lf\n", n, e_mul / kU2);
  std::printf("add %d %.3Lf\n", n, e_add / kU2);
  std::printf("add_same_sign %d %.3Lf\n", n, e_add_same / kU2);
  std::printf("add_float %d %.3Lf\n", n, e_addf / kU2);

  // the liquid and ice saturation polynomials (src/module_mp_tempo_utils.F90:285-331)
  static const double cl[9] = {.611583699E03, .444606896E02, .143177157e01, .264224321e-1,
                               .299291081e-3, .203154182e-5, .702620698e-8, .379534310e-11,
                               -.321582393e-13};
  static const double ci[9] = {.609868993e03, .499320233e02, .184672631e01, .402737184e-1,
                               .565392987e-3, .521693933e-5, .307839583e-7, .105785160e-9,
                               .161444444e-12};
  const double* polys[2] = {cl, ci};
  const char* names[2] = {"poly_liquid", "poly_ice"};
  for (int p = 0; p < 2; p++) {
    const double* c = polys[p];
    LD worst_scaled = 0, worst_rel_warm = 0;
    const int m = 100000;
    for (int i = 0; i < m; i++) {
      const df t = df(193.16 + 140.0 * uniform()) + df((float)(1e-4 * (uniform() - 0.5)));
      const df x = t - 273.16;
      df s = df(c[8]);
      for (int k = 7; k >= 0; k--) s = tg::horner_step(x, s, c[k]);
      const LD X = exact(x);
      LD want = c[8], mag = std::fabs((LD)c[8]);
      for (int k = 7; k >= 0; k--) {
        want = (LD)c[k] + X * want;
        mag = std::fabs((LD)c[k]) + std::fabs(X) * mag;
      }
      const LD err = std::fabs(exact(s) - want);
      if (err / mag > worst_scaled) worst_scaled = err / mag;
      if (X > -20 && rel(exact(s), want) > worst_rel_warm) worst_rel_warm = rel(exact(s), want);
    }
    std::printf("%s %d %.3Lf %.3Lf\n", names[p], m, worst_scaled / kU2, worst_rel_warm / kU2);
  }
  return 0;
}
